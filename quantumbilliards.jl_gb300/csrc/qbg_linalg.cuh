// Batched dense complex linear algebra for the Beyn contour step
// (beyn.jl:270-285: lu! of every T(z_j), ldiv! with the probe block V, and the
// A0/A1 moment sums).
#pragma once
#include "qbg_common.cuh"

namespace qbg {

// Factorisation workspace for a batch of n x n column-major matrices.
template <class T>
struct LUBatch {
  int n = 0, batch = 0, nb = 0, nblk = 0;
  cx<T>* A = nullptr;       // batch * n * n (factored in place)
  long long stride = 0;     // elements between matrices
  int* ipiv = nullptr;      // batch * n (0-based global row indices, LAPACK order)
  int* perm = nullptr;      // batch * n row permutation (P V gather)
  int* info = nullptr;      // batch
  cx<T>* Linv = nullptr;    // batch * nblk * nb * nb
  cx<T>* Uinv = nullptr;    // batch * nblk * nb * nb
};

template <class T>
int lu_factor(LUBatch<T>& f, cudaStream_t st);

// X[b] = A_b^{-1} P_b ... solve with V shared by the batch (ldv = n).
// V: n x L (cx<T>), X: batch * n * L (cx<T>), column-major, ld = n.
template <class T>
int lu_solve_shared(const LUBatch<T>& f, const cx<T>* V, int L, cx<T>* X, long long strideV, cudaStream_t st);

// Batched complex GEMM: C = alpha A B + beta C.
template <class T>
int gemm_batched(int M, int N, int K, cx<T> alpha, const cx<T>* A, long long lda, long long sA, const cx<T>* B,
                 long long ldb, long long sB, cx<T> beta, cx<T>* C, long long ldc, long long sC, int batch,
                 cudaStream_t st);

// A0 = sum_b w_b X_b, A1 = sum_b w_b z_b X_b  (outputs complex128, n x L)
template <class T>
int moments(const cx<T>* X, long long sX, int batch, int n, int L, const cxd* w, const cxd* z, cxd* A0, cxd* A1,
            int accumulate, cudaStream_t st);

// Mixed-form refinement pieces.
// R_b = V - (T_b + Tlo_b) X_b computed with compensated FP32 products
// (double-float) flushed to FP64 every 32 terms; T_b, Tlo_b complex64 (Tlo may
// be null), X_b complex128. rmax receives max |R| (|re|+|im|), must be zeroed.
int residual_df32(const cxf* Tm, const cxf* Tlo, long long sT, const cxd* X, long long sX, const cxd* V, cxd* R,
                  long long sR, int n, int L, int batch, double* rmax, cudaStream_t st);
int convert_d2f(const cxd* in, cxf* out, long long count, cudaStream_t st);
int broadcast_f(const cxf* in, long long count, int batch, cxf* out, cudaStream_t st);  // out[b] = in
int axpy_f2d(const cxf* d, cxd* x, long long count, cudaStream_t st);  // x += d

}  // namespace qbg
