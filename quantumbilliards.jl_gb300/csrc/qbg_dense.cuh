// FP64 dense building blocks on the library's own kernels (qbg_dense.cu):
// batched LU and inverses, the smallest singular value by a device-resident
// subspace iteration on the inverse, and the deflated shift of the Newton
// refinement.
#pragma once
#include <vector>

#include "qbg_handles.cuh"
#include "qbg_linalg.cuh"

namespace qbg {

constexpr int DENSE_P = 8;  // block size of the sigma_min subspace iteration

// A batch of n x n FP64 LU factorisations (pivots in LAPACK order), buffers
// from the library's allocator; f.A holds the matrices (factored in place).
struct Dense64 {
  LUBatch<double> f;
  int n = 0, batch = 0;
  cudaStream_t st = nullptr;
  std::vector<void*> mem;
  template <class P>
  int alloc(P** p, size_t bytes) {
    int s = dmalloc(p, bytes);
    if (!s) mem.push_back(*p);
    return s;
  }
  int create(int n, int batch, cudaStream_t st);
  // as create, with the matrices in caller-owned memory (batch * n * n at A)
  int bind(cxd* A, int n, int batch, cudaStream_t st);
  void release();
  cxd* A(int b) const { return f.A + (size_t)b * f.stride; }
  // factors every matrix; info_host (optional) receives LAPACK's info per
  // matrix (k > 0: U(k, k) == 0), which synchronizes the stream
  int factor(std::vector<int>* info_host = nullptr);
  int inverse(cxd* X) { return lu_inverse<double>(f, X, st); }
  ~Dense64();
};

// sigma_min of every A_b from Cinv_b = A_b^{-1} (see qbg_dense.cu); work:
// batch * 3 * n * DENSE_P elements; vec (optional): n per matrix.
int sigma_iterate(const cxd* Cinv, int n, int batch, const cxd* X0, cxd* work, int maxit, double tol, double* sig,
                  int* iters, cxd* vec, cudaStream_t st);
// the fixed n x DENSE_P start block of the iteration (host)
void dense_start_block(int n, std::vector<cxd>& hx);
// orthonormal columns of Q (n x p, column-major) in place on the device:
// modified Gram-Schmidt applied twice, vanishing columns refilled
int orth_columns(cxd* Q, int n, int p, cudaStream_t st);
// M = G - lam I + mu x x^H
int deflate_shift(const cxd* G, const cxd* x, int n, double lam, double mu, cxd* M, cudaStream_t st);

}  // namespace qbg
