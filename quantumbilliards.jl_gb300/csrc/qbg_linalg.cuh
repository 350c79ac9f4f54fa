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
  // Triangular solves in blocks of nbs = nb * 2^levels rows (levels 0..2):
  // inverses of the nbs x nbs diagonal blocks, built from the nb x nb ones by
  // doubling after the factorisation; the solve ping-pongs between X and Y.
  int levels = 0, nbs = 0, nblks = 0;
  cx<T>* Linv_mid = nullptr;  // batch * ceil(n / 2nb) * (2nb)^2 (levels == 2)
  cx<T>* Uinv_mid = nullptr;
  cx<T>* Linv2 = nullptr;     // batch * nblks * nbs^2
  cx<T>* Uinv2 = nullptr;
  cx<T>* W = nullptr;         // doubling scratch: batch * ceil(nblk / 2) * (nbs / 2)^2
  cx<T>* Y = nullptr;         // solve scratch: batch * n * ymax_L
  int ymax_L = 0;
  // optional extra streams (owned by the caller): with nsplit > 1, lu_factor
  // and lu_solve_shared run nsplit contiguous parts of the batch concurrently,
  // the first on the calling stream and part i on stx[i - 1], forked from and
  // joined back into the calling stream with these two events
  static constexpr int MAX_SPLIT = 8;
  int nsplit = 1;
  cudaStream_t stx[MAX_SPLIT - 1] = {};
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
};

// Sets levels/nbs/nblks and returns the device bytes the solve blocks need.
template <class T>
size_t lu_solve_blocks_bytes(LUBatch<T>& f, int levels, int ymax_L);
// Points the solve-block buffers into one device allocation of that size.
template <class T>
void lu_solve_blocks_bind(LUBatch<T>& f, void* mem);

template <class T>
int lu_factor(LUBatch<T>& f, cudaStream_t st);

// X[b] = A_b^{-1} P_b ... solve with V shared by the batch (ldv = n).
// V: n x L (cx<T>), X: batch * n * L (cx<T>), column-major, ld = n.
template <class T>
int lu_solve_shared(const LUBatch<T>& f, const cx<T>* V, int L, cx<T>* X, long long strideV, cudaStream_t st);

// A_b^{-1} of every matrix (X: batch * n * n, column-major). levels == 0.
template <class T>
int lu_inverse(const LUBatch<T>& f, cx<T>* X, cudaStream_t st);

// X_b = A_b^{-H} V_b (V_b = V + b strideV, n x L; X, Y: batch * n * L; Y is
// scratch). levels == 0.
template <class T>
int lu_solve_adjoint(const LUBatch<T>& f, const cx<T>* V, long long strideV, int L, cx<T>* X, cx<T>* Y,
                     cudaStream_t st);

// Batched complex GEMM: C = alpha A B + beta C.
template <class T>
int gemm_batched(int M, int N, int K, cx<T> alpha, const cx<T>* A, long long lda, long long sA, const cx<T>* B,
                 long long ldb, long long sB, cx<T> beta, cx<T>* C, long long ldc, long long sC, int batch,
                 cudaStream_t st);

// C = alpha A^H B + beta C with A^H the conjugate transpose of the K x M
// blocks stored at A (CUDA-core tiles).
template <class T>
int gemm_batched_ah(int M, int N, int K, cx<T> alpha, const cx<T>* A, long long lda, long long sA, const cx<T>* B,
                    long long ldb, long long sB, cx<T> beta, cx<T>* C, long long ldc, long long sC, int batch,
                    cudaStream_t st);

// The CUDA-core (FMA) tile GEMM, whatever the engine setting.
template <class T>
int gemm_batched_simt(int M, int N, int K, cx<T> alpha, const cx<T>* A, long long lda, long long sA, const cx<T>* B,
                      long long ldb, long long sB, cx<T> beta, cx<T>* C, long long ldc, long long sC, int batch,
                      cudaStream_t st);

// A0 = sum_b w_b X_b, A1 = sum_b w_b z_b X_b  (outputs complex128, n x L)
template <class T>
int moments(const cx<T>* X, long long sX, int batch, int n, int L, const cxd* w, const cxd* z, cxd* A0, cxd* A1,
            int accumulate, cudaStream_t st);

// Mixed-form refinement pieces.
// R_b = V_b - (T_b + Tlo_b) X_b computed with compensated FP32 products
// (double-float) flushed to FP64 every 256 terms; T_b, Tlo_b complex64 (Tlo
// may be null), X_b, V_b = V + b sV complex128 (sV = 0: one V for all). rmax
// receives max |R| (|re|+|im|), must be zeroed.
int residual_df32(const cxf* Tm, const cxf* Tlo, long long sT, const cxd* X, long long sX, const cxd* V,
                  long long sV, cxd* R, long long sR, int n, int L, int batch, double* rmax, cudaStream_t st);
int convert_d2f(const cxd* in, cxf* out, long long count, cudaStream_t st);
// out[b] = opnorm(A_b, 1) (out zeroed before the call)
int opnorm1_batched(const cxd* A, int n, long long sA, int batch, double* out, cudaStream_t st);
// out[4 b + q] = ||y_b||_2^2, ||y_b||_1, ||phi_b||_1, ||phi_b||_2^2 for n x batch column blocks
int vec_norms(const cxd* y, const cxd* phi, int n, int batch, double* out, cudaStream_t st);
// out = max(out, max_e |re x_e| + |im x_e|); out must be zeroed (or hold a
// previous maximum) before the first call
int maxabs_c64(const cxf* x, long long count, double* out, cudaStream_t st);
int broadcast_f(const cxf* in, long long count, int batch, cxf* out, cudaStream_t st);  // out[b] = in
int axpy_f2d(const cxf* d, cxd* x, long long count, cudaStream_t st);  // x += d

// Complex64 GEMM on the tcgen05 tensor cores (3xTF32 split, FP32-class
// accuracy); same argument meaning as gemm_batched. K must be positive.
// batch2 > 1 adds an inner batch index (strides sA2, sB2, sC2): matrix
// (outer o, inner q) starts at A + o sA + q sA2, and so on.
int tc_gemm_c64(int M, int N, int K, cxf alpha, const cxf* A, long long lda, long long sA, const cxf* B,
                long long ldb, long long sB, cxf beta, cxf* C, long long ldc, long long sC, int batch,
                cudaStream_t st, int batch2 = 1, long long sA2 = 0, long long sB2 = 0, long long sC2 = 0, bool allow_packed = true);
// Reads the tensor-core GEMM's device error flag (set, and kept set, once an
// mbarrier wait gave up); synchronizes the stream. Returns QBG_OK or QBG_ECUDA.
int tc_check(cudaStream_t st);
// pipeline-wait poll limit of the tensor-core GEMM (< 0: the built-in limit)
// and reset of its sticky error flag, on the current device (both synchronize
// the device first)
int tc_set_wait_limit(long long polls);
int tc_clear_error();
// returns the tensor-core GEMM's packing scratch of stream st to the pool
// (call before destroying a stream that ran library GEMMs)
void tc_release_scratch(cudaStream_t st);

// Refinement residual on the tensor cores (exact 7-bit digit products, see
// qbg_tc_resid.cu). The digit planes of the operators T = hi + lo are built
// once per factorisation; each residual splits X and forms R = V - T X.
struct TcResidT {
  int n = 0, batch = 0, MT = 0, KS = 0;  // 128-row tiles, 16-real-k stages
  void* TD = nullptr;   // bf16 digit planes, laid out as the kernel's stage images
  int* erow = nullptr;  // row exponents
};
size_t tc_resid_T_bytes(int n, int batch);
int tc_resid_bind_T(TcResidT& t, int n, int batch, void* mem, cudaStream_t st);  // zeroes mem
int tc_resid_prepare_T(TcResidT& t, const cxf* Th, const cxf* Tl, long long sT, int c, cudaStream_t st);
size_t tc_resid_X_bytes(int n, int L, int batch);  // scratch per residual call (zeroed once by the caller)
// ndig: 7 (the full digit product, ~2^-47 of the row and column scales) or 6
// (the leading six digits of T and X, ~2^-40: for a sweep that is not the last)
int tc_residual(const TcResidT& t, const cxd* X, long long sX, const cxd* V, long long sV, cxd* R, long long sR,
                int L, int c, double* rmax, void* xmem, cudaStream_t st, int ndig = 7);
// C_b -= A_b B_b in complex128 from eight-digit products on the tensor cores
// (qbg_tc_resid.cu); scratch from the pool, stream-ordered
int tc_gemm_sub_f64(int M, int N, int K, const cxd* A, long long lda, long long sA, const cxd* B, long long ldb,
                    long long sB, cxd* C, long long ldc, long long sC, int batch, cudaStream_t st);
// device address of the tensor-core error flag (shared by the GEMM and the residual)
int tc_error_ptr(int** p);

// Engine of the complex64 GEMMs inside gemm_batched<float> (LU trailing
// updates, triangular-solve updates, refinement products): 0 = CUDA-core FMA
// tiles, 1 = tcgen05 tensor cores. Process-wide.
constexpr int GEMM_ENGINE_SIMT = 0;
constexpr int GEMM_ENGINE_TCGEN05 = 1;
constexpr int GEMM_ENGINE_TCGEN05_STAGED = 2;  // tcgen05 with register-staged operands only
void set_gemm_engine(int e);
int gemm_engine();
// Plan of lu_factor, process-wide: panels per outer block (1..16; <= 0 keeps
// the current value), the panel form (< 0 automatic: a cluster of CTAs per
// complex64 panel for batches of at most 4 matrices; 0 one CTA; 1 a cluster)
// and the stream parts of a Beyn operator batch (1..MAX_SPLIT; <= 0 keeps).
void set_lu_plan(int outer, int cluster, int parts);
void get_lu_plan(int* outer, int* cluster, int* parts);

}  // namespace qbg
