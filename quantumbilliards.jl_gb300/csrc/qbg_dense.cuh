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
// One-matrix steps of the iteration for callers that run its products as
// split-k GEMMs over the whole GPU. state (device, 2 + 2 DENSE_P doubles):
// [est, done, z]; est starts negative. rr_step: G = W^H W, top eigenpair,
// est = 1/sqrt(lambda_max), done when est changed by <= tol relative; orth8:
// orthonormal columns of the n x DENSE_P block Y; topvec: x = W z / |W z|.
int rr_step(const cxd* W, int n, double tol, double* state, cudaStream_t st);
int orth8(cxd* Y, int n, int salt, cudaStream_t st);
int topvec(const cxd* W, const double* state, int n, cxd* x, cudaStream_t st);
// Y = A B for n x n A and n x q B (FP64), split over k to fill the GPU
// (qbg_ebim.cu); P: scratch of gemm_tall_scratch(n, q) elements
size_t gemm_tall_scratch(int n, int q);
int gemm_tall(const cxd* A, const cxd* B, cxd* Y, int n, int q, cxd* P, cudaStream_t st);
int conj_transpose(const cxd* A, cxd* AH, int n, cudaStream_t st);
// sigma_min (and, when x_out is given, the unit right singular vector) of one
// operator from its inverse Cinv, the products as split-k GEMMs over the whole
// GPU; CH: n x n scratch; X, W, Y: n x DENSE_P; P: gemm_tall_scratch(n,
// DENSE_P); state: 2 + 2 DENSE_P doubles; synchronizes st every 8 steps.
int sigma_single(const cxd* Cinv, cxd* CH, int n, const cxd* X0, cxd* X, cxd* W, cxd* Y, cxd* P, double* state,
                 int maxit, double tol, double* sig, cxd* x_out, cudaStream_t st);
// M = G - lam I + mu x x^H
int deflate_shift(const cxd* G, const cxd* x, int n, double lam, double mu, cxd* M, cudaStream_t st);

}  // namespace qbg
