// FP64 dense building blocks on the library's own kernels: batched LU
// (k_getrf_panel_smem + k_gemm, qbg_linalg.cu), explicit inverses, and the
// smallest singular value of A(k) by subspace iteration on A(k)^{-1}, one CTA
// per matrix with the whole iteration (products, Rayleigh-Ritz, Gram-Schmidt)
// on the device.
//
// sigma_min (the reference: svdvals(A)[end], macros.jl:159-161): with
// C = A^{-1} = V S^{-1} U^H, sigma_min(A) = 1 / sigma_max(C). A block X of
// DENSE_P orthonormal columns is iterated X <- orth(C^H C X); after W = C X,
// the Rayleigh-Ritz value lambda_max(W^H W) approaches sigma_max(C)^2 from
// below, and W z (z the top Ritz vector) approaches v_min / sigma_min, the
// right singular vector of A. Convergence per step goes like
// (sigma_1 / sigma_{DENSE_P + 1})^2 of A; the iteration stops when
// 1 / sqrt(lambda_max) changes by less than tol relative.
#include <algorithm>
#include <cmath>
#include <vector>

#include "qbg_dense.cuh"

namespace qbg {

namespace {

constexpr int SP = DENSE_P;
constexpr int KC = 128;  // rows of X staged per chunk of the product C X

// every thread receives the block total of v[0..NV) (256 threads)
template <int NV>
__device__ __forceinline__ void block_sum(double (&v)[NV], double* sh) {
#pragma unroll
  for (int i = 0; i < NV; ++i)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v[i] += __shfl_xor_sync(0xffffffffu, v[i], o);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0)
#pragma unroll
    for (int i = 0; i < NV; ++i) sh[wid * NV + i] = v[i];
  __syncthreads();
#pragma unroll
  for (int i = 0; i < NV; ++i) {
    double t = 0.0;
#pragma unroll
    for (int w = 0; w < 8; ++w) t += sh[w * NV + i];
    v[i] = t;
  }
}

// deterministic fill value in [-1, 1) for (row, column, salt)
__device__ __forceinline__ double fillv(int r, int c, int salt) {
  unsigned long long x = 0x9E3779B97F4A7C15ull * (unsigned long long)(r + 1) + 0xBF58476D1CE4E5B9ull * (c + 7) +
                         0x94D049BB133111EBull * (salt + 3);
  x ^= x >> 31;
  x *= 0xD6E8FEB86659FD93ull;
  x ^= x >> 29;
  return (double)(x >> 11) * (2.0 / 9007199254740992.0) - 1.0;
}

// orthonormal columns of Q (n x SP, column-major) in place: classical
// Gram-Schmidt applied twice per column; a column that vanishes against the
// earlier ones (below 1e-14 of its length) is refilled and orthogonalised again
__device__ void orth_cgs2(cxd* Q, int n, double* sh, int salt) {
  const int tid = threadIdx.x;
  for (int j = 0; j < SP; ++j) {
    cxd* qj = Q + (size_t)j * n;
    for (int attempt = 0; attempt < 3; ++attempt) {
      double v0[1] = {0.0};
      for (int r = tid; r < n; r += 256) v0[0] += cabs2(qj[r]);
      block_sum<1>(v0, sh);
      const double n0 = sqrt(v0[0]);
      for (int pass = 0; pass < 2 && j > 0; ++pass) {
        double c[2 * SP];
#pragma unroll
        for (int i = 0; i < 2 * SP; ++i) c[i] = 0.0;
        for (int r = tid; r < n; r += 256) {
          const cxd y = qj[r];
#pragma unroll
          for (int i = 0; i < SP; ++i)
            if (i < j) {
              const cxd qi = Q[(size_t)i * n + r];
              c[2 * i] += qi.re * y.re + qi.im * y.im;  // conj(qi) y
              c[2 * i + 1] += qi.re * y.im - qi.im * y.re;
            }
        }
        block_sum<2 * SP>(c, sh);
        for (int r = tid; r < n; r += 256) {
          cxd y = qj[r];
#pragma unroll
          for (int i = 0; i < SP; ++i)
            if (i < j) cfms(y, Q[(size_t)i * n + r], cxd(c[2 * i], c[2 * i + 1]));
          qj[r] = y;
        }
      }
      double v1[1] = {0.0};
      for (int r = tid; r < n; r += 256) v1[0] += cabs2(qj[r]);
      block_sum<1>(v1, sh);
      const double n1 = sqrt(v1[0]);
      if (n1 > 1e-14 * n0 && n1 > 1e-300 && isfinite(n1)) {
        const double s = 1.0 / n1;
        for (int r = tid; r < n; r += 256) qj[r] = qj[r] * s;
        break;
      }
      for (int r = tid; r < n; r += 256) qj[r] = cxd(fillv(r, j, salt + attempt), fillv(r, j + SP, salt + attempt));
      __syncthreads();
    }
  }
  __syncthreads();
}

// largest eigenvalue and its eigenvector of the Hermitian SP x SP matrix G
// (column-major, complex, exactly Hermitian) by cyclic Jacobi on its real
// 2SP x 2SP embedding [[Re G, -Im G], [Im G, Re G]], run by one whole warp on
// the shared scratch wk (2 (2SP)^2 doubles): for each rotation every lane
// derives the same (c, s) from the pivot entries, then lane k < 2SP rotates
// column k's pair (p, q) and row k's pair of the matrix, lanes 2SP.. the
// eigenvector columns. Lane 0 writes lam and z (SP complex). A one-thread
// version on thread-local 16 x 16 arrays lost the symmetry of the matrix
// after its first sweep when built with device optimisation for sm_103a
// (correct at -G and on the host), hence the shared-memory form.
__device__ void herm_top(const double* G, double* lam, double* z, double* wk) {
  constexpr int M2 = 2 * SP;
  const int lane = threadIdx.x & 31;
  double* a = wk;
  double* v = wk + M2 * M2;
  for (int e = lane; e < M2 * M2; e += 32) {
    const int r = e / M2, c = e % M2, gr = r % SP, gc = c % SP;
    const double re = G[2 * (gc * SP + gr)], im = G[2 * (gc * SP + gr) + 1];
    a[e] = (r < SP) == (c < SP) ? re : (r >= SP ? im : -im);
    v[e] = r == c ? 1.0 : 0.0;
  }
  __syncwarp();
  for (int sweep = 0; sweep < 40; ++sweep) {
    double off = 0.0, dia = 0.0;
    for (int e = lane; e < M2 * M2; e += 32) {
      const double t = a[e] * a[e];
      if (e / M2 == e % M2)
        dia += t;
      else
        off += t;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      off += __shfl_xor_sync(0xffffffffu, off, o);
      dia += __shfl_xor_sync(0xffffffffu, dia, o);
    }
    // lane 0's sums decide for the whole warp (the butterfly may round per lane).
    // Converged at an off-diagonal norm of 1e-15 of the diagonal's: rounding
    // keeps every rotated pair at ~eps of its entries, so a tighter stop is
    // never met and the sweeps would run to their limit.
    off = __shfl_sync(0xffffffffu, off, 0);
    dia = __shfl_sync(0xffffffffu, dia, 0);
    if (!(off > 1e-30 * dia)) break;
    for (int p = 0; p < M2 - 1; ++p)
      for (int q = p + 1; q < M2; ++q) {
        const double apq = a[p * M2 + q];
        // an entry at rounding level of its diagonal pair needs no rotation
        if (fabs(apq) < 1e-300 || fabs(apq) <= 1e-17 * sqrt(fabs(a[p * M2 + p] * a[q * M2 + q]))) continue;
        const double th = (a[q * M2 + q] - a[p * M2 + p]) / (2.0 * apq);
        const double t = (th >= 0.0 ? 1.0 : -1.0) / (fabs(th) + sqrt(th * th + 1.0));
        const double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
        __syncwarp();
        if (lane < M2) {
          const double akp = a[lane * M2 + p], akq = a[lane * M2 + q];
          a[lane * M2 + p] = c * akp - s * akq;
          a[lane * M2 + q] = s * akp + c * akq;
        } else {
          const int k = lane - M2;
          const double vkp = v[k * M2 + p], vkq = v[k * M2 + q];
          v[k * M2 + p] = c * vkp - s * vkq;
          v[k * M2 + q] = s * vkp + c * vkq;
        }
        __syncwarp();
        if (lane < M2) {
          const double apk = a[p * M2 + lane], aqk = a[q * M2 + lane];
          a[p * M2 + lane] = c * apk - s * aqk;
          a[q * M2 + lane] = s * apk + c * aqk;
        }
        __syncwarp();
      }
  }
  if (lane == 0) {
    int best = 0;
    for (int i = 1; i < M2; ++i)
      if (a[i * M2 + i] > a[best * M2 + best]) best = i;
    *lam = a[best * M2 + best];
    double nrm = 0.0;
    for (int i = 0; i < SP; ++i) {
      z[2 * i] = v[i * M2 + best];
      z[2 * i + 1] = v[(i + SP) * M2 + best];
      nrm += z[2 * i] * z[2 * i] + z[2 * i + 1] * z[2 * i + 1];
    }
    nrm = nrm > 0.0 ? 1.0 / sqrt(nrm) : 0.0;
    for (int i = 0; i < 2 * SP; ++i) z[i] *= nrm;
  }
  __syncwarp();
}

// One CTA per matrix: the subspace iteration on C_b = A_b^{-1} (n x n,
// column-major, stride n^2). X0: the shared n x SP start block; work: per
// matrix 3 n SP elements. sig[b] = sigma_min(A_b); iters[b] = steps taken;
// vec (optional): the unit right singular vector of A_b (n per matrix).
__global__ void __launch_bounds__(256) k_sigma_iter(const cxd* __restrict__ Cb, int n, const cxd* __restrict__ X0,
                                                    cxd* work, int maxit, double tol, double* sig, int* iters,
                                                    cxd* vec) {
  const int b = blockIdx.x, tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const cxd* C = Cb + (size_t)b * n * n;
  cxd* X = work + (size_t)b * 3 * n * SP;
  cxd* W = X + (size_t)n * SP;
  cxd* Y = W + (size_t)n * SP;
  __shared__ double sh[8 * SP * (SP + 1)];
  __shared__ cxd xs[KC][SP];
  __shared__ double Gs[2 * SP * SP];
  __shared__ double zs[2 * SP];
  __shared__ double lam_s;
  __shared__ double hw[2 * 4 * SP * SP];
  for (size_t e = tid; e < (size_t)n * SP; e += 256) X[e] = X0[e];
  __syncthreads();
  orth_cgs2(X, n, sh, 0);
  double est = -1.0;
  int it = 0;
  for (; it < maxit; ++it) {
    // W = C X
    for (int r0 = 0; r0 < n; r0 += 256) {
      const int r = r0 + tid;
      cxd acc[SP];
#pragma unroll
      for (int q = 0; q < SP; ++q) acc[q] = cxd(0.0, 0.0);
      for (int k0 = 0; k0 < n; k0 += KC) {
        __syncthreads();
        for (int e = tid; e < KC * SP; e += 256) {
          const int kk = e % KC, q = e / KC;
          xs[kk][q] = (k0 + kk < n) ? X[(size_t)q * n + k0 + kk] : cxd(0.0, 0.0);
        }
        __syncthreads();
        if (r < n) {
          const int kmax = min(KC, n - k0);
          const cxd* cp = C + r + (size_t)k0 * n;
          for (int kk = 0; kk < kmax; ++kk) {
            const cxd c = cp[(size_t)kk * n];
#pragma unroll
            for (int q = 0; q < SP; ++q) cfma(acc[q], c, xs[kk][q]);
          }
        }
      }
      if (r < n)
#pragma unroll
        for (int q = 0; q < SP; ++q) W[(size_t)q * n + r] = acc[q];
    }
    __syncthreads();
    // G = W^H W (upper triangle, then mirrored)
    {
      double g[SP * (SP + 1)];
#pragma unroll
      for (int i = 0; i < SP * (SP + 1); ++i) g[i] = 0.0;
      for (int r = tid; r < n; r += 256) {
        cxd w[SP];
#pragma unroll
        for (int q = 0; q < SP; ++q) w[q] = W[(size_t)q * n + r];
        int e = 0;
#pragma unroll
        for (int j = 0; j < SP; ++j)
#pragma unroll
          for (int i = 0; i <= j; ++i, e += 2) {
            g[e] += w[i].re * w[j].re + w[i].im * w[j].im;
            g[e + 1] += w[i].re * w[j].im - w[i].im * w[j].re;
          }
      }
      block_sum<SP * (SP + 1)>(g, sh);
      if (wid == 0) {
        if (lane == 0) {
          int e = 0;
          for (int j = 0; j < SP; ++j)
            for (int i = 0; i <= j; ++i, e += 2) {
              // exactly Hermitian: the diagonal of W^H W is real, the summed
              // products only leave a rounding residue there
              const double im = (i == j) ? 0.0 : g[e + 1];
              Gs[2 * (j * SP + i)] = g[e];
              Gs[2 * (j * SP + i) + 1] = im;
              Gs[2 * (i * SP + j)] = g[e];
              Gs[2 * (i * SP + j) + 1] = -im;
            }
        }
        __syncwarp();
        herm_top(Gs, &lam_s, zs, hw);
      }
      __syncthreads();
    }
    const double lam = lam_s;
    const double cur = (lam > 0.0 && isfinite(lam)) ? 1.0 / sqrt(lam) : 0.0;
    const bool done = (it > 0 && fabs(cur - est) <= tol * cur) || !(lam > 0.0 && isfinite(lam));
    est = cur;
    if (done || it + 1 == maxit) {
      ++it;
      break;
    }
    // Y = C^H W, one warp per column of C
    for (int r = wid; r < n; r += 8) {
      double acc[2 * SP];
#pragma unroll
      for (int i = 0; i < 2 * SP; ++i) acc[i] = 0.0;
      const cxd* cc = C + (size_t)r * n;
      for (int k = lane; k < n; k += 32) {
        const cxd c = conj(cc[k]);
#pragma unroll
        for (int q = 0; q < SP; ++q) {
          const cxd w = W[(size_t)q * n + k];
          acc[2 * q] += c.re * w.re - c.im * w.im;
          acc[2 * q + 1] += c.re * w.im + c.im * w.re;
        }
      }
#pragma unroll
      for (int i = 0; i < 2 * SP; ++i)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc[i] += __shfl_xor_sync(0xffffffffu, acc[i], o);
      if (lane == 0)
#pragma unroll
        for (int q = 0; q < SP; ++q) Y[(size_t)q * n + r] = cxd(acc[2 * q], acc[2 * q + 1]);
    }
    __syncthreads();
    orth_cgs2(Y, n, sh, 8 * (it + 1));
    cxd* t = X;  // X <- Y (Y is the old X's storage from now on)
    X = Y;
    Y = t;
  }
  if (tid == 0) {
    sig[b] = est;
    if (iters) iters[b] = it;
  }
  if (vec) {
    // W z / |W z|
    double nv[1] = {0.0};
    for (int r = tid; r < n; r += 256) {
      cxd v(0.0, 0.0);
#pragma unroll
      for (int q = 0; q < SP; ++q) cfma(v, W[(size_t)q * n + r], cxd(zs[2 * q], zs[2 * q + 1]));
      vec[(size_t)b * n + r] = v;
      nv[0] += cabs2(v);
    }
    block_sum<1>(nv, sh);
    const double s = nv[0] > 0.0 ? 1.0 / sqrt(nv[0]) : 0.0;
    for (int r = tid; r < n; r += 256) vec[(size_t)b * n + r] = vec[(size_t)b * n + r] * s;
  }
}

// One-matrix steps of the same iteration for callers that spread the products
// over the whole GPU (split-k GEMMs between these launches), one CTA each:
// k_rr_step: G = W^H W, its top eigenpair (lambda, z), est = 1/sqrt(lambda)
// and the convergence flag against the previous estimate (state: est, done,
// z[2 SP]); k_orth8: orthonormal columns of Y in place; k_topvec: x = W z / |W z|.
__global__ void __launch_bounds__(256) k_rr_step(const cxd* __restrict__ W, int n, double tol, double* state) {
  __shared__ double sh[8 * SP * (SP + 1)];
  __shared__ double Gs[2 * SP * SP];
  __shared__ double hw[2 * 4 * SP * SP];
  __shared__ double lam_s;
  const int tid = threadIdx.x;
  double g[SP * (SP + 1)];
#pragma unroll
  for (int i = 0; i < SP * (SP + 1); ++i) g[i] = 0.0;
  for (int r = tid; r < n; r += 256) {
    cxd w[SP];
#pragma unroll
    for (int q = 0; q < SP; ++q) w[q] = W[(size_t)q * n + r];
    int e = 0;
#pragma unroll
    for (int j = 0; j < SP; ++j)
#pragma unroll
      for (int i = 0; i <= j; ++i, e += 2) {
        g[e] += w[i].re * w[j].re + w[i].im * w[j].im;
        g[e + 1] += w[i].re * w[j].im - w[i].im * w[j].re;
      }
  }
  block_sum<SP * (SP + 1)>(g, sh);
  if (tid >= 32) return;
  if (tid == 0) {
    int e = 0;
    for (int j = 0; j < SP; ++j)
      for (int i = 0; i <= j; ++i, e += 2) {
        const double im = (i == j) ? 0.0 : g[e + 1];  // real diagonal (see k_sigma_iter)
        Gs[2 * (j * SP + i)] = g[e];
        Gs[2 * (j * SP + i) + 1] = im;
        Gs[2 * (i * SP + j)] = g[e];
        Gs[2 * (i * SP + j) + 1] = -im;
      }
  }
  __syncwarp();
  herm_top(Gs, &lam_s, state + 2, hw);
  if (tid == 0) {
    const double lam = lam_s;
    const bool ok = lam > 0.0 && isfinite(lam);
    const double cur = ok ? 1.0 / sqrt(lam) : 0.0;
    const double prev = state[0];
    state[1] = (prev >= 0.0 && fabs(cur - prev) <= tol * cur) || !ok ? 1.0 : 0.0;
    state[0] = cur;
  }
}

__global__ void __launch_bounds__(256) k_orth8(cxd* Y, int n, int salt) {
  __shared__ double sh[8 * 2 * SP];
  orth_cgs2(Y, n, sh, salt);
}

__global__ void __launch_bounds__(256) k_topvec(const cxd* __restrict__ W, const double* __restrict__ state, int n,
                                                cxd* __restrict__ x) {
  __shared__ double sh[8];
  const int tid = threadIdx.x;
  double nv[1] = {0.0};
  for (int r = tid; r < n; r += 256) {
    cxd v(0.0, 0.0);
#pragma unroll
    for (int q = 0; q < SP; ++q) cfma(v, W[(size_t)q * n + r], cxd(state[2 + 2 * q], state[3 + 2 * q]));
    x[r] = v;
    nv[0] += cabs2(v);
  }
  block_sum<1>(nv, sh);
  const double s = nv[0] > 0.0 ? 1.0 / sqrt(nv[0]) : 0.0;
  for (int r = tid; r < n; r += 256) x[r] = x[r] * s;
}

// M = G - lam I + mu x x^H (n x n, column-major)
__global__ void k_deflate_shift(const cxd* __restrict__ G, const cxd* __restrict__ x, int n, double lam, double mu,
                                cxd* __restrict__ M) {
  const size_t count = (size_t)n * n;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < count; e += (size_t)gridDim.x * blockDim.x) {
    const int r = (int)(e % n), c = (int)(e / n);
    cxd v = G[e];
    if (r == c) v.re -= lam;
    const cxd xr = x[r], xc = x[c];
    v.re += mu * (xr.re * xc.re + xr.im * xc.im);
    v.im += mu * (xr.im * xc.re - xr.re * xc.im);
    M[e] = v;
  }
}

}  // namespace

int Dense64::create(int n_, int batch_, cudaStream_t st_) {
  cxd* A = nullptr;
  st = st_;
  QBG_TRY(alloc(&A, sizeof(cxd) * (size_t)n_ * n_ * batch_));
  return bind(A, n_, batch_, st_);
}

int Dense64::bind(cxd* A, int n_, int batch_, cudaStream_t st_) {
  n = n_;
  batch = batch_;
  st = st_;
  f = LUBatch<double>();
  f.n = n;
  f.batch = batch;
  f.nb = 64;
  f.nblk = (n + f.nb - 1) / f.nb;
  f.stride = (long long)n * n;
  f.A = A;
  QBG_TRY(alloc(&f.ipiv, sizeof(int) * (size_t)n * batch));
  QBG_TRY(alloc(&f.perm, sizeof(int) * (size_t)n * batch));
  QBG_TRY(alloc(&f.info, sizeof(int) * batch));
  QBG_TRY(alloc(&f.Linv, sizeof(cxd) * (size_t)f.nblk * f.nb * f.nb * batch));
  QBG_TRY(alloc(&f.Uinv, sizeof(cxd) * (size_t)f.nblk * f.nb * f.nb * batch));
  return QBG_OK;
}

int Dense64::factor(std::vector<int>* info_host) {
  QBG_TRY(lu_factor<double>(f, st));
  if (!info_host) return QBG_OK;
  info_host->assign(batch, 0);
  QBG_CUDA(cudaMemcpyAsync(info_host->data(), f.info, sizeof(int) * batch, cudaMemcpyDeviceToHost, st));
  QBG_CUDA(cudaStreamSynchronize(st));
  return QBG_OK;
}

void Dense64::release() {
  if (st && !mem.empty()) cudaStreamSynchronize(st);
  for (void* q : mem) dfree(q, st);
  mem.clear();
}

Dense64::~Dense64() { release(); }

namespace {
// one CTA: modified Gram-Schmidt, each column projected twice against the
// earlier ones; a column that vanishes (below 1e-14 of its length) is refilled
__global__ void __launch_bounds__(256) k_orth_mgs2(cxd* Q, int n, int p) {
  __shared__ double sh[8 * 2];
  const int tid = threadIdx.x;
  for (int j = 0; j < p; ++j) {
    cxd* qj = Q + (size_t)j * n;
    for (int attempt = 0; attempt < 3; ++attempt) {
      double v0[1] = {0.0};
      for (int r = tid; r < n; r += 256) v0[0] += cabs2(qj[r]);
      block_sum<1>(v0, sh);
      for (int pass = 0; pass < 2; ++pass)
        for (int i = 0; i < j; ++i) {
          const cxd* qi = Q + (size_t)i * n;
          double c[2] = {0.0, 0.0};
          for (int r = tid; r < n; r += 256) {
            const cxd a = qi[r], y = qj[r];
            c[0] += a.re * y.re + a.im * y.im;
            c[1] += a.re * y.im - a.im * y.re;
          }
          block_sum<2>(c, sh);
          for (int r = tid; r < n; r += 256) {
            cxd y = qj[r];
            cfms(y, qi[r], cxd(c[0], c[1]));
            qj[r] = y;
          }
        }
      double v1[1] = {0.0};
      for (int r = tid; r < n; r += 256) v1[0] += cabs2(qj[r]);
      block_sum<1>(v1, sh);
      const double n1 = sqrt(v1[0]);
      if (n1 > 1e-14 * sqrt(v0[0]) && n1 > 1e-300 && isfinite(n1)) {
        const double s = 1.0 / n1;
        for (int r = tid; r < n; r += 256) qj[r] = qj[r] * s;
        break;
      }
      for (int r = tid; r < n; r += 256) qj[r] = cxd(fillv(r, j, 97 + attempt), fillv(r, j + p, 97 + attempt));
      __syncthreads();
    }
    __syncthreads();
  }
}
}  // namespace

int orth_columns(cxd* Q, int n, int p, cudaStream_t st) {
  k_orth_mgs2<<<1, 256, 0, st>>>(Q, n, p);
  QBG_LAUNCH_CHECK("k_orth_mgs2");
  return QBG_OK;
}

int sigma_iterate(const cxd* Cinv, int n, int batch, const cxd* X0, cxd* work, int maxit, double tol, double* sig,
                  int* iters, cxd* vec, cudaStream_t st) {
  if (batch < 1) return QBG_OK;
  k_sigma_iter<<<batch, 256, 0, st>>>(Cinv, n, X0, work, maxit, tol, sig, iters, vec);
  QBG_LAUNCH_CHECK("k_sigma_iter");
  return QBG_OK;
}

void dense_start_block(int n, std::vector<cxd>& hx) {
  // fixed (reproducible) start block: entries of a 64-bit LCG in [-1, 1)
  hx.resize((size_t)n * DENSE_P);
  unsigned long long lcg = 0x9E3779B97F4A7C15ull;
  auto nxt = [&]() {
    lcg = lcg * 6364136223846793005ull + 1442695040888963407ull;
    return (double)(lcg >> 11) * (2.0 / 9007199254740992.0) - 1.0;
  };
  for (auto& v : hx) {
    v.re = nxt();
    v.im = nxt();
  }
}

int rr_step(const cxd* W, int n, double tol, double* state, cudaStream_t st) {
  k_rr_step<<<1, 256, 0, st>>>(W, n, tol, state);
  QBG_LAUNCH_CHECK("k_rr_step");
  return QBG_OK;
}

int orth8(cxd* Y, int n, int salt, cudaStream_t st) {
  k_orth8<<<1, 256, 0, st>>>(Y, n, salt);
  QBG_LAUNCH_CHECK("k_orth8");
  return QBG_OK;
}

int topvec(const cxd* W, const double* state, int n, cxd* x, cudaStream_t st) {
  k_topvec<<<1, 256, 0, st>>>(W, state, n, x);
  QBG_LAUNCH_CHECK("k_topvec");
  return QBG_OK;
}

int sigma_single(const cxd* Cinv, cxd* CH, int n, const cxd* X0, cxd* X, cxd* W, cxd* Y, cxd* P, double* state,
                 int maxit, double tol, double* sig, cxd* x_out, cudaStream_t st) {
  QBG_TRY(conj_transpose(Cinv, CH, n, st));
  QBG_CUDA(cudaMemcpyAsync(X, X0, sizeof(cxd) * (size_t)n * DENSE_P, cudaMemcpyDeviceToDevice, st));
  QBG_TRY(orth8(X, n, 0, st));
  static const double init[2] = {-1.0, 0.0};
  QBG_CUDA(cudaMemcpyAsync(state, init, sizeof(init), cudaMemcpyHostToDevice, st));
  double h[2] = {0.0, 0.0};
  for (int it = 0; it < maxit; ++it) {
    QBG_TRY(gemm_tall(Cinv, X, W, n, DENSE_P, P, st));
    // the Rayleigh-Ritz step only tests convergence (the iteration itself is
    // X <- orth(C^H C X)): every fourth step, always before the host reads the
    // state, so the estimate and the Ritz vector belong to the last W
    const bool check = (it % 8 == 7) || it + 1 == maxit;
    if (check || it % 4 == 3) QBG_TRY(rr_step(W, n, tol, state, st));
    if (check) {
      QBG_CUDA(cudaMemcpyAsync(h, state, sizeof(h), cudaMemcpyDeviceToHost, st));
      QBG_CUDA(cudaStreamSynchronize(st));
      if (h[1] != 0.0 || it + 1 == maxit) break;
    }
    QBG_TRY(gemm_tall(CH, W, Y, n, DENSE_P, P, st));
    QBG_TRY(orth8(Y, n, 8 * (it + 1), st));
    cxd* t = X;
    X = Y;
    Y = t;
  }
  *sig = h[0];
  if (x_out) QBG_TRY(topvec(W, state, n, x_out, st));
  return QBG_OK;
}

int deflate_shift(const cxd* G, const cxd* x, int n, double lam, double mu, cxd* M, cudaStream_t st) {
  k_deflate_shift<<<2048, 256, 0, st>>>(G, x, n, lam, mu, M);
  QBG_LAUNCH_CHECK("k_deflate_shift");
  return QBG_OK;
}

}  // namespace qbg
