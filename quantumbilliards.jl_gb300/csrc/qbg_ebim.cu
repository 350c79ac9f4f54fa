// EBIM eigen step on the device: the second-order expansion of the boundary
// operator about a trial k (A(k + eps) = A + eps A' + eps^2/2 A'' + ...).
//
// The eigenpairs of the pencil A v = lambda A' v nearest 0 are those of
// largest |mu| of C = A^{-1} A' (mu = 1 / lambda). They are found by block
// shift-invert iteration: one FP64 LU of A (cuSOLVER getrf), C = A^-1 A' from
// it (one solve with N right-hand sides) and C^H, then Q <- orth(C Q) with p
// vectors (one skinny split-k product; Cholesky QR twice for orth), Rayleigh-Ritz on the p x p projection
// Q^H C Q (formed on the device, eigen-decomposed on the host: a few
// microseconds at this size) after every step, until the nev largest Ritz
// values change by less than 1e-13 relative (1e-8 for those well outside the
// acceptance box, which only place it). The left vectors u come from the same
// iteration on C^H = A'^H A^{-H}, paired with the right ones by
// mu_l ~ conj(mu_r). Then, per accepted lambda (|Re|, |Im| < dk):
//   eps1 = -lambda, eps2 = -eps1^2 / 2 (u^H A'' v) / (u^H A' v)
// (0 when |u^H A' v| <= 1e-15), corrected k = k + eps1 + eps2, tension
// |eps1 + eps2|.
//
// Two conventions, as in the reference:
// * solve_krylov! (ebim.jl:464-537): the nev eigenvalues of largest |mu|; u is
//   the eigenvector of C^H itself (the reference pairs it with v as is), and a
//   corrected k is kept only when |Re(k_c) - k| < dk.
// * solve_full! (ebim.jl:336-375, QBG_EBIM_FULL): every eigenvalue inside the
//   dk box; u is the left eigenvector of the pencil, u~ = A^{-H} u
//   (u~^H A = lambda u~^H A'), as LAPACK's generalized eigensolver returns it.
//   The block grows (nev doubles) until the nev-th eigenvalue lies outside the
//   disk |lambda| < sqrt(2) dk that contains the box, so none is missed.
// Results do not depend on how the eigenpairs are converged: the reference
// uses Arnoldi (KrylovKit) and QZ (LAPACK); here a block iteration converges
// the same eigenpairs to FP64 accuracy.
#include <algorithm>
#include <cmath>
#include <complex>
#include <vector>
#include "qbg_common.cuh"
#include "qbg_handles.cuh"
#include "qbg_linalg.cuh"
#include "qbg_dense.cuh"
#include "qbgpu.h"

using namespace qbg;

namespace {

typedef std::complex<double> zc;

// G[a + b p] = sum_r conj(X[r, a]) Y[r, b], a < p, b < q; one CTA per entry
__global__ void k_inner(const cxd* __restrict__ X, const cxd* __restrict__ Y, int n, int p, cxd* __restrict__ G) {
  const int a = blockIdx.x % p, b = blockIdx.x / p;
  const cxd* x = X + (size_t)a * n;
  const cxd* y = Y + (size_t)b * n;
  double re = 0.0, im = 0.0;
  for (int r = threadIdx.x; r < n; r += blockDim.x) {
    const cxd u = x[r], v = y[r];
    re = fma(u.re, v.re, fma(u.im, v.im, re));
    im = fma(u.re, v.im, fma(-u.im, v.re, im));
  }
  __shared__ double sr[8], si[8];
  for (int o = 16; o > 0; o >>= 1) {
    re += __shfl_xor_sync(0xffffffffu, re, o);
    im += __shfl_xor_sync(0xffffffffu, im, o);
  }
  if ((threadIdx.x & 31) == 0) {
    sr[threadIdx.x >> 5] = re;
    si[threadIdx.x >> 5] = im;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double tr = 0.0, ti = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
      tr += sr[w];
      ti += si[w];
    }
    G[blockIdx.x] = cxd(tr, ti);
  }
}

// AH = A^H for n x n column-major A, through 32 x 32 shared-memory tiles
__global__ void k_conj_transpose(const cxd* __restrict__ A, cxd* __restrict__ AH, int n) {
  __shared__ cxd t[32][33];
  const int bx = blockIdx.x * 32, by = blockIdx.y * 32;
  for (int j = threadIdx.y; j < 32; j += blockDim.y) {
    const int r = bx + threadIdx.x, c = by + j;
    if (r < n && c < n) t[j][threadIdx.x] = A[r + (size_t)c * n];
  }
  __syncthreads();
  for (int j = threadIdx.y; j < 32; j += blockDim.y) {
    const int r = by + threadIdx.x, c = bx + j;  // AH[r, c] = conj(A[c, r]) = conj(t[r - by][c - bx])
    if (r < n && c < n) {
      const cxd v = t[threadIdx.x][j];
      AH[r + (size_t)c * n] = cxd(v.re, -v.im);
    }
  }
}

// Adjoint Fredholm matrix from the Fredholm matrix F = I - D of the DLP:
// Aadj[a, b] = delta_ab - D[b, a] ds_b / ds_a = F[b, a] ds_b / ds_a (the
// diagonal ratio is 1). ds: arc-length weights of the full boundary; with a
// reduction, fund maps reduced index -> full node. 32 x 32 shared-memory tiles.
__global__ void k_adjoint_fredholm(const cxd* __restrict__ F, const double* __restrict__ ds,
                                   const int* __restrict__ fund, int m, cxd* __restrict__ out) {
  __shared__ cxd t[32][33];
  const int bx = blockIdx.x * 32, by = blockIdx.y * 32;
  for (int j = threadIdx.y; j < 32; j += blockDim.y) {
    const int r = bx + threadIdx.x, c = by + j;
    if (r < m && c < m) t[j][threadIdx.x] = F[r + (size_t)c * m];
  }
  __syncthreads();
  for (int j = threadIdx.y; j < 32; j += blockDim.y) {
    const int a = by + threadIdx.x, b = bx + j;  // out[a, b] = F[b, a] ds_b / ds_a = t[a - by][b - bx] ...
    if (a < m && b < m) {
      const double da = ds[fund ? fund[a] : a], db = ds[fund ? fund[b] : b];
      const cxd v = t[threadIdx.x][j];
      const double sc = (a == b) ? 1.0 : db / da;
      out[a + (size_t)b * m] = cxd(v.re * sc, v.im * sc);
    }
  }
}

// ---------------------------------------------------------------------------
// Y = A X for n x n A and n x q X, q <= TALL_MAXQ (FP64 complex, column-major):
// split over k into ks slices so that a skinny product still fills the device;
// each CTA computes a 64-row block of one slice's partial product, and a
// second kernel sums the slices in a fixed order (deterministic).
// ---------------------------------------------------------------------------
constexpr int TALL_MAXQ = 128, TALL_KC = 16;  // 16 KB + 32 KB of static shared memory

// CPT: columns per thread (q <= 4 CPT)
template <int CPT>
__global__ void __launch_bounds__(256) k_zgemm_tall(const cxd* __restrict__ A, const cxd* __restrict__ X, int n,
                                                    int q, int kslice, cxd* __restrict__ P) {
  __shared__ cxd As[TALL_KC][64];
  __shared__ cxd Xs[TALL_KC][4 * CPT];
  const int r0 = blockIdx.x * 64, s = blockIdx.y;
  const int k0 = s * kslice, k1 = min(n, k0 + kslice);
  const int tr = threadIdx.x & 63, tg = threadIdx.x >> 6;  // row, column group (columns tg, tg + 4, ...)
  double ar[CPT], ai[CPT];
#pragma unroll
  for (int c = 0; c < CPT; ++c) ar[c] = ai[c] = 0.0;
  for (int kc = k0; kc < k1; kc += TALL_KC) {
    for (int e = threadIdx.x; e < TALL_KC * 64; e += 256) {
      const int rr = e & 63, kk = e >> 6;
      const int r = r0 + rr, k = kc + kk;
      As[kk][rr] = (r < n && k < k1) ? A[r + (size_t)k * n] : cxd(0, 0);
    }
    for (int e = threadIdx.x; e < TALL_KC * q; e += 256) {
      const int kk = e % TALL_KC, j = e / TALL_KC;
      const int k = kc + kk;
      Xs[kk][j] = (k < k1) ? X[k + (size_t)j * n] : cxd(0, 0);
    }
    __syncthreads();
#pragma unroll 2
    for (int kk = 0; kk < TALL_KC; ++kk) {
      const cxd a = As[kk][tr];
#pragma unroll
      for (int c = 0; c < CPT; ++c) {
        const int j = tg + 4 * c;
        if (j < q) {
          const cxd x = Xs[kk][j];
          ar[c] = fma(a.re, x.re, fma(-a.im, x.im, ar[c]));
          ai[c] = fma(a.re, x.im, fma(a.im, x.re, ai[c]));
        }
      }
    }
    __syncthreads();
  }
  const int r = r0 + tr;
  if (r < n) {
    cxd* ps = P + (size_t)s * n * q;
#pragma unroll
    for (int c = 0; c < CPT; ++c) {
      const int j = tg + 4 * c;
      if (j < q) ps[r + (size_t)j * n] = cxd(ar[c], ai[c]);
    }
  }
}

__global__ void k_sum_slices(const cxd* __restrict__ P, int ks, size_t count, cxd* __restrict__ Y) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < count; i += (size_t)gridDim.x * blockDim.x) {
    double re = 0.0, im = 0.0;
    for (int s = 0; s < ks; ++s) {
      re += P[s * count + i].re;
      im += P[s * count + i].im;
    }
    Y[i] = cxd(re, im);
  }
}

// ---------------------------------------------------------------------------
// Eigen-decomposition of a small complex matrix on the host (the Rayleigh-Ritz
// step): Householder reduction to Hessenberg form, single-shift QR sweeps with
// Givens rotations and Wilkinson shifts (exceptional shifts after 10 sweeps
// without deflation) to the Schur form T = Z^H H Z, eigenvectors of T by
// back substitution, V = Z Y with unit columns. Golub and Van Loan, Matrix
// Computations, algorithms 7.4.2 (Hessenberg), 7.5 (shifted QR), 7.6.4
// (eigenvectors of a triangular matrix).
// ---------------------------------------------------------------------------
int small_eig(int p, std::vector<zc>& H, std::vector<zc>& w, std::vector<zc>& V) {
  auto h = [&](int i, int j) -> zc& { return H[(size_t)j * p + i]; };
  std::vector<zc> Z((size_t)p * p, zc(0.0, 0.0));
  auto z = [&](int i, int j) -> zc& { return Z[(size_t)j * p + i]; };
  for (int i = 0; i < p; ++i) z(i, i) = 1.0;
  double hnorm = 0.0;
  for (const zc& x : H) hnorm = std::max(hnorm, std::abs(x));
  // Hessenberg reduction
  std::vector<zc> v(p);
  for (int j = 0; j + 2 < p; ++j) {
    double xn = 0.0;
    for (int i = j + 1; i < p; ++i) xn += std::norm(h(i, j));
    xn = std::sqrt(xn);
    if (xn == 0.0) continue;
    const zc x0 = h(j + 1, j);
    const zc ph = std::abs(x0) > 0.0 ? x0 / std::abs(x0) : zc(1.0, 0.0);
    const zc alpha = -ph * xn;
    for (int i = j + 1; i < p; ++i) v[i] = h(i, j);
    v[j + 1] -= alpha;
    double vn = 0.0;
    for (int i = j + 1; i < p; ++i) vn += std::norm(v[i]);
    if (vn == 0.0) continue;
    const double beta = 2.0 / vn;
    // H = (I - beta v v^H) H
    for (int c = 0; c < p; ++c) {
      zc t(0.0, 0.0);
      for (int i = j + 1; i < p; ++i) t += std::conj(v[i]) * h(i, c);
      t *= beta;
      for (int i = j + 1; i < p; ++i) h(i, c) -= v[i] * t;
    }
    // H = H (I - beta v v^H), Z = Z (I - beta v v^H)
    for (int rr = 0; rr < p; ++rr) {
      zc t(0.0, 0.0), tz(0.0, 0.0);
      for (int i = j + 1; i < p; ++i) {
        t += h(rr, i) * v[i];
        tz += z(rr, i) * v[i];
      }
      t *= beta;
      tz *= beta;
      for (int i = j + 1; i < p; ++i) {
        h(rr, i) -= t * std::conj(v[i]);
        z(rr, i) -= tz * std::conj(v[i]);
      }
    }
    for (int i = j + 2; i < p; ++i) h(i, j) = 0.0;
  }
  // shifted QR on the active window [lo, hi]
  const double eps = 2.220446049250313e-16;
  int hi = p - 1, since = 0, total = 0;
  while (hi > 0) {
    if (++total > 100 * p) {
      set_error("small_eig: QR iteration did not converge");
      return QBG_ECUDA;
    }
    int lo = hi;
    while (lo > 0) {
      const double sc = std::abs(h(lo - 1, lo - 1)) + std::abs(h(lo, lo));
      if (std::abs(h(lo, lo - 1)) <= eps * (sc > 0.0 ? sc : hnorm)) {
        h(lo, lo - 1) = 0.0;
        break;
      }
      --lo;
    }
    if (lo == hi) {  // 1 x 1 block converged
      --hi;
      since = 0;
      continue;
    }
    zc mu;
    if (since > 0 && since % 10 == 0) {
      mu = h(hi, hi) + zc(0.75 * std::abs(h(hi, hi - 1)), 0.0);  // exceptional shift
    } else {
      const zc a = h(hi - 1, hi - 1), b = h(hi - 1, hi), c = h(hi, hi - 1), d = h(hi, hi);
      const zc tr = 0.5 * (a + d), det = a * d - b * c;
      const zc disc = std::sqrt(tr * tr - det);
      const zc m1 = tr + disc, m2 = tr - disc;
      mu = std::abs(m1 - d) < std::abs(m2 - d) ? m1 : m2;
    }
    ++since;
    zc x = h(lo, lo) - mu, y = h(lo + 1, lo);
    for (int k = lo; k < hi; ++k) {
      if (k > lo) {
        x = h(k, k - 1);
        y = h(k + 1, k - 1);
      }
      const double ax = std::abs(x), ay = std::abs(y);
      if (ay == 0.0) continue;
      const double r = std::hypot(ax, ay);
      double c;
      zc sgn, sn;
      if (ax == 0.0) {
        c = 0.0;
        sn = std::conj(y) / ay;
      } else {
        c = ax / r;
        sgn = x / ax;
        sn = sgn * std::conj(y) / r;
      }
      // rows k, k + 1 (every column from k - 1 on)
      for (int col = std::max(k - 1, 0); col < p; ++col) {
        const zc a = h(k, col), b = h(k + 1, col);
        h(k, col) = c * a + sn * b;
        h(k + 1, col) = -std::conj(sn) * a + c * b;
      }
      // columns k, k + 1 (rows 0 .. min(k + 2, hi)) and Z
      const int rmax = std::min(k + 2, hi);
      for (int rr = 0; rr <= rmax; ++rr) {
        const zc a = h(rr, k), b = h(rr, k + 1);
        h(rr, k) = c * a + std::conj(sn) * b;
        h(rr, k + 1) = -sn * a + c * b;
      }
      for (int rr = 0; rr < p; ++rr) {
        const zc a = z(rr, k), b = z(rr, k + 1);
        z(rr, k) = c * a + std::conj(sn) * b;
        z(rr, k + 1) = -sn * a + c * b;
      }
      if (k > lo) h(k + 1, k - 1) = 0.0;
    }
  }
  // eigenvalues and eigenvectors of the triangular T
  w.assign(p, zc(0.0, 0.0));
  for (int i = 0; i < p; ++i) w[i] = h(i, i);
  V.assign((size_t)p * p, zc(0.0, 0.0));
  std::vector<zc> x(p);
  const double smin = std::max(eps * hnorm, 1e-300);
  for (int k = 0; k < p; ++k) {
    std::fill(x.begin(), x.end(), zc(0.0, 0.0));
    x[k] = 1.0;
    for (int i = k - 1; i >= 0; --i) {
      zc t = h(i, k);
      for (int j = i + 1; j < k; ++j) t += h(i, j) * x[j];
      zc den = h(i, i) - w[k];
      if (std::abs(den) < smin) den = smin;
      x[i] = -t / den;
    }
    double nrm = 0.0;
    for (int rr = 0; rr < p; ++rr) {
      zc t(0.0, 0.0);
      for (int j = 0; j <= k; ++j) t += z(rr, j) * x[j];
      V[(size_t)k * p + rr] = t;
      nrm += std::norm(t);
    }
    nrm = std::sqrt(nrm);
    if (nrm > 0.0)
      for (int rr = 0; rr < p; ++rr) V[(size_t)k * p + rr] /= nrm;
  }
  return QBG_OK;
}

struct Ebim {
  int n = 0;
  cudaStream_t st = nullptr;
  cudaEvent_t ev = nullptr;
  cxd *LU = nullptr, *dA = nullptr, *ddA = nullptr;
  cxd *C = nullptr, *CH = nullptr;  // A^-1 A' and its conjugate transpose
  Dense64 D;                        // the library's FP64 LU of the matrix in LU
  std::vector<void*> tmp;
  ~Ebim() {
    if (st) cudaStreamSynchronize(st);
    D.release();
    for (void* q : tmp) dfree(q, st);
    if (ev) cudaEventDestroy(ev);
    if (st) cudaStreamDestroy(st);
  }
  // LU of the n x n matrix in LU, in place; QBG_ESINGULAR (with what) if U is exactly singular
  int factor(const char* what) {
    QBG_TRY(D.bind(LU, n, 1, st));
    std::vector<int> info;
    QBG_TRY(D.factor(&info));
    if (info[0] > 0) {
      set_error("%s is exactly singular (U(%d, %d) = 0)", what, info[0], info[0]);
      return QBG_ESINGULAR;
    }
    return QBG_OK;
  }
  template <class P>
  int alloc(P** q, size_t bytes) {
    int s = dmalloc(q, bytes);
    if (!s) tmp.push_back(*q);
    return s;
  }
  int wait() {
    cudaError_t e = cudaEventRecord(ev, st);
    if (e == cudaSuccess) e = cudaEventSynchronize(ev);
    return e == cudaSuccess ? QBG_OK : cuda_status(e, "EBIM wait");
  }
};

// Y = A B for n x n A and n x q B (FP64 complex); P: scratch of
// tall_scratch(n, q) elements
int tall_slices(int n) {
  const int rb = (n + 63) / 64;
  const int want = std::max(1, std::min(16, (2 * 152 + rb - 1) / rb));
  return std::min(want, std::max(1, n / TALL_KC));
}
size_t tall_scratch(int n, int q) { return (size_t)tall_slices(n) * n * q; }

int gemm_nq(const cxd* A, const cxd* B, cxd* Y, int n, int q, cxd* P, cudaStream_t st) {
  if (q > TALL_MAXQ) return gemm_batched<double>(n, q, n, cxd(1, 0), A, n, 0, B, n, 0, cxd(0, 0), Y, n, 0, 1, st);
  const int ks = tall_slices(n);
  const int kslice = ((n + ks - 1) / ks + TALL_KC - 1) / TALL_KC * TALL_KC;
  const int nsl = (n + kslice - 1) / kslice;
  const dim3 grd((n + 63) / 64, nsl);
  if (q <= 32)
    k_zgemm_tall<8><<<grd, 256, 0, st>>>(A, B, n, q, kslice, P);
  else if (q <= 64)
    k_zgemm_tall<16><<<grd, 256, 0, st>>>(A, B, n, q, kslice, P);
  else
    k_zgemm_tall<32><<<grd, 256, 0, st>>>(A, B, n, q, kslice, P);
  QBG_LAUNCH_CHECK("k_zgemm_tall");
  const size_t count = (size_t)n * q;
  k_sum_slices<<<(unsigned)std::min<size_t>((count + 255) / 256, 4096), 256, 0, st>>>(P, nsl, count, Y);
  QBG_LAUNCH_CHECK("k_sum_slices");
  return QBG_OK;
}

// Buffers of the orthonormalisation: Gram matrix, its factor, a copy of W.
struct OrthWork {
  cxd *G = nullptr, *M = nullptr, *Wt = nullptr;
  std::vector<cxd> hg, hm;
};

// Orthonormal basis of the columns of W (n x p) in place by Cholesky QR, twice
// (the second pass restores orthogonality to rounding): G = W^H W on the
// device; on the host, with D = diag(G)^(1/2), the Cholesky factor R of
// D^-1 G D^-1 and M = D^-1 R^-1; then W <- W M. Falls back to Gram-Schmidt
// on the device (twice per column) when the scaled Gram matrix is not
// numerically positive definite.
int orthonormalize(Ebim& E, cxd* W, int p, OrthWork& o) {
  const int n = E.n;
  o.hg.resize((size_t)p * p);
  o.hm.resize((size_t)p * p);
  std::vector<zc> R((size_t)p * p), Ri((size_t)p * p);
  std::vector<double> d(p);
  for (int pass = 0; pass < 2; ++pass) {
    k_inner<<<p * p, 256, 0, E.st>>>(W, W, n, p, o.G);
    QBG_LAUNCH_CHECK("k_inner");
    QBG_CUDA(cudaMemcpyAsync(o.hg.data(), o.G, sizeof(cxd) * o.hg.size(), cudaMemcpyDeviceToHost, E.st));
    QBG_TRY(E.wait());
    auto g = [&](int i, int j) { return zc(o.hg[(size_t)j * p + i].re, o.hg[(size_t)j * p + i].im); };
    bool ok = true;
    for (int i = 0; i < p && ok; ++i) {
      const double gi = g(i, i).real();
      ok = std::isfinite(gi) && gi > 0.0;
      d[i] = ok ? std::sqrt(gi) : 1.0;
    }
    // Cholesky of the scaled Gram matrix, S = R^H R with R upper triangular
    std::fill(R.begin(), R.end(), zc(0.0, 0.0));
    for (int j = 0; j < p && ok; ++j) {
      double djj = g(j, j).real() / (d[j] * d[j]);
      for (int k = 0; k < j; ++k) djj -= std::norm(R[(size_t)j * p + k]);
      if (!(djj > 1e-13)) {
        ok = false;
        break;
      }
      const double rjj = std::sqrt(djj);
      R[(size_t)j * p + j] = rjj;
      for (int i = j + 1; i < p; ++i) {
        zc t = g(j, i) / (d[j] * d[i]);
        for (int k = 0; k < j; ++k) t -= std::conj(R[(size_t)j * p + k]) * R[(size_t)i * p + k];
        R[(size_t)i * p + j] = t / rjj;
      }
    }
    if (!ok) return orth_columns(W, n, p, E.st);
    // Ri = R^-1 (upper triangular), M = D^-1 Ri
    std::fill(Ri.begin(), Ri.end(), zc(0.0, 0.0));
    for (int j = 0; j < p; ++j) {
      Ri[(size_t)j * p + j] = 1.0 / R[(size_t)j * p + j];
      for (int i = j - 1; i >= 0; --i) {
        zc t(0.0, 0.0);
        for (int k = i + 1; k <= j; ++k) t += R[(size_t)k * p + i] * Ri[(size_t)j * p + k];
        Ri[(size_t)j * p + i] = -t / R[(size_t)i * p + i];
      }
    }
    for (int j = 0; j < p; ++j)
      for (int i = 0; i < p; ++i) {
        const zc m = Ri[(size_t)j * p + i] / d[i];
        o.hm[(size_t)j * p + i] = cxd(m.real(), m.imag());
      }
    QBG_CUDA(cudaMemcpyAsync(o.M, o.hm.data(), sizeof(cxd) * o.hm.size(), cudaMemcpyHostToDevice, E.st));
    QBG_CUDA(cudaMemcpyAsync(o.Wt, W, sizeof(cxd) * (size_t)n * p, cudaMemcpyDeviceToDevice, E.st));
    QBG_TRY(gemm_batched<double>(n, p, p, cxd(1, 0), o.Wt, n, 0, o.M, p, 0, cxd(0, 0), W, n, 0, 1, E.st));
  }
  return QBG_OK;
}

// The nev eigenvalues of largest modulus of C = A^{-1} A' (adjoint: of
// C^H = A'^H A^{-H}) and their eigenvectors (device, n x nev), largest first.
// V0 (optional, n x n0): vectors that seed the first n0 columns of the block
// Ritz values with |lambda| = 1/|mu| below r_tight must settle to 1e-13
// relative; the others (outside the acceptance box, used only to place it) to
// 1e-8.
int block_eigs(Ebim& E, bool adjoint, int p, int nev, std::vector<zc>& mu, cxd* V, int* iters, double r_tight,
               const cxd* V0 = nullptr, int n0 = 0) {
  const int n = E.n;
  constexpr int MAXIT = 400;
  constexpr double TOL = 1e-13;
  cxd *Q = nullptr, *Y = nullptr, *H = nullptr, *Xs = nullptr, *P = nullptr;
  const size_t np = (size_t)n * p, pp = (size_t)p * p;
  OrthWork o;
  QBG_TRY(E.alloc(&Q, sizeof(cxd) * np));
  QBG_TRY(E.alloc(&Y, sizeof(cxd) * np));
  QBG_TRY(E.alloc(&H, sizeof(cxd) * pp));
  QBG_TRY(E.alloc(&Xs, sizeof(cxd) * (size_t)p * nev));
  QBG_TRY(E.alloc(&P, sizeof(cxd) * std::max<size_t>(tall_scratch(n, p), 1)));
  QBG_TRY(E.alloc(&o.G, sizeof(cxd) * pp));
  QBG_TRY(E.alloc(&o.M, sizeof(cxd) * pp));
  QBG_TRY(E.alloc(&o.Wt, sizeof(cxd) * np));
  // fixed starting block (reproducible): entries of a 64-bit LCG in [-1, 1)
  std::vector<cxd> hq(np);
  unsigned long long lcg = adjoint ? 0xD1B54A32D192ED03ull : 0x9E3779B97F4A7C15ull;
  for (auto& v : hq) {
    lcg = lcg * 6364136223846793005ull + 1442695040888963407ull;
    v.re = (double)(lcg >> 11) * (2.0 / 9007199254740992.0) - 1.0;
    lcg = lcg * 6364136223846793005ull + 1442695040888963407ull;
    v.im = (double)(lcg >> 11) * (2.0 / 9007199254740992.0) - 1.0;
  }
  QBG_CUDA(cudaMemcpyAsync(Q, hq.data(), sizeof(cxd) * np, cudaMemcpyHostToDevice, E.st));
  if (V0 && n0 > 0)
    QBG_CUDA(cudaMemcpyAsync(Q, V0, sizeof(cxd) * (size_t)n * std::min(n0, p), cudaMemcpyDeviceToDevice, E.st));
  QBG_TRY(orthonormalize(E, Q, p, o));
  std::vector<cxd> hh(pp), hx((size_t)p * nev);
  std::vector<zc> Hz(pp), w, X;
  std::vector<zc> prev(nev, zc(0.0, 0.0));
  std::vector<int> order(p);
  for (int it = 0; it < MAXIT; ++it) {
    // Y = C Q, or C^H Q
    QBG_TRY(gemm_nq(adjoint ? E.CH : E.C, Q, Y, n, p, P, E.st));
    // Rayleigh-Ritz on the projection Q^H Y
    k_inner<<<p * p, 256, 0, E.st>>>(Q, Y, n, p, H);
    QBG_LAUNCH_CHECK("k_inner");
    QBG_CUDA(cudaMemcpyAsync(hh.data(), H, sizeof(cxd) * pp, cudaMemcpyDeviceToHost, E.st));
    QBG_TRY(E.wait());
    for (size_t i = 0; i < pp; ++i) Hz[i] = zc(hh[i].re, hh[i].im);
    QBG_TRY(small_eig(p, Hz, w, X));
    for (int i = 0; i < p; ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return std::abs(w[a]) > std::abs(w[b]); });
    bool conv = it >= 2;
    for (int j = 0; j < nev; ++j) {
      const zc m = w[order[j]];
      const double tol = (1.0 < r_tight * std::abs(m)) ? TOL : 1e-8;
      if (!(std::abs(m - prev[j]) <= tol * std::abs(m))) conv = false;
      prev[j] = m;
    }
    if (conv || it + 1 == MAXIT) {
      // Ritz vectors of the nev largest: V = Q X(:, order[0..nev))
      for (int j = 0; j < nev; ++j)
        for (int i = 0; i < p; ++i) {
          const zc x = X[(size_t)order[j] * p + i];
          hx[(size_t)j * p + i] = cxd(x.real(), x.imag());
        }
      QBG_CUDA(cudaMemcpyAsync(Xs, hx.data(), sizeof(cxd) * hx.size(), cudaMemcpyHostToDevice, E.st));
      QBG_TRY(gemm_batched<double>(n, nev, p, cxd(1, 0), Q, n, 0, Xs, p, 0, cxd(0, 0), V, n, 0, 1, E.st));
      QBG_TRY(E.wait());
      mu = prev;
      *iters = it + 1;
      return QBG_OK;
    }
    QBG_TRY(orthonormalize(E, Y, p, o));
    std::swap(Q, Y);
  }
  return QBG_OK;  // not reached
}

// Everything after the three matrices are on the device (LU is overwritten).
int ebim_run(Ebim& E, double k, double dk, int nev_req, int flags, int cap, double* out_k, double* out_tens,
             int32_t* count, int32_t* iters_out) {
  const int n = E.n;
  const bool full = (flags & QBG_EBIM_FULL) != 0;
  // LU of A (the reference's lu!(A)), the library's batched FP64 LU with one matrix
  QBG_TRY(E.factor("EBIM: A(k)"));
  // C = A^-1 A' and C^H from the factors (one solve with n right-hand sides):
  // every application of the shift-invert operator is then one skinny product
  QBG_TRY(E.alloc(&E.C, sizeof(cxd) * (size_t)n * n));
  QBG_TRY(E.alloc(&E.CH, sizeof(cxd) * (size_t)n * n));
  QBG_TRY(lu_solve_shared<double>(E.D.f, E.dA, n, E.C, 0, E.st));
  k_conj_transpose<<<dim3((n + 31) / 32, (n + 31) / 32), dim3(32, 8), 0, E.st>>>(E.C, E.CH, n);
  QBG_LAUNCH_CHECK("k_conj_transpose");
  int nev = std::min(nev_req, n);
  std::vector<zc> mur, mul;
  cxd *V = nullptr, *U = nullptr, *W1 = nullptr, *W2 = nullptr;
  int itr = 0, itl = 0;
  cxd* Vprev = nullptr;
  int nprev = 0;
  const double r_tight = 1.25 * std::sqrt(2.0) * dk;  // the box |Re|, |Im| < dk with a margin
  for (;;) {
    const int p = std::min(n, 2 * nev + 12);
    QBG_TRY(E.alloc(&V, sizeof(cxd) * (size_t)n * nev));
    // a grown block starts from the Ritz vectors of the smaller one
    QBG_TRY(block_eigs(E, false, p, nev, mur, V, &itr, r_tight, Vprev, nprev));
    Vprev = V;
    nprev = nev;
    // full: the box |Re|, |Im| < dk lies inside |lambda| < sqrt(2) dk
    const double lam_last = 1.0 / std::abs(mur[nev - 1]);
    if (!full || nev >= n || lam_last >= std::sqrt(2.0) * dk) {
      QBG_TRY(E.alloc(&U, sizeof(cxd) * (size_t)n * nev));
      QBG_TRY(block_eigs(E, true, p, nev, mul, U, &itl, r_tight));
      break;
    }
    nev = std::min(n, 2 * nev);
  }
  // pair left with right: perm[j] = argmin_i |mu_l[i] - conj(mu_r[j])|
  std::vector<int> perm(nev);
  for (int j = 0; j < nev; ++j) {
    int bi = 0;
    double bd = INFINITY;
    for (int i = 0; i < nev; ++i) {
      const double d = std::abs(mul[i] - std::conj(mur[j]));
      if (d < bd) {
        bd = d;
        bi = i;
      }
    }
    perm[j] = bi;
  }
  cxd* P = nullptr;
  QBG_TRY(E.alloc(&W1, sizeof(cxd) * (size_t)n * nev));
  QBG_TRY(E.alloc(&W2, sizeof(cxd) * (size_t)n * nev));
  QBG_TRY(E.alloc(&P, sizeof(cxd) * std::max<size_t>(tall_scratch(n, nev), 1)));
  if (full) {  // left eigenvectors of the pencil: u~ = A^{-H} u
    cxd* Us = nullptr;
    QBG_TRY(E.alloc(&Us, sizeof(cxd) * (size_t)n * nev));
    QBG_TRY(lu_solve_adjoint<double>(E.D.f, U, 0, nev, U, Us, E.st));
  }
  QBG_TRY(gemm_nq(E.ddA, V, W1, n, nev, P, E.st));
  QBG_TRY(gemm_nq(E.dA, V, W2, n, nev, P, E.st));
  std::vector<cxd> hu((size_t)n * nev), h1((size_t)n * nev), h2((size_t)n * nev);
  QBG_CUDA(cudaMemcpyAsync(hu.data(), U, sizeof(cxd) * hu.size(), cudaMemcpyDeviceToHost, E.st));
  QBG_CUDA(cudaMemcpyAsync(h1.data(), W1, sizeof(cxd) * h1.size(), cudaMemcpyDeviceToHost, E.st));
  QBG_CUDA(cudaMemcpyAsync(h2.data(), W2, sizeof(cxd) * h2.size(), cudaMemcpyDeviceToHost, E.st));
  QBG_TRY(E.wait());
  int m = 0;
  for (int j = 0; j < nev; ++j) {
    const zc lam = 1.0 / mur[j];
    if (!(std::fabs(lam.real()) < dk && std::fabs(lam.imag()) < dk)) continue;
    const cxd* u = hu.data() + (size_t)perm[j] * n;
    const cxd* a1 = h1.data() + (size_t)j * n;
    const cxd* a2 = h2.data() + (size_t)j * n;
    zc num(0.0, 0.0), den(0.0, 0.0);
    for (int r = 0; r < n; ++r) {
      const zc ur(u[r].re, -u[r].im);
      num += ur * zc(a1[r].re, a1[r].im);
      den += ur * zc(a2[r].re, a2[r].im);
    }
    const zc c1 = -lam;
    zc c2(0.0, 0.0);
    if (std::abs(den) > 1e-15) c2 = -0.5 * c1 * c1 * (num / den);
    const zc t = c1 + c2;
    const zc kc = zc(k, 0.0) + t;
    if (!full && !(std::fabs(kc.real() - k) < dk)) continue;
    if (m < cap) {
      out_k[2 * m] = kc.real();
      out_k[2 * m + 1] = kc.imag();
      out_tens[m] = std::abs(t);
    }
    ++m;
  }
  *count = m;
  if (iters_out) {
    iters_out[0] = itr;
    iters_out[1] = itl;
    iters_out[2] = nev;
  }
  return QBG_OK;
}

int ebim_setup(Ebim& E, int n) {
  E.n = n;
  cudaError_t e = stream_create(&E.st);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&E.ev, cudaEventBlockingSync | cudaEventDisableTiming);
  return e == cudaSuccess ? QBG_OK : cuda_status(e, "EBIM stream");
}

bool ebim_args_ok(double k, double dk, int32_t nev, int32_t cap, const double* out_k, const double* out_tens,
                  const int32_t* count) {
  return std::isfinite(k) && dk > 0.0 && nev >= 1 && cap >= 0 && count && (cap == 0 || (out_k && out_tens));
}

}  // namespace

size_t qbg::gemm_tall_scratch(int n, int q) { return tall_scratch(n, q); }
int qbg::gemm_tall(const cxd* A, const cxd* B, cxd* Y, int n, int q, cxd* P, cudaStream_t st) {
  return gemm_nq(A, B, Y, n, q, P, st);
}
int qbg::conj_transpose(const cxd* A, cxd* AH, int n, cudaStream_t st) {
  k_conj_transpose<<<dim3((n + 31) / 32, (n + 31) / 32), dim3(32, 8), 0, st>>>(A, AH, n);
  QBG_LAUNCH_CHECK("k_conj_transpose");
  return QBG_OK;
}

extern "C" {

qbg_status qbg_ebim_eig(int64_t n, const void* A, const void* dA, const void* ddA, double k, double dk, int32_t nev,
                        int32_t flags, int32_t cap, double* out_k, double* out_tens, int32_t* count,
                        int32_t* iters) {
  if (n < 1 || n > (1 << 20) || !A || !dA || !ddA || !ebim_args_ok(k, dk, nev, cap, out_k, out_tens, count)) {
    set_error("qbg_ebim_eig: invalid arguments");
    return QBG_EINVAL;
  }
  Ebim E;
  QBG_TRY(ebim_setup(E, (int)n));
  const size_t bytes = sizeof(cxd) * (size_t)n * n;
  QBG_TRY(E.alloc(&E.LU, bytes));
  QBG_TRY(E.alloc(&E.dA, bytes));
  QBG_TRY(E.alloc(&E.ddA, bytes));
  const cudaMemcpyKind kind = (flags & QBG_PTR_DEVICE) ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
  QBG_CUDA(cudaMemcpyAsync(E.LU, A, bytes, kind, E.st));
  QBG_CUDA(cudaMemcpyAsync(E.dA, dA, bytes, kind, E.st));
  QBG_CUDA(cudaMemcpyAsync(E.ddA, ddA, bytes, kind, E.st));
  return ebim_run(E, k, dk, nev, flags, cap, out_k, out_tens, count, iters);
}

// ---------------------------------------------------------------------------
// Newton refinement of a sweep minimum (newton_refine_svd!,
// sweepmethods.jl:307-368): f(k) = lambda_min(G(k)), G = A^H A, with
// G' = A'^H A + A^H A' and G'' = A''^H A + 2 A'^H A' + A^H A''. The
// reference takes lambda = lambda_min, x and every eigenpair (lambda_j, v_j)
// from a full Hermitian eigen-decomposition of G and forms
//   lambda1 = x^H G' x,
//   lambda2 = x^H G'' x + 2 sum_{j != min} |v_j^H G' x|^2 / (lambda - lambda_j).
// Here, per step, on the device:
//  * lambda = sigma_min(A)^2 and x = the right singular vector of A, from the
//    library's FP64 LU of A, its inverse and the subspace iteration on the
//    inverse (sigma_single: products over the whole GPU), iterated to rounding;
//  * with u = A x, u1 = A' x, u2 = A'' x: G' x = A'^H u + A^H u1 and
//    x^H G'' x = 2 Re(u2^H u) + 2 |u1|^2 (matrix-vector products only);
//  * the eigen-sum is -b^H y with b = G' x - lambda1 x and y the solution of
//    (G - lambda I + mu x x^H) y = b (mu = trace(G) / n): b has no x
//    component, so y = sum_{j != min} v_j (v_j^H b) / (lambda_j - lambda);
//    G = A^H A is formed once per step and factored by the library's LU.
// The reference's skip of terms with |lambda - lambda_j| < eps has no
// counterpart (a numerically degenerate pair makes either form blow up).
// Steps, clamping, stopping rules and the best-k fallback are the reference's.
// ---------------------------------------------------------------------------
struct Newton {
  Ebim E;
  Dense64 DM;  // LU of the deflated shift M
  cxd *Ac = nullptr, *G = nullptr, *M = nullptr, *Cinv = nullptr, *CH = nullptr, *X0 = nullptr, *Xb = nullptr,
      *Wb = nullptr, *Yb = nullptr, *Ps = nullptr, *xv = nullptr, *u = nullptr, *u1 = nullptr, *u2 = nullptr,
      *gx = nullptr, *bv = nullptr, *yv = nullptr;
  double* state = nullptr;
  cxd* dks = nullptr;
  void** dptrs = nullptr;
  ~Newton() {
    if (E.st) cudaStreamSynchronize(E.st);
    DM.release();
  }
};

struct NewtonEval {
  double lam = 0.0, l1 = 0.0, l2 = 0.0;
};

int newton_eval(qbg_geom* g, Newton& W, double k, bool derivs, NewtonEval& out) {
  Ebim& E = W.E;
  const int n = E.n;
  const cxd kk(k, 0.0);
  void* hp[3] = {W.Ac, E.dA, E.ddA};
  QBG_CUDA(cudaMemcpyAsync(W.dks, &kk, sizeof(cxd), cudaMemcpyHostToDevice, E.st));
  QBG_CUDA(cudaMemcpyAsync(W.dptrs, hp, sizeof(hp), cudaMemcpyHostToDevice, E.st));
  QBG_TRY(launch_assemble(g->d, W.dks, 1, derivs ? 1 : 0, QBG_PREC_FP64, W.dptrs, n, E.st));
  const size_t nn = (size_t)n * n;
  QBG_CUDA(cudaMemcpyAsync(E.LU, W.Ac, sizeof(cxd) * nn, cudaMemcpyDeviceToDevice, E.st));
  std::vector<int> info;
  QBG_TRY(E.D.factor(&info));  // synchronizes: k and the pointer table are staged from this frame
  double sig = 0.0;
  if (info[0] > 0) {
    out.lam = 0.0;  // A(k) exactly singular: sigma_min = 0
    if (!derivs) return QBG_OK;
    set_error("Newton refinement: A(k) is exactly singular at k = %.17g", k);
    return QBG_ESINGULAR;
  }
  QBG_TRY(E.D.inverse(W.Cinv));
  QBG_TRY(sigma_single(W.Cinv, W.CH, n, W.X0, W.Xb, W.Wb, W.Yb, W.Ps, W.state, 64, 1e-15, &sig,
                       derivs ? W.xv : nullptr, E.st));
  if (!derivs) {
    out.lam = sig * sig;
    return QBG_OK;
  }
  const cxd one(1, 0), zero(0, 0);
  QBG_TRY(gemm_batched<double>(n, 1, n, one, W.Ac, n, 0, W.xv, n, 0, zero, W.u, n, 0, 1, E.st));     // A x
  QBG_TRY(gemm_batched<double>(n, 1, n, one, E.dA, n, 0, W.xv, n, 0, zero, W.u1, n, 0, 1, E.st));    // A' x
  QBG_TRY(gemm_batched<double>(n, 1, n, one, E.ddA, n, 0, W.xv, n, 0, zero, W.u2, n, 0, 1, E.st));   // A'' x
  QBG_TRY(gemm_batched_ah<double>(n, 1, n, one, E.dA, n, 0, W.u, n, 0, zero, W.gx, n, 0, 1, E.st));  // A'^H A x
  QBG_TRY(gemm_batched_ah<double>(n, 1, n, one, W.Ac, n, 0, W.u1, n, 0, one, W.gx, n, 0, 1, E.st));  // + A^H A' x
  QBG_TRY(gemm_batched_ah<double>(n, n, n, one, W.Ac, n, 0, W.Ac, n, 0, zero, W.G, n, 0, 1, E.st));  // G = A^H A
  std::vector<cxd> hx(n), hu(n), h1(n), h2(n), hg(n), hd(n);
  QBG_CUDA(cudaMemcpyAsync(hx.data(), W.xv, sizeof(cxd) * n, cudaMemcpyDeviceToHost, E.st));
  QBG_CUDA(cudaMemcpyAsync(hu.data(), W.u, sizeof(cxd) * n, cudaMemcpyDeviceToHost, E.st));
  QBG_CUDA(cudaMemcpyAsync(h1.data(), W.u1, sizeof(cxd) * n, cudaMemcpyDeviceToHost, E.st));
  QBG_CUDA(cudaMemcpyAsync(h2.data(), W.u2, sizeof(cxd) * n, cudaMemcpyDeviceToHost, E.st));
  QBG_CUDA(cudaMemcpyAsync(hg.data(), W.gx, sizeof(cxd) * n, cudaMemcpyDeviceToHost, E.st));
  QBG_CUDA(cudaMemcpy2DAsync(hd.data(), sizeof(cxd), W.G, sizeof(cxd) * (n + 1), sizeof(cxd), n,
                             cudaMemcpyDeviceToHost, E.st));  // diag(G)
  QBG_TRY(E.wait());
  const double lam = sig * sig;
  double l1 = 0.0, g2 = 0.0, tr = 0.0;
  for (int r = 0; r < n; ++r) {
    l1 += hx[r].re * hg[r].re + hx[r].im * hg[r].im;                           // Re(x^H G' x)
    g2 += 2.0 * (h2[r].re * hu[r].re + h2[r].im * hu[r].im) + 2.0 * cabs2(h1[r]);  // x^H G'' x
    tr += hd[r].re;
  }
  std::vector<cxd> hb(n);
  for (int r = 0; r < n; ++r) hb[r] = cxd(hg[r].re - l1 * hx[r].re, hg[r].im - l1 * hx[r].im);
  const double mu = tr > 0.0 ? tr / n : 1.0;
  QBG_TRY(deflate_shift(W.G, W.xv, n, lam, mu, W.M, E.st));
  std::vector<int> infm;
  QBG_TRY(W.DM.factor(&infm));
  if (infm[0] > 0) {
    set_error("Newton refinement: G - lambda I + mu x x^H is singular (a repeated smallest eigenvalue)");
    return QBG_ESINGULAR;
  }
  QBG_CUDA(cudaMemcpyAsync(W.bv, hb.data(), sizeof(cxd) * n, cudaMemcpyHostToDevice, E.st));
  QBG_TRY(lu_solve_shared<double>(W.DM.f, W.bv, 1, W.yv, 0, E.st));
  std::vector<cxd> hy(n);
  QBG_CUDA(cudaMemcpyAsync(hy.data(), W.yv, sizeof(cxd) * n, cudaMemcpyDeviceToHost, E.st));
  QBG_TRY(E.wait());
  double s2 = 0.0;
  for (int r = 0; r < n; ++r) s2 += hb[r].re * hy[r].re + hb[r].im * hy[r].im;  // Re(b^H y)
  out.lam = lam;
  out.l1 = l1;
  out.l2 = g2 - 2.0 * s2;
  return QBG_OK;
}

qbg_status newton_impl(qbg_geom* g, double k0, double a, double b, int maxiter, double tol, double* k_out,
                       double* t_out, int32_t* iters) {
  Newton W;
  Ebim& E = W.E;
  const int n = (int)g->dim;
  QBG_TRY(ebim_setup(E, n));
  cudaEvent_t ev_in = nullptr;
  QBG_CUDA(cudaEventCreateWithFlags(&ev_in, cudaEventDisableTiming));
  cudaError_t e = cudaEventRecord(ev_in, g->stream);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(E.st, ev_in, 0);
  cudaEventDestroy(ev_in);
  if (e != cudaSuccess) return cuda_status(e, "Newton stream order");
  const size_t bytes = sizeof(cxd) * (size_t)n * n;
  for (cxd** q : {&E.LU, &E.dA, &E.ddA, &W.Ac, &W.G, &W.M, &W.Cinv, &W.CH}) QBG_TRY(E.alloc(q, bytes));
  for (cxd** q : {&W.xv, &W.u, &W.u1, &W.u2, &W.gx, &W.bv, &W.yv}) QBG_TRY(E.alloc(q, sizeof(cxd) * n));
  for (cxd** q : {&W.X0, &W.Xb, &W.Wb, &W.Yb}) QBG_TRY(E.alloc(q, sizeof(cxd) * (size_t)n * DENSE_P));
  QBG_TRY(E.alloc(&W.Ps, sizeof(cxd) * std::max<size_t>(tall_scratch(n, DENSE_P), 1)));
  QBG_TRY(E.alloc(&W.state, sizeof(double) * (2 + 2 * DENSE_P)));
  QBG_TRY(E.alloc(&W.dks, sizeof(cxd)));
  QBG_TRY(E.alloc(&W.dptrs, sizeof(void*) * 3));
  QBG_TRY(E.D.bind(E.LU, n, 1, E.st));
  QBG_TRY(W.DM.bind(W.M, n, 1, E.st));
  {
    std::vector<cxd> hx0;
    dense_start_block(n, hx0);
    QBG_CUDA(cudaMemcpyAsync(W.X0, hx0.data(), sizeof(cxd) * hx0.size(), cudaMemcpyHostToDevice, E.st));
  }
  double k = std::min(std::max(k0, a), b), kbest = k, lbest = INFINITY;
  int it = 0;
  const double eps = 2.220446049250313e-16;
  NewtonEval ev;
  for (; it < maxiter; ++it) {
    QBG_TRY(newton_eval(g, W, k, true, ev));
    if (std::isfinite(ev.lam) && ev.lam < lbest) {
      lbest = ev.lam;
      kbest = k;
    }
    const double l1 = ev.l1, l2 = ev.l2;
    if (!std::isfinite(l1) || !std::isfinite(l2) || std::fabs(l2) < std::sqrt(eps)) break;
    const double knew = std::min(std::max(k - l1 / l2, a), b);
    if (!std::isfinite(knew)) break;
    if (std::fabs(knew - k) < tol) {
      k = knew;
      ++it;
      break;
    }
    k = knew;
  }
  QBG_TRY(newton_eval(g, W, k, false, ev));
  double lmin = ev.lam;
  if (!(std::isfinite(lmin) && lmin <= lbest)) {
    k = kbest;
    QBG_TRY(newton_eval(g, W, k, false, ev));
    lmin = ev.lam;
  }
  *k_out = k;
  *t_out = std::sqrt(std::max(0.0, lmin));
  if (iters) *iters = it;
  return QBG_OK;
}

// Assembles the DLP Fredholm matrix at real k into E.LU and overwrites E.C
// with its adjoint form (both m x m).
int adjoint_into(qbg_geom* g, Ebim& E, double k, const double* ds_host) {
  const int m = E.n, n = (int)g->d.n;
  cxd* dks = nullptr;
  void** dptrs = nullptr;
  double* dds = nullptr;
  QBG_TRY(E.alloc(&dks, sizeof(cxd)));
  QBG_TRY(E.alloc(&dptrs, sizeof(void*)));
  QBG_TRY(E.alloc(&dds, sizeof(double) * n));
  const cxd kk(k, 0.0);
  void* hp[1] = {E.LU};
  QBG_CUDA(cudaMemcpyAsync(dks, &kk, sizeof(cxd), cudaMemcpyHostToDevice, E.st));
  QBG_CUDA(cudaMemcpyAsync(dptrs, hp, sizeof(hp), cudaMemcpyHostToDevice, E.st));
  QBG_CUDA(cudaMemcpyAsync(dds, ds_host, sizeof(double) * n, cudaMemcpyHostToDevice, E.st));
  QBG_TRY(launch_assemble(g->d, dks, 1, 0, QBG_PREC_FP64, dptrs, m, E.st));
  k_adjoint_fredholm<<<dim3((m + 31) / 32, (m + 31) / 32), dim3(32, 8), 0, E.st>>>(
      E.LU, dds, g->d.m != g->d.n ? g->d.fund : nullptr, m, E.C);
  QBG_LAUNCH_CHECK("k_adjoint_fredholm");
  return E.wait();  // k, the pointer table and ds are staged from this frame
}

int adjoint_setup(qbg_geom* g, Ebim& E) {
  if (g->d.form != 0 || g->d.quad != 0) {
    set_error("the adjoint Fredholm matrix is defined for the DLP Kress formulation");
    return QBG_ENOTSUP;
  }
  QBG_TRY(ebim_setup(E, (int)g->dim));
  cudaEvent_t ev_in = nullptr;
  QBG_CUDA(cudaEventCreateWithFlags(&ev_in, cudaEventDisableTiming));
  cudaError_t e = cudaEventRecord(ev_in, g->stream);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(E.st, ev_in, 0);
  cudaEventDestroy(ev_in);
  if (e != cudaSuccess) return cuda_status(e, "adjoint stream order");
  const size_t bytes = sizeof(cxd) * (size_t)E.n * E.n;
  QBG_TRY(E.alloc(&E.LU, bytes));
  QBG_TRY(E.alloc(&E.C, bytes));
  return QBG_OK;
}

qbg_status qbg_small_eig(int32_t p, const double* H, double* w, double* V) {
  if (p < 1 || p > 4096 || !H || !w || !V) {
    set_error("qbg_small_eig: invalid arguments");
    return QBG_EINVAL;
  }
  std::vector<zc> Hz((size_t)p * p), wz, Vz;
  for (size_t i = 0; i < Hz.size(); ++i) Hz[i] = zc(H[2 * i], H[2 * i + 1]);
  QBG_TRY(small_eig(p, Hz, wz, Vz));
  for (int i = 0; i < p; ++i) {
    w[2 * i] = wz[i].real();
    w[2 * i + 1] = wz[i].imag();
  }
  for (size_t i = 0; i < Vz.size(); ++i) {
    V[2 * i] = Vz[i].real();
    V[2 * i + 1] = Vz[i].imag();
  }
  return QBG_OK;
}

qbg_status qbg_newton_refine(qbg_geom* g, double k0, double a, double b, int32_t maxiter, double tol,
                             double* k_out, double* t_out, int32_t* iters) {
  if (!g || !k_out || !t_out || !std::isfinite(k0) || !(a <= b) || maxiter < 0 || !(tol >= 0.0)) {
    set_error("qbg_newton_refine: invalid arguments");
    return QBG_EINVAL;
  }
  std::lock_guard<std::mutex> lk(g->mu);
  return newton_impl(g, k0, a, b, maxiter, tol, k_out, t_out, iters);
}

qbg_status qbg_adjoint_fredholm(qbg_geom* g, double k, const double* ds, void* out, int32_t flags) {
  if (!g || !ds || !out || !std::isfinite(k) || !(k > 0.0)) {
    set_error("qbg_adjoint_fredholm: invalid arguments");
    return QBG_EINVAL;
  }
  std::lock_guard<std::mutex> lk(g->mu);
  Ebim E;
  QBG_TRY(adjoint_setup(g, E));
  QBG_TRY(adjoint_into(g, E, k, ds));
  const size_t bytes = sizeof(cxd) * (size_t)E.n * E.n;
  QBG_CUDA(cudaMemcpyAsync(out, E.C, bytes, (flags & QBG_PTR_DEVICE) ? cudaMemcpyDeviceToDevice
                                                                     : cudaMemcpyDeviceToHost, E.st));
  return E.wait();
}

qbg_status qbg_solve_vect(qbg_geom* g, double k, const double* ds, double* sigma, double* u) {
  if (!g || !ds || !sigma || !u || !std::isfinite(k) || !(k > 0.0)) {
    set_error("qbg_solve_vect: invalid arguments");
    return QBG_EINVAL;
  }
  std::lock_guard<std::mutex> lk(g->mu);
  Ebim E;
  QBG_TRY(adjoint_setup(g, E));
  QBG_TRY(adjoint_into(g, E, k, ds));
  const int n = E.n;
  // LU of the adjoint matrix (in E.LU), then C = A^-1 for the block iteration
  QBG_CUDA(cudaMemcpyAsync(E.LU, E.C, sizeof(cxd) * (size_t)n * n, cudaMemcpyDeviceToDevice, E.st));
  QBG_TRY(E.factor("solve_vect: the adjoint Fredholm matrix"));
  QBG_TRY(E.D.inverse(E.C));
  // the eigenvalue of largest modulus of A^-1 (smallest_nullvec_krylov!, dlp.jl:991-1004)
  const int nev = 1, p = std::min(n, 12);
  std::vector<zc> mu;
  cxd* V = nullptr;
  int it = 0;
  QBG_TRY(E.alloc(&V, sizeof(cxd) * (size_t)n));
  QBG_TRY(block_eigs(E, false, p, nev, mu, V, &it, INFINITY));
  std::vector<cxd> hv(n);
  QBG_CUDA(cudaMemcpyAsync(hv.data(), V, sizeof(cxd) * n, cudaMemcpyDeviceToHost, E.st));
  QBG_TRY(E.wait());
  double nrm = 0.0;
  for (const cxd& x : hv) nrm += x.re * x.re + x.im * x.im;
  nrm = std::sqrt(nrm);
  for (int i = 0; i < n; ++i) {
    u[2 * i] = hv[i].re / nrm;
    u[2 * i + 1] = hv[i].im / nrm;
  }
  *sigma = 1.0 / std::abs(mu[0]);
  return QBG_OK;
}

qbg_status qbg_ebim_solve(qbg_geom* g, double k, double dk, int32_t nev, int32_t flags, int32_t cap, double* out_k,
                          double* out_tens, int32_t* count, int32_t* iters) {
  if (!g || !ebim_args_ok(k, dk, nev, cap, out_k, out_tens, count) || !(k > 0.0)) {
    set_error("qbg_ebim_solve: invalid arguments");
    return QBG_EINVAL;
  }
  std::lock_guard<std::mutex> lk(g->mu);
  Ebim E;
  const int n = (int)g->dim;
  QBG_TRY(ebim_setup(E, n));
  // after the geometry stream's earlier work (its uploads)
  cudaEvent_t ev_in = nullptr;
  QBG_CUDA(cudaEventCreateWithFlags(&ev_in, cudaEventDisableTiming));
  cudaError_t e = cudaEventRecord(ev_in, g->stream);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(E.st, ev_in, 0);
  cudaEventDestroy(ev_in);
  if (e != cudaSuccess) return cuda_status(e, "EBIM stream order");
  const size_t bytes = sizeof(cxd) * (size_t)n * n;
  QBG_TRY(E.alloc(&E.LU, bytes));
  QBG_TRY(E.alloc(&E.dA, bytes));
  QBG_TRY(E.alloc(&E.ddA, bytes));
  cxd* dks = nullptr;
  void** dptrs = nullptr;
  QBG_TRY(E.alloc(&dks, sizeof(cxd)));
  QBG_TRY(E.alloc(&dptrs, sizeof(void*) * 3));
  const cxd kk(k, 0.0);
  void* hp[3] = {E.LU, E.dA, E.ddA};
  QBG_CUDA(cudaMemcpyAsync(dks, &kk, sizeof(cxd), cudaMemcpyHostToDevice, E.st));
  QBG_CUDA(cudaMemcpyAsync(dptrs, hp, sizeof(hp), cudaMemcpyHostToDevice, E.st));
  QBG_TRY(launch_assemble(g->d, dks, 1, 1, QBG_PREC_FP64, dptrs, n, E.st));
  QBG_TRY(E.wait());  // the host staging of k and the pointers is on this frame
  return ebim_run(E, k, dk, nev, flags, cap, out_k, out_tens, count, iters);
}

}  // extern "C"
