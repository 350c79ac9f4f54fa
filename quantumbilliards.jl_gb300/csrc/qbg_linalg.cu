// Batched complex LU with partial pivoting, blocked triangular solves with a
// probe block shared by the batch, contour moments and the mixed-form
// refinement residual.
//
// Algorithm (right-looking blocked LU, the same factorisation LAPACK zgetrf
// computes; the reference calls lu!(T; check=false), beyn.jl:270-277):
//   for each block column [j0, j0+nb):
//     1. k_getf2_panel   one CTA per matrix factors the n-j0 x nb panel
//                        column by column (pivot = first max of |re|+|im|,
//                        as izamax); zero pivots are recorded in info and
//                        skipped, matching check=false.
//     2. k_laswp         applies the panel's row interchanges to the columns
//                        left and right of the panel.
//     3. k_trtri         inverts the unit-lower diagonal block L11.
//     4. gemm            U12 = inv(L11) A12   (in place, one M tile)
//     5. gemm            A22 -= L21 U12       (trailing update)
//   After the last panel the upper diagonal blocks are inverted so that the
//   triangular solves are sequences of GEMMs.
#include <atomic>
#include <algorithm>
#include <cooperative_groups.h>
#include <cstdlib>
#include <type_traits>
#include "qbg_linalg.cuh"
#include "qbg_handles.cuh"

namespace qbg {

// ---------------------------------------------------------------------------
// batched complex GEMM  C = alpha A B + beta C   (column-major)
// 64 x 64 tile, K step 16, 256 threads, 4 x 4 outputs per thread.
// Thread (tx, ty): rows tx + 16 a, columns ty + 16 b, so that the 16 lanes
// with consecutive tx store 16 consecutive rows of a column.
// Safe for C == B when one M tile covers all of K (used for inv(L11) A12).
// CA: the A operand is the conjugate transpose of the K x M block stored at A
// (leading dimension lda), op(A)[i, k] = conj(A[k + i lda]).
// ---------------------------------------------------------------------------
// One 64 x 64 tile of op(A) B over k in [kb, ke) accumulated in acc (the
// thread's 4 x 4 outputs); Ab, Bb point at the batch entry.
template <class T, bool CA>
__device__ __forceinline__ void gemm_tile(int M, int N, int K, int kb, int ke, const cx<T>* __restrict__ Ab,
                                          long long lda, const cx<T>* Bb, long long ldb, int m0, int n0,
                                          cx<T> (&acc)[4][4]) {
  constexpr int BM = 64, BN = 64, BK = 16;
  __shared__ cx<T> As[BK][BM];
  __shared__ cx<T> Bs[BK][BN + 1];
  const int tid = threadIdx.x;
  const int tx = tid & 15, ty = tid >> 4;
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) acc[a][b] = cx<T>(0, 0);
  for (int k0 = kb; k0 < ke; k0 += BK) {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int idx = tid + q * 256;
      if (CA) {  // consecutive threads walk k, the contiguous index of the stored block
        const int kk = idx & (BK - 1), i = idx >> 4;
        const int gi = m0 + i, gk = k0 + kk;
        As[kk][i] = (gi < M && gk < ke) ? conj(Ab[(long long)gk + (long long)gi * lda]) : cx<T>(0, 0);
      } else {
        const int i = idx & (BM - 1), kk = idx >> 6;
        const int gi = m0 + i, gk = k0 + kk;
        As[kk][i] = (gi < M && gk < ke) ? Ab[(long long)gi + (long long)gk * lda] : cx<T>(0, 0);
      }
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int idx = tid + q * 256;
      const int kk = idx & (BK - 1), jj = idx >> 4;
      const int gk = k0 + kk, gj = n0 + jj;
      Bs[kk][jj] = (gk < ke && gj < N) ? Bb[(long long)gk + (long long)gj * ldb] : cx<T>(0, 0);
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < BK; ++kk) {
      cx<T> ar[4], br[4];
#pragma unroll
      for (int a = 0; a < 4; ++a) ar[a] = As[kk][tx + 16 * a];
#pragma unroll
      for (int b = 0; b < 4; ++b) br[b] = Bs[kk][ty + 16 * b];
#pragma unroll
      for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) cfma(acc[a][b], ar[a], br[b]);
    }
    __syncthreads();
  }
  (void)K;
}

template <class T, bool CA = false>
__global__ void __launch_bounds__(256) k_gemm(int M, int N, int K, cx<T> alpha, const cx<T>* __restrict__ A,
                                              long long lda, long long sA, const cx<T>* B, long long ldb,
                                              long long sB, cx<T> beta, cx<T>* C, long long ldc, long long sC) {
  const int tid = threadIdx.x;
  const int tx = tid & 15, ty = tid >> 4;
  const int m0 = blockIdx.x * 64, n0 = blockIdx.y * 64;
  const long long bz = blockIdx.z;
  cx<T>* Cb = C + bz * sC;
  cx<T> acc[4][4];
  gemm_tile<T, CA>(M, N, K, 0, K, A + bz * sA, lda, B + bz * sB, ldb, m0, n0, acc);
  const bool use_beta = !(beta.re == T(0) && beta.im == T(0));
#pragma unroll
  for (int b = 0; b < 4; ++b) {
    const int gj = n0 + ty + 16 * b;
    if (gj >= N) continue;
#pragma unroll
    for (int a = 0; a < 4; ++a) {
      const int gi = m0 + tx + 16 * a;
      if (gi >= M) continue;
      cx<T>* c = Cb + (long long)gi + (long long)gj * ldc;
      cx<T> v = alpha * acc[a][b];
      if (use_beta) v += beta * (*c);
      *c = v;
    }
  }
}

// Split-K partial products in one launch: z = b * ns + q computes
// P[q, b] = op(A_b) B_b over k in [q kc, min(K, (q + 1) kc)).
template <class T, bool CA>
__global__ void __launch_bounds__(256) k_gemm_sk(int M, int N, int K, int kc, int ns, const cx<T>* __restrict__ A,
                                                 long long lda, long long sA, const cx<T>* B, long long ldb,
                                                 long long sB, cx<T>* P, int batch) {
  const int tid = threadIdx.x;
  const int tx = tid & 15, ty = tid >> 4;
  const int m0 = blockIdx.x * 64, n0 = blockIdx.y * 64;
  const long long b = blockIdx.z / ns, q = blockIdx.z % ns;
  const int kb = (int)q * kc, ke = min(K, kb + kc);
  cx<T> acc[4][4];
  gemm_tile<T, CA>(M, N, K, kb, ke, A + b * sA, lda, B + b * sB, ldb, m0, n0, acc);
  cx<T>* Pq = P + (q * batch + b) * (long long)M * N;
#pragma unroll
  for (int bb = 0; bb < 4; ++bb) {
    const int gj = n0 + ty + 16 * bb;
    if (gj >= N) continue;
#pragma unroll
    for (int a = 0; a < 4; ++a) {
      const int gi = m0 + tx + 16 * a;
      if (gi < M) Pq[(long long)gi + (long long)gj * M] = acc[a][bb];
    }
  }
}

// C = alpha sum_s P_s + beta C over the split-K partial products P_s (s
// slices of M x N, column-major, stride M N), summed in slice order
template <class T>
__global__ void k_splitk_sum(const cx<T>* __restrict__ P, int splits, int M, int N, int batch, cx<T> alpha, cx<T> beta,
                             cx<T>* C, long long ldc, long long sC) {
  const long long mn = (long long)M * N, total = mn * batch;
  const bool use_beta = !(beta.re == T(0) && beta.im == T(0));
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total; e += (long long)gridDim.x * blockDim.x) {
    const long long b = e / mn, r = e % mn;
    const int i = (int)(r % M), j = (int)(r / M);
    cx<T> v(0, 0);
    for (int q = 0; q < splits; ++q) v += P[((long long)q * batch + b) * mn + r];
    cx<T>* c = C + b * sC + (long long)i + (long long)j * ldc;
    v = alpha * v;
    if (use_beta) v += beta * (*c);
    *c = v;
  }
}

// FP64 on this part is ~2 FMA per clock per SM: a 64 x 64 tile with K = 256
// is ~1 ms of one SM's FP64 pipe, so a complex128 product with fewer tiles
// than SMs is split over K into slices of at least 16 (about two CTAs per
// SM); the partial products are summed in a fixed order by a second kernel,
// so the result does not depend on scheduling. Returns false when the
// product is left to the plain launch.
template <class T, bool CA>
static bool gemm_split_k(int M, int N, int K, cx<T> alpha, const cx<T>* A, long long lda, long long sA,
                         const cx<T>* B, long long ldb, long long sB, cx<T> beta, cx<T>* C, long long ldc,
                         long long sC, int batch, cudaStream_t st, int* status) {
  const long long tiles = (long long)((M + 63) / 64) * ((N + 63) / 64) * batch;
  if (sizeof(T) != 8 || tiles >= 152 || K < 64 || (long long)batch * 16 > 65535) return false;
  const int splits = (int)std::min<long long>(std::min<long long>((304 + tiles - 1) / tiles, K / 16), 16);
  if (splits < 2) return false;
  const int kc = ((K + splits - 1) / splits + 15) / 16 * 16;
  const int ns = (K + kc - 1) / kc;
  cx<T>* P = nullptr;
  if ((*status = dmalloc(&P, sizeof(cx<T>) * (size_t)ns * batch * M * N))) return true;
  {
    dim3 grd((M + 63) / 64, (N + 63) / 64, batch * ns);
    k_gemm_sk<T, CA><<<grd, 256, 0, st>>>(M, N, K, kc, ns, A, lda, sA, B, ldb, sB, P, batch);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
      *status = cuda_status(e, "k_gemm_sk");
      dfree(P, st);
      return true;
    }
  }
  const long long total = (long long)M * N * batch;
  k_splitk_sum<T><<<(unsigned)std::min<long long>((total + 255) / 256, 4096), 256, 0, st>>>(P, ns, M, N, batch, alpha,
                                                                                         beta, C, ldc, sC);
  const cudaError_t e = cudaGetLastError();
  *status = e == cudaSuccess ? QBG_OK : cuda_status(e, "k_splitk_sum");
  dfree(P, st);
  return true;
}

template <class T>
int gemm_batched_simt(int M, int N, int K, cx<T> alpha, const cx<T>* A, long long lda, long long sA, const cx<T>* B,
                      long long ldb, long long sB, cx<T> beta, cx<T>* C, long long ldc, long long sC, int batch,
                      cudaStream_t st) {
  if (M <= 0 || N <= 0 || batch <= 0) return QBG_OK;
  int status = QBG_OK;
  if (gemm_split_k<T, false>(M, N, K, alpha, A, lda, sA, B, ldb, sB, beta, C, ldc, sC, batch, st, &status))
    return status;
  dim3 grd((M + 63) / 64, (N + 63) / 64, batch);
  k_gemm<T><<<grd, 256, 0, st>>>(M, N, K, alpha, A, lda, sA, B, ldb, sB, beta, C, ldc, sC);
  QBG_LAUNCH_CHECK("k_gemm");
  return QBG_OK;
}

// C = alpha A^H B + beta C, A^H of the K x M blocks stored at A (CUDA-core tiles)
template <class T>
int gemm_batched_ah(int M, int N, int K, cx<T> alpha, const cx<T>* A, long long lda, long long sA,
                           const cx<T>* B, long long ldb, long long sB, cx<T> beta, cx<T>* C, long long ldc,
                           long long sC, int batch, cudaStream_t st) {
  if (M <= 0 || N <= 0 || batch <= 0) return QBG_OK;
  int status = QBG_OK;
  if (gemm_split_k<T, true>(M, N, K, alpha, A, lda, sA, B, ldb, sB, beta, C, ldc, sC, batch, st, &status))
    return status;
  dim3 grd((M + 63) / 64, (N + 63) / 64, batch);
  k_gemm<T, true><<<grd, 256, 0, st>>>(M, N, K, alpha, A, lda, sA, B, ldb, sB, beta, C, ldc, sC);
  QBG_LAUNCH_CHECK("k_gemm (A^H)");
  return QBG_OK;
}

template <class T>
int gemm_batched(int M, int N, int K, cx<T> alpha, const cx<T>* A, long long lda, long long sA, const cx<T>* B,
                 long long ldb, long long sB, cx<T> beta, cx<T>* C, long long ldc, long long sC, int batch,
                 cudaStream_t st) {
  if (M <= 0 || N <= 0 || batch <= 0) return QBG_OK;
  if constexpr (std::is_same<T, float>::value) {
    if (K > 0 && gemm_engine() == GEMM_ENGINE_TCGEN05)
      return tc_gemm_c64(M, N, K, alpha, A, lda, sA, B, ldb, sB, beta, C, ldc, sC, batch, st);
  }
  return gemm_batched_simt<T>(M, N, K, alpha, A, lda, sA, B, ldb, sB, beta, C, ldc, sC, batch, st);
}

// ---------------------------------------------------------------------------
// panel factorisation (one CTA per matrix)
// ---------------------------------------------------------------------------
template <class T>
__device__ __forceinline__ void argmax_merge(T& v, int& i, T ov, int oi) {
  if (ov > v || (ov == v && oi < i)) {
    v = ov;
    i = oi;
  }
}

template <class T>
__global__ void __launch_bounds__(512) k_getf2_panel(cx<T>* A, int n, long long stride, int j0, int nb,
                                                     int* ipiv, int* info) {
  cx<T>* a = A + (long long)blockIdx.x * stride;
  int* piv = ipiv + (long long)blockIdx.x * n;
  __shared__ cx<T> urow[64];
  __shared__ T wv[16];
  __shared__ int wi[16];
  __shared__ int s_p;
  const int tid = threadIdx.x, nt = blockDim.x;
  const int jend = min(j0 + nb, n);
  for (int c = j0; c < jend; ++c) {
    cx<T>* col = a + (long long)c * n;
    T best = T(-1);
    int bi = 0x7fffffff;
    for (int r = c + tid; r < n; r += nt) {
      T v = cabs1(col[r]);
      if (v > best) { best = v; bi = r; }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      T ov = __shfl_down_sync(0xffffffffu, best, o);
      int oi = __shfl_down_sync(0xffffffffu, bi, o);
      argmax_merge(best, bi, ov, oi);
    }
    if ((tid & 31) == 0) { wv[tid >> 5] = best; wi[tid >> 5] = bi; }
    __syncthreads();
    if (tid < 32) {
      const int nw = nt >> 5;
      best = (tid < nw) ? wv[tid] : T(-1);
      bi = (tid < nw) ? wi[tid] : 0x7fffffff;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        T ov = __shfl_down_sync(0xffffffffu, best, o);
        int oi = __shfl_down_sync(0xffffffffu, bi, o);
        argmax_merge(best, bi, ov, oi);
      }
      if (tid == 0) {
        if (bi >= n) bi = c;
        s_p = bi;
        piv[c] = bi;
        if (!(best > T(0)) && info[blockIdx.x] == 0) info[blockIdx.x] = c + 1;
      }
    }
    __syncthreads();
    const int p = s_p;
    if (p != c) {
      for (int cc = j0 + tid; cc < jend; cc += nt) {
        cx<T> t0 = a[c + (long long)cc * n];
        a[c + (long long)cc * n] = a[p + (long long)cc * n];
        a[p + (long long)cc * n] = t0;
      }
    }
    __syncthreads();
    const cx<T> pv = col[c];
    const int nrem = jend - c - 1;
    if (tid < nrem) urow[tid] = a[c + (long long)(c + 1 + tid) * n];
    __syncthreads();
    const bool nz = (pv.re != T(0) || pv.im != T(0));
    const cx<T> inv = nz ? cinv(pv) : cx<T>(0, 0);
    for (int r = c + 1 + tid; r < n; r += nt) {
      cx<T> l = col[r];
      if (nz) {
        l = l * inv;
        col[r] = l;
      }
      for (int q = 0; q < nrem; ++q) cfms(a[r + (long long)(c + 1 + q) * n], l, urow[q]);
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// Panel factorisation with shared-memory sub-panels (one CTA per matrix).
// The panel [j0, jend) is factored in sub-panels of `sub` columns. A
// sub-panel (rows s0..n-1) is loaded into shared memory and factored column
// by column there: warp 0 finishes the block's pivot search, swaps the pivot
// row into place and publishes it; every thread then scales its rows, applies
// the rank-1 update and searches its rows of the next column (two block
// barriers per column). The sub-panel's interchanges reach the other panel
// columns afterwards as one composed permutation of at most 2 sub rows, and
// the rest of the panel is updated by one rank-`sub` step
// (U12 = inv(L11) A12 by forward substitution, A22 -= L21 U12). The factors
// and pivots are those of column-by-column partial pivoting (largest
// |re| + |im|, first index on ties; a zero pivot sets info and skips the
// scaling, as LAPACK's getf2 does).
// Dynamic smem: (n - j0) * sub * sizeof(cx<T>) (host picks sub so this fits).
// ---------------------------------------------------------------------------
template <class T>
__device__ __forceinline__ void warp_argmax(T& best, int& bi) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const T ov = __shfl_down_sync(0xffffffffu, best, o);
    const int oi = __shfl_down_sync(0xffffffffu, bi, o);
    argmax_merge(best, bi, ov, oi);
  }
}

// dst[c * ldd + i] = src[i + c * lds] for i < rows, c < cols (a column block
// from global to shared memory), eight columns at a time (four for
// complex128): a thread issues the loads of its row in those columns before it
// stores them, so that the loads
// overlap instead of each waiting for the previous shared-memory store, and
// no index is divided.
template <class T>
__device__ __forceinline__ void load_block(cx<T>* dst, int ldd, const cx<T>* src, long long lds, int rows, int cols,
                                           int tid, int nt) {
  constexpr int G = sizeof(T) == 4 ? 8 : 4;  // columns per group (registers)
  for (int c0 = 0; c0 < cols; c0 += G)
    for (int i = tid; i < rows; i += nt) {
      cx<T> v[G];
#pragma unroll
      for (int u = 0; u < G; ++u)
        if (c0 + u < cols) v[u] = src[i + (long long)(c0 + u) * lds];
#pragma unroll
      for (int u = 0; u < G; ++u)
        if (c0 + u < cols) dst[(c0 + u) * ldd + i] = v[u];
    }
}

// the reverse copy, shared to global memory
template <class T>
__device__ __forceinline__ void store_block(cx<T>* dst, long long ldd, const cx<T>* src, int lds, int rows, int cols,
                                            int tid, int nt) {
  for (int c = 0; c < cols; ++c)
    for (int i = tid; i < rows; i += nt) dst[i + (long long)c * ldd] = src[c * lds + i];
}

template <class T>
__global__ void __launch_bounds__(1024) k_getrf_panel_smem(cx<T>* A, int n, long long stride, int j0, int nb,
                                                          int sub, int* ipiv, int* info) {
  extern __shared__ unsigned char smraw[];
  cx<T>* S = reinterpret_cast<cx<T>*>(smraw);
  __shared__ T wv[32];
  __shared__ int wi[32];
  __shared__ cx<T> urow[8];        // pivot row of the current column on the sub-panel's columns
  __shared__ int spiv[8];          // the sub-panel's pivots (local rows)
  __shared__ int tpos[16], tsrc[16];  // rows moved by the sub-panel's interchanges: tpos[t] <- row tsrc[t]
  __shared__ int s_cnt;
  __shared__ cx<T> Us[8 * 64];     // U rows of the sub-panel on the remaining panel columns
  cx<T>* a = A + (long long)blockIdx.x * stride;
  int* piv = ipiv + (long long)blockIdx.x * n;
  const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, wid = tid >> 5, nw = nt >> 5;
  const int jend = min(j0 + nb, n);
  for (int s0 = j0; s0 < jend; s0 += sub) {
    const int w = min(sub, jend - s0);
    const int m = n - s0;  // rows held in smem
    load_block<T>(S, m, a + s0 + (long long)s0 * n, n, m, w, tid, nt);
    __syncthreads();
    T best = T(-1);
    int bi = 0x7fffffff;
    for (int r = tid; r < m; r += nt) {
      const T v = cabs1(S[r]);
      if (v > best) { best = v; bi = r; }
    }
    for (int c = 0; c < w; ++c) {
      warp_argmax(best, bi);
      if (lane == 0) { wv[wid] = best; wi[wid] = bi; }
      __syncthreads();  // partial maxima of column c; the update of column c - 1 is complete
      if (wid == 0) {
        best = (lane < nw) ? wv[lane] : T(-1);
        bi = (lane < nw) ? wi[lane] : 0x7fffffff;
        warp_argmax(best, bi);
        int p = __shfl_sync(0xffffffffu, bi, 0);
        const T pb = __shfl_sync(0xffffffffu, best, 0);
        if (p >= m) p = c;
        if (lane < w) {
          const cx<T> vp = S[lane * m + p];
          S[lane * m + p] = S[lane * m + c];
          S[lane * m + c] = vp;
          urow[lane] = vp;
        }
        if (lane == 0) {
          spiv[c] = p;
          piv[s0 + c] = s0 + p;
          if (!(pb > T(0)) && info[blockIdx.x] == 0) info[blockIdx.x] = s0 + c + 1;
        }
      }
      __syncthreads();  // pivot row in urow and in place
      const cx<T> pv = urow[c];
      const bool nz = (pv.re != T(0) || pv.im != T(0));
      const cx<T> inv = nz ? cinv(pv) : cx<T>(0, 0);
      const bool search = c + 1 < w;
      best = T(-1);
      bi = 0x7fffffff;
      for (int r = c + 1 + tid; r < m; r += nt) {
        cx<T> l = S[c * m + r];
        if (nz) {
          l = l * inv;
          S[c * m + r] = l;
        }
        for (int q = c + 1; q < w; ++q) cfms(S[q * m + r], l, urow[q]);
        if (search) {
          const T v = cabs1(S[(c + 1) * m + r]);
          if (v > best) { best = v; bi = r; }
        }
      }
    }
    if (tid == 0) {  // compose the sub-panel's interchanges
      int cnt = 0;
      for (int c = 0; c < w; ++c) {
        const int r1 = s0 + c, r2 = s0 + spiv[c];
        if (r1 == r2) continue;
        int i1 = -1, i2 = -1;
        for (int t = 0; t < cnt; ++t) {
          if (tpos[t] == r1) i1 = t;
          if (tpos[t] == r2) i2 = t;
        }
        if (i1 < 0) { tpos[cnt] = r1; tsrc[cnt] = r1; i1 = cnt++; }
        if (i2 < 0) { tpos[cnt] = r2; tsrc[cnt] = r2; i2 = cnt++; }
        const int t0 = tsrc[i1];
        tsrc[i1] = tsrc[i2];
        tsrc[i2] = t0;
      }
      s_cnt = cnt;
    }
    __syncthreads();  // sub-panel factored; permutation composed
    store_block<T>(a + s0 + (long long)s0 * n, n, S, m, m, w, tid, nt);
    // the interchanges on the other panel columns [j0, s0) and [s0 + w, jend):
    // whole columns per round, every read of a round before its writes
    const int cnt = s_cnt;
    const int nother = (s0 - j0) + (jend - s0 - w);
    if (cnt > 0) {
      const int per = nt / cnt;
      for (int q0 = 0; q0 < nother; q0 += per) {
        const int q = q0 + tid / cnt, t = tid % cnt;
        const bool act = tid < per * cnt && q < nother;
        cx<T> v(0, 0);
        cx<T>* pc = nullptr;
        if (act) {
          const int col = (q < s0 - j0) ? (j0 + q) : (s0 + w + (q - (s0 - j0)));
          pc = a + (long long)col * n;
          v = pc[tsrc[t]];
        }
        __syncthreads();
        if (act) pc[tpos[t]] = v;
        __syncthreads();
      }
    }
    // rank-w update of the rest of the panel: columns [s0 + w, jend)
    const int nr = jend - s0 - w;
    if (nr > 0) {
      // U12 = inv(L11) A12 : forward substitution, one thread per column
      for (int q = tid; q < nr; q += nt) {
        cx<T>* pc = a + (long long)(s0 + w + q) * n + s0;
        cx<T> x[8];
        for (int k = 0; k < w; ++k) {
          cx<T> v = pc[k];
          for (int l = 0; l < k; ++l) cfms(v, S[l * m + k], x[l]);
          x[k] = v;
          pc[k] = v;
          Us[k * 64 + q] = v;
        }
      }
      __syncthreads();
      // A22 -= L21 U12, one thread per row; the row's entries of CH columns are
      // loaded together before they are updated, so the global-memory latency
      // is paid once per CH columns instead of once per column (within the 64
      // registers a thread has at 1024 threads)
      constexpr int CH = sizeof(T) == 4 ? 8 : 4;
      for (int r = w + tid; r < m; r += nt) {
        cx<T> lr[8];
#pragma unroll
        for (int l = 0; l < 8; ++l) lr[l] = l < w ? S[l * m + r] : cx<T>(0, 0);
        cx<T>* pr = a + (s0 + r) + (long long)(s0 + w) * n;
        for (int q0 = 0; q0 < nr; q0 += CH) {
          cx<T> v[CH];
#pragma unroll
          for (int u = 0; u < CH; ++u)
            if (q0 + u < nr) v[u] = pr[(long long)(q0 + u) * n];
#pragma unroll
          for (int u = 0; u < CH; ++u)
            if (q0 + u < nr) {
#pragma unroll
              for (int l = 0; l < 8; ++l)
                if (l < w) cfms(v[u], lr[l], Us[l * 64 + q0 + u]);
              pr[(long long)(q0 + u) * n] = v[u];
            }
        }
      }
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// Panel factorisation on a cluster of PC_CS CTAs per matrix: the m x w panel
// (m = n - j0 rows, w <= 64 columns) is held in the CTAs' shared memory, rows
// in blocks of rpc = ceil(m / PC_CS) per CTA. One cluster barrier per column:
// before it, every CTA pushes into every CTA's shared memory its candidate
// (the largest |re| + |im| of the column over its rows at or below the
// diagonal, lowest row on ties, as izamax) together with that whole candidate
// row, and the owner of the diagonal row pushes the diagonal row; after it,
// every CTA picks the pivot from the eight candidates locally, so the pivot
// row and the displaced row are already on chip, the two owners write the
// interchange into their rows and every CTA scales and updates its own rows.
// The push buffers alternate between two copies by column parity: a CTA
// pushing column c + 1 writes the other copy than the one a slower CTA may
// still read for column c, and cannot reach column c + 2 before that CTA has
// passed the barrier of column c + 1. Same factors, pivots and info as
// k_getrf_panel_smem. (Measured on 2048 x 64 panels: 228 us with 256 threads
// per CTA; 1024 threads sharing each row's columns took 274 us, the per-thread
// pivot bookkeeping then outweighing the split update.)
// ---------------------------------------------------------------------------
constexpr int PC_THREADS = 256;
// largest rows per CTA: 64 columns within the dynamic shared memory left
// beside the push buffers, whose static size grows with the cluster: 8 CTAs
// 432 complex64 / 200 complex128 rows, 16 CTAs 416 / 192 rows
template <class T, int CS>
constexpr int pc_max_rpc() { return sizeof(T) == 4 ? (CS == 8 ? 432 : 416) : (CS == 8 ? 200 : 192); }

// CS = 8 (portable cluster size) or 16 (non-portable, for panels too tall for
// 8 CTAs' shared memory, used when the device can hold such a cluster)
template <class T, int CS>
__global__ void __cluster_dims__(CS, 1, 1) __launch_bounds__(PC_THREADS)
    k_getrf_panel_cluster(cx<T>* A, int n, long long stride, int j0, int nb, int rpc, int* ipiv, int* info) {
  constexpr int PC_CS = CS;
  namespace cg = cooperative_groups;
  cg::cluster_group cl = cg::this_cluster();
  extern __shared__ unsigned char smraw[];
  cx<T>* P = reinterpret_cast<cx<T>*>(smraw);  // column c of the own rows at P + c * rpc
  __shared__ cx<T> crow[2][PC_CS][64];  // candidate rows pushed by every CTA
  __shared__ cx<T> drow[2][64];         // the diagonal row, pushed by its owner
  __shared__ T cv[2][PC_CS];
  __shared__ int ci[2][PC_CS];
  __shared__ T wv[PC_THREADS / 32];
  __shared__ int wi[PC_THREADS / 32];
  __shared__ int s_bi;
  const int rank = (int)cl.block_rank();
  const int mat = blockIdx.x / PC_CS;
  cx<T>* a = A + (long long)mat * stride;
  int* piv = ipiv + (long long)mat * n;
  const int m = n - j0, w = min(nb, n - j0);
  const int r0 = rank * rpc;
  const int rows = max(0, min(rpc, m - r0));
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  load_block<T>(P, rpc, a + (j0 + r0) + (long long)j0 * n, n, rows, w, tid, PC_THREADS);
  __syncthreads();
  cl.sync();  // every CTA of the cluster runs before the first remote store
  for (int c = 0; c < w; ++c) {
    const int buf = c & 1;
    T best = T(-1);
    int bi = 0x7fffffff;
    for (int i = tid; i < rows; i += PC_THREADS) {
      const int pr = r0 + i;
      if (pr >= c) argmax_merge(best, bi, cabs1(P[c * rpc + i]), pr);
    }
    warp_argmax(best, bi);
    if (lane == 0) {
      wv[wid] = best;
      wi[wid] = bi;
    }
    __syncthreads();
    if (wid == 0) {
      best = lane < PC_THREADS / 32 ? wv[lane] : T(-1);
      bi = lane < PC_THREADS / 32 ? wi[lane] : 0x7fffffff;
      warp_argmax(best, bi);  // the result is in lane 0
      best = __shfl_sync(0xffffffffu, best, 0);
      bi = __shfl_sync(0xffffffffu, bi, 0);
      if (lane == 0) s_bi = bi;
      if (lane < PC_CS) {  // the candidate to CTA `lane`
        *cl.map_shared_rank(&cv[buf][rank], lane) = best;
        *cl.map_shared_rank(&ci[buf][rank], lane) = bi;
      }
    }
    __syncthreads();
    {
      const int mine = s_bi;  // the candidate row (global panel row), or none
      const int oc = c / rpc;
      for (int e = tid; e < PC_CS * w; e += PC_THREADS) {
        const int q = e / w, col = e % w;  // destination CTA, column
        if (mine < m) *cl.map_shared_rank(&crow[buf][rank][col], q) = P[col * rpc + (mine - r0)];
        if (rank == oc) *cl.map_shared_rank(&drow[buf][col], q) = P[col * rpc + (c - r0)];
      }
    }
    cl.sync();  // candidates, candidate rows and the diagonal row of column c everywhere
    T bv = T(-1);
    int p = 0x7fffffff, ps = 0;
#pragma unroll
    for (int q = 0; q < PC_CS; ++q) {
      const T v = cv[buf][q];
      const int ix = ci[buf][q];
      if (v > bv || (v == bv && ix < p)) {
        bv = v;
        p = ix;
        ps = q;
      }
    }
    if (p >= m) {  // no row at or below the diagonal compared (NaN column): no interchange
      p = c;
      ps = -1;
    }
    if (rank == 0 && tid == 0) {
      piv[j0 + c] = j0 + p;
      if (!(bv > T(0)) && info[mat] == 0) info[mat] = j0 + c + 1;
    }
    const cx<T>* prow = ps >= 0 ? crow[buf][ps] : drow[buf];  // the new row c
    if (p != c) {
      if (c >= r0 && c < r0 + rows)
        for (int q = tid; q < w; q += PC_THREADS) P[q * rpc + (c - r0)] = prow[q];
      if (p >= r0 && p < r0 + rows)
        for (int q = tid; q < w; q += PC_THREADS) P[q * rpc + (p - r0)] = drow[buf][q];
    }
    __syncthreads();
    const cx<T> pv = prow[c];
    const bool nz = (pv.re != T(0) || pv.im != T(0));
    if (nz) {  // multipliers of column c
      const cx<T> inv = cinv(pv);
      for (int i = tid; i < rows; i += PC_THREADS)
        if (r0 + i > c) P[c * rpc + i] = P[c * rpc + i] * inv;
      __syncthreads();
    }
    // rank-1 update of the trailing columns as (row, 8-column chunk) items
    // over all threads, so that short row blocks (small n, or 16 CTAs) still
    // keep every thread busy; a chunk goes through registers, its
    // shared-memory loads independent of its stores
    const int i0 = max(0, c + 1 - r0);  // first own row below the diagonal
    const int nrow = rows - i0, nch = (w - c - 1 + 7) >> 3;
    for (int it = tid; it < nrow * nch; it += PC_THREADS) {
      const int i = i0 + it % nrow, q0 = c + 1 + 8 * (it / nrow);
      const cx<T> l = P[c * rpc + i];
      cx<T> u[8], v[8];
#pragma unroll
      for (int t = 0; t < 8; ++t)
        if (q0 + t < w) {
          u[t] = prow[q0 + t];
          v[t] = P[(q0 + t) * rpc + i];
        }
#pragma unroll
      for (int t = 0; t < 8; ++t)
        if (q0 + t < w) {
          cfms(v[t], l, u[t]);
          P[(q0 + t) * rpc + i] = v[t];
        }
    }
    __syncthreads();
  }
  store_block<T>(a + (j0 + r0) + (long long)j0 * n, n, P, rpc, rows, w, tid, PC_THREADS);
}

// row interchanges of one panel on the columns outside the panel
template <class T>
__global__ void k_laswp(cx<T>* A, int n, long long stride, int j0, int nb, const int* ipiv) {
  const int col = blockIdx.x * blockDim.x + threadIdx.x;
  const int jend = min(j0 + nb, n);
  if (col >= n || (col >= j0 && col < jend)) return;
  cx<T>* a = A + (long long)blockIdx.y * stride + (long long)col * n;
  const int* piv = ipiv + (long long)blockIdx.y * n;
  for (int c = j0; c < jend; ++c) {
    const int p = piv[c];
    if (p != c) {
      cx<T> t0 = a[c];
      a[c] = a[p];
      a[p] = t0;
    }
  }
}

// ---------------------------------------------------------------------------
// inverse of one nb x nb diagonal block by recursive doubling:
// lower unit:  inv([A 0; C B]) = [Ai 0; -Bi C Ai  Bi]
// upper:       inv([A C; 0 B]) = [Ai -Ai C Bi; 0  Bi]
// A partial last block is padded with the identity.
// grid (nblocks_to_do, batch); block 256; dynamic smem = 1.25 nb^2 cx<T>
// ---------------------------------------------------------------------------
template <class T, bool UPPER>
__global__ void __launch_bounds__(256) k_trtri(const cx<T>* A, int n, long long stride, int nb, int blk0,
                                               cx<T>* inv, int nblk) {
  extern __shared__ unsigned char smraw[];
  cx<T>* S = reinterpret_cast<cx<T>*>(smraw);  // nb x nb, column-major
  cx<T>* Tm = S + nb * nb;                       // scratch, nb*nb/4
  const int blk = blk0 + blockIdx.x;
  const int b = blockIdx.y;
  const int r0 = blk * nb;
  const int nr = min(nb, n - r0);
  const cx<T>* a = A + (long long)b * stride;
  const int tid = threadIdx.x;
  for (int e = tid; e < nb * nb; e += blockDim.x) {
    const int i = e % nb, j = e / nb;
    cx<T> v(0, 0);
    if (i < nr && j < nr) {
      if (UPPER) {
        if (i < j) v = a[(r0 + i) + (long long)(r0 + j) * n];
        else if (i == j) v = cinv(a[(r0 + i) + (long long)(r0 + j) * n]);
      } else {
        if (i > j) v = a[(r0 + i) + (long long)(r0 + j) * n];
        else if (i == j) v = cx<T>(1, 0);
      }
    } else if (i == j) {
      v = cx<T>(1, 0);
    }
    S[i + j * nb] = v;
  }
  __syncthreads();
  for (int s = 1; s < nb; s <<= 1) {
    const int npair = nb / (2 * s);
    // T = C * Xi  (lower: C = S[o+s.., o..], Xi = Ai = S[o.., o..])
    //             (upper: C = S[o.., o+s..], Xi = Bi = S[o+s.., o+s..])
    for (int e = tid; e < npair * s * s; e += blockDim.x) {
      const int pr = e / (s * s), rem = e % (s * s);
      const int i = rem % s, j = rem / s;
      const int o = pr * 2 * s;
      cx<T> acc(0, 0);
      if (!UPPER) {
        for (int q = 0; q < s; ++q) cfma(acc, S[(o + s + i) + (o + q) * nb], S[(o + q) + (o + j) * nb]);
      } else {
        for (int q = 0; q < s; ++q) cfma(acc, S[(o + i) + (o + s + q) * nb], S[(o + s + q) + (o + s + j) * nb]);
      }
      Tm[pr * s * s + i + j * s] = acc;
    }
    __syncthreads();
    for (int e = tid; e < npair * s * s; e += blockDim.x) {
      const int pr = e / (s * s), rem = e % (s * s);
      const int i = rem % s, j = rem / s;
      const int o = pr * 2 * s;
      cx<T> acc(0, 0);
      if (!UPPER) {
        // -Bi T, Bi = S[o+s.., o+s..]
        for (int q = 0; q < s; ++q) cfma(acc, S[(o + s + i) + (o + s + q) * nb], Tm[pr * s * s + q + j * s]);
        S[(o + s + i) + (o + j) * nb] = -acc;
      } else {
        // -Ai T, Ai = S[o.., o..]
        for (int q = 0; q < s; ++q) cfma(acc, S[(o + i) + (o + q) * nb], Tm[pr * s * s + q + j * s]);
        S[(o + i) + (o + s + j) * nb] = -acc;
      }
    }
    __syncthreads();
  }
  cx<T>* out = inv + ((long long)b * nblk + blk) * nb * nb;
  for (int e = tid; e < nb * nb; e += blockDim.x) out[e] = S[e];
}

// row permutation from the interchange list (sequential per matrix)
__global__ void k_perm_from_ipiv(const int* ipiv, int* perm, int n) {
  extern __shared__ int pm[];
  const int b = blockIdx.x;
  const int* piv = ipiv + (long long)b * n;
  for (int i = threadIdx.x; i < n; i += blockDim.x) pm[i] = i;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int c = 0; c < n; ++c) {
      const int p = piv[c];
      const int t0 = pm[c];
      pm[c] = pm[p];
      pm[p] = t0;
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < n; i += blockDim.x) perm[(long long)b * n + i] = pm[i];
}

template <class T>
__global__ void k_gather_rows(const cx<T>* V, long long strideV, const int* perm, int n, int L, cx<T>* X) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int b = blockIdx.y;
  if (e >= (long long)n * L) return;
  const int i = (int)(e % n), l = (int)(e / n);
  X[(long long)b * n * L + e] = V[(long long)b * strideV + perm[(long long)b * n + i] + (long long)l * n];
}

// ---------------------------------------------------------------------------
// solve blocks of nbs = nb * 2^levels rows: doubling of the diagonal-block
// inverses (the same identities as k_trtri, one level per pass):
//   lower unit: inv([A 0; C B]) = [Ai 0; -Bi (C Ai)  Bi]
//   upper:      inv([A C; 0 B]) = [Ai -Ai (C Bi); 0  Bi]
// ---------------------------------------------------------------------------
template <class T>
static int gemm_batched2(int M, int N, int K, cx<T> alpha, const cx<T>* A, long long lda, long long sA,
                         long long sA2, const cx<T>* B, long long ldb, long long sB, long long sB2, cx<T> beta,
                         cx<T>* C, long long ldc, long long sC, long long sC2, int batch, int batch2,
                         cudaStream_t st) {
  if constexpr (std::is_same<T, float>::value) {
    if (gemm_engine() == GEMM_ENGINE_TCGEN05)
      return tc_gemm_c64(M, N, K, alpha, A, lda, sA, B, ldb, sB, beta, C, ldc, sC, batch, st, batch2, sA2, sB2,
                         sC2);
  }
  for (int q = 0; q < batch2; ++q) {
    int s = gemm_batched<T>(M, N, K, alpha, A + q * sA2, lda, sA, B + q * sB2, ldb, sB, beta, C + q * sC2, ldc, sC,
                            batch, st);
    if (s) return s;
  }
  return QBG_OK;
}

// out block p (2b x 2b, ld 2b): diagonal b x b blocks from in[2p], in[2p+1]
// (identity where the second block lies beyond the matrix), zeros elsewhere.
template <class T>
__global__ void k_place_diag(const cx<T>* Lin, const cx<T>* Uin, int b, int nin, cx<T>* Lout, cx<T>* Uout,
                             int nout) {
  const long long per = (long long)nout * 4 * b * b;
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= per) return;
  const long long node = blockIdx.y;
  const int b2 = 2 * b;
  const int p = (int)(e / ((long long)b2 * b2));
  const int rem = (int)(e % ((long long)b2 * b2));
  const int i = rem % b2, j = rem / b2;
  const int hi = i >= b, hj = j >= b;
  cx<T> lv(0, 0), uv(0, 0);
  if (hi == hj) {
    const int q = 2 * p + hi, ii = i - hi * b, jj = j - hj * b;
    if (q < nin) {
      const long long o = node * nin * (long long)b * b + (long long)q * b * b + ii + (long long)jj * b;
      lv = Lin[o];
      uv = Uin[o];
    } else if (ii == jj) {
      lv = cx<T>(1, 0);
      uv = cx<T>(1, 0);
    }
  }
  Lout[node * per + e] = lv;
  Uout[node * per + e] = uv;
}

// one doubling pass: b x b block inverses (nin per matrix) -> 2b x 2b (ceil(nin/2))
template <class T>
static int double_level(const LUBatch<T>& f, const cx<T>* Lin, const cx<T>* Uin, int b, int nin, cx<T>* Lout,
                        cx<T>* Uout, cudaStream_t st) {
  const int n = f.n, batch = f.batch, b2 = 2 * b, nout = (nin + 1) / 2;
  const long long per = (long long)nout * b2 * b2;
  dim3 g((unsigned)((per + 255) / 256), batch);
  k_place_diag<T><<<g, 256, 0, st>>>(Lin, Uin, b, nin, Lout, Uout, nout);
  QBG_LAUNCH_CHECK("k_place_diag");
  const int npairs = nin / 2;
  if (npairs == 0) return QBG_OK;
  const long long sIn = (long long)nin * b * b, sOut = per;
  const long long sW = (long long)((f.nblk + 1) / 2) * (f.nbs / 2) * (f.nbs / 2);
  // the second block of the last pair may be partial
  const int wlast = min(b, n - (2 * npairs - 1) * b);
  const int nfull = wlast < b ? npairs - 1 : npairs;
  const cx<T> one(1, 0), mone(-1, 0), zero(0, 0);
  auto run = [&](int p0, int np, int w2) -> int {
    const long long sA2 = 2LL * b * (n + 1), sB2 = 2LL * b * b, sC2 = (long long)b2 * b2, sW2 = (long long)b * b;
    // lower: W = L21 Ai (w2 x b), then bottom-left = -Bi W
    const cx<T>* L21 = f.A + (long long)(2 * p0 + 1) * b + (long long)(2 * p0) * b * n;
    int s = gemm_batched2<T>(w2, b, b, one, L21, n, f.stride, sA2, Lin + 2LL * p0 * b * b, b, sIn, sB2, zero,
                             f.W, b, sW, sW2, batch, np, st);
    if (!s)
      s = gemm_batched2<T>(w2, b, w2, mone, Lin + (2LL * p0 + 1) * b * b, b, sIn, sB2, f.W, b, sW, sW2, zero,
                           Lout + (long long)p0 * b2 * b2 + b, b2, sOut, sC2, batch, np, st);
    // upper: W = U12 Bi (b x w2), then top-right = -Ai W
    const cx<T>* U12 = f.A + (long long)(2 * p0) * b + (long long)(2 * p0 + 1) * b * n;
    if (!s)
      s = gemm_batched2<T>(b, w2, w2, one, U12, n, f.stride, sA2, Uin + (2LL * p0 + 1) * b * b, b, sIn, sB2, zero,
                           f.W, b, sW, sW2, batch, np, st);
    if (!s)
      s = gemm_batched2<T>(b, w2, b, mone, Uin + 2LL * p0 * b * b, b, sIn, sB2, f.W, b, sW, sW2, zero,
                           Uout + (long long)p0 * b2 * b2 + (long long)b * b2, b2, sOut, sC2, batch, np, st);
    return s;
  };
  if (nfull > 0)
    if (int s = run(0, nfull, b)) return s;
  if (nfull < npairs)
    if (int s = run(nfull, 1, wlast)) return s;
  return QBG_OK;
}

template <class T>
size_t lu_solve_blocks_bytes(LUBatch<T>& f, int levels, int ymax_L) {
  f.levels = levels;
  f.nbs = f.nb << levels;
  f.nblks = (f.n + f.nbs - 1) / f.nbs;
  f.ymax_L = levels > 0 ? ymax_L : 0;
  if (levels == 0) return 0;
  const size_t e = sizeof(cx<T>);
  const size_t mid = levels == 2 ? (size_t)((f.nblk + 1) / 2) * (2 * f.nb) * (2 * f.nb) : 0;
  const size_t fin = (size_t)f.nblks * f.nbs * f.nbs;
  const size_t w = (size_t)((f.nblk + 1) / 2) * (f.nbs / 2) * (f.nbs / 2);
  const size_t y = (size_t)f.n * f.ymax_L;
  auto r256 = [](size_t x) { return (x + 255) & ~(size_t)255; };
  return r256(e * mid * f.batch) * 2 + r256(e * fin * f.batch) * 2 + r256(e * w * f.batch) + r256(e * y * f.batch);
}

template <class T>
void lu_solve_blocks_bind(LUBatch<T>& f, void* mem) {
  if (f.levels == 0) return;
  auto r256 = [](size_t x) { return (x + 255) & ~(size_t)255; };
  const size_t e = sizeof(cx<T>);
  const size_t mid = f.levels == 2 ? (size_t)((f.nblk + 1) / 2) * (2 * f.nb) * (2 * f.nb) : 0;
  const size_t fin = (size_t)f.nblks * f.nbs * f.nbs;
  const size_t w = (size_t)((f.nblk + 1) / 2) * (f.nbs / 2) * (f.nbs / 2);
  unsigned char* p = static_cast<unsigned char*>(mem);
  f.Linv_mid = reinterpret_cast<cx<T>*>(p); p += r256(e * mid * f.batch);
  f.Uinv_mid = reinterpret_cast<cx<T>*>(p); p += r256(e * mid * f.batch);
  f.Linv2 = reinterpret_cast<cx<T>*>(p); p += r256(e * fin * f.batch);
  f.Uinv2 = reinterpret_cast<cx<T>*>(p); p += r256(e * fin * f.batch);
  f.W = reinterpret_cast<cx<T>*>(p); p += r256(e * w * f.batch);
  f.Y = reinterpret_cast<cx<T>*>(p);
}

template <class T>
static int build_solve_blocks(const LUBatch<T>& f, cudaStream_t st) {
  if (f.levels == 1) return double_level<T>(f, f.Linv, f.Uinv, f.nb, f.nblk, f.Linv2, f.Uinv2, st);
  const int nmid = (f.nblk + 1) / 2;
  int s = double_level<T>(f, f.Linv, f.Uinv, f.nb, f.nblk, f.Linv_mid, f.Uinv_mid, st);
  if (!s) s = double_level<T>(f, f.Linv_mid, f.Uinv_mid, 2 * f.nb, nmid, f.Linv2, f.Uinv2, st);
  return s;
}

// process-wide plan of lu_factor: panels per outer block (1..16), the panel
// form (-1 automatic, 0 one CTA per panel, 1 a cluster of CTAs) and the
// number of stream parts a Beyn operator batch is factored and solved in;
// the environment variables QBG_LU_OUTER, QBG_LU_CLUSTER and QBG_LU_SPLIT give
// the initial values
static std::atomic<int> g_lu_outer{[] {
  const char* e = std::getenv("QBG_LU_OUTER");
  const int v = (e && *e) ? std::atoi(e) : 4;
  return std::max(1, std::min(v, 16));
}()};
static std::atomic<int> g_lu_cluster{[] {
  const char* e = std::getenv("QBG_LU_CLUSTER");
  return (e && *e) ? (*e == '0' ? 0 : 1) : -1;
}()};

static std::atomic<int> g_lu_parts{[] {
  const char* e = std::getenv("QBG_LU_SPLIT");
  const int v = (e && *e) ? std::atoi(e) : 4;
  return std::max(1, std::min(v, LUBatch<float>::MAX_SPLIT));
}()};

void set_lu_plan(int outer, int cluster, int parts) {
  if (outer > 0) g_lu_outer.store(std::max(1, std::min(outer, 16)));
  g_lu_cluster.store(cluster < 0 ? -1 : (cluster ? 1 : 0));
  if (parts > 0) g_lu_parts.store(std::min(parts, LUBatch<float>::MAX_SPLIT));
}
void get_lu_plan(int* outer, int* cluster, int* parts) {
  if (outer) *outer = g_lu_outer.load();
  if (cluster) *cluster = g_lu_cluster.load();
  if (parts) *parts = g_lu_parts.load();
}

// complex128 blocked updates C -= A B on the tensor cores (eight-digit
// products, tc_gemm_sub_f64) where the product fills the device; QBG_F64_TC=0
// keeps every FP64 product on the FP64 CUDA-core kernels
static std::atomic<int> g_f64_tc{[] {
  const char* e = std::getenv("QBG_F64_TC");
  return (e && *e) ? (std::atoi(e) != 0 ? 1 : 0) : 1;
}()};

template <class T>
static int gemm_sub(int M, int N, int K, const cx<T>* A, long long lda, long long sA, const cx<T>* B, long long ldb,
                    long long sB, cx<T>* C, long long ldc, long long sC, int batch, cudaStream_t st) {
  if constexpr (sizeof(T) == 8) {
    if (g_f64_tc.load() && M >= 256 && N >= 64 && K >= 16 && batch <= 65535)
      return tc_gemm_sub_f64(M, N, K, reinterpret_cast<const cxd*>(A), lda, sA, reinterpret_cast<const cxd*>(B), ldb,
                             sB, reinterpret_cast<cxd*>(C), ldc, sC, batch, st);
  }
  return gemm_batched<T>(M, N, K, cx<T>(-1, 0), A, lda, sA, B, ldb, sB, cx<T>(1, 0), C, ldc, sC, batch, st);
}

template <class T>
static int lu_factor_one(LUBatch<T>& f, cudaStream_t st, cudaEvent_t after_first_panel = nullptr) {
  const int n = f.n, nb = f.nb, batch = f.batch;
  const size_t sm = (size_t)nb * nb * sizeof(cx<T>) * 5 / 4;
  static bool attr_set[2] = {false, false};
  if (!attr_set[sizeof(T) == 8]) {
    QBG_CUDA(cudaFuncSetAttribute(k_trtri<T, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, 96 * 1024));
    QBG_CUDA(cudaFuncSetAttribute(k_trtri<T, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, 96 * 1024));
    attr_set[sizeof(T) == 8] = true;
  }
  // shared-memory sub-panel width: the widest of 8, 4, 2, 1 columns whose n-row sub-panel fits 160 KiB
  constexpr size_t kPanelSmem = 160 * 1024;
  int sub = 8;
  while (sub > 1 && (size_t)n * sub * sizeof(cx<T>) > kPanelSmem) sub >>= 1;
  const bool smem_panel = (size_t)n * sub * sizeof(cx<T>) <= kPanelSmem;
  static bool panel_attr[2] = {false, false};
  if (smem_panel && !panel_attr[sizeof(T) == 8]) {
    QBG_CUDA(cudaFuncSetAttribute(k_getrf_panel_smem<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)kPanelSmem));
    panel_attr[sizeof(T) == 8] = true;
  }
  // panels of up to 64 columns and n <= 8 (or 16) * pc_max_rpc rows of a small
  // batch (at most 4 matrices, where one CTA per panel leaves most SMs idle;
  // for complex128 one SM's FP64 pipe takes ~1 ms per 500 x 64 panel) go to
  // a cluster of CTAs. For larger batches the one-CTA panels of
  // several matrices already run side by side with other matrices' updates,
  // and the cluster form measured slower (48 operators of 2048 in four
  // stream parts: factor phase 38.5 ms with clusters against 34.0 ms without).
  // set_lu_plan (or QBG_LU_CLUSTER=0 / =1 in the environment) forces either form.
  const int cluster_set = g_lu_cluster.load();
  const bool cluster_on = cluster_set < 0 ? batch <= 4 : cluster_set == 1;
  static bool cluster_attr[2] = {false, false};
  static bool cluster16_ok[2] = {false, false};
  if (cluster_on && nb <= 64 && !cluster_attr[sizeof(T) == 8]) {
    QBG_CUDA(cudaFuncSetAttribute(k_getrf_panel_cluster<T, 8>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  pc_max_rpc<T, 8>() * 64 * (int)sizeof(cx<T>)));
    // 16-CTA clusters exist on this part as a non-portable size: allowed only
    // when the occupancy query finds room for at least one
    bool ok = cudaFuncSetAttribute(k_getrf_panel_cluster<T, 16>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) ==
                  cudaSuccess &&
              cudaFuncSetAttribute(k_getrf_panel_cluster<T, 16>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   pc_max_rpc<T, 16>() * 64 * (int)sizeof(cx<T>)) == cudaSuccess;
    if (ok) {
      cudaLaunchConfig_t cfg = {};
      cfg.gridDim = dim3(16, 1, 1);
      cfg.blockDim = dim3(PC_THREADS, 1, 1);
      cfg.dynamicSmemBytes = (size_t)pc_max_rpc<T, 16>() * 64 * sizeof(cx<T>);
      int nclusters = 0;
      ok = cudaOccupancyMaxActiveClusters(&nclusters, (void*)k_getrf_panel_cluster<T, 16>, &cfg) == cudaSuccess &&
           nclusters >= 1;
    }
    (void)cudaGetLastError();  // a refused attribute or query leaves 16-CTA clusters off, nothing else
    cluster16_ok[sizeof(T) == 8] = ok;
    cluster_attr[sizeof(T) == 8] = true;
  }
  const int pcs = !(cluster_on && nb <= 64)                  ? 0
                  : n <= 8 * pc_max_rpc<T, 8>()               ? 8
                  : (cluster16_ok[sizeof(T) == 8] && n <= 16 * pc_max_rpc<T, 16>()) ? 16
                                                              : 0;
  const bool use_cluster = pcs > 0;
  QBG_CUDA(cudaMemsetAsync(f.info, 0, sizeof(int) * batch, st));
  // two-level right-looking LU: panels of nb columns inside outer blocks of
  // LU_OUTER panels. A panel's updates reach only the columns of its outer
  // block; the trailing matrix right of an outer block is updated once, with
  // K = LU_OUTER * nb, after the outer block's U rows are formed by block
  // forward substitution (the nb x nb inverses of L from k_trtri). The row
  // interchanges of every panel still apply to all columns at once (k_laswp),
  // so the factors are those of the one-level algorithm.
  // panels per outer block: set_lu_plan (or QBG_LU_OUTER in the environment), 1..16, default 4
  const int LU_OUTER = g_lu_outer.load();
  const cx<T> one(1, 0), mone(-1, 0), zero(0, 0);
  auto linv = [&](int j) { return f.Linv + (long long)(j / nb) * nb * nb; };
  const long long sLinv = (long long)f.nblk * nb * nb;
  for (int J0 = 0; J0 < n; J0 += LU_OUTER * nb) {
    const int E = min(n, J0 + LU_OUTER * nb);  // outer block columns [J0, E)
    for (int j0 = J0; j0 < E; j0 += nb) {
      const int w = min(nb, n - j0);
      if (use_cluster) {
        const int rpc = (n - j0 + pcs - 1) / pcs;
        const size_t smem = (size_t)rpc * 64 * sizeof(cx<T>);
        if (pcs == 8)
          k_getrf_panel_cluster<T, 8><<<batch * 8, PC_THREADS, smem, st>>>(f.A, n, f.stride, j0, nb, rpc, f.ipiv,
                                                                           f.info);
        else
          k_getrf_panel_cluster<T, 16><<<batch * 16, PC_THREADS, smem, st>>>(f.A, n, f.stride, j0, nb, rpc, f.ipiv,
                                                                             f.info);
        QBG_LAUNCH_CHECK("k_getrf_panel_cluster");
      } else if (smem_panel) {
        const size_t smem = (size_t)(n - j0) * sub * sizeof(cx<T>);
        k_getrf_panel_smem<T><<<batch, 1024, smem, st>>>(f.A, n, f.stride, j0, nb, sub, f.ipiv, f.info);
        QBG_LAUNCH_CHECK("k_getrf_panel_smem");
      } else {
        k_getf2_panel<T><<<batch, 512, 0, st>>>(f.A, n, f.stride, j0, nb, f.ipiv, f.info);
        QBG_LAUNCH_CHECK("k_getf2_panel");
      }
      dim3 g2((n + 255) / 256, batch);
      k_laswp<T><<<g2, 256, 0, st>>>(f.A, n, f.stride, j0, nb, f.ipiv);
      QBG_LAUNCH_CHECK("k_laswp");
      k_trtri<T, false><<<dim3(1, batch), 256, sm, st>>>(f.A, n, f.stride, nb, j0 / nb, f.Linv, f.nblk);
      QBG_LAUNCH_CHECK("k_trtri lower");
      if (j0 == 0 && after_first_panel) QBG_CUDA(cudaEventRecord(after_first_panel, st));
      const int rin = E - j0 - w;  // columns of this outer block right of the panel
      if (rin > 0) {
        // U12 = inv(L11) A12 and A22 -= L21 U12 on the outer block's columns
        int s = gemm_batched<T>(w, rin, w, one, linv(j0), nb, sLinv, f.A + j0 + (long long)(j0 + w) * n, n,
                                f.stride, zero, f.A + j0 + (long long)(j0 + w) * n, n, f.stride, batch, st);
        if (s) return s;
        s = gemm_sub<T>(n - j0 - w, rin, w, f.A + (j0 + w) + (long long)j0 * n, n, f.stride,
                        f.A + j0 + (long long)(j0 + w) * n, n, f.stride, f.A + (j0 + w) + (long long)(j0 + w) * n, n,
                        f.stride, batch, st);
        if (s) return s;
      }
    }
    const int rest = n - E;
    if (rest > 0) {
      // U rows of the outer block on the trailing columns: U_b = inv(L_bb) (A_b - sum_{b'<b} L_bb' U_b')
      for (int j0 = J0; j0 < E; j0 += nb) {
        const int w = min(nb, E - j0);
        int s = gemm_batched<T>(w, rest, w, one, linv(j0), nb, sLinv, f.A + j0 + (long long)E * n, n, f.stride,
                                zero, f.A + j0 + (long long)E * n, n, f.stride, batch, st);
        if (s) return s;
        const int below = E - j0 - w;
        if (below > 0) {
          s = gemm_sub<T>(below, rest, w, f.A + (j0 + w) + (long long)j0 * n, n, f.stride,
                          f.A + j0 + (long long)E * n, n, f.stride, f.A + (j0 + w) + (long long)E * n, n, f.stride,
                          batch, st);
          if (s) return s;
        }
      }
      // trailing update, K = E - J0
      int s = gemm_sub<T>(rest, rest, E - J0, f.A + E + (long long)J0 * n, n, f.stride, f.A + J0 + (long long)E * n,
                          n, f.stride, f.A + E + (long long)E * n, n, f.stride, batch, st);
      if (s) return s;
    }
  }
  k_trtri<T, true><<<dim3(f.nblk, batch), 256, sm, st>>>(f.A, n, f.stride, nb, 0, f.Uinv, f.nblk);
  QBG_LAUNCH_CHECK("k_trtri upper");
  if (sizeof(int) * (size_t)n > 48 * 1024)
    QBG_CUDA(cudaFuncSetAttribute(k_perm_from_ipiv, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)(sizeof(int) * (size_t)n)));
  k_perm_from_ipiv<<<batch, 256, sizeof(int) * n, st>>>(f.ipiv, f.perm, n);
  QBG_LAUNCH_CHECK("k_perm_from_ipiv");
  if (f.levels > 0) return build_solve_blocks<T>(f, st);
  return QBG_OK;
}

template <class T>
static int lu_trsolve(const LUBatch<T>& f, int L, cx<T>* X, cudaStream_t st);

template <class T>
static int lu_solve_one(const LUBatch<T>& f, const cx<T>* V, int L, cx<T>* X, long long strideV, cudaStream_t st) {
  const int n = f.n, batch = f.batch;
  dim3 g((unsigned)(((long long)n * L + 255) / 256), batch);
  k_gather_rows<T><<<g, 256, 0, st>>>(V, strideV, f.perm, n, L, X);
  QBG_LAUNCH_CHECK("k_gather_rows");
  return lu_trsolve<T>(f, L, X, st);
}

// X = P (the row permutation of the factorisation, as a matrix)
template <class T>
__global__ void k_perm_matrix(const int* perm, int n, cx<T>* X) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int b = blockIdx.y;
  if (e >= (long long)n * n) return;
  const int i = (int)(e % n), l = (int)(e / n);
  X[(long long)b * n * n + e] = cx<T>(perm[(long long)b * n + i] == l ? T(1) : T(0), T(0));
}

// X[perm[i]] = Y[i]: applies P^T to every column
template <class T>
__global__ void k_scatter_rows(const cx<T>* Y, const int* perm, int n, int L, cx<T>* X) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int b = blockIdx.y;
  if (e >= (long long)n * L) return;
  const int i = (int)(e % n), l = (int)(e / n);
  X[(long long)b * n * L + perm[(long long)b * n + i] + (long long)l * n] = Y[(long long)b * n * L + e];
}

template <class T>
__global__ void k_copy_rhs(const cx<T>* V, long long strideV, int n, int L, cx<T>* X) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int b = blockIdx.y;
  if (e >= (long long)n * L) return;
  X[(long long)b * n * L + e] = V[(long long)b * strideV + e];
}

// A_b^{-1} for every matrix of the batch (X: batch * n * n)
template <class T>
int lu_inverse(const LUBatch<T>& f, cx<T>* X, cudaStream_t st) {
  const int n = f.n;
  dim3 g((unsigned)(((long long)n * n + 255) / 256), f.batch);
  k_perm_matrix<T><<<g, 256, 0, st>>>(f.perm, n, X);
  QBG_LAUNCH_CHECK("k_perm_matrix");
  return lu_trsolve<T>(f, n, X, st);
}

// X_b = A_b^{-H} V_b with P A = L U: A^{-H} = P^T L^{-H} U^{-H}. U^H is lower
// and L^H unit upper; both use the nb x nb diagonal-block inverses of the
// factorisation (levels 0). Y: scratch of batch * n * L elements.
template <class T>
int lu_solve_adjoint(const LUBatch<T>& f, const cx<T>* V, long long strideV, int L, cx<T>* X, cx<T>* Y,
                     cudaStream_t st) {
  const int n = f.n, nb = f.nb, batch = f.batch;
  const long long sY = (long long)n * L;
  const long long sInv = (long long)f.nblk * nb * nb;
  const cx<T> one(1, 0), mone(-1, 0), zero(0, 0);
  dim3 g((unsigned)(((long long)n * L + 255) / 256), batch);
  k_copy_rhs<T><<<g, 256, 0, st>>>(V, strideV, n, L, Y);
  QBG_LAUNCH_CHECK("k_copy_rhs");
  for (int blk = 0; blk < f.nblk; ++blk) {  // U^H y = v, forward
    const int r0 = blk * nb, w = min(nb, n - r0), rest = n - r0 - w;
    QBG_TRY(gemm_batched_ah<T>(w, L, w, one, f.Uinv + (long long)blk * nb * nb, nb, sInv, Y + r0, n, sY, zero,
                               Y + r0, n, sY, batch, st));
    if (rest > 0)
      QBG_TRY(gemm_batched_ah<T>(rest, L, w, mone, f.A + r0 + (long long)(r0 + w) * n, n, f.stride, Y + r0, n, sY,
                                 one, Y + r0 + w, n, sY, batch, st));
  }
  for (int blk = f.nblk - 1; blk >= 0; --blk) {  // L^H x = y, backward
    const int r0 = blk * nb;
    const int w = min(nb, n - r0);
    QBG_TRY(gemm_batched_ah<T>(w, L, w, one, f.Linv + (long long)blk * nb * nb, nb, sInv, Y + r0, n, sY, zero,
                               Y + r0, n, sY, batch, st));
    if (r0 > 0)
      QBG_TRY(gemm_batched_ah<T>(r0, L, w, mone, f.A + r0, n, f.stride, Y + r0, n, sY, one, Y, n, sY, batch, st));
  }
  k_scatter_rows<T><<<g, 256, 0, st>>>(Y, f.perm, n, L, X);
  QBG_LAUNCH_CHECK("k_scatter_rows");
  return QBG_OK;
}

template <class T>
static int lu_trsolve(const LUBatch<T>& f, int L, cx<T>* X, cudaStream_t st) {
  const int n = f.n, nb = f.nb, batch = f.batch;
  const long long sX = (long long)n * L;
  if (f.levels > 0) {
    // blocks of nbs rows; forward: Y_b = Linv_b X_b, X_rest -= L_rest,b Y_b;
    // backward: X_b = Uinv_b Y_b, Y_above -= U_above,b X_b (no in-place products)
    const int bs = f.nbs;
    const long long sI2 = (long long)f.nblks * bs * bs;
    const cx<T> one(1, 0), mone(-1, 0), zero(0, 0);
    for (int c0 = 0; c0 < L; c0 += f.ymax_L) {
      const int Lc = min(f.ymax_L, L - c0);
      cx<T>* Xc = X + (long long)c0 * n;
      cx<T>* Yc = f.Y;
      const long long sY = (long long)n * Lc;
      for (int blk = 0; blk < f.nblks; ++blk) {
        const int r0 = blk * bs, w = min(bs, n - r0), rest = n - r0 - w;
        int s = gemm_batched<T>(w, Lc, w, one, f.Linv2 + (long long)blk * bs * bs, bs, sI2, Xc + r0, n, sX, zero,
                                Yc + r0, n, sY, batch, st);
        if (!s && rest > 0)
          s = gemm_sub<T>(rest, Lc, w, f.A + (r0 + w) + (long long)r0 * n, n, f.stride, Yc + r0, n, sY,
                          Xc + r0 + w, n, sX, batch, st);
        if (s) return s;
      }
      for (int blk = f.nblks - 1; blk >= 0; --blk) {
        const int r0 = blk * bs, w = min(bs, n - r0);
        int s = gemm_batched<T>(w, Lc, w, one, f.Uinv2 + (long long)blk * bs * bs, bs, sI2, Yc + r0, n, sY, zero,
                                Xc + r0, n, sX, batch, st);
        if (!s && r0 > 0)
          s = gemm_sub<T>(r0, Lc, w, f.A + (long long)r0 * n, n, f.stride, Xc + r0, n, sX, Yc, n, sY, batch, st);
        if (s) return s;
      }
    }
    return QBG_OK;
  }
  const long long sInv = (long long)f.nblk * nb * nb;
  for (int blk = 0; blk < f.nblk; ++blk) {
    const int r0 = blk * nb, w = min(nb, n - r0);
    int s = gemm_batched<T>(w, L, w, cx<T>(1, 0), f.Linv + (long long)blk * nb * nb, nb, sInv, X + r0, n, sX,
                            cx<T>(0, 0), X + r0, n, sX, batch, st);
    if (s) return s;
    const int rest = n - r0 - w;
    if (rest > 0) {
      s = gemm_sub<T>(rest, L, w, f.A + (r0 + w) + (long long)r0 * n, n, f.stride, X + r0, n, sX, X + r0 + w, n, sX,
                      batch, st);
      if (s) return s;
    }
  }
  for (int blk = f.nblk - 1; blk >= 0; --blk) {
    const int r0 = blk * nb, w = min(nb, n - r0);
    int s = gemm_batched<T>(w, L, w, cx<T>(1, 0), f.Uinv + (long long)blk * nb * nb, nb, sInv, X + r0, n, sX,
                            cx<T>(0, 0), X + r0, n, sX, batch, st);
    if (s) return s;
    if (r0 > 0) {
      s = gemm_sub<T>(r0, L, w, f.A + (long long)r0 * n, n, f.stride, X + r0, n, sX, X, n, sX, batch, st);
      if (s) return s;
    }
  }
  return QBG_OK;
}

// ---------------------------------------------------------------------------
// contour moments, one thread per (i, l), loop over contour nodes
// ---------------------------------------------------------------------------
template <class T>
__global__ void k_moments(const cx<T>* X, long long sX, int batch, long long count, const cxd* w, const cxd* z,
                          cxd* A0, cxd* A1, int accumulate) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= count) return;
  cxd a0(0, 0), a1(0, 0);
  if (accumulate) { a0 = A0[e]; a1 = A1[e]; }
  for (int b = 0; b < batch; ++b) {
    const cxd x(X[(long long)b * sX + e]);
    const cxd wx = w[b] * x;
    a0 += wx;
    a1 += z[b] * wx;
  }
  A0[e] = a0;
  A1[e] = a1;
}

template <class T>
int moments(const cx<T>* X, long long sX, int batch, int n, int L, const cxd* w, const cxd* z, cxd* A0, cxd* A1,
            int accumulate, cudaStream_t st) {
  const long long count = (long long)n * L;
  k_moments<T><<<(unsigned)((count + 255) / 256), 256, 0, st>>>(X, sX, batch, count, w, z, A0, A1, accumulate);
  QBG_LAUNCH_CHECK("k_moments");
  return QBG_OK;
}

// ---------------------------------------------------------------------------
// refinement residual R = V - T X with compensated FP32 arithmetic.
// Each real product a*(xh + xl) is split exactly (p + e via FMA); the hi
// parts are accumulated with Knuth's TwoSum, the error terms in a second FP32
// word, and the (hi, lo) pair is flushed into an FP64 accumulator after every
// 32-term K tile so the low word never grows.
// tile: 64 rows x 32 columns, K step 32; 256 threads, 4 x 2 outputs each.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void df_acc(float& sh, float& sl, float a, float bh, float bl) {
  const float p = a * bh;
  float e = fmaf(a, bh, -p);
  e = fmaf(a, bl, e);
  const float s = sh + p;
  const float v = s - sh;
  const float err = (sh - (s - v)) + (p - v);
  sh = s;
  sl += err + e;
}

template <bool LO>
__global__ void __launch_bounds__(256) k_residual_df32(const cxf* __restrict__ Tm, const cxf* __restrict__ Tl,
                                                       long long sT, const cxd* __restrict__ X, long long sX,
                                                       const cxd* __restrict__ V, long long sV, cxd* R,
                                                       long long sR, int n, int L, unsigned long long* rmax) {
  constexpr int BM = 64, BN = 32, BK = 32;
  __shared__ cxf Ts[BK][BM];
  __shared__ cxf Tls[LO ? BK : 1][LO ? BM : 1];
  __shared__ float4 Xs[BK][BN + 1];  // (re_hi, re_lo, im_hi, im_lo)
  const int tid = threadIdx.x;
  const int tx = tid & 15, ty = tid >> 4;  // rows tx + 16a (a<4), cols ty + 16b (b<2)
  const int m0 = blockIdx.x * BM, n0 = blockIdx.y * BN;
  const long long bz = blockIdx.z;
  const cxf* Tb = Tm + bz * sT;
  const cxf* Tlb = LO ? Tl + bz * sT : nullptr;
  const cxd* Xb = X + bz * sX;
  const cxd* Vb = V + bz * sV;
  float hr[4][2], lr[4][2], hi_[4][2], li[4][2];
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 2; ++b) { hr[a][b] = 0.f; lr[a][b] = 0.f; hi_[a][b] = 0.f; li[a][b] = 0.f; }
  double accr[4][2], acci[4][2];
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 2; ++b) { accr[a][b] = 0.0; acci[a][b] = 0.0; }
  for (int k0 = 0; k0 < n; k0 += BK) {
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const int idx = tid + q * 256;
      const int i = idx & (BM - 1), kk = idx >> 6;
      const int gi = m0 + i, gk = k0 + kk;
      Ts[kk][i] = (gi < n && gk < n) ? Tb[(long long)gi + (long long)gk * n] : cxf(0.f, 0.f);
      if (LO) Tls[kk][i] = (gi < n && gk < n) ? Tlb[(long long)gi + (long long)gk * n] : cxf(0.f, 0.f);
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int idx = tid + q * 256;
      const int kk = idx & (BK - 1), jj = idx >> 5;
      const int gk = k0 + kk, gj = n0 + jj;
      float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
      if (gk < n && gj < L) {
        const cxd x = Xb[(long long)gk + (long long)gj * n];
        const float rh = (float)x.re, ih = (float)x.im;
        v = make_float4(rh, (float)(x.re - (double)rh), ih, (float)(x.im - (double)ih));
      }
      Xs[kk][jj] = v;
    }
    __syncthreads();
#pragma unroll 4
    for (int kk = 0; kk < BK; ++kk) {
      cxf t[4];
      float4 x[2];
#pragma unroll
      for (int a = 0; a < 4; ++a) t[a] = Ts[kk][tx + 16 * a];
#pragma unroll
      for (int b = 0; b < 2; ++b) x[b] = Xs[kk][ty + 16 * b];
#pragma unroll
      for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 2; ++b) {
          // re += t.re*x.re - t.im*x.im ; im += t.re*x.im + t.im*x.re
          df_acc(hr[a][b], lr[a][b], t[a].re, x[b].x, x[b].y);
          df_acc(hr[a][b], lr[a][b], -t[a].im, x[b].z, x[b].w);
          df_acc(hi_[a][b], li[a][b], t[a].re, x[b].z, x[b].w);
          df_acc(hi_[a][b], li[a][b], t[a].im, x[b].x, x[b].y);
        }
      if (LO) {
        // lo part of the operator (|lo| <= 2^-24 |hi|): plain FP32 products into the low words
#pragma unroll
        for (int a = 0; a < 4; ++a) {
          const cxf tl = Tls[kk][tx + 16 * a];
#pragma unroll
          for (int b = 0; b < 2; ++b) {
            lr[a][b] = fmaf(tl.re, x[b].x, lr[a][b]);
            lr[a][b] = fmaf(-tl.im, x[b].z, lr[a][b]);
            li[a][b] = fmaf(tl.re, x[b].z, li[a][b]);
            li[a][b] = fmaf(tl.im, x[b].x, li[a][b]);
          }
        }
      }
    }
    // flush the (hi, lo) float pairs into FP64 every 8 tiles (256 terms) and at the end:
    // the low word then holds at most ~256 rounding errors of the high word, far below
    // the residual levels the refinement tests (the FP64 pipe of GB300 is 1/64 rate)
    if (((k0 / BK) & 7) == 7 || k0 + BK >= n) {
#pragma unroll
      for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 2; ++b) {
          accr[a][b] += (double)hr[a][b] + (double)lr[a][b];
          acci[a][b] += (double)hi_[a][b] + (double)li[a][b];
          hr[a][b] = 0.f; lr[a][b] = 0.f; hi_[a][b] = 0.f; li[a][b] = 0.f;
        }
    }
    __syncthreads();
  }
  double lmax = 0.0;
  bool bad = false;
#pragma unroll
  for (int b = 0; b < 2; ++b) {
    const int gj = n0 + ty + 16 * b;
    if (gj >= L) continue;
#pragma unroll
    for (int a = 0; a < 4; ++a) {
      const int gi = m0 + tx + 16 * a;
      if (gi >= n) continue;
      const cxd v = Vb[(long long)gi + (long long)gj * n];
      const cxd r(v.re - accr[a][b], v.im - acci[a][b]);
      R[bz * sR + (long long)gi + (long long)gj * n] = r;
      const double m = fabs(r.re) + fabs(r.im);
      bad |= !(m == m);
      lmax = fmax(lmax, m);
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) lmax = fmax(lmax, __shfl_down_sync(0xffffffffu, lmax, o));
  bad = __any_sync(0xffffffffu, bad);
  // a NaN (bit pattern above +Inf) wins the unsigned maximum
  if ((tid & 31) == 0 && rmax)
    atomicMax(rmax, bad ? 0x7FF8000000000000ull : (unsigned long long)__double_as_longlong(lmax));
}

int residual_df32(const cxf* Tm, const cxf* Tlo, long long sT, const cxd* X, long long sX, const cxd* V,
                  long long sV, cxd* R, long long sR, int n, int L, int batch, double* rmax, cudaStream_t st) {
  dim3 grd((n + 63) / 64, (L + 31) / 32, batch);
  auto* rm = reinterpret_cast<unsigned long long*>(rmax);
  if (Tlo)
    k_residual_df32<true><<<grd, 256, 0, st>>>(Tm, Tlo, sT, X, sX, V, sV, R, sR, n, L, rm);
  else
    k_residual_df32<false><<<grd, 256, 0, st>>>(Tm, nullptr, sT, X, sX, V, sV, R, sR, n, L, rm);
  QBG_LAUNCH_CHECK("k_residual_df32");
  return QBG_OK;
}

__global__ void k_d2f(const cxd* in, cxf* out, long long count) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e < count) out[e] = cxf(in[e]);
}
__global__ void k_axpy_f2d(const cxf* d, cxd* x, long long count) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e < count) {
    x[e].re += (double)d[e].re;
    x[e].im += (double)d[e].im;
  }
}
__global__ void k_bcast_f(const cxf* in, long long count, int batch, cxf* out) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= count) return;
  const cxf v = in[e];
  for (int b = 0; b < batch; ++b) out[(long long)b * count + e] = v;
}
int broadcast_f(const cxf* in, long long count, int batch, cxf* out, cudaStream_t st) {
  k_bcast_f<<<(unsigned)((count + 255) / 256), 256, 0, st>>>(in, count, batch, out);
  QBG_LAUNCH_CHECK("k_bcast_f");
  return QBG_OK;
}
__global__ void k_maxabs_c64(const cxf* __restrict__ x, long long count, unsigned long long* out) {
  float m = 0.f;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < count;
       e += (long long)gridDim.x * blockDim.x)
    m = fmaxf(m, fabsf(x[e].re) + fabsf(x[e].im));
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  // non-negative doubles order like their bit patterns
  if ((threadIdx.x & 31) == 0) atomicMax(out, (unsigned long long)__double_as_longlong((double)m));
}
int maxabs_c64(const cxf* x, long long count, double* out, cudaStream_t st) {
  if (count <= 0) return QBG_OK;
  const long long blocks = std::min<long long>((count + 255) / 256, 152 * 8);
  k_maxabs_c64<<<(unsigned)blocks, 256, 0, st>>>(x, count, reinterpret_cast<unsigned long long*>(out));
  QBG_LAUNCH_CHECK("k_maxabs_c64");
  return QBG_OK;
}
// column |.|-sums of a batch of n x n complex128 matrices: out[b] = max_j sum_i |A_b(i, j)|
// (opnorm(A, 1)); one CTA per (column, matrix); out holds non-negative double bits, zeroed
__global__ void k_opnorm1(const cxd* __restrict__ A, int n, long long sA, unsigned long long* out) {
  const int j = blockIdx.x, b = blockIdx.y;
  const cxd* col = A + (long long)b * sA + (long long)j * n;
  double s = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) s += hypot(col[i].re, col[i].im);
  __shared__ double red[32];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    s = threadIdx.x < (int)(blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (threadIdx.x == 0) atomicMax(&out[b], (unsigned long long)__double_as_longlong(s));
  }
}

// per column b of the n x batch blocks y, phi: out[4 b + 0..3] = ||y||_2^2, ||y||_1, ||phi||_1, ||phi||_2^2
__global__ void k_vec_norms(const cxd* __restrict__ y, const cxd* __restrict__ phi, int n, double* out) {
  const int b = blockIdx.x;
  double a[4] = {0.0, 0.0, 0.0, 0.0};
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const cxd u = y[(long long)b * n + i], v = phi[(long long)b * n + i];
    a[0] += u.re * u.re + u.im * u.im;
    a[1] += hypot(u.re, u.im);
    a[2] += hypot(v.re, v.im);
    a[3] += v.re * v.re + v.im * v.im;
  }
  __shared__ double red[4][32];
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    double s = a[q];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) red[q][threadIdx.x >> 5] = s;
  }
  __syncthreads();
  if (threadIdx.x < 32) {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      double s = threadIdx.x < (int)(blockDim.x >> 5) ? red[q][threadIdx.x] : 0.0;
      for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
      if (threadIdx.x == 0) out[4 * b + q] = s;
    }
  }
}

int opnorm1_batched(const cxd* A, int n, long long sA, int batch, double* out, cudaStream_t st) {
  k_opnorm1<<<dim3(n, batch), 256, 0, st>>>(A, n, sA, reinterpret_cast<unsigned long long*>(out));
  QBG_LAUNCH_CHECK("k_opnorm1");
  return QBG_OK;
}

int vec_norms(const cxd* y, const cxd* phi, int n, int batch, double* out, cudaStream_t st) {
  k_vec_norms<<<batch, 256, 0, st>>>(y, phi, n, out);
  QBG_LAUNCH_CHECK("k_vec_norms");
  return QBG_OK;
}

int convert_d2f(const cxd* in, cxf* out, long long count, cudaStream_t st) {
  k_d2f<<<(unsigned)((count + 255) / 256), 256, 0, st>>>(in, out, count);
  QBG_LAUNCH_CHECK("k_d2f");
  return QBG_OK;
}
int axpy_f2d(const cxf* d, cxd* x, long long count, cudaStream_t st) {
  k_axpy_f2d<<<(unsigned)((count + 255) / 256), 256, 0, st>>>(d, x, count);
  QBG_LAUNCH_CHECK("k_axpy_f2d");
  return QBG_OK;
}

// matrices [b0, b0 + cnt) of a batch as a batch of their own (every
// per-matrix buffer offset by its allocation stride)
template <class T>
static LUBatch<T> lu_view(const LUBatch<T>& f, int b0, int cnt) {
  LUBatch<T> v = f;
  v.batch = cnt;
  v.nsplit = 1;
  const long long b = b0;
  v.A = f.A + b * f.stride;
  v.ipiv = f.ipiv + b * f.n;
  v.perm = f.perm + b * f.n;
  v.info = f.info + b;
  const long long sinv = (long long)f.nblk * f.nb * f.nb;
  v.Linv = f.Linv + b * sinv;
  v.Uinv = f.Uinv + b * sinv;
  if (f.levels > 0) {
    const long long mid = f.levels == 2 ? (long long)((f.nblk + 1) / 2) * (2 * f.nb) * (2 * f.nb) : 0;
    const long long fin = (long long)f.nblks * f.nbs * f.nbs;
    const long long w = (long long)((f.nblk + 1) / 2) * (f.nbs / 2) * (f.nbs / 2);
    if (f.Linv_mid) v.Linv_mid = f.Linv_mid + b * mid;
    if (f.Uinv_mid) v.Uinv_mid = f.Uinv_mid + b * mid;
    v.Linv2 = f.Linv2 + b * fin;
    v.Uinv2 = f.Uinv2 + b * fin;
    v.W = f.W + b * w;
    v.Y = f.Y + b * (long long)f.n * f.ymax_L;
  }
  return v;
}

// With extra streams the parts of the batch are factored (solved)
// concurrently: the panel factorisations and the short GEMM chains of one part
// leave most SMs idle, which the other parts' kernels fill. The matrices are
// independent, so the results are those of one stream.
template <class T>
static int split_parts(const LUBatch<T>& f) {
  return std::max(1, std::min(std::min(f.nsplit, LUBatch<T>::MAX_SPLIT), f.batch));
}

template <class T>
int lu_factor(LUBatch<T>& f, cudaStream_t st) {
  const int P = split_parts(f);
  if (P < 2) return lu_factor_one<T>(f, st);
  // part i + 1 starts one panel behind part i, so that the panels of one part
  // run under the updates of the others
  int s = QBG_OK;
  for (int i = 0; i < P && !s; ++i) {
    const int b0 = (int)((long long)i * f.batch / P), b1 = (int)((long long)(i + 1) * f.batch / P);
    LUBatch<T> v = lu_view<T>(f, b0, b1 - b0);
    cudaStream_t si = i == 0 ? st : f.stx[i - 1];
    if (i > 0) QBG_CUDA(cudaStreamWaitEvent(si, f.ev_fork, 0));
    s = lu_factor_one<T>(v, si, i + 1 < P ? f.ev_fork : nullptr);
  }
  for (int i = 1; i < P; ++i) {
    QBG_CUDA(cudaEventRecord(f.ev_join, f.stx[i - 1]));
    QBG_CUDA(cudaStreamWaitEvent(st, f.ev_join, 0));
  }
  return s;
}

template <class T>
int lu_solve_shared(const LUBatch<T>& f, const cx<T>* V, int L, cx<T>* X, long long strideV, cudaStream_t st) {
  const int P = split_parts(f);
  if (P < 2) return lu_solve_one<T>(f, V, L, X, strideV, st);
  QBG_CUDA(cudaEventRecord(f.ev_fork, st));
  int s = QBG_OK;
  for (int i = 0; i < P && !s; ++i) {
    const int b0 = (int)((long long)i * f.batch / P), b1 = (int)((long long)(i + 1) * f.batch / P);
    const LUBatch<T> v = lu_view<T>(f, b0, b1 - b0);
    cudaStream_t si = i == 0 ? st : f.stx[i - 1];
    if (i > 0) QBG_CUDA(cudaStreamWaitEvent(si, f.ev_fork, 0));
    s = lu_solve_one<T>(v, V + (long long)b0 * strideV, L, X + (long long)b0 * f.n * L, strideV, si);
  }
  for (int i = 1; i < P; ++i) {
    QBG_CUDA(cudaEventRecord(f.ev_join, f.stx[i - 1]));
    QBG_CUDA(cudaStreamWaitEvent(st, f.ev_join, 0));
  }
  return s;
}

template int lu_factor<double>(LUBatch<double>&, cudaStream_t);
template int lu_inverse<double>(const LUBatch<double>&, cxd*, cudaStream_t);
template int gemm_batched_ah<double>(int, int, int, cxd, const cxd*, long long, long long, const cxd*, long long,
                                     long long, cxd, cxd*, long long, long long, int, cudaStream_t);
template int lu_solve_adjoint<double>(const LUBatch<double>&, const cxd*, long long, int, cxd*, cxd*, cudaStream_t);

template size_t lu_solve_blocks_bytes<double>(LUBatch<double>&, int, int);
template size_t lu_solve_blocks_bytes<float>(LUBatch<float>&, int, int);
template void lu_solve_blocks_bind<double>(LUBatch<double>&, void*);
template void lu_solve_blocks_bind<float>(LUBatch<float>&, void*);
template int lu_factor<float>(LUBatch<float>&, cudaStream_t);
template int lu_inverse<float>(const LUBatch<float>&, cxf*, cudaStream_t);
template int lu_solve_shared<double>(const LUBatch<double>&, const cxd*, int, cxd*, long long, cudaStream_t);
template int lu_solve_shared<float>(const LUBatch<float>&, const cxf*, int, cxf*, long long, cudaStream_t);
template int gemm_batched<double>(int, int, int, cxd, const cxd*, long long, long long, const cxd*, long long,
                                  long long, cxd, cxd*, long long, long long, int, cudaStream_t);
template int gemm_batched_simt<float>(int, int, int, cxf, const cxf*, long long, long long, const cxf*, long long,
                                      long long, cxf, cxf*, long long, long long, int, cudaStream_t);
template int gemm_batched<float>(int, int, int, cxf, const cxf*, long long, long long, const cxf*, long long,
                                 long long, cxf, cxf*, long long, long long, int, cudaStream_t);
template int moments<double>(const cxd*, long long, int, int, int, const cxd*, const cxd*, cxd*, cxd*, int,
                             cudaStream_t);
template int moments<float>(const cxf*, long long, int, int, int, const cxd*, const cxd*, cxd*, cxd*, int,
                            cudaStream_t);

}  // namespace qbg
