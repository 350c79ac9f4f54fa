// Refinement residual R = V - T X on the tensor cores with exact digit
// products (tcgen05, kind::f16 with bf16 operands, FP32 accumulation in TMEM).
//
// T (the FP64 value hi + lo of each operator entry) is scaled per row and X
// (complex128) per column so that every scaled value t satisfies |t| < 1/2,
// rounded to the fixed-point integer V = round(t 2^49) (|V| <= 2^48) and
// split into 7 balanced base-128 digits,
//   V = sum_{a=1..7} d_a 128^{7-a},  |d_a| <= 64,
// each digit an integer that bf16 holds exactly. The rounding and the
// splitting are integer operations on the IEEE bit fields (FP64 arithmetic
// is slow on this part); the fixed point drops at most 2^-50 of the row or
// column scale per value. Rows of T or columns of X holding a non-finite
// value give NaN in R and in rmax. The product of two digits
// is at most 2^12 and is exact in FP32; the digit pairs (a, b) with
// a + b = g <= 8 (28 pairs, 7 levels g = 2..8) are summed per level in its
// own TMEM accumulator. A level collects at most 7 pairs, so over 512 real
// terms its partial sum stays below 7 * 2^21 < 2^24 and is exact; every 512
// terms the levels are read back and added, scaled by 2^{-7g}, into
// double-float (hi + lo FP32) sums, which carry ~48 bits. (A residual for a
// refinement sweep that is not the last may use the leading six digits of
// both operands: 21 pairs in 6 levels, ~2^-40 of the scales.) The pairs left out
// (a + b >= 9) and the truncation of both digit expansions are below 2^-47 of
// max|T_i.| max|X_.l| per term, the accuracy of the compensated FP32 kernel
// this replaces. The complex product uses the real mapping of the complex
// GEMM kernel: A' rows interleave (Re, Im) along k, B' rows are (Re, -Im) for
// the real part of an output column and (Im, Re) for its imaginary part.
//
// Layouts (bf16): the digit planes are written as the shared-memory images of
// the kernel's stages, so that a stage is two bulk copies. Stage ks covers 16
// real k (8 complex k); a plane image of R rows holds R x 16 bf16 in the
// canonical K-major no-swizzle layout (8-row x 16-byte core matrices, the two
// along k 128 B apart, 8-row groups 256 B apart):
//   T tile (node, 128-row tile mt, ks): planes a = 1..7 of 128 rows (28 KB)
//   X tile (node, 32-column tile nt, ks): planes b = 1..7 of 64 B' rows (14 KB)
// One CTA (128 threads) owns 128 rows x 32 complex columns of R: 7 levels x
// 64 FP32 TMEM columns. Thread 0 streams the stages through a four-stage
// ring (full / empty mbarriers, cp.async.bulk) and issues the 28 MMAs of a
// stage (K = 16 each); every 32 stages (512 real k) it waits for the MMAs and
// all threads add the level sums into their double-float accumulators. Every
// wait is bounded (1e9 SM cycles): on a timeout the CTA records an error,
// waits (bounded) for the copies and MMAs it started, frees its TMEM and
// returns without writing R.
#include <cstdint>
#include <cuda_bf16.h>
#include "qbg_common.cuh"
#include "qbg_handles.cuh"
#include "qbg_linalg.cuh"

namespace qbg {
namespace {

constexpr int RD = 7;                 // digits per operand (levels g = 2..8 of the full product)
constexpr int RBM = 128;              // rows of R per CTA
constexpr int RBN = 32;               // complex columns of R per CTA (B' rows: 64)
constexpr int RKS = 16;               // real k per stage (one MMA k-step)
constexpr int RCHUNK = 32;            // stages between exact flushes (512 real k)
constexpr int RNST = 4;               // stages in the ring
constexpr int RA_PLANE = RBM * RKS * 2;         // bytes of one T plane image (4096)
constexpr int RB_PLANE = 2 * RBN * RKS * 2;     // bytes of one X plane image (2048)
constexpr int RA_TILE = RD * RA_PLANE;          // 28672
constexpr int RB_TILE = RD * RB_PLANE;          // 14336
constexpr int RSTAGE = RA_TILE + RB_TILE;       // 43008
// stage layout for P digit planes per operand (P = RD for the refinement
// residual, 8 for the FP64 products of tc_gemm_sub_f64)
template <int P>
struct RLay {
  static constexpr int A_TILE = P * RA_PLANE;
  static constexpr int B_TILE = P * RB_PLANE;
  static constexpr int STAGE = A_TILE + B_TILE;
};
constexpr uint32_t RTMEM_COLS = 512;
constexpr long long RSPIN = 1ll << 26;
// D f32, A/B bf16, K-major, N = 64, M = 128
constexpr uint32_t R_IDESC = (1u << 4) | (1u << 7) | (1u << 10) | ((64u >> 3) << 17) | ((128u >> 4) << 24);

__device__ __forceinline__ uint32_t r_smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ uint64_t r_desc(uint32_t saddr) {
  uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)((128u >> 4) & 0x3FFFu) << 16;  // LBO: the two core matrices along k
  d |= (uint64_t)((256u >> 4) & 0x3FFFu) << 32;  // SBO: consecutive 8-row groups
  d |= (uint64_t)1 << 46;
  return d;
}

__device__ __forceinline__ void r_mma(uint32_t dtmem, uint64_t da, uint64_t db, uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(dtmem),
      "l"(da), "l"(db), "r"(R_IDESC), "r"(acc));
}

__device__ __forceinline__ void r_commit(uint32_t mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar) : "memory");
}

__device__ __forceinline__ bool r_wait(uint32_t mbar, uint32_t parity) {
  const long long t0 = clock64();
  for (long long it = 0; it < RSPIN; ++it) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(mbar), "r"(parity)
        : "memory");
    if (ok) return true;
    if (clock64() - t0 > 1000000000ll) break;
  }
  return false;
}


// byte offset of (row, real k kl < 16) inside a plane image (canonical K-major)
__device__ __forceinline__ uint32_t img_off(int row, int kl) {
  return (uint32_t)((row >> 3) * 256 + (kl >> 3) * 128 + (row & 7) * 16 + (kl & 7) * 2);
}

__device__ __forceinline__ void r_expect(uint32_t mbar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mbar), "r"(bytes) : "memory");
}

__device__ __forceinline__ void r_bulk(uint32_t dst, const void* src, uint32_t bytes, uint32_t mbar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
      "l"(src), "r"(bytes), "r"(mbar)
      : "memory");
}

// exact df32 accumulation of one FP32 value
__device__ __forceinline__ void df_add(float& hi, float& lo, float x) {
  const float s = hi + x;
  const float bb = s - hi;
  const float e = (hi - (s - bb)) + (x - bb);
  lo += e;
  const float h2 = s + lo;
  lo -= h2 - s;
  hi = h2;
}

}  // namespace

// ---------------------------------------------------------------------------
// digit preparation
// ---------------------------------------------------------------------------
constexpr int R_NONFINITE = 0x40000000;  // row / column exponent of a row / column with Inf or NaN

// round(v 2^Q) of an FP32 value as an integer, from its bit fields; the caller
// guarantees |v| 2^Q < 2^49 (so a shift left stays below 2^49)
__device__ __forceinline__ long long fx_f32(float v, int Q) {
  const uint32_t u = __float_as_uint(v);
  const int ex = (int)((u >> 23) & 255u);
  long long m = (long long)(ex ? ((u & 0x7FFFFFu) | 0x800000u) : (u & 0x7FFFFFu));
  const int sh = (ex ? ex : 1) - 150 + Q;
  if (sh >= 0) m <<= sh;
  else if (sh > -26) m = (m + (1ll << (-sh - 1))) >> (-sh);
  else m = 0;
  return (u >> 31) ? -m : m;
}

// round(v 2^Q) of an FP64 value as an integer (|v| 2^Q < 2^49)
__device__ __forceinline__ long long fx_f64(double v, int Q) {
  const unsigned long long u = (unsigned long long)__double_as_longlong(v);
  const int ex = (int)((u >> 52) & 2047u);
  long long m = (long long)(u & 0xFFFFFFFFFFFFFull);
  if (ex) m |= 1ll << 52;
  const int sh = (ex ? ex : 1) - 1075 + Q;
  if (sh >= 0) m <<= sh;
  else if (sh > -55) m = (m + (1ll << (-sh - 1))) >> (-sh);
  else m = 0;
  return (u >> 63) ? -m : m;
}

// P balanced base-128 digits of V (|V| <= 2^(7P - 1) + 1): d[0] most significant, |d| <= 64
template <int P>
__device__ __forceinline__ void digitsP(long long V, float* d) {
#pragma unroll
  for (int a = P - 1; a > 0; --a) {
    const int q = (int)(((uint32_t)V + 64u) & 127u) - 64;
    d[a] = (float)q;
    V = (V - q) >> 7;
  }
  d[0] = (float)V;
}

__device__ __forceinline__ void digits7(long long V, float* d) { digitsP<RD>(V, d); }

// row exponent e_i with max_k |T_ik| < 2^(e_i - 1) (re and im parts; T = hi + lo).
// From FP32 maxima: |hi + lo| <= max|hi| + max|lo|, and that sum rounded to
// FP32 is below a power of two whenever the exact sum is. Block (32, 8): 32
// rows, 8 column strides; grid (n/32, batch).
__global__ void k_t_rowexp(const cxf* __restrict__ Th, const cxf* __restrict__ Tl, long long sT, int n,
                           int* __restrict__ erow) {
  __shared__ float red[3][8][33];
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int i = blockIdx.x * 32 + tx;
  const long long b = blockIdx.y;
  const cxf* h = Th + b * sT;
  const cxf* l = Tl ? Tl + b * sT : nullptr;
  float mh = 0.f, ml = 0.f, chk = 0.f;  // chk turns NaN on any Inf or NaN (x * 0)
  if (i < n) {
    for (int j = ty; j < n; j += 8) {
      const long long e = (long long)i + (long long)j * n;
      const cxf v = h[e];
      mh = fmaxf(mh, fmaxf(fabsf(v.re), fabsf(v.im)));
      chk = fmaf(v.re, 0.f, fmaf(v.im, 0.f, chk));
      if (l) {
        const cxf w = l[e];
        ml = fmaxf(ml, fmaxf(fabsf(w.re), fabsf(w.im)));
        chk = fmaf(w.re, 0.f, fmaf(w.im, 0.f, chk));
      }
    }
  }
  red[0][ty][tx] = mh;
  red[1][ty][tx] = ml;
  red[2][ty][tx] = chk;
  __syncthreads();
  if (ty == 0 && i < n) {
    bool bad = false;
#pragma unroll
    for (int r = 0; r < 8; ++r) {
      mh = fmaxf(mh, red[0][r][tx]);
      ml = fmaxf(ml, red[1][r][tx]);
      bad |= (red[2][r][tx] != 0.f);
    }
    const float m = mh + ml;
    bad |= !(m <= 3.40282346638528859812e38f);  // the bound itself overflowed
    int E = 0;
    frexpf(m, &E);
    erow[b * n + i] = bad ? R_NONFINITE : (m > 0.f ? E + 1 : 0);
  }
}

// T digit planes through a 32 x 32 shared-memory transpose (column-major in,
// stage images out); grid (n/32, n/32, batch), block (32, 8). Each warp
// writes 128 contiguous bytes per plane: 8 rows x 4 complex k of one
// 16-byte core-matrix column.
__global__ void k_t_digits(const cxf* __restrict__ Th, const cxf* __restrict__ Tl, long long sT, int n, int MT,
                           int KS, const int* __restrict__ erow, unsigned char* __restrict__ TD) {
  __shared__ cxf th[32][33], tl[32][33];  // [column][row]
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int i0 = blockIdx.x * 32, k0 = blockIdx.y * 32;
  const long long b = blockIdx.z;
  const cxf* h = Th + b * sT;
  const cxf* l = Tl ? Tl + b * sT : nullptr;
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    const int c = ty + 8 * r, i = i0 + tx, k = k0 + c;
    cxf vh(0.f, 0.f), vl(0.f, 0.f);
    if (i < n && k < n) {
      const long long e = (long long)i + (long long)k * n;
      vh = h[e];
      if (l) vl = l[e];
    }
    th[c][tx] = vh;
    tl[c][tx] = vl;
  }
  __syncthreads();
  const int t = ty * 32 + tx;
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    const int w = t + 256 * r;
    const int e4 = w & 3, rr = (w >> 2) & 7, rg = (w >> 5) & 3, cs = w >> 7;  // cs: (stage, core column)
    const int il = rg * 8 + rr, kloc = (cs >> 1) * 8 + (cs & 1) * 4 + e4;
    const int i = i0 + il, k = k0 + kloc;
    if (i >= n || k >= n) continue;
    const cxf vh = th[kloc][il], vl = tl[kloc][il];
    const int e = erow[b * n + i];
    float dr[RD], di[RD];
    if (e == R_NONFINITE) {
#pragma unroll
      for (int a = 0; a < RD; ++a) { dr[a] = 0.f; di[a] = 0.f; }
    } else {
      const int Q = 49 - e;
      digits7(fx_f32(vh.re, Q) + fx_f32(vl.re, Q), dr);
      digits7(fx_f32(vh.im, Q) + fx_f32(vl.im, Q), di);
    }
    unsigned char* tile = TD + ((b * MT + (i >> 7)) * (long long)KS + (k >> 3)) * RA_TILE + img_off(i & 127, (2 * k) & 15);
#pragma unroll
    for (int a = 0; a < RD; ++a) {
      __nv_bfloat162 p;
      p.x = __float2bfloat16_rn(dr[a]);
      p.y = __float2bfloat16_rn(di[a]);
      *reinterpret_cast<__nv_bfloat162*>(tile + a * RA_PLANE) = p;
    }
  }
}

// column exponent f_l with max_k |X_kl| < 2^(f_l - 1); grid (L, batch)
__global__ void k_x_colexp(const cxd* __restrict__ X, long long sX, long long ldx, int n, int L,
                           int* __restrict__ fcol) {
  const int l = blockIdx.x;
  const long long b = blockIdx.y;
  const cxd* x = X + b * sX + (long long)l * ldx;
  double m = 0.0;
  int bad = 0;
  for (int k = threadIdx.x; k < n; k += blockDim.x) {
    const double a = fmax(fabs(x[k].re), fabs(x[k].im));
    bad |= !(a <= 1.79769313486231570815e308);  // Inf or NaN
    m = fmax(m, a);
  }
  __shared__ double red[32];
  __shared__ int redb[32];
  for (int o = 16; o > 0; o >>= 1) {
    m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    bad |= __shfl_xor_sync(0xffffffffu, bad, o);
  }
  if ((threadIdx.x & 31) == 0) { red[threadIdx.x >> 5] = m; redb[threadIdx.x >> 5] = bad; }
  __syncthreads();
  if (threadIdx.x < 32) {
    const bool in = threadIdx.x < (int)(blockDim.x >> 5);
    m = in ? red[threadIdx.x] : 0.0;
    bad = in ? redb[threadIdx.x] : 0;
    for (int o = 16; o > 0; o >>= 1) {
      m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
      bad |= __shfl_xor_sync(0xffffffffu, bad, o);
    }
    if (threadIdx.x == 0) {
      int E = 0;
      frexp(m, &E);
      fcol[b * L + l] = bad ? R_NONFINITE : (m > 0.0 ? E + 1 : 0);
    }
  }
}

// X digit planes (P per value, fixed point 2^(7P)) as stage images: column l
// of tile nt = l / 32 gives B' rows j = l % 32 (Re, -Im) and 32 + j (Im, Re)
// along k; columns l in [L, Lp) are zero. X: n rows (the k extent) per
// column, leading dimension ldx. grid (n/256, Lp, batch)
template <int P>
__global__ void k_x_digits(const cxd* __restrict__ X, long long sX, long long ldx, int n, int L, int NT, int KS,
                           const int* __restrict__ fcol, unsigned char* __restrict__ XD) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  const int l = blockIdx.y;
  const long long b = blockIdx.z;
  if (k >= n) return;
  float dr[P], di[P];
  const int f = l < L ? fcol[b * L + l] : R_NONFINITE;
  if (f == R_NONFINITE) {  // padding column, or a column holding Inf / NaN
#pragma unroll
    for (int a = 0; a < P; ++a) { dr[a] = 0.f; di[a] = 0.f; }
  } else {
    const cxd v = X[b * sX + (long long)l * ldx + k];
    digitsP<P>(fx_f64(v.re, 7 * P - f), dr);
    digitsP<P>(fx_f64(v.im, 7 * P - f), di);
  }
  const int j = l & (RBN - 1);
  unsigned char* tile = XD + ((b * NT + (l / RBN)) * (long long)KS + (k >> 3)) * RLay<P>::B_TILE;
  const uint32_t o_re = img_off(j, (2 * k) & 15), o_im = img_off(RBN + j, (2 * k) & 15);
#pragma unroll
  for (int a = 0; a < P; ++a) {
    __nv_bfloat162 pr, pi;
    pr.x = __float2bfloat16_rn(dr[a]);
    pr.y = __float2bfloat16_rn(-di[a]);
    pi.x = __float2bfloat16_rn(di[a]);
    pi.y = __float2bfloat16_rn(dr[a]);
    *reinterpret_cast<__nv_bfloat162*>(tile + a * RB_PLANE + o_re) = pr;
    *reinterpret_cast<__nv_bfloat162*>(tile + a * RB_PLANE + o_im) = pi;
  }
}

// A operand of tc_gemm_sub_f64 (complex128, M x K, leading dimension lda):
// row exponents e_i with max_k |A_ik| < 2^(e_i - 1); block (32, 8), grid
// (ceil(M / 32), batch)
__global__ void k_a_rowexp_f64(const cxd* __restrict__ A, long long sA, long long lda, int M, int K,
                               int* __restrict__ erow) {
  __shared__ double red[8][33];
  __shared__ int redb[8][33];
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int i = blockIdx.x * 32 + tx;
  const long long b = blockIdx.y;
  const cxd* a = A + b * sA;
  double m = 0.0;
  int bad = 0;
  if (i < M)
    for (int k = ty; k < K; k += 8) {
      const cxd v = a[(long long)i + (long long)k * lda];
      const double x = fmax(fabs(v.re), fabs(v.im));
      bad |= !(x <= 1.79769313486231570815e308);
      m = fmax(m, x);
    }
  red[ty][tx] = m;
  redb[ty][tx] = bad;
  __syncthreads();
  if (ty == 0 && i < M) {
#pragma unroll
    for (int r = 1; r < 8; ++r) {
      m = fmax(m, red[r][tx]);
      bad |= redb[r][tx];
    }
    int E = 0;
    frexp(m, &E);
    erow[b * M + i] = bad ? R_NONFINITE : (m > 0.0 ? E + 1 : 0);
  }
}

// A digit planes (P per value) as stage images, as k_t_digits for a
// complex128 M x K block; grid (ceil(M / 32), ceil(K / 32), batch), block
// (32, 8): a 32 x 32 shared-memory transpose, then each warp writes 8 rows x
// 4 complex k of one 16-byte core-matrix column per plane
template <int P>
__global__ void k_a_digits_f64(const cxd* __restrict__ A, long long sA, long long lda, int M, int K, int MT, int KS,
                               const int* __restrict__ erow, unsigned char* __restrict__ TD) {
  __shared__ cxd tv[32][33];  // [column][row]
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int i0 = blockIdx.x * 32, k0 = blockIdx.y * 32;
  const long long b = blockIdx.z;
  const cxd* a = A + b * sA;
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    const int c = ty + 8 * r, i = i0 + tx, k = k0 + c;
    tv[c][tx] = (i < M && k < K) ? a[(long long)i + (long long)k * lda] : cxd(0.0, 0.0);
  }
  __syncthreads();
  const int t = ty * 32 + tx;
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    const int w = t + 256 * r;
    const int e4 = w & 3, rr = (w >> 2) & 7, rg = (w >> 5) & 3, cs = w >> 7;  // cs: (stage, core column)
    const int il = rg * 8 + rr, kloc = (cs >> 1) * 8 + (cs & 1) * 4 + e4;
    const int i = i0 + il, k = k0 + kloc;
    if (i >= M || k >= K) continue;
    const cxd v = tv[kloc][il];
    const int e = erow[b * M + i];
    float dr[P], di[P];
    if (e == R_NONFINITE) {
#pragma unroll
      for (int q = 0; q < P; ++q) { dr[q] = 0.f; di[q] = 0.f; }
    } else {
      digitsP<P>(fx_f64(v.re, 7 * P - e), dr);
      digitsP<P>(fx_f64(v.im, 7 * P - e), di);
    }
    unsigned char* tile =
        TD + ((b * MT + (i >> 7)) * (long long)KS + (k >> 3)) * RLay<P>::A_TILE + img_off(i & 127, (2 * k) & 15);
#pragma unroll
    for (int q = 0; q < P; ++q) {
      __nv_bfloat162 pq;
      pq.x = __float2bfloat16_rn(dr[q]);
      pq.y = __float2bfloat16_rn(di[q]);
      *reinterpret_cast<__nv_bfloat162*>(tile + q * RA_PLANE) = pq;
    }
  }
}

// ---------------------------------------------------------------------------
// R = V - T X from the digit planes; grid (Lp / 32, ceil(n / 128), batch)
// ---------------------------------------------------------------------------
// ND <= RD: the leading ND digits of T and X, pairs a + b <= ND + 1 (ND levels);
// ND = RD is the full product, a smaller ND a residual to ~2^-(7 ND) of the
// scales (for refinement sweeps whose correction is not the last)
// P: digit planes per operand image (ND <= P); n: rows of T, V and R; ldv:
// leading dimension of V and R (column l of row i at i + l ldv)
template <int ND, int P>
__global__ void __launch_bounds__(128, 1) k_resid_tc(const unsigned char* __restrict__ TD,
                                                     const int* __restrict__ erow,
                                                     const unsigned char* __restrict__ XD,
                                                     const int* __restrict__ fcol, int n, int L, int MT, int NT, int KS,
                                                     const cxd* __restrict__ V, long long sV, cxd* R, long long sR,
                                                     long long ldv, unsigned long long* rmax, int* err) {
  constexpr int RA_TILE = RLay<P>::A_TILE, RB_TILE = RLay<P>::B_TILE, RSTAGE = RLay<P>::STAGE;
  // stages between exact flushes: a level of ND digits collects up to ND
  // pairs, so 16 stages (256 real k) keep eight-digit level sums below 2^23
  constexpr int RCHUNK = ND >= 8 ? 16 : 32;
  extern __shared__ __align__(1024) unsigned char r_smem[];
  uint64_t* full = reinterpret_cast<uint64_t*>(r_smem + RNST * RSTAGE);  // [RNST]
  uint64_t* empty = full + RNST;                                         // [RNST]
  uint64_t* fbar = empty + RNST;                                         // [1]
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(fbar + 1);
  int* abort_flag = reinterpret_cast<int*>(tmem_slot + 1);

  const int tid = threadIdx.x, warp = tid >> 5;
  const int nt = blockIdx.x, mt = blockIdx.y;
  const long long z = blockIdx.z;
  const int n0 = nt * RBN, m0 = mt * RBM;

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(r_smem_u32(tmem_slot)),
                 "r"(RTMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    for (int s = 0; s < RNST; ++s) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(r_smem_u32(full + s)) : "memory");
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(r_smem_u32(empty + s)) : "memory");
    }
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(r_smem_u32(fbar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    *abort_flag = (*reinterpret_cast<volatile int*>(err) != 0) ? 1 : 0;
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;
  const uint32_t sbase = r_smem_u32(r_smem);

  float acc_hi[2 * RBN], acc_lo[2 * RBN];
#pragma unroll
  for (int c = 0; c < 2 * RBN; ++c) { acc_hi[c] = 0.f; acc_lo[c] = 0.f; }

  // thread 0: producer and MMA issuer
  const unsigned char* ta = TD + (z * MT + mt) * (long long)KS * RA_TILE;
  const unsigned char* xb = XD + (z * NT + nt) * (long long)KS * RB_TILE;
  int issued = 0, consumed = 0, committed = 0, freed = 0;
  bool good = (*abort_flag == 0);
  // the leading ND planes of each tile image (planes are stored most significant first)
  auto issue = [&](int t) {
    const int s = t % RNST;
    const uint32_t fb = r_smem_u32(full + s);
    r_expect(fb, (uint32_t)(ND * (RA_PLANE + RB_PLANE)));
    r_bulk(sbase + (uint32_t)(s * RSTAGE), ta + (long long)t * RA_TILE, (uint32_t)(ND * RA_PLANE), fb);
    r_bulk(sbase + (uint32_t)(s * RSTAGE + RA_TILE), xb + (long long)t * RB_TILE, (uint32_t)(ND * RB_PLANE), fb);
  };
  if (tid == 0 && good)
    for (; issued < KS && issued < RNST; ++issued) issue(issued);

  const int nch = (KS + RCHUNK - 1) / RCHUNK;
  for (int ch = 0; ch < nch; ++ch) {
    if (tid == 0 && good) {
      uint32_t started = 0u;  // levels whose accumulator holds this chunk's sum (bit g - 2)
      const int k1 = min(KS, (ch + 1) * RCHUNK);
      for (int kt = ch * RCHUNK; kt < k1; ++kt) {
        const int s = kt % RNST;
        if (!r_wait(r_smem_u32(full + s), (uint32_t)((kt / RNST) & 1))) {
          good = false;
          break;
        }
        ++consumed;
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t so = sbase + (uint32_t)(s * RSTAGE);
#pragma unroll
        for (int a = 1; a <= ND; ++a) {
          const uint64_t da = r_desc(so + (uint32_t)((a - 1) * RA_PLANE));
#pragma unroll
          for (int bq = 1; bq + a <= ND + 1; ++bq) {
            const int g = a + bq;  // 2 .. 8
            const uint64_t db = r_desc(so + (uint32_t)(RA_TILE + (bq - 1) * RB_PLANE));
            const uint32_t bit = 1u << (g - 2);
            r_mma(tmem + (uint32_t)((g - 2) * 2 * RBN), da, db, (started & bit) ? 1u : 0u);
            started |= bit;
          }
        }
        r_commit(r_smem_u32(empty + s));
        ++committed;
        // refill the stage of tile kt - 1 once its MMAs are done
        if (kt >= 1 && issued < KS) {
          const int t = kt - 1;
          if (!r_wait(r_smem_u32(empty + t % RNST), (uint32_t)((t / RNST) & 1))) {
            good = false;
            break;
          }
          ++freed;
          issue(issued);
          ++issued;
        }
      }
      // every MMA of the chunk completes before the exact level sums are read back
      if (good) {
        r_commit(r_smem_u32(fbar));
        if (!r_wait(r_smem_u32(fbar), (uint32_t)(ch & 1))) good = false;
      }
      if (!good) *abort_flag = 1;
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const bool flush = (*abort_flag == 0);
    if (flush) {
      __syncwarp();
      const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16);
#pragma unroll 1
      for (int lev = 0; lev < ND; ++lev) {
        const float sc = ldexpf(1.f, -7 * (lev + 2));
#pragma unroll
        for (int qt = 0; qt < 4; ++qt) {
          uint32_t v[16];
          asm volatile(
              "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
              : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
                "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]),
                "=r"(v[15])
              : "r"(taddr + (uint32_t)(lev * 2 * RBN + qt * 16)));
          asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
          for (int c = 0; c < 16; ++c) df_add(acc_hi[qt * 16 + c], acc_lo[qt * 16 + c], __uint_as_float(v[c]) * sc);
        }
      }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (*abort_flag) break;
  }
  if (tid == 0 && *abort_flag) {
    atomicExch(err, 1);
    // bounded drain of what this thread started: copies, then MMA groups
    for (int t = consumed; t < issued; ++t) r_wait(r_smem_u32(full + t % RNST), (uint32_t)((t / RNST) & 1));
    for (int t = freed; t < committed; ++t) r_wait(r_smem_u32(empty + t % RNST), (uint32_t)((t / RNST) & 1));
  }
  if (*abort_flag == 0) {
    const int i = m0 + tid;
    if (i < n) {
      const int ei = erow[z * n + i];
      const cxd* Vb = V + z * sV;
      cxd* Rb = R + z * sR;
      double lmax = 0.0;
      bool bad = false;
#pragma unroll
      for (int c = 0; c < RBN; ++c) {
        const int col = n0 + c;
        if (col >= L) continue;  // full unroll keeps the sums in registers
        const int f = fcol[z * L + col];
        const long long e = (long long)i + (long long)col * ldv;
        const cxd v = Vb[e];
        cxd r;
        if (ei == R_NONFINITE || f == R_NONFINITE) {
          r = cxd(__longlong_as_double(0x7FF8000000000000ll), __longlong_as_double(0x7FF8000000000000ll));
        } else {
          const double re = ldexp((double)acc_hi[c] + (double)acc_lo[c], ei + f);
          const double im = ldexp((double)acc_hi[RBN + c] + (double)acc_lo[RBN + c], ei + f);
          r = cxd(v.re - re, v.im - im);
        }
        Rb[e] = r;
        const double a = fabs(r.re) + fabs(r.im);
        bad |= !(a == a);
        lmax = fmax(lmax, a);
      }
      // a NaN (bit pattern above +Inf) wins the unsigned maximum
      if (rmax)
        atomicMax(rmax, bad ? 0x7FF8000000000000ull : (unsigned long long)__double_as_longlong(lmax));
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(RTMEM_COLS) : "memory");
  }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
static int ks_of(int n) { return (2 * n + RKS - 1) / RKS; }
static int mt_of(int n) { return (n + RBM - 1) / RBM; }
static int lp_of(int L) { return ((L + RBN - 1) / RBN) * RBN; }
template <int P = RD>
static size_t r_smem_bytes() { return (size_t)RNST * RLay<P>::STAGE + 128; }

size_t tc_resid_T_bytes(int n, int batch) {
  const size_t dig = (size_t)batch * mt_of(n) * ks_of(n) * RA_TILE;
  return ((dig + 255) & ~(size_t)255) + (size_t)batch * n * sizeof(int);
}

int tc_resid_bind_T(TcResidT& t, int n, int batch, void* mem, cudaStream_t st) {
  t.n = n;
  t.batch = batch;
  t.MT = mt_of(n);
  t.KS = ks_of(n);
  const size_t dig = (size_t)batch * t.MT * t.KS * RA_TILE;
  t.TD = mem;
  t.erow = reinterpret_cast<int*>(static_cast<unsigned char*>(mem) + ((dig + 255) & ~(size_t)255));
  // rows beyond n and k beyond n stay zero in every image
  QBG_CUDA(cudaMemsetAsync(mem, 0, tc_resid_T_bytes(n, batch), st));
  return QBG_OK;
}

int tc_resid_prepare_T(TcResidT& t, const cxf* Th, const cxf* Tl, long long sT, int c, cudaStream_t st) {
  if (c > t.batch) {
    set_error("tc_resid_prepare_T: %d operators, room for %d", c, t.batch);
    return QBG_EINVAL;
  }
  const int n = t.n;
  k_t_rowexp<<<dim3((n + 31) / 32, c), dim3(32, 8), 0, st>>>(Th, Tl, sT, n, t.erow);
  QBG_LAUNCH_CHECK("k_t_rowexp");
  k_t_digits<<<dim3((n + 31) / 32, (n + 31) / 32, c), dim3(32, 8), 0, st>>>(
      Th, Tl, sT, n, t.MT, t.KS, t.erow, static_cast<unsigned char*>(t.TD));
  QBG_LAUNCH_CHECK("k_t_digits");
  return QBG_OK;
}

size_t tc_resid_X_bytes(int n, int L, int batch) {
  const size_t dig = (size_t)batch * (lp_of(L) / RBN) * ks_of(n) * RB_TILE;
  return ((dig + 255) & ~(size_t)255) + (size_t)batch * L * sizeof(int);
}

int tc_residual(const TcResidT& t, const cxd* X, long long sX, const cxd* V, long long sV, cxd* R, long long sR,
                int L, int c, double* rmax, void* xmem, cudaStream_t st, int ndig) {
  const int n = t.n, Lp = lp_of(L), NT = Lp / RBN;
  if (c > t.batch || c < 1 || c > 65535 || L < 1 || (ndig != RD && ndig != 6)) {
    set_error("tc_residual: bad sizes");
    return QBG_EINVAL;
  }
  const size_t dig = (size_t)c * NT * t.KS * RB_TILE;
  unsigned char* XD = static_cast<unsigned char*>(xmem);
  int* fcol = reinterpret_cast<int*>(XD + ((dig + 255) & ~(size_t)255));
  int* derr = nullptr;
  QBG_TRY(tc_error_ptr(&derr));
  static bool attr[64] = {};
  int dev = 0;
  QBG_CUDA(cudaGetDevice(&dev));
  if (dev >= 0 && dev < 64 && !attr[dev]) {
    QBG_CUDA(cudaFuncSetAttribute(k_resid_tc<RD, RD>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)r_smem_bytes()));
    QBG_CUDA(cudaFuncSetAttribute(k_resid_tc<6, RD>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)r_smem_bytes()));
    attr[dev] = true;
  }
  k_x_colexp<<<dim3(L, c), 256, 0, st>>>(X, sX, n, n, L, fcol);
  QBG_LAUNCH_CHECK("k_x_colexp");
  k_x_digits<RD><<<dim3((n + 255) / 256, Lp, c), 256, 0, st>>>(X, sX, n, n, L, NT, t.KS, fcol, XD);
  QBG_LAUNCH_CHECK("k_x_digits");
  if (ndig == 6)
    k_resid_tc<6, RD><<<dim3(NT, t.MT, c), 128, r_smem_bytes(), st>>>(
        static_cast<const unsigned char*>(t.TD), t.erow, XD, fcol, n, L, t.MT, NT, t.KS, V, sV, R, sR, n,
        reinterpret_cast<unsigned long long*>(rmax), derr);
  else
    k_resid_tc<RD, RD><<<dim3(NT, t.MT, c), 128, r_smem_bytes(), st>>>(
        static_cast<const unsigned char*>(t.TD), t.erow, XD, fcol, n, L, t.MT, NT, t.KS, V, sV, R, sR, n,
        reinterpret_cast<unsigned long long*>(rmax), derr);
  QBG_LAUNCH_CHECK("k_resid_tc");
  return QBG_OK;
}

// C_b -= A_b B_b (complex128; A: M x K, B: K x N, C: M x N, column-major with
// leading dimensions lda, ldb, ldc and batch strides sA, sB, sC). Both
// operands are cut into eight balanced 7-bit digits against the row maxima of
// A and the column maxima of B (56-bit fixed point), the 36 digit pairs with
// a + b <= 9 are multiplied exactly on the tensor cores into 8 TMEM level
// sums (exact FP32 integers over 256 real k), the levels are added in
// double-float and subtracted from C in FP64: per product term the error is
// ~2^-56 of max_k |A_ik| max_k |B_kj|, the order of an FP64 GEMM's rounding.
int tc_gemm_sub_f64(int M, int N, int K, const cxd* A, long long lda, long long sA, const cxd* B, long long ldb,
                    long long sB, cxd* C, long long ldc, long long sC, int batch, cudaStream_t st) {
  constexpr int P = 8;
  if (M < 1 || N < 1 || K < 1 || batch < 1 || batch > 65535 || lda < M || ldb < K || ldc < M) {
    set_error("tc_gemm_sub_f64: bad sizes");
    return QBG_EINVAL;
  }
  const int MT = (M + RBM - 1) / RBM, KS = (2 * K + RKS - 1) / RKS, Lp = lp_of(N), NT = Lp / RBN;
  const size_t td = (size_t)batch * MT * KS * RLay<P>::A_TILE;
  const size_t xd = (size_t)batch * NT * KS * RLay<P>::B_TILE;
  const size_t td_r = (td + 255) & ~(size_t)255, xd_r = (xd + 255) & ~(size_t)255;
  const size_t er = (((size_t)batch * M * sizeof(int)) + 255) & ~(size_t)255;
  const size_t bytes = td_r + xd_r + er + (size_t)batch * N * sizeof(int);
  int* derr = nullptr;
  QBG_TRY(tc_error_ptr(&derr));
  static bool attr[64] = {};
  int dev = 0;
  QBG_CUDA(cudaGetDevice(&dev));
  if (dev >= 0 && dev < 64 && !attr[dev]) {
    QBG_CUDA(cudaFuncSetAttribute(k_resid_tc<P, P>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)r_smem_bytes<P>()));
    attr[dev] = true;
  }
  unsigned char* mem = nullptr;
  QBG_TRY(dmalloc(&mem, bytes));
  unsigned char* TDm = mem;
  unsigned char* XDm = mem + td_r;
  int* erow = reinterpret_cast<int*>(mem + td_r + xd_r);
  int* fcol = reinterpret_cast<int*>(mem + td_r + xd_r + er);
  int s = QBG_OK;
  // images of rows past M, k past K or columns past N stay zero
  if (M % RBM || K % 8) {
    cudaError_t e = cudaMemsetAsync(TDm, 0, td, st);
    if (e != cudaSuccess) s = cuda_status(e, "tc_gemm_sub_f64 memset");
  }
  if (!s && (K % 8 || N % RBN)) {
    cudaError_t e = cudaMemsetAsync(XDm, 0, xd, st);
    if (e != cudaSuccess) s = cuda_status(e, "tc_gemm_sub_f64 memset");
  }
  auto launched = [&](const char* what) {
    note_launch();
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) s = cuda_status(e, what);
    return s == QBG_OK;
  };
  if (!s) {
    k_a_rowexp_f64<<<dim3((M + 31) / 32, batch), dim3(32, 8), 0, st>>>(A, sA, lda, M, K, erow);
    if (launched("k_a_rowexp_f64")) {
      k_a_digits_f64<P><<<dim3((M + 31) / 32, (K + 31) / 32, batch), dim3(32, 8), 0, st>>>(A, sA, lda, M, K, MT, KS,
                                                                                         erow, TDm);
      launched("k_a_digits_f64");
    }
  }
  if (!s) {
    k_x_colexp<<<dim3(N, batch), 256, 0, st>>>(B, sB, ldb, K, N, fcol);
    if (launched("k_x_colexp"))
      k_x_digits<P><<<dim3((K + 255) / 256, Lp, batch), 256, 0, st>>>(B, sB, ldb, K, N, NT, KS, fcol, XDm);
    launched("k_x_digits");
  }
  if (!s) {
    k_resid_tc<P, P><<<dim3(NT, MT, batch), 128, r_smem_bytes<P>(), st>>>(TDm, erow, XDm, fcol, M, N, MT, NT, KS,
                                                                           C, sC, C, sC, ldc, nullptr, derr);
    launched("k_resid_tc");
  }
  dfree(mem, st);
  return s;
}

}  // namespace qbg
