// Complex FP32 GEMM on the 5th-generation tensor cores (tcgen05, sm_103a).
//
//   C = alpha A B + beta C,  A: M x K, B: K x N, C: M x N complex64,
//   column-major, batched by blockIdx.z.
//
// Mapping of the complex product onto one real product D = A' B'^T:
//   A'[i][2k] = Re A(i,k), A'[i][2k+1] = Im A(i,k)                 (M x 2K)
//   B'[j][2k] = Re B(k,j), B'[j][2k+1] = -Im B(k,j)                 (rows 0..BN-1)
//   B'[BN+j][2k] = Im B(k,j), B'[BN+j][2k+1] = Re B(k,j)            (rows BN..2BN-1)
//   Re C(i,j) = D[i][j],  Im C(i,j) = D[i][BN+j].
// FP32 accuracy from TF32 units (3xTF32): every operand x is split as
// x = big + small with big = tf32(x), small = tf32(x - big), and
// D += A_big B_big + A_big B_small + A_small B_big (the dropped small*small
// term is ~2^-22 relative).
//
// One CTA (128 threads) computes a 128 x 32 complex tile (real 128 x 64,
// tcgen05.mma.cta_group::1.kind::tf32 with M = 128, N = 64, K = 8). Threads
// stage the operands in shared memory in the canonical K-major layout without
// swizzle (8-row x 16-byte core matrices; LBO = 128 B between the two core
// matrices along K, SBO = 256 B between 8-row groups) with 16-byte stores, in
// two stages of 16 complex k (48 KB each, two CTAs per SM); thread 0 issues
// the MMAs and commits each stage to its own mbarrier; the accumulator lives in
// 64 TMEM columns and is read back with tcgen05.ld.32x32b. C is fetched into
// registers before the k loop. Every mbarrier wait is
// bounded: on timeout the kernel records an error, waits (bounded) for its own
// MMAs, frees its TMEM and returns without writing C.
#include <algorithm>
#include <atomic>
#include <type_traits>
#include <cstdlib>
#include <cstdint>
#include <mutex>
#include <vector>
#include "qbg_common.cuh"
#include "qbg_handles.cuh"
#include "qbg_linalg.cuh"

namespace qbg {
namespace {

constexpr int TC_BM = 128;        // rows of C per CTA
constexpr int TC_BN = 32;         // complex columns of C per CTA (real N = 64)
constexpr int TC_BK = 16;         // complex k per stage (real K = 32 = 4 MMA steps of 8)
constexpr int TC_KSTEPS = 4;
constexpr int TC_A_STEP = TC_BM * 8;        // floats per operand block per MMA step (4 KB)
constexpr int TC_B_STEP = 2 * TC_BN * 8;    // floats (2 KB)
constexpr int TC_STAGE_FLOATS = 2 * TC_KSTEPS * (TC_A_STEP + TC_B_STEP);  // big + small, A and B (48 KB)
constexpr uint32_t TC_TMEM_COLS = 64;
constexpr long long TC_SPIN_LIMIT = 1ll << 26;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ float tf32_rna(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}


__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr) {
  const uint64_t lbo = 128, sbo = 256;
  uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= ((lbo >> 4) & 0x3FFFu) << 16;
  d |= ((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;  // descriptor version of this architecture family
  return d;                 // base offset 0, layout type 0 (no swizzle)
}

// instruction descriptor: D f32, A/B tf32, both K-major, N = 64, M = 128
constexpr uint32_t TC_IDESC = (1u << 4) | (2u << 7) | (2u << 10) | ((64u >> 3) << 17) | ((128u >> 4) << 24);

__device__ __forceinline__ void mma_tf32(uint32_t dtmem, uint64_t da, uint64_t db, uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(dtmem),
      "l"(da), "l"(db), "r"(TC_IDESC), "r"(acc));
}

__device__ __forceinline__ void mma_commit(uint32_t mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar) : "memory");
}

__device__ __forceinline__ bool mbar_try(uint32_t mbar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(mbar), "r"(parity)
      : "memory");
  return ok != 0;
}

// Poll limit of the pipeline waits (not of the drains that follow a give-up):
// TC_SPIN_LIMIT unless lowered by qbg_set_tc_wait_limit, which lets a test make
// a wait run out on purpose and check the error path. One copy per device.
__device__ long long g_tc_wait_polls = TC_SPIN_LIMIT;

// bounded wait: gives up after ~0.5 s of SM clock (1e9 cycles) or `polls` polls
__device__ __forceinline__ bool mbar_wait_bounded(uint32_t mbar, uint32_t parity,
                                                  long long polls = TC_SPIN_LIMIT) {
  const long long t0 = clock64();
  for (long long it = 0; it < polls; ++it) {
    if (mbar_try(mbar, parity)) return true;
    if (clock64() - t0 > 1000000000ll) break;
  }
  return false;
}


// Operand staging. A tile: thread = row i, 16 complex k of one k-tile, held in
// registers between the global load and the shared-memory store so that the
// loads of tile kt+1 are in flight while the tensor cores work on tile kt.
struct TcRegs {
  cxf a[TC_BK];   // A(m0 + tid, k0 + kc)
  cxf b[2][2];    // B(k0 + 2p + {0,1}, n0 + j) for the two (p, j) items of this thread
};

__device__ __forceinline__ void tc_load(TcRegs& r, const cxf* __restrict__ Ab, long long lda, const cxf* __restrict__ Bb,
                                        long long ldb, int M, int N, int K, int m0, int n0, int k0, int tid) {
  const int gi = m0 + tid;
  const bool rowok = gi < M;
#pragma unroll
  for (int kc = 0; kc < TC_BK; ++kc) {
    const int gk = k0 + kc;
    r.a[kc] = (rowok && gk < K) ? Ab[(long long)gi + (long long)gk * lda] : cxf(0.f, 0.f);
  }
#pragma unroll
  for (int q = 0; q < 2; ++q) {
    const int item = tid + 128 * q;
    const int j = item & (TC_BN - 1), p = item >> 5;  // j fastest: conflict-free shared stores
    const int gj = n0 + j, gk = k0 + 2 * p;
    const bool colok = gj < N;
    r.b[q][0] = (colok && gk < K) ? Bb[(long long)gk + (long long)gj * ldb] : cxf(0.f, 0.f);
    r.b[q][1] = (colok && gk + 1 < K) ? Bb[(long long)(gk + 1) + (long long)gj * ldb] : cxf(0.f, 0.f);
  }
}

// 16-byte row segment (k = 4c .. 4c+3) of core matrices in the K-major layout
__device__ __forceinline__ int kmaj4(int row, int c) { return (row >> 3) * 64 + c * 32 + (row & 7) * 4; }

__device__ __forceinline__ void split4(float x0, float x1, float x2, float x3, float4& big, float4& small) {
  big = make_float4(tf32_rna(x0), tf32_rna(x1), tf32_rna(x2), tf32_rna(x3));
  small = make_float4(tf32_rna(x0 - big.x), tf32_rna(x1 - big.y), tf32_rna(x2 - big.z), tf32_rna(x3 - big.w));
}

__device__ __forceinline__ void tc_store(const TcRegs& r, float* sAb, float* sAs, float* sBb, float* sBs, int tid) {
  // A'[i][2k] = Re, A'[i][2k+1] = Im; pair p = complex k 2p, 2p+1 -> MMA step p/2, 16-byte segment p%2
#pragma unroll
  for (int p = 0; p < TC_BK / 2; ++p) {
    float4 big, small;
    split4(r.a[2 * p].re, r.a[2 * p].im, r.a[2 * p + 1].re, r.a[2 * p + 1].im, big, small);
    const int off = (p >> 1) * TC_A_STEP + kmaj4(tid, p & 1);
    *reinterpret_cast<float4*>(sAb + off) = big;
    *reinterpret_cast<float4*>(sAs + off) = small;
  }
  // B'[j] = (Re, -Im) and B'[BN + j] = (Im, Re) along k
#pragma unroll
  for (int q = 0; q < 2; ++q) {
    const int item = tid + 128 * q;
    const int j = item & (TC_BN - 1), p = item >> 5;
    const cxf v0 = r.b[q][0], v1 = r.b[q][1];
    float4 big, small;
    const int base = (p >> 1) * TC_B_STEP;
    split4(v0.re, -v0.im, v1.re, -v1.im, big, small);
    *reinterpret_cast<float4*>(sBb + base + kmaj4(j, p & 1)) = big;
    *reinterpret_cast<float4*>(sBs + base + kmaj4(j, p & 1)) = small;
    split4(v0.im, v0.re, v1.im, v1.re, big, small);
    *reinterpret_cast<float4*>(sBb + base + kmaj4(TC_BN + j, p & 1)) = big;
    *reinterpret_cast<float4*>(sBs + base + kmaj4(TC_BN + j, p & 1)) = small;
  }
}

}  // namespace

// Two shared-memory stages: while the tensor cores read stage kt&1, the
// threads hold tile kt+1 in registers and then store it into the other stage
// once the MMAs of tile kt-1 (which read that stage) have been observed done.
__global__ void __launch_bounds__(128) k_tc_cgemm(int M, int N, int K, cxf alpha, const cxf* __restrict__ A,
                                                  long long lda, long long sA, const cxf* B, long long ldb,
                                                  long long sB, cxf beta, cxf* C, long long ldc, long long sC,
                                                  int batch2, long long sA2, long long sB2, long long sC2,
                                                  int* err) {
  extern __shared__ __align__(1024) unsigned char tc_smem[];
  float* stage_base = reinterpret_cast<float*>(tc_smem);  // [2][sAb | sAs | sBb | sBs]
  uint64_t* mbar = reinterpret_cast<uint64_t*>(stage_base + 2 * TC_STAGE_FLOATS);  // [2]
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(mbar + 2);
  int* abort_flag = reinterpret_cast<int*>(tmem_slot + 1);

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int m0 = blockIdx.x * TC_BM, n0 = blockIdx.y * TC_BN;
  const long long bo = blockIdx.z / batch2, bi = blockIdx.z % batch2;  // outer, inner batch index
  const cxf* Ab = A + bo * sA + bi * sA2;
  const cxf* Bb = B + bo * sB + bi * sB2;
  cxf* Cb = C + bo * sC + bi * sC2;

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(TC_TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(mbar)) : "memory");
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(mbar + 1)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    *abort_flag = (*reinterpret_cast<volatile int*>(err) != 0) ? 1 : 0;
  }

  // C of this thread's row, fetched now so that its latency hides behind the k loop
  const int i = m0 + warp * 32 + lane;  // TMEM lane = row within the tile = tid
  const bool use_beta = !(beta.re == 0.f && beta.im == 0.f);
  cxf cold[TC_BN];
#pragma unroll
  for (int j = 0; j < TC_BN; ++j) {
    const int gj = n0 + j;
    cold[j] = (use_beta && i < M && gj < N) ? Cb[(long long)i + (long long)gj * ldc] : cxf(0.f, 0.f);
  }

  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;
  const uint32_t mb0 = smem_u32(mbar), mb1 = smem_u32(mbar + 1);
  // per stage: parity of the next completion of its barrier, and whether a
  // commit to it has not been observed complete yet (uniform over the CTA)
  uint32_t wph0 = 0u, wph1 = 0u;
  bool pend0 = false, pend1 = false;
  const int ktiles = (K + TC_BK - 1) / TC_BK;
  bool ok = (*abort_flag == 0);

  TcRegs regs;
  if (ok && ktiles > 0) tc_load(regs, Ab, lda, Bb, ldb, M, N, K, m0, n0, 0, tid);
  for (int kt = 0; kt < ktiles && ok; ++kt) {
    const int st = kt & 1;
    float* sAb = stage_base + st * TC_STAGE_FLOATS;
    float* sAs = sAb + TC_KSTEPS * TC_A_STEP;
    float* sBb = sAs + TC_KSTEPS * TC_A_STEP;
    float* sBs = sBb + TC_KSTEPS * TC_B_STEP;
    if (st ? pend1 : pend0) {
      // the MMAs of tile kt-2 read this stage
      if (mbar_wait_bounded(st ? mb1 : mb0, st ? wph1 : wph0, g_tc_wait_polls)) {
        if (st) { wph1 ^= 1u; pend1 = false; } else { wph0 ^= 1u; pend0 = false; }
      } else {
        atomicExch(abort_flag, 1);
      }
    }
    tc_store(regs, sAb, sAs, sBb, sBs, tid);
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    if (*abort_flag) {
      ok = false;
      break;
    }
    if (kt + 1 < ktiles) tc_load(regs, Ab, lda, Bb, ldb, M, N, K, m0, n0, (kt + 1) * TC_BK, tid);
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll
      for (int s = 0; s < TC_KSTEPS; ++s) {
        const uint64_t dab = smem_desc(smem_u32(sAb + s * TC_A_STEP));
        const uint64_t das = smem_desc(smem_u32(sAs + s * TC_A_STEP));
        const uint64_t dbb = smem_desc(smem_u32(sBb + s * TC_B_STEP));
        const uint64_t dbs = smem_desc(smem_u32(sBs + s * TC_B_STEP));
        mma_tf32(tmem, das, dbb, (kt | s) != 0);
        mma_tf32(tmem, dab, dbs, 1);
        mma_tf32(tmem, dab, dbb, 1);
      }
      mma_commit(st ? mb1 : mb0);
    }
    if (st) pend1 = true; else pend0 = true;
  }
  // drain: every committed group must be observed before TMEM is read or released
  bool drained = true;
  if (pend0 && !mbar_wait_bounded(mb0, wph0)) drained = false;
  if (pend1 && !mbar_wait_bounded(mb1, wph1)) drained = false;
  if (!drained) atomicExch(abort_flag, 1);
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (*abort_flag || ktiles == 0) {
    if (tid == 0 && *abort_flag) atomicExch(err, 1);
  } else {
    const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16);
    uint32_t re[32], im[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(re[0]), "=r"(re[1]), "=r"(re[2]), "=r"(re[3]), "=r"(re[4]), "=r"(re[5]), "=r"(re[6]), "=r"(re[7]),
          "=r"(re[8]), "=r"(re[9]), "=r"(re[10]), "=r"(re[11]), "=r"(re[12]), "=r"(re[13]), "=r"(re[14]),
          "=r"(re[15]), "=r"(re[16]), "=r"(re[17]), "=r"(re[18]), "=r"(re[19]), "=r"(re[20]), "=r"(re[21]),
          "=r"(re[22]), "=r"(re[23]), "=r"(re[24]), "=r"(re[25]), "=r"(re[26]), "=r"(re[27]), "=r"(re[28]),
          "=r"(re[29]), "=r"(re[30]), "=r"(re[31])
        : "r"(taddr));
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(im[0]), "=r"(im[1]), "=r"(im[2]), "=r"(im[3]), "=r"(im[4]), "=r"(im[5]), "=r"(im[6]), "=r"(im[7]),
          "=r"(im[8]), "=r"(im[9]), "=r"(im[10]), "=r"(im[11]), "=r"(im[12]), "=r"(im[13]), "=r"(im[14]),
          "=r"(im[15]), "=r"(im[16]), "=r"(im[17]), "=r"(im[18]), "=r"(im[19]), "=r"(im[20]), "=r"(im[21]),
          "=r"(im[22]), "=r"(im[23]), "=r"(im[24]), "=r"(im[25]), "=r"(im[26]), "=r"(im[27]), "=r"(im[28]),
          "=r"(im[29]), "=r"(im[30]), "=r"(im[31])
        : "r"(taddr + (uint32_t)TC_BN));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
    if (i < M) {
#pragma unroll
      for (int j = 0; j < TC_BN; ++j) {
        const int gj = n0 + j;
        if (gj < N) {
          cxf v = alpha * cxf(__uint_as_float(re[j]), __uint_as_float(im[j]));
          if (use_beta) v += beta * cold[j];
          Cb[(long long)i + (long long)gj * ldc] = v;
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TC_TMEM_COLS) : "memory");
  }
}

// ---------------------------------------------------------------------------
// Packed-operand path: A and B are split and laid out once per call in the
// exact shared-memory images of the stages (k_tc_pack_a / k_tc_pack_b), and
// the GEMM streams them with one bulk copy per operand and stage through a
// four-stage ring; thread 0 issues the copies and the MMAs (full / empty
// mbarriers per stage), all threads prefetch C and run the epilogue.
//   PA tile (b, mt, kt): [big | small] x 4 MMA steps x 128 rows x 8 real k (32 KB)
//   PB tile (b, nt, kt): [big | small] x 4 MMA steps x 64 B' rows x 8 real k (16 KB)
// Every wait is bounded; on a timeout thread 0 records the error, waits
// (bounded) for the copies and MMAs it issued, and the CTA frees its TMEM and
// returns without writing C.
// ---------------------------------------------------------------------------
constexpr int PK_NST = 4;                                   // stages in the ring
constexpr int PK_A_TILE = 2 * TC_KSTEPS * TC_A_STEP;        // 8192 floats
constexpr int PK_B_TILE = 2 * TC_KSTEPS * TC_B_STEP;        // 4096 floats
constexpr int PK_STAGE = PK_A_TILE + PK_B_TILE;             // 12288 floats (48 KB)

// grid (MT, KT, batch * batch2), 128 threads: thread = row of the tile
__global__ void __launch_bounds__(128) k_tc_pack_a(const cxf* __restrict__ A, long long lda, long long sA,
                                                   long long sA2, int batch2, int M, int K, float* __restrict__ PA) {
  const int tid = threadIdx.x;
  const int mt = blockIdx.x, kt = blockIdx.y, MT = gridDim.x, KT = gridDim.y;
  const long long z = blockIdx.z, bo = z / batch2, bi = z % batch2;
  const cxf* Ab = A + bo * sA + bi * sA2;
  const int gi = mt * TC_BM + tid, k0 = kt * TC_BK;
  const bool rowok = gi < M;
  cxf a[TC_BK];
#pragma unroll
  for (int kc = 0; kc < TC_BK; ++kc) {
    const int gk = k0 + kc;
    a[kc] = (rowok && gk < K) ? Ab[(long long)gi + (long long)gk * lda] : cxf(0.f, 0.f);
  }
  float* tile = PA + ((z * MT + mt) * (long long)KT + kt) * PK_A_TILE;
#pragma unroll
  for (int p = 0; p < TC_BK / 2; ++p) {
    float4 big, small;
    split4(a[2 * p].re, a[2 * p].im, a[2 * p + 1].re, a[2 * p + 1].im, big, small);
    const int off = (p >> 1) * TC_A_STEP + kmaj4(tid, p & 1);
    *reinterpret_cast<float4*>(tile + off) = big;
    *reinterpret_cast<float4*>(tile + TC_KSTEPS * TC_A_STEP + off) = small;
  }
}

// grid (NT, KT, batch * batch2), 128 threads: two (column, k pair) items each
__global__ void __launch_bounds__(128) k_tc_pack_b(const cxf* __restrict__ B, long long ldb, long long sB,
                                                   long long sB2, int batch2, int N, int K, float* __restrict__ PB) {
  const int tid = threadIdx.x;
  const int nt = blockIdx.x, kt = blockIdx.y, NT = gridDim.x, KT = gridDim.y;
  const long long z = blockIdx.z, bo = z / batch2, bi = z % batch2;
  const cxf* Bb = B + bo * sB + bi * sB2;
  const int n0 = nt * TC_BN, k0 = kt * TC_BK;
  float* tile = PB + ((z * NT + nt) * (long long)KT + kt) * PK_B_TILE;
#pragma unroll
  for (int q = 0; q < 2; ++q) {
    const int item = tid + 128 * q;
    const int j = item & (TC_BN - 1), p = item >> 5;
    const int gj = n0 + j, gk = k0 + 2 * p;
    const bool colok = gj < N;
    const cxf v0 = (colok && gk < K) ? Bb[(long long)gk + (long long)gj * ldb] : cxf(0.f, 0.f);
    const cxf v1 = (colok && gk + 1 < K) ? Bb[(long long)(gk + 1) + (long long)gj * ldb] : cxf(0.f, 0.f);
    const int base = (p >> 1) * TC_B_STEP;
    float4 big, small;
    split4(v0.re, -v0.im, v1.re, -v1.im, big, small);
    *reinterpret_cast<float4*>(tile + base + kmaj4(j, p & 1)) = big;
    *reinterpret_cast<float4*>(tile + TC_KSTEPS * TC_B_STEP + base + kmaj4(j, p & 1)) = small;
    split4(v0.im, v0.re, v1.im, v1.re, big, small);
    *reinterpret_cast<float4*>(tile + base + kmaj4(TC_BN + j, p & 1)) = big;
    *reinterpret_cast<float4*>(tile + TC_KSTEPS * TC_B_STEP + base + kmaj4(TC_BN + j, p & 1)) = small;
  }
}

namespace {
__device__ __forceinline__ void pk_expect(uint32_t mbar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mbar), "r"(bytes) : "memory");
}

__device__ __forceinline__ void pk_bulk(uint32_t dst, const void* src, uint32_t bytes, uint32_t mbar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
      "l"(src), "r"(bytes), "r"(mbar)
      : "memory");
}
}  // namespace

// grid (MT, NT, batch * batch2), 128 threads
__global__ void __launch_bounds__(128, 1) k_tc_cgemm_pk(int M, int N, int KT, cxf alpha, const float* __restrict__ PA,
                                                        const float* __restrict__ PB, cxf beta, cxf* C, long long ldc,
                                                        long long sC, int batch2, long long sC2, int* err) {
  extern __shared__ __align__(1024) unsigned char pk_smem[];
  float* stages = reinterpret_cast<float*>(pk_smem);  // [PK_NST][A tile | B tile]
  uint64_t* full = reinterpret_cast<uint64_t*>(stages + PK_NST * PK_STAGE);  // [PK_NST]
  uint64_t* empty = full + PK_NST;                                          // [PK_NST]
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(empty + PK_NST);
  int* abort_flag = reinterpret_cast<int*>(tmem_slot + 1);

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int mt = blockIdx.x, nt = blockIdx.y, MT = gridDim.x, NT = gridDim.y;
  const long long z = blockIdx.z, bo = z / batch2, bi = z % batch2;
  const int m0 = mt * TC_BM, n0 = nt * TC_BN;
  cxf* Cb = C + bo * sC + bi * sC2;

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(TC_TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    for (int s = 0; s < PK_NST; ++s) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(full + s)) : "memory");
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(empty + s)) : "memory");
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    *abort_flag = (*reinterpret_cast<volatile int*>(err) != 0) ? 1 : 0;
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;
  // C of this thread's row, in flight while the k loop runs
  const int i = m0 + warp * 32 + lane;
  const bool use_beta = !(beta.re == 0.f && beta.im == 0.f);
  cxf cold[TC_BN];
#pragma unroll
  for (int j = 0; j < TC_BN; ++j) {
    const int gj = n0 + j;
    cold[j] = (use_beta && i < M && gj < N) ? Cb[(long long)i + (long long)gj * ldc] : cxf(0.f, 0.f);
  }

  if (tid == 0 && *abort_flag == 0) {
    const float* pa = PA + (z * MT + mt) * (long long)KT * PK_A_TILE;
    const float* pb = PB + (z * NT + nt) * (long long)KT * PK_B_TILE;
    const uint32_t sbase = smem_u32(stages);
    auto issue = [&](int t) {
      const int s = t % PK_NST;
      const uint32_t fb = smem_u32(full + s);
      pk_expect(fb, (uint32_t)(PK_STAGE * sizeof(float)));
      pk_bulk(sbase + (uint32_t)(s * PK_STAGE * sizeof(float)), pa + (long long)t * PK_A_TILE,
              (uint32_t)(PK_A_TILE * sizeof(float)), fb);
      pk_bulk(sbase + (uint32_t)((s * PK_STAGE + PK_A_TILE) * sizeof(float)), pb + (long long)t * PK_B_TILE,
              (uint32_t)(PK_B_TILE * sizeof(float)), fb);
    };
    int issued = 0;     // tiles whose copies were issued
    int consumed = 0;   // tiles whose full barrier was observed
    int committed = 0;  // tiles whose MMAs were committed
    int freed = 0;      // tiles whose empty barrier was observed
    bool good = true;
    for (; issued < KT && issued < PK_NST; ++issued) issue(issued);
    for (int kt = 0; kt < KT && good; ++kt) {
      const int s = kt % PK_NST;
      if (!mbar_wait_bounded(smem_u32(full + s), (uint32_t)((kt / PK_NST) & 1), g_tc_wait_polls)) {
        good = false;
        break;
      }
      ++consumed;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const float* sA = stages + s * PK_STAGE;
      const float* sB = sA + PK_A_TILE;
#pragma unroll
      for (int q = 0; q < TC_KSTEPS; ++q) {
        const uint64_t dab = smem_desc(smem_u32(sA + q * TC_A_STEP));
        const uint64_t das = smem_desc(smem_u32(sA + TC_KSTEPS * TC_A_STEP + q * TC_A_STEP));
        const uint64_t dbb = smem_desc(smem_u32(sB + q * TC_B_STEP));
        const uint64_t dbs = smem_desc(smem_u32(sB + TC_KSTEPS * TC_B_STEP + q * TC_B_STEP));
        mma_tf32(tmem, das, dbb, (kt | q) != 0);
        mma_tf32(tmem, dab, dbs, 1);
        mma_tf32(tmem, dab, dbb, 1);
      }
      mma_commit(smem_u32(empty + s));
      ++committed;
      // refill the stage of tile kt - 1 once its MMAs are done
      if (kt >= 1 && issued < KT) {
        const int t = kt - 1;
        if (!mbar_wait_bounded(smem_u32(empty + t % PK_NST), (uint32_t)((t / PK_NST) & 1), g_tc_wait_polls)) {
          good = false;
          break;
        }
        ++freed;
        issue(issued);
        ++issued;
      }
    }
    // every committed MMA group completes before TMEM is read or freed
    for (; good && freed < committed; ++freed)
      if (!mbar_wait_bounded(smem_u32(empty + freed % PK_NST), (uint32_t)((freed / PK_NST) & 1), g_tc_wait_polls))
        good = false;
    if (!good) {
      *abort_flag = 1;
      atomicExch(err, 1);
      // bounded drain of what this thread started: copies, then MMA groups
      for (int t = consumed; t < issued; ++t)
        mbar_wait_bounded(smem_u32(full + t % PK_NST), (uint32_t)((t / PK_NST) & 1));
      for (int t = freed; t < committed; ++t)
        mbar_wait_bounded(smem_u32(empty + t % PK_NST), (uint32_t)((t / PK_NST) & 1));
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (*abort_flag == 0 && KT > 0) {
    const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16);
    uint32_t re[32], im[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(re[0]), "=r"(re[1]), "=r"(re[2]), "=r"(re[3]), "=r"(re[4]), "=r"(re[5]), "=r"(re[6]), "=r"(re[7]),
          "=r"(re[8]), "=r"(re[9]), "=r"(re[10]), "=r"(re[11]), "=r"(re[12]), "=r"(re[13]), "=r"(re[14]),
          "=r"(re[15]), "=r"(re[16]), "=r"(re[17]), "=r"(re[18]), "=r"(re[19]), "=r"(re[20]), "=r"(re[21]),
          "=r"(re[22]), "=r"(re[23]), "=r"(re[24]), "=r"(re[25]), "=r"(re[26]), "=r"(re[27]), "=r"(re[28]),
          "=r"(re[29]), "=r"(re[30]), "=r"(re[31])
        : "r"(taddr));
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(im[0]), "=r"(im[1]), "=r"(im[2]), "=r"(im[3]), "=r"(im[4]), "=r"(im[5]), "=r"(im[6]), "=r"(im[7]),
          "=r"(im[8]), "=r"(im[9]), "=r"(im[10]), "=r"(im[11]), "=r"(im[12]), "=r"(im[13]), "=r"(im[14]),
          "=r"(im[15]), "=r"(im[16]), "=r"(im[17]), "=r"(im[18]), "=r"(im[19]), "=r"(im[20]), "=r"(im[21]),
          "=r"(im[22]), "=r"(im[23]), "=r"(im[24]), "=r"(im[25]), "=r"(im[26]), "=r"(im[27]), "=r"(im[28]),
          "=r"(im[29]), "=r"(im[30]), "=r"(im[31])
        : "r"(taddr + (uint32_t)TC_BN));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
    if (i < M) {
#pragma unroll
      for (int j = 0; j < TC_BN; ++j) {
        const int gj = n0 + j;
        if (gj < N) {
          cxf v = alpha * cxf(__uint_as_float(re[j]), __uint_as_float(im[j]));
          if (use_beta) v += beta * cold[j];
          Cb[(long long)i + (long long)gj * ldc] = v;
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TC_TMEM_COLS) : "memory");
  }
}

// ---------------------------------------------------------------------------
// Wide packed GEMM for large products (the LU's trailing updates): one CTA
// computes a 128 x 128 complex tile as one real M = 128, N = 256 MMA per k
// step (B' rows 0..127 = (Re, -Im) of the tile's columns, 128..255 =
// (Im, Re)), so an A tile read from L2 feeds four times the MMA work of the
// 128 x 32 tile. Accumulator: 256 TMEM columns (Re C in 0..127, Im C in
// 128..255). Operands are packed (split into big and small TF32 parts) in
// tiles of 4 KS complex k (KS MMA k steps), one bulk copy per operand and
// stage, through a four-stage ring:
//   PAW tile (b, mt, kt): [big | small] x KS MMA steps x 128 rows x 8 real k (8 KS KB)
//   PBW tile (b, nt, kt): [big | small] x KS MMA steps x 256 B' rows x 8 real k (16 KS KB)
// The epilogue reads the accumulator in 32-column chunks and updates C
// (beta C read there, not prefetched). Waits bounded as in k_tc_cgemm_pk.
// ---------------------------------------------------------------------------
constexpr int PW_BN = 128;                                  // complex columns per CTA (real N = 256)
constexpr int PW_NST = 4;                                   // stages in the ring
constexpr int PW_B_STEP = 2 * PW_BN * 8;                    // floats per B' block per MMA step (8 KB)
constexpr uint32_t PW_TMEM_COLS = 256;
// KS MMA k steps (4 KS complex k) per stage: KS = 2, 48 KB stages, one CTA per
// SM; KS = 1, 24 KB stages, two CTAs per SM (96 KB of stages and 256 TMEM
// columns each), so one CTA's epilogue and pipeline fill overlap the other's MMAs
template <int KS> struct PW {
  static constexpr int BK = 4 * KS;                           // complex k per stage
  static constexpr int A_TILE = 2 * KS * TC_A_STEP;           // floats
  static constexpr int B_TILE = 2 * KS * PW_B_STEP;
  static constexpr int STAGE = A_TILE + B_TILE;
  static constexpr int CTAS = KS == 1 ? 2 : 1;                // resident CTAs per SM
};
// instruction descriptor: D f32, A/B tf32, both K-major, N = 256, M = 128
constexpr uint32_t PW_IDESC = (1u << 4) | (2u << 7) | (2u << 10) | ((256u >> 3) << 17) | ((128u >> 4) << 24);

__device__ __forceinline__ void mma_tf32_w(uint32_t dtmem, uint64_t da, uint64_t db, uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(dtmem),
      "l"(da), "l"(db), "r"(PW_IDESC), "r"(acc));
}

// grid (MT, KTW, batch * batch2), 128 threads: thread = row of the tile
template <int KS>
__global__ void __launch_bounds__(128) k_tc_pack_aw(const cxf* __restrict__ A, long long lda, long long sA,
                                                    long long sA2, int batch2, int M, int K, float* __restrict__ PA) {
  constexpr int PW_BK = PW<KS>::BK, PW_KSTEPS = KS, PW_A_TILE = PW<KS>::A_TILE;
  const int tid = threadIdx.x;
  const int mt = blockIdx.x, kt = blockIdx.y, MT = gridDim.x, KT = gridDim.y;
  const long long z = blockIdx.z, bo = z / batch2, bi = z % batch2;
  const cxf* Ab = A + bo * sA + bi * sA2;
  const int gi = mt * TC_BM + tid, k0 = kt * PW_BK;
  const bool rowok = gi < M;
  cxf a[PW_BK];
#pragma unroll
  for (int kc = 0; kc < PW_BK; ++kc) {
    const int gk = k0 + kc;
    a[kc] = (rowok && gk < K) ? Ab[(long long)gi + (long long)gk * lda] : cxf(0.f, 0.f);
  }
  float* tile = PA + ((z * MT + mt) * (long long)KT + kt) * PW_A_TILE;
#pragma unroll
  for (int p = 0; p < PW_BK / 2; ++p) {
    float4 big, small;
    split4(a[2 * p].re, a[2 * p].im, a[2 * p + 1].re, a[2 * p + 1].im, big, small);
    const int off = (p >> 1) * TC_A_STEP + kmaj4(tid, p & 1);
    *reinterpret_cast<float4*>(tile + off) = big;
    *reinterpret_cast<float4*>(tile + PW_KSTEPS * TC_A_STEP + off) = small;
  }
}

// grid (NTW, KTW, batch * batch2), 128 threads: 2 KS (column, k pair) items each
template <int KS>
__global__ void __launch_bounds__(128) k_tc_pack_bw(const cxf* __restrict__ B, long long ldb, long long sB,
                                                    long long sB2, int batch2, int N, int K, float* __restrict__ PB) {
  constexpr int PW_BK = PW<KS>::BK, PW_KSTEPS = KS, PW_B_TILE = PW<KS>::B_TILE;
  const int tid = threadIdx.x;
  const int nt = blockIdx.x, kt = blockIdx.y, NT = gridDim.x, KT = gridDim.y;
  const long long z = blockIdx.z, bo = z / batch2, bi = z % batch2;
  const cxf* Bb = B + bo * sB + bi * sB2;
  const int n0 = nt * PW_BN, k0 = kt * PW_BK;
  float* tile = PB + ((z * NT + nt) * (long long)KT + kt) * PW_B_TILE;
#pragma unroll
  for (int q = 0; q < 2 * KS; ++q) {
    const int item = tid + 128 * q;
    const int j = item & (PW_BN - 1), p = item >> 7;  // j fastest: consecutive columns per warp
    const int gj = n0 + j, gk = k0 + 2 * p;
    const bool colok = gj < N;
    const cxf v0 = (colok && gk < K) ? Bb[(long long)gk + (long long)gj * ldb] : cxf(0.f, 0.f);
    const cxf v1 = (colok && gk + 1 < K) ? Bb[(long long)(gk + 1) + (long long)gj * ldb] : cxf(0.f, 0.f);
    const int base = (p >> 1) * PW_B_STEP;
    float4 big, small;
    split4(v0.re, -v0.im, v1.re, -v1.im, big, small);
    *reinterpret_cast<float4*>(tile + base + kmaj4(j, p & 1)) = big;
    *reinterpret_cast<float4*>(tile + PW_KSTEPS * PW_B_STEP + base + kmaj4(j, p & 1)) = small;
    split4(v0.im, v0.re, v1.im, v1.re, big, small);
    *reinterpret_cast<float4*>(tile + base + kmaj4(PW_BN + j, p & 1)) = big;
    *reinterpret_cast<float4*>(tile + PW_KSTEPS * PW_B_STEP + base + kmaj4(PW_BN + j, p & 1)) = small;
  }
}

// grid (MT, NTW, batch * batch2), 128 threads
template <int KS>
__global__ void __launch_bounds__(128, PW<KS>::CTAS) k_tc_cgemm_pkw(int M, int N, int KT, cxf alpha,
                                                                   const float* __restrict__ PA,
                                                                   const float* __restrict__ PB, cxf beta, cxf* C,
                                                                   long long ldc, long long sC, int batch2,
                                                                   long long sC2, int* err) {
  constexpr int PW_KSTEPS = KS, PW_A_TILE = PW<KS>::A_TILE, PW_B_TILE = PW<KS>::B_TILE, PW_STAGE = PW<KS>::STAGE;
  extern __shared__ __align__(1024) unsigned char pw_smem[];
  float* stages = reinterpret_cast<float*>(pw_smem);  // [PW_NST][A tile | B tile]
  uint64_t* full = reinterpret_cast<uint64_t*>(stages + PW_NST * PW_STAGE);  // [PW_NST]
  uint64_t* empty = full + PW_NST;                                          // [PW_NST]
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(empty + PW_NST);
  int* abort_flag = reinterpret_cast<int*>(tmem_slot + 1);

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int mt = blockIdx.x, nt = blockIdx.y, MT = gridDim.x, NT = gridDim.y;
  const long long z = blockIdx.z, bo = z / batch2, bi = z % batch2;
  const int m0 = mt * TC_BM, n0 = nt * PW_BN;
  cxf* Cb = C + bo * sC + bi * sC2;

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(PW_TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    for (int s = 0; s < PW_NST; ++s) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(full + s)) : "memory");
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(empty + s)) : "memory");
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    *abort_flag = (*reinterpret_cast<volatile int*>(err) != 0) ? 1 : 0;
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;

  if (tid == 0 && *abort_flag == 0) {
    const float* pa = PA + (z * MT + mt) * (long long)KT * PW_A_TILE;
    const float* pb = PB + (z * NT + nt) * (long long)KT * PW_B_TILE;
    const uint32_t sbase = smem_u32(stages);
    auto issue = [&](int t) {
      const int s = t % PW_NST;
      const uint32_t fb = smem_u32(full + s);
      pk_expect(fb, (uint32_t)(PW_STAGE * sizeof(float)));
      pk_bulk(sbase + (uint32_t)(s * PW_STAGE * sizeof(float)), pa + (long long)t * PW_A_TILE,
              (uint32_t)(PW_A_TILE * sizeof(float)), fb);
      pk_bulk(sbase + (uint32_t)((s * PW_STAGE + PW_A_TILE) * sizeof(float)), pb + (long long)t * PW_B_TILE,
              (uint32_t)(PW_B_TILE * sizeof(float)), fb);
    };
    int issued = 0, consumed = 0, committed = 0, freed = 0;
    bool good = true;
    for (; issued < KT && issued < PW_NST; ++issued) issue(issued);
    for (int kt = 0; kt < KT && good; ++kt) {
      const int s = kt % PW_NST;
      if (!mbar_wait_bounded(smem_u32(full + s), (uint32_t)((kt / PW_NST) & 1), g_tc_wait_polls)) {
        good = false;
        break;
      }
      ++consumed;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const float* sA = stages + s * PW_STAGE;
      const float* sB = sA + PW_A_TILE;
#pragma unroll
      for (int q = 0; q < PW_KSTEPS; ++q) {
        const uint64_t dab = smem_desc(smem_u32(sA + q * TC_A_STEP));
        const uint64_t das = smem_desc(smem_u32(sA + PW_KSTEPS * TC_A_STEP + q * TC_A_STEP));
        const uint64_t dbb = smem_desc(smem_u32(sB + q * PW_B_STEP));
        const uint64_t dbs = smem_desc(smem_u32(sB + PW_KSTEPS * PW_B_STEP + q * PW_B_STEP));
        mma_tf32_w(tmem, das, dbb, (kt | q) != 0);
        mma_tf32_w(tmem, dab, dbs, 1);
        mma_tf32_w(tmem, dab, dbb, 1);
      }
      mma_commit(smem_u32(empty + s));
      ++committed;
      if (kt >= 1 && issued < KT) {  // refill the stage of tile kt - 1 once its MMAs are done
        const int t = kt - 1;
        if (!mbar_wait_bounded(smem_u32(empty + t % PW_NST), (uint32_t)((t / PW_NST) & 1), g_tc_wait_polls)) {
          good = false;
          break;
        }
        ++freed;
        issue(issued);
        ++issued;
      }
    }
    for (; good && freed < committed; ++freed)
      if (!mbar_wait_bounded(smem_u32(empty + freed % PW_NST), (uint32_t)((freed / PW_NST) & 1), g_tc_wait_polls))
        good = false;
    if (!good) {
      *abort_flag = 1;
      atomicExch(err, 1);
      for (int t = consumed; t < issued; ++t)
        mbar_wait_bounded(smem_u32(full + t % PW_NST), (uint32_t)((t / PW_NST) & 1));
      for (int t = freed; t < committed; ++t)
        mbar_wait_bounded(smem_u32(empty + t % PW_NST), (uint32_t)((t / PW_NST) & 1));
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (*abort_flag == 0 && KT > 0) {
    const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16);
    const int i = m0 + warp * 32 + lane;
    const bool use_beta = !(beta.re == 0.f && beta.im == 0.f);
#pragma unroll 1
    for (int ch = 0; ch < PW_BN / 32; ++ch) {
      uint32_t re[32], im[32];
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
          "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
          : "=r"(re[0]), "=r"(re[1]), "=r"(re[2]), "=r"(re[3]), "=r"(re[4]), "=r"(re[5]), "=r"(re[6]), "=r"(re[7]),
            "=r"(re[8]), "=r"(re[9]), "=r"(re[10]), "=r"(re[11]), "=r"(re[12]), "=r"(re[13]), "=r"(re[14]),
            "=r"(re[15]), "=r"(re[16]), "=r"(re[17]), "=r"(re[18]), "=r"(re[19]), "=r"(re[20]), "=r"(re[21]),
            "=r"(re[22]), "=r"(re[23]), "=r"(re[24]), "=r"(re[25]), "=r"(re[26]), "=r"(re[27]), "=r"(re[28]),
            "=r"(re[29]), "=r"(re[30]), "=r"(re[31])
          : "r"(taddr + (uint32_t)(ch * 32)));
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
          "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
          : "=r"(im[0]), "=r"(im[1]), "=r"(im[2]), "=r"(im[3]), "=r"(im[4]), "=r"(im[5]), "=r"(im[6]), "=r"(im[7]),
            "=r"(im[8]), "=r"(im[9]), "=r"(im[10]), "=r"(im[11]), "=r"(im[12]), "=r"(im[13]), "=r"(im[14]),
            "=r"(im[15]), "=r"(im[16]), "=r"(im[17]), "=r"(im[18]), "=r"(im[19]), "=r"(im[20]), "=r"(im[21]),
            "=r"(im[22]), "=r"(im[23]), "=r"(im[24]), "=r"(im[25]), "=r"(im[26]), "=r"(im[27]), "=r"(im[28]),
            "=r"(im[29]), "=r"(im[30]), "=r"(im[31])
          : "r"(taddr + (uint32_t)(PW_BN + ch * 32)));
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
      if (i < M) {
        cxf cold[32];
#pragma unroll
        for (int j = 0; j < 32; ++j) {
          const int gj = n0 + ch * 32 + j;
          cold[j] = (use_beta && gj < N) ? Cb[(long long)i + (long long)gj * ldc] : cxf(0.f, 0.f);
        }
#pragma unroll
        for (int j = 0; j < 32; ++j) {
          const int gj = n0 + ch * 32 + j;
          if (gj < N) {
            cxf v = alpha * cxf(__uint_as_float(re[j]), __uint_as_float(im[j]));
            if (use_beta) v += beta * cold[j];
            Cb[(long long)i + (long long)gj * ldc] = v;
          }
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(PW_TMEM_COLS) : "memory");
  }
}

// device error flag of the tensor-core GEMM (one per device, found by symbol)
__device__ int g_tc_err;

static size_t tc_smem_bytes() { return sizeof(float) * (size_t)(2 * TC_STAGE_FLOATS) + 64; }
static size_t pk_smem_bytes() { return sizeof(float) * (size_t)(PK_NST * PK_STAGE) + 16 * PK_NST + 64; }
template <int KS>
static size_t pw_smem_bytes() { return sizeof(float) * (size_t)(PW_NST * PW<KS>::STAGE) + 16 * PW_NST + 64; }

namespace {
constexpr int TC_MAX_DEV = 64;
std::mutex g_tc_mu;
int* g_tc_err_addr[TC_MAX_DEV] = {};
bool g_tc_attr[TC_MAX_DEV] = {};
std::atomic<int> g_engine{GEMM_ENGINE_TCGEN05};
std::atomic<bool> g_pk_enabled{true};  // packed-operand path of tc_gemm_c64
// wide-tile packed path: QBG_GEMM_WIDE in the environment, 0 keeps the
// 128 x 32 tiles, 1 one wide CTA per SM (48 KB stages), 2 (default) two per
// SM (24 KB stages; C2 factor phase 28.1 -> 26.7 ms against 1)
std::atomic<int> g_pkw_mode{[] {
  const char* e = std::getenv("QBG_GEMM_WIDE");
  return (e && *e) ? std::max(0, std::min(std::atoi(e), 2)) : 2;
}()};

int tc_device_setup(int** err_out) {
  int dev = 0;
  QBG_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= TC_MAX_DEV) {
    set_error("device ordinal %d out of range", dev);
    return QBG_ECUDA;
  }
  std::lock_guard<std::mutex> lk(g_tc_mu);
  if (!g_tc_attr[dev]) {
    QBG_CUDA(cudaFuncSetAttribute(k_tc_cgemm, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tc_smem_bytes()));
    QBG_CUDA(cudaFuncSetAttribute(k_tc_cgemm_pk, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)pk_smem_bytes()));
    QBG_CUDA(cudaFuncSetAttribute(k_tc_cgemm_pkw<2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)pw_smem_bytes<2>()));
    QBG_CUDA(cudaFuncSetAttribute(k_tc_cgemm_pkw<1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)pw_smem_bytes<1>()));
    void* a = nullptr;
    QBG_CUDA(cudaGetSymbolAddress(&a, g_tc_err));
    g_tc_err_addr[dev] = static_cast<int*>(a);
    g_tc_attr[dev] = true;
  }
  *err_out = g_tc_err_addr[dev];
  return QBG_OK;
}

// Packing scratch, one buffer per (device, stream): the GEMMs of one stream
// run in order, so a stream reuses its buffer without waiting; a larger
// request replaces it (the old block goes back to the pool behind the stream's
// work). The owner of a stream returns its buffer with tc_release_scratch
// before destroying the stream.
struct PackScratch {
  int dev;
  cudaStream_t st;
  void* p;
  size_t bytes;
};
std::mutex g_pack_mu;
std::vector<PackScratch> g_pack;

int pack_scratch(cudaStream_t st, size_t bytes, void** out) {
  int dev = 0;
  QBG_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(g_pack_mu);
  for (auto& e : g_pack)
    if (e.dev == dev && e.st == st) {
      if (e.bytes < bytes) {
        void* q = nullptr;
        QBG_TRY(dmalloc(&q, bytes));
        dfree(e.p, st);
        e.p = q;
        e.bytes = bytes;
      }
      *out = e.p;
      return QBG_OK;
    }
  void* q = nullptr;
  QBG_TRY(dmalloc(&q, bytes));
  g_pack.push_back({dev, st, q, bytes});
  *out = q;
  return QBG_OK;
}
}  // namespace

int tc_error_ptr(int** p) { return tc_device_setup(p); }

void tc_release_scratch(cudaStream_t st) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return;
  std::lock_guard<std::mutex> lk(g_pack_mu);
  for (size_t q = 0; q < g_pack.size(); ++q)
    if (g_pack[q].dev == dev && g_pack[q].st == st) {
      dfree(g_pack[q].p, st);
      g_pack.erase(g_pack.begin() + (long)q);
      return;
    }
}

void set_gemm_engine(int e) {
  g_engine.store(e == GEMM_ENGINE_SIMT ? GEMM_ENGINE_SIMT : GEMM_ENGINE_TCGEN05);
  g_pk_enabled.store(e != GEMM_ENGINE_TCGEN05_STAGED);
}
int gemm_engine() { return g_engine.load(); }

int tc_gemm_c64(int M, int N, int K, cxf alpha, const cxf* A, long long lda, long long sA, const cxf* B,
                long long ldb, long long sB, cxf beta, cxf* C, long long ldc, long long sC, int batch,
                cudaStream_t st, int batch2, long long sA2, long long sB2, long long sC2, bool allow_packed) {
  if (M <= 0 || N <= 0 || batch <= 0 || batch2 <= 0) return QBG_OK;
  if (K <= 0 || (long long)batch * batch2 > 65535) {
    set_error("tc_gemm_c64: K = %d, batch = %d x %d out of range", K, batch, batch2);
    return QBG_EINVAL;
  }
  int* derr = nullptr;
  if (int s = tc_device_setup(&derr)) return s;
  const int MT = (M + TC_BM - 1) / TC_BM, NT = (N + TC_BN - 1) / TC_BN, KT = (K + TC_BK - 1) / TC_BK;
  const int nb = batch * batch2;
  // packed path where packing pays: each packed A tile is read by NT CTAs and
  // each B tile by MT CTAs (measured on the FP32 LU of 48 operators of
  // N = 2048: faster from the 512 x 512 trailing updates up; the skinny solve
  // products, N = 64, and the updates inside an outer block are faster staged)
  // wide tiles (128 x 128 complex) for the large products: N of at least two
  // wide tiles and enough tiles to fill the device, or one mostly full wide
  // tile (the triangular-solve products of a 128-column block) and half as
  // many tiles (the other stream parts' products fill the rest; C2 solve
  // phase 33.7 -> 29.0 ms)
  const int wide = g_pkw_mode.load();  // 0 off, 1 one CTA per SM (KS = 2), 2 two CTAs per SM (KS = 1)
  const int NTW = (N + PW_BN - 1) / PW_BN, KTW8 = (K + 7) / 8;
  if (allow_packed && g_pk_enabled.load() && wide > 0 && KTW8 >= 4 && (NTW >= 2 || N >= 96) &&
      (long long)MT * NTW * nb >= (NTW >= 2 ? 152 : 64)) {
    auto run = [&](auto ks) -> int {
      constexpr int KS = decltype(ks)::value;
      const int KTW = (K + PW<KS>::BK - 1) / PW<KS>::BK;
      const size_t pa = (size_t)nb * MT * KTW * PW<KS>::A_TILE, pb = (size_t)nb * NTW * KTW * PW<KS>::B_TILE;
      void* scr = nullptr;
      QBG_TRY(pack_scratch(st, sizeof(float) * (pa + pb), &scr));
      float* PA = static_cast<float*>(scr);
      float* PB = PA + pa;
      k_tc_pack_aw<KS><<<dim3(MT, KTW, nb), 128, 0, st>>>(A, lda, sA, sA2, batch2, M, K, PA);
      QBG_LAUNCH_CHECK("k_tc_pack_aw");
      k_tc_pack_bw<KS><<<dim3(NTW, KTW, nb), 128, 0, st>>>(B, ldb, sB, sB2, batch2, N, K, PB);
      QBG_LAUNCH_CHECK("k_tc_pack_bw");
      k_tc_cgemm_pkw<KS><<<dim3(MT, NTW, nb), 128, pw_smem_bytes<KS>(), st>>>(M, N, KTW, alpha, PA, PB, beta, C,
                                                                               ldc, sC, batch2, sC2, derr);
      QBG_LAUNCH_CHECK("k_tc_cgemm_pkw");
      return QBG_OK;
    };
    return wide == 2 ? run(std::integral_constant<int, 1>{}) : run(std::integral_constant<int, 2>{});
  }
  if (allow_packed && g_pk_enabled.load() && KT >= 2 && MT >= 4 && NT >= 8) {
    const size_t pa = (size_t)nb * MT * KT * PK_A_TILE, pb = (size_t)nb * NT * KT * PK_B_TILE;
    void* scr = nullptr;
    QBG_TRY(pack_scratch(st, sizeof(float) * (pa + pb), &scr));
    float* PA = static_cast<float*>(scr);
    float* PB = PA + pa;
    k_tc_pack_a<<<dim3(MT, KT, nb), 128, 0, st>>>(A, lda, sA, sA2, batch2, M, K, PA);
    QBG_LAUNCH_CHECK("k_tc_pack_a");
    k_tc_pack_b<<<dim3(NT, KT, nb), 128, 0, st>>>(B, ldb, sB, sB2, batch2, N, K, PB);
    QBG_LAUNCH_CHECK("k_tc_pack_b");
    k_tc_cgemm_pk<<<dim3(MT, NT, nb), 128, pk_smem_bytes(), st>>>(M, N, KT, alpha, PA, PB, beta, C, ldc, sC, batch2,
                                                                   sC2, derr);
    QBG_LAUNCH_CHECK("k_tc_cgemm_pk");
    return QBG_OK;
  }
  dim3 grd(MT, NT, nb);
  k_tc_cgemm<<<grd, 128, tc_smem_bytes(), st>>>(M, N, K, alpha, A, lda, sA, B, ldb, sB, beta, C, ldc, sC, batch2,
                                                 sA2, sB2, sC2, derr);
  QBG_LAUNCH_CHECK("k_tc_cgemm");
  return QBG_OK;
}

// runtime pipeline-wait limit (polls; < 0 restores the built-in limit) and
// reset of the sticky error flag, on the current device
int tc_set_wait_limit(long long polls) {
  int* derr = nullptr;
  if (int s = tc_device_setup(&derr)) return s;
  const long long v = polls < 0 ? TC_SPIN_LIMIT : polls;
  QBG_CUDA(cudaDeviceSynchronize());
  QBG_CUDA(cudaMemcpyToSymbol(g_tc_wait_polls, &v, sizeof(v)));
  return QBG_OK;
}

int tc_clear_error() {
  int* derr = nullptr;
  if (int s = tc_device_setup(&derr)) return s;
  QBG_CUDA(cudaDeviceSynchronize());
  QBG_CUDA(cudaMemset(derr, 0, sizeof(int)));
  return QBG_OK;
}

int tc_check(cudaStream_t st) {
  int* derr = nullptr;
  if (int s = tc_device_setup(&derr)) return s;
  QBG_CUDA(cudaStreamSynchronize(st));
  int h = 0;
  QBG_CUDA(cudaMemcpy(&h, derr, sizeof(int), cudaMemcpyDeviceToHost));
  if (h != 0) {
    // sticky for the process, like a CUDA context error: every handle sees it
    set_error("tensor-core GEMM: an mbarrier wait gave up; results discarded");
    return QBG_ECUDA;
  }
  return QBG_OK;
}

}  // namespace qbg
