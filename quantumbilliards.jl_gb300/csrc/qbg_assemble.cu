// Fused multi-k assembly of the Kress-corrected boundary operators.
//
// One thread owns one matrix entry (i, j) and loops over all wavenumbers of
// the batch: the k-independent pair geometry (distance, source-normal inner
// product, periodic log term, circulant Kress weight, quadrature weight) is
// formed once in registers and reused for every k. Consecutive threads of a
// warp own consecutive rows i of the same column j, so every store of every
// k is a coalesced 32 x 16 B (FP64) or 32 x 8 B (mixed) segment of the
// column-major output (Julia Matrix{ComplexF64} layout).
//
// Formulas (all cited from QuantumBilliards.jl):
//   DLP  F = I - D                                  dlp_kress.jl:906-932
//        D_ij = R_ij l1 + w_j l2,  l1 = -(k/2pi) inner J1(kr)/r,
//        l2 = (ik/2) inner H1(kr)/r - l1 log(4 sin^2((t_i-t_j)/2)),
//        D_ii = w_i kappa_i
//   dF/dk, d2F/dk2 (diagonal 0)                      dlp_kress.jl:975-1075
//   CFIE A = I - (D + ik S), same component:         cfie_kress.jl:416-480
//        S_ij = R_ij m1 + w_j m2, m1 = -J0 s_j/2pi, m2 = (i/2) H0 s_j - m1 lt
//        diagonal with the finite part log(k^2 s^2/4)   cfie_kress.jl:436-445
//   CFIE cross-component (smooth kernel)              cfie_kress.jl:480-503
//   complex k: J0/J1 evaluated separately from H0/H1 and the coefficients
//   hoisted exactly as chebyshev_euclidian_helmholtz_cfie_kress.jl:596-611.
#include "qbg_assemble.cuh"
#include "qbg_bessel.cuh"

namespace qbg {

static __device__ __forceinline__ double pair_logterm(double ti, double tj) {
  double s = sin(0.5 * (ti - tj));
  return log(4.0 * s * s);
}

struct PairGeom {
  bool same;
  double r, invr, inn, lt, Rk, wj, sj;
};

static __device__ __forceinline__ PairGeom pair_geom(const GeomDev& g, int i, int j) {
  PairGeom p;
  const double dxij = g.x[i] - g.x[j], dyij = g.y[i] - g.y[j];
  p.r = hypot(dxij, dyij);
  p.invr = 1.0 / p.r;
  p.inn = g.dy[j] * dxij - g.dx[j] * dyij;
  p.wj = g.ws[j];
  p.sj = g.speed[j];
  const int ci = g.comp[i], cj = g.comp[j];
  p.same = (ci == cj);
  if (p.same) {
    const int o = g.coff[ci], na = g.coff[ci + 1] - o;
    int d = g.lidx[i] - g.lidx[j];
    d += (d < 0) ? na : 0;
    p.Rk = g.kcol[o + d];
    p.lt = pair_logterm(g.ts[i], g.ts[j]);
  } else {
    p.Rk = 0.0;
    p.lt = 0.0;
  }
  return p;
}

// ---------------------------------------------------------------------------
// FP64 entry for one wavenumber
// ---------------------------------------------------------------------------
template <int FORM, int DERIV>
static __device__ __forceinline__ void entry_fp64(const PairGeom& p, cxd k, bool realk, cxd* F, cxd* F1,
                                                  cxd* F2) {
  const double inv2pi = 0.15915494309189533577;
  cxd z = p.r * k;
  Bessel01d b = bessel01(z);
  if (realk) {  // reference: J = Re H for real k (dlp_kress.jl:821-822)
    b.j0.im = 0.0;
    b.j1.im = 0.0;
  }
  const cxd h0 = b.h0(), h1 = b.h1(), j0 = b.j0, j1 = b.j1;
  const cxd ik = cmul_i(k);
  const cxd aL1 = (-inv2pi) * k;
  const cxd aL2 = 0.5 * ik;
  if (FORM == 1 && !p.same) {
    // smooth cross-component kernel
    cxd dval = (p.wj * p.inn * p.invr) * (aL2 * h1);
    cxd sval = (p.wj * p.sj) * cmul_i(0.5 * h0);
    *F = -(dval + ik * sval);
    return;
  }
  const double cD1 = p.Rk * p.inn * p.invr, cD2 = p.wj * p.inn * p.invr, cD3 = p.wj * p.lt * p.inn * p.invr;
  const cxd L1 = aL1 * j1, L2 = aL2 * h1;
  cxd dval = cD1 * L1 + cD2 * L2 - cD3 * L1;
  if (FORM == 0) {
    *F = -dval;
    if (DERIV) {
      const cxd kr = p.r * k;
      const cxd ipi_h0 = cmul_i(3.14159265358979323846 * h0);
      // l1' = -inner k J0/2pi ; l2' = inner k (lt J0 + i pi H0)/2pi
      cxd l1_1 = (-p.inn * inv2pi) * (k * j0);
      cxd l2_1 = (p.inn * inv2pi) * (k * (p.lt * j0 + ipi_h0));
      // l1'' = inner (kr J1 - J0)/2pi ; l2'' = inner (lt (J0 - kr J1) + i pi (H0 - kr H1))/2pi
      cxd l1_2 = (p.inn * inv2pi) * (kr * j1 - j0);
      cxd l2_2 = (p.inn * inv2pi) * (p.lt * (j0 - kr * j1) + cmul_i(3.14159265358979323846 * (h0 - kr * h1)));
      *F1 = -(p.Rk * l1_1 + p.wj * l2_1);
      *F2 = -(p.Rk * l1_2 + p.wj * l2_2);
    }
  } else {
    const double cS1 = p.Rk * p.sj, cS2 = p.wj * p.sj, cS3 = p.wj * p.sj * p.lt;
    const cxd M1 = (-inv2pi) * j0, M2 = cmul_i(0.5 * h0);
    cxd sval = cS1 * M1 + cS2 * M2 - cS3 * M1;
    *F = -(dval + ik * sval);
  }
}

template <int FORM>
static __device__ __forceinline__ cxd diag_fp64(const GeomDev& g, int i, cxd k) {
  const double wi = g.ws[i], ki = g.kappa[i];
  if (FORM == 0) return cxd(1.0 - wi * ki, 0.0);
  const double inv2pi = 0.15915494309189533577, euler_over_pi = 0.18373345259830797886;  // gamma/pi
  const double si = g.speed[i];
  const int o = g.coff[g.comp[i]];
  const double rii = g.kcol[o];
  const cxd ik = cmul_i(k);
  const double m1 = -inv2pi * si;
  // log((k^2/4) s^2) principal branch
  cxd q = (0.25 * si * si) * (k * k);
  cxd lg = clog_d(q);
  cxd m2 = (cxd(-euler_over_pi, 0.5) - inv2pi * lg) * si;
  cxd sval = cxd(rii * m1, 0.0) + wi * m2;
  return cxd(1.0, 0.0) - (cxd(wi * ki, 0.0) + ik * sval);
}

template <int FORM, int DERIV>
__global__ void __launch_bounds__(256) k_assemble_fp64(GeomDev g, const cxd* __restrict__ ks, int nk,
                                                       cxd* const* __restrict__ outs, long long ld) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= g.n || j >= g.n) return;
  const size_t off = (size_t)i + (size_t)j * (size_t)ld;
  if (i == j) {
    for (int q = 0; q < nk; ++q) {
      outs[q][off] = diag_fp64<FORM>(g, i, ks[q]);
      if (DERIV) {
        outs[nk + q][off] = cxd(0.0, 0.0);
        outs[2 * nk + q][off] = cxd(0.0, 0.0);
      }
    }
    return;
  }
  PairGeom p = pair_geom(g, i, j);
  if (FORM == 1 && !p.same && p.r * p.r <= 4.93038065763132e-32) {  // eps(T)^2 guard, cfie_kress.jl:494
    for (int q = 0; q < nk; ++q) outs[q][off] = cxd(0.0, 0.0);
    return;
  }
  for (int q = 0; q < nk; ++q) {
    const cxd k = ks[q];
    cxd F, F1, F2;
    entry_fp64<FORM, DERIV>(p, k, k.im == 0.0, &F, &F1, &F2);
    outs[q][off] = F;
    if (DERIV) {
      outs[nk + q][off] = F1;
      outs[2 * nk + q][off] = F2;
    }
  }
}

// ---------------------------------------------------------------------------
// Mixed form: kernel values in FP64, written as an FP32 pair (hi, lo) with
// hi = fl32(F) and lo = fl32(F - hi). The LU factors hi in FP32; the
// refinement residual uses hi + lo, so the refined solves see the FP64
// operator (to ~2^-48) although every bulk O(N^3) step runs in FP32.
// ---------------------------------------------------------------------------
template <int FORM>
__global__ void __launch_bounds__(256) k_assemble_split(GeomDev g, const cxd* __restrict__ ks, int nk,
                                                        cxf* const* __restrict__ his, cxf* const* __restrict__ los,
                                                        long long ld) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= g.n || j >= g.n) return;
  const size_t off = (size_t)i + (size_t)j * (size_t)ld;
  PairGeom p;
  const bool diag = (i == j);
  bool zero = false;
  if (!diag) {
    p = pair_geom(g, i, j);
    zero = (FORM == 1 && !p.same && p.r * p.r <= 4.93038065763132e-32);
  }
  for (int q = 0; q < nk; ++q) {
    cxd F(0.0, 0.0), F1, F2;
    if (diag) F = diag_fp64<FORM>(g, i, ks[q]);
    else if (!zero) entry_fp64<FORM, 0>(p, ks[q], ks[q].im == 0.0, &F, &F1, &F2);
    const cxf hi(F);
    his[q][off] = hi;
    if (los) los[q][off] = cxf((float)(F.re - (double)hi.re), (float)(F.im - (double)hi.im));
  }
}

// ---------------------------------------------------------------------------
// FP32 form: FP32 kernel values with FP64 pair geometry and FP64 phase
// reduction; entries whose argument |k r| < 12 (the near-diagonal band, where
// the Kress log split is most delicate) are evaluated entirely in FP64 and
// rounded once. Accuracy is bounded by FP32 rounding of the operator itself.
// ---------------------------------------------------------------------------
template <int FORM>
__global__ void __launch_bounds__(256) k_assemble_fp32(GeomDev g, const cxd* __restrict__ ks, int nk,
                                                        cxf* const* __restrict__ outs, long long ld) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= g.n || j >= g.n) return;
  const size_t off = (size_t)i + (size_t)j * (size_t)ld;
  if (i == j) {
    for (int q = 0; q < nk; ++q) outs[q][off] = cxf(diag_fp64<FORM>(g, i, ks[q]));
    return;
  }
  PairGeom p = pair_geom(g, i, j);
  if (FORM == 1 && !p.same && p.r * p.r <= 4.93038065763132e-32) {
    for (int q = 0; q < nk; ++q) outs[q][off] = cxf(0.f, 0.f);
    return;
  }
  const float inv2pi = 0.159154943091895f;
  const bool cross = (FORM == 1 && !p.same);
  const float cD1 = (float)(p.Rk * p.inn * p.invr), cD2 = (float)(p.wj * p.inn * p.invr),
              cD3 = (float)(p.wj * p.lt * p.inn * p.invr);
  const float cS1 = (float)(p.Rk * p.sj), cS2 = (float)(p.wj * p.sj), cS3 = (float)(p.wj * p.sj * p.lt);
  for (int q = 0; q < nk; ++q) {
    const cxd k = ks[q];
    const cxd z = p.r * k;
    if (z.re * z.re + z.im * z.im < 144.0) {
      cxd F, F1, F2;
      entry_fp64<FORM, 0>(p, k, k.im == 0.0, &F, &F1, &F2);
      outs[q][off] = cxf(F);
      continue;
    }
    Bessel01f b = bessel01_asym_f32(z);
    if (k.im == 0.0) { b.j0.im = 0.f; b.j1.im = 0.f; }
    const cxf kf((float)k.re, (float)k.im);
    const cxf ik = cmul_i(kf);
    const cxf aL1 = (-inv2pi) * kf, aL2 = 0.5f * ik;
    cxf F;
    if (cross) {
      cxf dval = (float)(p.wj * p.inn * p.invr) * (aL2 * b.h1());
      cxf sval = (float)(p.wj * p.sj) * cmul_i(0.5f * b.h0());
      F = -(dval + ik * sval);
    } else {
      const cxf L1 = aL1 * b.j1, L2 = aL2 * b.h1();
      cxf dval = cD1 * L1 + cD2 * L2 - cD3 * L1;
      if (FORM == 0) {
        F = -dval;
      } else {
        const cxf M1 = (-inv2pi) * b.j0, M2 = cmul_i(0.5f * b.h0());
        cxf sval = cS1 * M1 + cS2 * M2 - cS3 * M1;
        F = -(dval + ik * sval);
      }
    }
    outs[q][off] = F;
  }
}

// ---------------------------------------------------------------------------
// Symmetry-reduced DLP (dlp_kress.jl:1151-1189 and derivatives :1293-1345):
// D_red[a,b] = D_full[I_a, I_b] (Kress split) + sum over images q != I_b of
// scale_q (ik/2) c H1(kr) |t_q| w_q, c = n_q.(x_i - x_q)/r.
// ---------------------------------------------------------------------------
template <int DERIV>
__global__ void __launch_bounds__(256) k_assemble_dlp_reduced_fp64(GeomDev g, const cxd* __restrict__ ks,
                                                                   int nk, cxd* const* __restrict__ outs,
                                                                   long long ld) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  const int bcol = blockIdx.y * blockDim.y + threadIdx.y;
  if (a >= g.m || bcol >= g.m) return;
  const int i = g.fund[a], j = g.fund[bcol];
  const size_t off = (size_t)a + (size_t)bcol * (size_t)ld;
  const double xi = g.x[i], yi = g.y[i];
  PairGeom p;
  if (i != j) p = pair_geom(g, i, j);
  for (int q = 0; q < nk; ++q) {
    const cxd k = ks[q];
    const bool realk = (k.im == 0.0);
    cxd F, F1(0.0, 0.0), F2(0.0, 0.0);
    if (i == j) {
      F = cxd(1.0 - g.ws[i] * g.kappa[i], 0.0);
    } else {
      entry_fp64<0, DERIV>(p, k, realk, &F, &F1, &F2);
    }
    // image contributions (regular kernel), subtracted because F = I - D
    for (int l = 0; l < g.norb; ++l) {
      const int qn = g.orb[bcol * g.norb + l];
      if (qn == j) continue;
      const double dxq = xi - g.x[qn], dyq = yi - g.y[qn];
      const double r = hypot(dxq, dyq);
      if (r < 2.220446049250313e-16) continue;
      const double c = (g.nx[qn] * dxq + g.ny[qn] * dyq) / r;
      const cxd sc(g.orb_scale[2 * (bcol * g.norb + l)], g.orb_scale[2 * (bcol * g.norb + l) + 1]);
      const double wq = g.speed[qn] * g.ws[qn];
      Bessel01d bb = bessel01(r * k);
      if (realk) { bb.j0.im = 0.0; bb.j1.im = 0.0; }
      const cxd h0 = bb.h0(), h1 = bb.h1();
      F -= (c * wq) * (sc * (cmul_i(0.5 * k) * h1));
      if (DERIV) {
        const cxd kr = r * k;
        F1 -= (c * wq) * (sc * cmul_i(0.5 * (kr * h0)));
        F2 -= (c * wq) * (sc * cmul_i(0.5 * (r * h0 - (r * r) * (k * h1))));
      }
    }
    outs[q][off] = F;
    if (DERIV) {
      outs[nk + q][off] = F1;
      outs[2 * nk + q][off] = F2;
    }
  }
}

// ---------------------------------------------------------------------------
// Kress first column per component: c_m = -(4 pi/N) sum_{p=1}^{n-1} cos(2 pi p m/N)/p
//   - (4 pi/N^2) (-1)^m   (N = 2n even),   without the last term for odd N
// (the closed form of the ifft in boundarypoints.jl:310-345). The phase
// p*m mod N is reduced exactly in integers before sinpi/cospi.
// ---------------------------------------------------------------------------
__global__ void k_kress_column(double* out, int N) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= N) return;
  const bool even = (N % 2) == 0;
  const int nmax = even ? N / 2 - 1 : (N - 1) / 2;
  double s = 0.0;
  long long pm = 0;
  for (int p = 1; p <= nmax; ++p) {
    pm += m;
    if (pm >= N) pm -= N;  // (p*m) mod N, m < N so one subtraction suffices
    s += cospi(2.0 * (double)pm / (double)N) / (double)p;
  }
  double c = -(4.0 * 3.14159265358979323846 / (double)N) * s;
  if (even) c -= (4.0 * 3.14159265358979323846 / ((double)N * (double)N)) * ((m & 1) ? -1.0 : 1.0);
  out[m] = c;
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
int launch_kress_column(double* out, int N, cudaStream_t st) {
  k_kress_column<<<(N + 255) / 256, 256, 0, st>>>(out, N);
  QBG_LAUNCH_CHECK("k_kress_column");
  return QBG_OK;
}

int launch_assemble(const GeomDev& g, const cxd* ks, int nk, int deriv, int prec, void* const* outs_dev,
                    long long ld, cudaStream_t st, void* const* lo_outs_dev) {
  const bool reduced = (g.m != g.n);
  const int dim = reduced ? g.m : g.n;
  dim3 blk(32, 8);
  dim3 grd((dim + 31) / 32, (dim + 7) / 8);
  if (reduced) {
    if (g.form != 0 || prec != 0) {
      set_error("symmetry-reduced assembly is implemented for DLP in FP64");
      return QBG_ENOTSUP;
    }
    if (deriv)
      k_assemble_dlp_reduced_fp64<1><<<grd, blk, 0, st>>>(g, ks, nk, (cxd* const*)outs_dev, ld);
    else
      k_assemble_dlp_reduced_fp64<0><<<grd, blk, 0, st>>>(g, ks, nk, (cxd* const*)outs_dev, ld);
    QBG_LAUNCH_CHECK("k_assemble_dlp_reduced_fp64");
    return QBG_OK;
  }
  if (prec == QBG_PREC_FP64) {
    if (g.form == 0) {
      if (deriv)
        k_assemble_fp64<0, 1><<<grd, blk, 0, st>>>(g, ks, nk, (cxd* const*)outs_dev, ld);
      else
        k_assemble_fp64<0, 0><<<grd, blk, 0, st>>>(g, ks, nk, (cxd* const*)outs_dev, ld);
    } else {
      if (deriv) {
        set_error("CFIE derivative assembly is not available");
        return QBG_ENOTSUP;
      }
      k_assemble_fp64<1, 0><<<grd, blk, 0, st>>>(g, ks, nk, (cxd* const*)outs_dev, ld);
    }
    QBG_LAUNCH_CHECK("k_assemble_fp64");
    return QBG_OK;
  }
  if (deriv) {
    set_error("the complex64 forms have no derivative assembly");
    return QBG_ENOTSUP;
  }
  if (prec == QBG_PREC_MIXED) {
    if (g.form == 0)
      k_assemble_split<0><<<grd, blk, 0, st>>>(g, ks, nk, (cxf* const*)outs_dev, (cxf* const*)lo_outs_dev, ld);
    else
      k_assemble_split<1><<<grd, blk, 0, st>>>(g, ks, nk, (cxf* const*)outs_dev, (cxf* const*)lo_outs_dev, ld);
    QBG_LAUNCH_CHECK("k_assemble_split");
    return QBG_OK;
  }
  if (g.form == 0)
    k_assemble_fp32<0><<<grd, blk, 0, st>>>(g, ks, nk, (cxf* const*)outs_dev, ld);
  else
    k_assemble_fp32<1><<<grd, blk, 0, st>>>(g, ks, nk, (cxf* const*)outs_dev, ld);
  QBG_LAUNCH_CHECK("k_assemble_fp32");
  return QBG_OK;
}

// Bessel self-test entry (used by the GPU tests through the C-ABI).
__global__ void k_bessel_eval(const cxd* z, int n, cxd* out) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  Bessel01d b = bessel01(z[t]);
  out[4 * t + 0] = b.j0;
  out[4 * t + 1] = b.j1;
  out[4 * t + 2] = b.y0;
  out[4 * t + 3] = b.y1;
}
__global__ void k_bessel_eval_f32(const cxd* z, int n, cxd* out) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  Bessel01f b = bessel01_asym_f32(z[t]);
  out[4 * t + 0] = cxd(b.j0);
  out[4 * t + 1] = cxd(b.j1);
  out[4 * t + 2] = cxd(b.y0);
  out[4 * t + 3] = cxd(b.y1);
}
int launch_bessel_eval(const cxd* z, int n, cxd* out, int f32, cudaStream_t st) {
  if (f32)
    k_bessel_eval_f32<<<(n + 127) / 128, 128, 0, st>>>(z, n, out);
  else
    k_bessel_eval<<<(n + 127) / 128, 128, 0, st>>>(z, n, out);
  QBG_LAUNCH_CHECK("k_bessel_eval");
  return QBG_OK;
}

}  // namespace qbg
