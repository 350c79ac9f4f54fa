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
#include <algorithm>
#include <cstring>

#include <vector>
#include "qbg_assemble.cuh"
#include "qbg_handles.cuh"
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

// pair_geom of (i, j) and of (j, i) together: the distance, its reciprocal
// and the Kress log term are symmetric and computed once (FP64 is 1/64 of the
// FP32 rate on this part)
static __device__ __forceinline__ void pair_geom_sym(const GeomDev& g, int i, int j, PairGeom& a, PairGeom& b) {
  const double dxij = g.x[i] - g.x[j], dyij = g.y[i] - g.y[j];
  a.r = b.r = hypot(dxij, dyij);
  a.invr = b.invr = 1.0 / a.r;
  a.inn = g.dy[j] * dxij - g.dx[j] * dyij;
  b.inn = g.dx[i] * dyij - g.dy[i] * dxij;
  a.wj = g.ws[j];
  a.sj = g.speed[j];
  b.wj = g.ws[i];
  b.sj = g.speed[i];
  const int ci = g.comp[i], cj = g.comp[j];
  a.same = b.same = (ci == cj);
  if (a.same) {
    const int o = g.coff[ci], na = g.coff[ci + 1] - o;
    int d = g.lidx[i] - g.lidx[j];
    d += (d < 0) ? na : 0;
    a.Rk = g.kcol[o + d];
    int e = g.lidx[j] - g.lidx[i];
    e += (e < 0) ? na : 0;
    b.Rk = g.kcol[o + e];
    a.lt = b.lt = pair_logterm(g.ts[i], g.ts[j]);
  } else {
    a.Rk = b.Rk = 0.0;
    a.lt = b.lt = 0.0;
  }
}

// ---------------------------------------------------------------------------
// FP64 entry for one wavenumber
// ---------------------------------------------------------------------------
template <int FORM, int DERIV>
static __device__ __forceinline__ void entry_vals(const PairGeom& p, cxd k, cxd h0, cxd h1, cxd j0, cxd j1, cxd* F,
                                                  cxd* F1, cxd* F2) {
  const double inv2pi = 0.15915494309189533577;
  const cxd ik = cmul_i(k);
  const cxd aL1 = (-inv2pi) * k;
  const cxd aL2 = 0.5 * ik;
  if (FORM == 1 && !p.same) {
    // smooth cross-component kernel
    cxd dval = (p.wj * p.inn * p.invr) * (aL2 * h1);
    cxd sval = (p.wj * p.sj) * cmul_i(0.5 * h0);
    *F = -(dval + ik * sval);
    if (DERIV) {
      // cfie_kress.jl:729-734 (and the Chebyshev route,
      // chebyshev_euclidian_helmholtz_cfie_kress.jl:1041-1045): the k-derivatives
      // of the double-layer part carry the sign written there
      const cxd kr = p.r * k;
      const double cD = p.wj * p.inn, cS = p.wj * p.sj;
      cxd dval1 = cmul_i(-0.5 * cD * (k * h0));
      cxd dval2 = cmul_i(-0.5 * cD * (h0 - kr * h1));
      cxd sval1 = cmul_i(-0.5 * cS * p.r * h1);
      cxd sval2 = cmul_i(0.5 * cS * p.r * (h1 - kr * h0)) / k;
      *F1 = -(dval1 + cmul_i(sval) + ik * sval1);
      *F2 = -(dval2 + cmul_i(2.0 * sval1) + ik * sval2);
    }
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
    if (DERIV) {
      // cfie_kress.jl:658-681
      const double pi = 3.14159265358979323846;
      const cxd kr = p.r * k;
      cxd l1_1 = (-p.inn * inv2pi) * (k * j0);
      cxd l2_1 = (p.inn * inv2pi) * (k * (p.lt * j0 + cmul_i(pi * h0)));
      cxd l1_2 = (p.inn * inv2pi) * (kr * j1 - j0);
      cxd l2_2 = (p.inn * inv2pi) * (p.lt * (j0 - kr * j1) + cmul_i(pi * (h0 - kr * h1)));
      const cxd dval1 = p.Rk * l1_1 + p.wj * l2_1;
      const cxd dval2 = p.Rk * l1_2 + p.wj * l2_2;
      const double rs = p.r * p.sj * inv2pi;
      cxd m1_1 = rs * j1;
      cxd m1_2 = (rs * (kr * j0 - j1)) / k;
      cxd m2_1 = (-rs) * (p.lt * j1 + cmul_i(pi * h1));
      cxd m2_2 = (rs * (p.lt * (j1 - kr * j0) + cmul_i(pi * (h1 - kr * h0)))) / k;
      const cxd sval1 = p.Rk * m1_1 + p.wj * m2_1;
      const cxd sval2 = p.Rk * m1_2 + p.wj * m2_2;
      *F1 = -(dval1 + cmul_i(sval) + ik * sval1);
      *F2 = -(dval2 + cmul_i(2.0 * sval1) + ik * sval2);
    }
  }
}

// direct evaluation: H0, H1, J0, J1 from the device Bessel routines
template <int FORM, int DERIV>
static __device__ __forceinline__ void entry_fp64(const PairGeom& p, cxd k, bool realk, cxd* F, cxd* F1,
                                                  cxd* F2) {
  Bessel01d b = bessel01(p.r * k);
  if (realk) {  // reference: J = Re H for real k (dlp_kress.jl:821-822)
    b.j0.im = 0.0;
    b.j1.im = 0.0;
  }
  entry_vals<FORM, DERIV>(p, k, b.h0(), b.h1(), b.j0, b.j1, F, F1, F2);
}

// diagonal and its k-derivatives (DLP: zero; CFIE: cfie_kress.jl:636-646)
template <int FORM>
static __device__ __forceinline__ void diag_derivs(const GeomDev& g, int i, cxd k, cxd* F1, cxd* F2) {
  if (FORM == 0) {
    *F1 = cxd(0.0, 0.0);
    *F2 = cxd(0.0, 0.0);
    return;
  }
  const double inv2pi = 0.15915494309189533577, euler_over_pi = 0.18373345259830797886;
  const double pi = 3.14159265358979323846;
  const double wi = g.ws[i], si = g.speed[i];
  const double rii = g.kcol[g.coff[g.comp[i]]];
  const cxd ik = cmul_i(k);
  cxd lg = clog_d((0.25 * si * si) * (k * k));
  cxd m2 = (cxd(-euler_over_pi, 0.5) - inv2pi * lg) * si;
  const cxd sval = cxd(rii * (-inv2pi * si), 0.0) + wi * m2;
  const cxd sval1 = cxd(-wi * si / pi, 0.0) / k;
  const cxd sval2 = cxd(wi * si / pi, 0.0) / (k * k);
  *F1 = -(cmul_i(sval) + ik * sval1);
  *F2 = -(cmul_i(2.0 * sval1) + ik * sval2);
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
      if (DERIV) diag_derivs<FORM>(g, i, ks[q], &outs[nk + q][off], &outs[2 * nk + q][off]);
    }
    return;
  }
  PairGeom p = pair_geom(g, i, j);
  if (FORM == 1 && !p.same && p.r * p.r <= 4.93038065763132e-32) {  // eps(T)^2 guard, cfie_kress.jl:494
    for (int q = 0; q < nk; ++q) {
      outs[q][off] = cxd(0.0, 0.0);
      if (DERIV) { outs[nk + q][off] = cxd(0.0, 0.0); outs[2 * nk + q][off] = cxd(0.0, 0.0); }
    }
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
// value store for the entry at `off`: OUT 0 = complex128, 1 = complex64 hi
// (+ lo = fl32(v - hi) when los != nullptr)
template <int OUT>
static __device__ __forceinline__ void store_entry(void* const* outs, void* const* los, int slot, size_t off,
                                                   cxd v) {
  if (OUT == 0) {
    reinterpret_cast<cxd*>(outs[slot])[off] = v;
  } else {
    const cxf hi(v);
    reinterpret_cast<cxf*>(outs[slot])[off] = hi;
    if (los) reinterpret_cast<cxf*>(los[slot])[off] = cxf((float)(v.re - (double)hi.re), (float)(v.im - (double)hi.im));
  }
}

// regular image kernel of orbit member qn seen from node (xi, yi), subtracted
// from F = I - D (dlp_kress.jl:1081-1100): D += sc (ik/2) c H1(kr) speed_q w_q,
// dD/dk = sc (i/2) c kr H0 speed_q w_q, d2D/dk2 = sc (i/2) c (r H0 - k r^2 H1) speed_q w_q
template <int DERIV>
static __device__ __forceinline__ void image_terms(double c, double wq, cxd sc, double r, cxd k, cxd h0, cxd h1,
                                                   cxd& F, cxd& F1, cxd& F2) {
  F -= (c * wq) * (sc * (cmul_i(0.5 * k) * h1));
  if (DERIV) {
    const cxd kr = r * k;
    F1 -= (c * wq) * (sc * cmul_i(0.5 * (kr * h0)));
    F2 -= (c * wq) * (sc * cmul_i(0.5 * (r * h0 - (r * r) * (k * h1))));
  }
}

template <int DERIV, int OUT>
__global__ void __launch_bounds__(256) k_assemble_dlp_reduced(GeomDev g, const cxd* __restrict__ ks, int nk,
                                                              void* const* __restrict__ outs,
                                                              void* const* __restrict__ los, long long ld) {
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
    for (int l = 0; l < g.norb; ++l) {
      const int qn = g.orb[bcol * g.norb + l];
      if (qn == j) continue;
      const double dxq = xi - g.x[qn], dyq = yi - g.y[qn];
      const double r = hypot(dxq, dyq);
      if (r < 2.220446049250313e-16) continue;
      const double c = (g.nx[qn] * dxq + g.ny[qn] * dyq) / r;
      const cxd sc(g.orb_scale[2 * (bcol * g.norb + l)], g.orb_scale[2 * (bcol * g.norb + l) + 1]);
      const Bessel01d bb = bessel01(r * k);
      image_terms<DERIV>(c, g.speed[qn] * g.ws[qn], sc, r, k, bb.h0(), bb.h1(), F, F1, F2);
    }
    store_entry<OUT>(outs, los, q, off, F);
    if (DERIV) {
      store_entry<OUT>(outs, los, nk + q, off, F1);
      store_entry<OUT>(outs, los, 2 * nk + q, off, F2);
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
// Chebyshev-panel evaluation (the reference's complex-k route,
// chebyshev_bessels.jl:316-528, 950-1241, chebyshev_core.jl:67-345):
// for every wavenumber, H0/H1 are tabulated on np_h uniform panels of
// [rmin, rmax] and J0/J1 on np_j uniform panels of [0, rmax]; on each panel a
// degree-M Chebyshev-Lobatto interpolant (DCT-I of the values at
// t_j = cos(pi j / M), c_0 halved) is evaluated by Clenshaw's recurrence at
// t = (2 r - (a + b)) / (b - a). The tables are built on the device from the
// direct evaluator. Hankel values at |k r| below `small_cut` (0.2 on the CFIE
// route, chebyshev_bessels.jl:1190-1207) and at r < rmin use the direct
// evaluator; J always uses its panels, which start at r = 0.
// ---------------------------------------------------------------------------
__global__ void k_pair_rminmax(GeomDev g, unsigned long long* out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  double lo = 1e300, hi = 0.0;
  if (i < g.n && j < g.n && i != j) {
    const double r = hypot(g.x[i] - g.x[j], g.y[i] - g.y[j]);
    if (r > 2.220446049250313e-16) { lo = r; hi = r; }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    lo = fmin(lo, __shfl_down_sync(0xffffffffu, lo, o));
    hi = fmax(hi, __shfl_down_sync(0xffffffffu, hi, o));
  }
  if (((threadIdx.y * blockDim.x + threadIdx.x) & 31) == 0) {
    atomicMin(&out[0], (unsigned long long)__double_as_longlong(lo));  // positive doubles order as integers
    atomicMax(&out[1], (unsigned long long)__double_as_longlong(hi));
  }
}

__global__ void k_cheb_build(ChebTables t, const cxd* __restrict__ ks) {
  constexpr int MMAX = QBG_CHEB_MAX_DEGREE;
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  const int q = blockIdx.y;
  const int tab = blockIdx.z;  // 0: (H0, H1) on [rmin, rmax]; 1: (J0, J1) on [0, rmax]
  const int np = tab ? t.nj : t.nh;
  const int M = tab ? t.Mj : t.Mh;
  if (p >= np) return;
  const double lo = tab ? 0.0 : t.rmin;
  const double h = tab ? t.dr_j : t.dr_h;
  const double a = fma((double)p, h, lo);
  const double b = (p + 1 == np) ? t.rmax : fma((double)(p + 1), h, lo);
  const cxd k = ks[q];
  const bool realk = (k.im == 0.0);
  cxd f0[MMAX + 1], f1[MMAX + 1];
  for (int jn = 0; jn <= M; ++jn) {
    const double tn = cospi((double)jn / (double)M);
    const double r = 0.5 * ((b + a) + (b - a) * tn);
    if (r == 0.0) {  // J0(0) = 1, J1(0) = 0 (only the J table reaches r = 0)
      f0[jn] = cxd(1.0, 0.0);
      f1[jn] = cxd(0.0, 0.0);
      continue;
    }
    Bessel01d bz = bessel01(r * k);
    if (tab == 0) {
      f0[jn] = bz.h0();
      f1[jn] = bz.h1();
    } else {
      if (realk) { bz.j0.im = 0.0; bz.j1.im = 0.0; }
      f0[jn] = bz.j0;
      f1[jn] = bz.j1;
    }
  }
  cxd* out = (tab ? t.J : t.H) + (((size_t)q * np + p) * (M + 1)) * 2;
  for (int m = 0; m <= M; ++m) {
    const double sg = (m & 1) ? -1.0 : 1.0;
    cxd s0 = 0.5 * f0[0] + (0.5 * sg) * f0[M];
    cxd s1 = 0.5 * f1[0] + (0.5 * sg) * f1[M];
    for (int jn = 1; jn < M; ++jn) {
      const double c = cospi((double)(jn * m) / (double)M);
      s0 += c * f0[jn];
      s1 += c * f1[jn];
    }
    double sc = 2.0 / (double)M;
    if (m == 0) sc *= 0.5;
    out[2 * m] = sc * s0;
    out[2 * m + 1] = sc * s1;
  }
}

// Clenshaw for two interleaved series: c[2m], c[2m+1], m = 0..M
static __device__ __forceinline__ void clenshaw2(const cxd* __restrict__ c, int M, double t, cxd& v0, cxd& v1) {
  const double u = 2.0 * t;
  cxd b1a(0.0, 0.0), b2a(0.0, 0.0), b1b(0.0, 0.0), b2b(0.0, 0.0);
  for (int m = M; m >= 1; --m) {
    const cxd ca = c[2 * m], cb = c[2 * m + 1];
    cxd b0a(fma(u, b1a.re, -b2a.re) + ca.re, fma(u, b1a.im, -b2a.im) + ca.im);
    cxd b0b(fma(u, b1b.re, -b2b.re) + cb.re, fma(u, b1b.im, -b2b.im) + cb.im);
    b2a = b1a; b1a = b0a;
    b2b = b1b; b1b = b0b;
  }
  v0 = cxd(fma(t, b1a.re, -b2a.re) + c[0].re, fma(t, b1a.im, -b2a.im) + c[0].im);
  v1 = cxd(fma(t, b1b.re, -b2b.re) + c[1].re, fma(t, b1b.im, -b2b.im) + c[1].im);
}

static __device__ __forceinline__ void panel_of(double r, double lo, double hi, double h, double invh, int np,
                                                int& p, double& t) {
  int q = (int)floor((r - lo) * invh);
  q = q < 0 ? 0 : (q >= np ? np - 1 : q);
  const double a = fma((double)q, h, lo);
  const double b = (q + 1 == np) ? hi : fma((double)(q + 1), h, lo);
  p = q;
  t = (2.0 * r - (b + a)) / (b - a);
}

// OUT: 0 = complex128, 1 = complex64 hi (+ lo when los != nullptr)
template <int FORM, int DERIV, int OUT>
__global__ void __launch_bounds__(256) k_assemble_cheb(GeomDev g, ChebTables t, const cxd* __restrict__ ks,
                                                       int nk, int kchunk, void* const* __restrict__ outs,
                                                       void* const* __restrict__ los, long long ld) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= g.n || j >= g.n) return;
  const int q0 = blockIdx.z * kchunk, q1 = min(nk, q0 + kchunk);
  const size_t off = (size_t)i + (size_t)j * (size_t)ld;
  auto store = [&](int slot, cxd v) {
    if (OUT == 0) {
      reinterpret_cast<cxd*>(outs[slot])[off] = v;
    } else {
      const cxf hi(v);
      reinterpret_cast<cxf*>(outs[slot])[off] = hi;
      if (los) reinterpret_cast<cxf*>(los[slot])[off] = cxf((float)(v.re - (double)hi.re), (float)(v.im - (double)hi.im));
    }
  };
  if (i == j) {
    for (int q = q0; q < q1; ++q) {
      store(q, diag_fp64<FORM>(g, i, ks[q]));
      if (DERIV) {
        cxd d1, d2;
        diag_derivs<FORM>(g, i, ks[q], &d1, &d2);
        store(nk + q, d1);
        store(2 * nk + q, d2);
      }
    }
    return;
  }
  const PairGeom p = pair_geom(g, i, j);
  if (FORM == 1 && !p.same && p.r * p.r <= 4.93038065763132e-32) {
    for (int q = q0; q < q1; ++q) {
      store(q, cxd(0.0, 0.0));
      if (DERIV) { store(nk + q, cxd(0.0, 0.0)); store(2 * nk + q, cxd(0.0, 0.0)); }
    }
    return;
  }
  int ph, pj;
  double th, tj;
  panel_of(p.r, t.rmin, t.rmax, t.dr_h, t.invdr_h, t.nh, ph, th);
  panel_of(p.r, 0.0, t.rmax, t.dr_j, t.invdr_j, t.nj, pj, tj);
  const bool below = p.r < t.rmin;
  const bool needj = !(FORM == 1 && !p.same);
  for (int q = q0; q < q1; ++q) {
    const cxd k = ks[q];
    const double az = p.r * hypot(k.re, k.im);
    cxd h0, h1, j0(0.0, 0.0), j1(0.0, 0.0);
    if (below || az < t.small_cut) {
      const Bessel01d b = bessel01(p.r * k);
      h0 = b.h0();
      h1 = b.h1();
    } else {
      clenshaw2(t.H + (((size_t)q * t.nh + ph) * (t.Mh + 1)) * 2, t.Mh, th, h0, h1);
    }
    if (needj) clenshaw2(t.J + (((size_t)q * t.nj + pj) * (t.Mj + 1)) * 2, t.Mj, tj, j0, j1);
    cxd F, F1, F2;
    entry_vals<FORM, DERIV>(p, k, h0, h1, j0, j1, &F, &F1, &F2);
    store(q, F);
    if (DERIV) { store(nk + q, F1); store(2 * nk + q, F2); }
  }
}

// ---------------------------------------------------------------------------
// Symmetry-reduced DLP through the Chebyshev panels (the reduced multi-k route,
// chebyshev_euclidian_helmholtz_dlp_kress.jl:771-847, derivatives :953-1054):
// entry (a, b) = Kress-split entry of the full operator at (fund[a], fund[b])
// minus the regular image kernels of the other members of orbit b. Image
// distances are node-pair distances of the full boundary, so they lie inside
// the panel range [rmin, rmax] built over all pairs.
// ---------------------------------------------------------------------------
static __device__ __forceinline__ void cheb_h01(const ChebTables& t, int q, double r, cxd k, cxd& h0, cxd& h1) {
  const double az = r * hypot(k.re, k.im);
  if (r < t.rmin || az < t.small_cut) {
    const Bessel01d b = bessel01(r * k);
    h0 = b.h0();
    h1 = b.h1();
    return;
  }
  int ph;
  double th;
  panel_of(r, t.rmin, t.rmax, t.dr_h, t.invdr_h, t.nh, ph, th);
  clenshaw2(t.H + (((size_t)q * t.nh + ph) * (t.Mh + 1)) * 2, t.Mh, th, h0, h1);
}

// ---------------------------------------------------------------------------
// CFIE with Alpert quadrature (cfie_alpert.jl:947-1087 self blocks,
// 1261-1350 off-component blocks; through the panels,
// chebyshev_euclidian_helmholtz_cfie_alpert.jl:533-1253). Kernel terms with
// weight w (cfie_alpert.jl:233-287):
//   d0 = w (ik/2) inner H1 / r, d1 = w (i/2) inner k H0, d2 = w (i/2) inner (H0 - k r H1),
//   s0 = w (i/2) H0 s, s1 = -w (i/2) r H1 s, s2 = w (i/2) r (H1 - k r H0) s / k;
// an entry loses d0 + ik s0, its k-derivatives d1 + i s0 + ik s1 and
// d2 + 2i s1 + ik s2. The self block keeps the identity, drops the trapezoid
// band |i - j| < a and gets the correction nodes' terms spread over the
// interpolation stencil.
// ---------------------------------------------------------------------------
struct AlpTerms {
  cxd v0, v1, v2;
};

// H0, H1 at k r: the device Bessel routines, or (CHEB) the Chebyshev panels of
// wavenumber slot q (direct below r_min or the small-|z| cut-off; the Alpert
// route interpolates H only, chebyshev_euclidian_helmholtz_cfie_alpert.jl:404-470)
template <int CHEB>
static __device__ __forceinline__ void alpert_h01(const ChebTables& t, int q, cxd k, double r, cxd& h0, cxd& h1) {
  if (CHEB) {
    cheb_h01(t, q, r, k, h0, h1);
  } else {
    const Bessel01d b = bessel01(r * k);
    h0 = b.h0();
    h1 = b.h1();
  }
}

template <int DERIV, int CHEB>
static __device__ __forceinline__ AlpTerms alpert_terms(const ChebTables& tb, int q, cxd k, double r, double inn,
                                                        double s, double w) {
  cxd h0, h1;
  alpert_h01<CHEB>(tb, q, k, r, h0, h1);
  const cxd ik = cmul_i(k);
  const cxd d0 = (w * inn / r) * cmul_i(0.5 * (k * h1));
  const cxd s0 = (w * s) * cmul_i(0.5 * h0);
  AlpTerms t;
  t.v0 = d0 + ik * s0;
  if (DERIV) {
    const cxd kr = r * k;
    const cxd d1 = (w * inn) * cmul_i(0.5 * (k * h0));
    const cxd d2 = (w * inn) * cmul_i(0.5 * (h0 - kr * h1));
    const cxd s1 = (w * s * r) * cmul_i(-0.5 * h1);
    const cxd s2 = cmul_i(0.5 * (w * s * r) * (h1 - kr * h0)) / k;
    t.v1 = d1 + cmul_i(s0) + ik * s1;
    t.v2 = d2 + cmul_i(2.0 * s1) + ik * s2;
  } else {
    t.v1 = t.v2 = cxd(0.0, 0.0);
  }
  return t;
}

template <int DERIV, int CHEB>
__global__ void __launch_bounds__(256) k_assemble_alpert(GeomDev g, ChebTables tb, const cxd* __restrict__ ks,
                                                         int nk, cxd* const* __restrict__ outs, long long ld) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= g.n || j >= g.n) return;
  const size_t off = (size_t)i + (size_t)j * (size_t)ld;
  bool zero = false;
  double r = 0.0, inn = 0.0;
  if (i != j) {
    const int ci = g.comp[i], cj = g.comp[j];
    const double dx = g.x[i] - g.x[j], dy = g.y[i] - g.y[j];
    const double r2 = dx * dx + dy * dy;
    if (ci == cj) {
      const int na = g.coff[ci + 1] - g.coff[ci];
      int d = abs(g.lidx[i] - g.lidx[j]);
      d = min(d, na - d);
      zero = d < g.aa;  // trapezoid band replaced by the correction nodes
    } else {
      zero = r2 <= 4.93038065763132e-32;
    }
    r = sqrt(r2);
    inn = g.dy[j] * dx - g.dx[j] * dy;
  }
  for (int q = 0; q < nk; ++q) {
    cxd F(0.0, 0.0), F1(0.0, 0.0), F2(0.0, 0.0);
    if (i == j) {
      F = cxd(1.0, 0.0);
    } else if (!zero) {
      const AlpTerms t = alpert_terms<DERIV, CHEB>(tb, q, ks[q], r, inn, g.speed[j], g.ws[j]);
      F = -t.v0;
      F1 = -t.v1;
      F2 = -t.v2;
    }
    outs[q][off] = F;
    if (DERIV) {
      outs[nk + q][off] = F1;
      outs[2 * nk + q][off] = F2;
    }
  }
}

// one thread per (row, wavenumber): the row's correction nodes, scattered into
// its own row only, so no two threads touch one entry
template <int DERIV, int CHEB>
__global__ void __launch_bounds__(128) k_alpert_corrections(GeomDev g, ChebTables tb, const cxd* __restrict__ ks,
                                                            int nk, cxd* const* __restrict__ outs, long long ld) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int q = blockIdx.y;
  if (i >= g.n || q >= nk) return;
  const int c = g.comp[i], o = g.coff[c], na = g.coff[c + 1] - o, li = g.lidx[i];
  const double h = g.ws[o];
  const cxd k = ks[q];
  const size_t n = (size_t)g.n, plane = (size_t)g.aj * n;
  for (int p = 0; p < g.aj; ++p) {
    const double fac = h * g.aw[p];
    for (int side = 0; side < 2; ++side) {
      const double r = g.anodes[(size_t)side * plane + (size_t)p * n + i];
      if (!isfinite(r)) continue;
      const double inn = g.anodes[(size_t)(2 + side) * plane + (size_t)p * n + i];
      const double sp = g.anodes[(size_t)(4 + side) * plane + (size_t)p * n + i];
      const AlpTerms t = alpert_terms<DERIV, CHEB>(tb, q, k, r, inn, sp, fac);
      const int* so = g.aoff + ((size_t)side * g.aj + p) * g.ani;
      const double* sw = g.awt + ((size_t)side * g.aj + p) * g.ani;
      for (int m = 0; m < g.ani; ++m) {
        int col = (li + so[m]) % na;
        col += col < 0 ? na : 0;
        const size_t e = (size_t)i + (size_t)(o + col) * (size_t)ld;
        outs[q][e] -= sw[m] * t.v0;
        if (DERIV) {
          outs[nk + q][e] -= sw[m] * t.v1;
          outs[2 * nk + q][e] -= sw[m] * t.v2;
        }
      }
    }
  }
}

// complex128 staging -> complex64 hi (+ lo) through the output pointer table
__global__ void k_split_slots(const cxd* __restrict__ src, long long count, int q0, int cnt, void* const* his,
                              void* const* los) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int q = blockIdx.y;
  if (e >= count || q >= cnt) return;
  const cxd v = src[(size_t)q * count + e];
  const cxf hi(v);
  reinterpret_cast<cxf*>(his[q0 + q])[e] = hi;
  if (los) reinterpret_cast<cxf*>(los[q0 + q])[e] = cxf((float)(v.re - (double)hi.re), (float)(v.im - (double)hi.im));
}

// cheb == nullptr: direct Hankel values; otherwise the panels of `cheb`
static int launch_alpert(const GeomDev& g, const ChebTables* cheb, const cxd* ks, int nk, int deriv, int prec,
                         void* const* outs_dev, long long ld, cudaStream_t st, void* const* lo_outs_dev) {
  dim3 blk(32, 8), grd((g.n + 31) / 32, (g.n + 7) / 8);
  const ChebTables tb = cheb ? *cheb : ChebTables();
  if (prec == QBG_PREC_FP64) {
    dim3 cg((g.n + 127) / 128, nk);
    cxd* const* o = (cxd* const*)outs_dev;
#define QBG_ALP(D, C)                                                        \
  k_assemble_alpert<D, C><<<grd, blk, 0, st>>>(g, tb, ks, nk, o, ld);        \
  QBG_LAUNCH_CHECK("k_assemble_alpert");                                     \
  k_alpert_corrections<D, C><<<cg, 128, 0, st>>>(g, tb, ks, nk, o, ld);      \
  QBG_LAUNCH_CHECK("k_alpert_corrections")
    if (cheb) {
      if (deriv) { QBG_ALP(1, 1); } else { QBG_ALP(0, 1); }
    } else {
      if (deriv) { QBG_ALP(1, 0); } else { QBG_ALP(0, 0); }
    }
#undef QBG_ALP
    return QBG_OK;
  }
  if (deriv) {
    set_error("derivative assembly is available in FP64");
    return QBG_ENOTSUP;
  }
  // complex64 forms: the corrections accumulate into FP64 entries, so groups
  // of wavenumbers are assembled in FP64 staging and then split
  const int grp = nk < 4 ? nk : 4;
  const long long count = (long long)g.n * ld;
  cxd* stage = nullptr;
  cxd** dp = nullptr;
  QBG_TRY(dmalloc(&stage, sizeof(cxd) * (size_t)count * grp));
  if (int sa = dmalloc(&dp, sizeof(cxd*) * grp)) { dfree(stage, st); return sa; }
  std::vector<cxd*> hp(grp);
  for (int q = 0; q < grp; ++q) hp[q] = stage + (size_t)q * count;
  cudaError_t e = cudaMemcpyAsync(dp, hp.data(), sizeof(cxd*) * grp, cudaMemcpyHostToDevice, st);
  int s = e == cudaSuccess ? QBG_OK : cuda_status(e, "Alpert staging pointers");
  for (int q0 = 0; !s && q0 < nk; q0 += grp) {
    const int c = nk - q0 < grp ? nk - q0 : grp;
    ChebTables sub;
    if (cheb) {  // the tables of wavenumbers q0 .. q0 + c
      sub = *cheb;
      sub.H = cheb->H + (size_t)q0 * cheb->nh * (cheb->Mh + 1) * 2;
      sub.J = cheb->J + (size_t)q0 * cheb->nj * (cheb->Mj + 1) * 2;
    }
    s = launch_alpert(g, cheb ? &sub : nullptr, ks + q0, c, 0, QBG_PREC_FP64, (void* const*)dp, ld, st, nullptr);
    if (!s) {
      dim3 sg((unsigned)((count + 255) / 256), c);
      k_split_slots<<<sg, 256, 0, st>>>(stage, count, q0, c, outs_dev,
                                        prec == QBG_PREC_MIXED ? lo_outs_dev : nullptr);
      QBG_LAUNCH_CHECK("k_split_slots");
    }
  }
  e = cudaStreamSynchronize(st);  // the staging buffers are freed below
  dfree(stage, st);
  dfree(dp, st);
  if (s) return s;
  if (e != cudaSuccess) return cuda_status(e, "Alpert assembly");
  return QBG_OK;
}

template <int DERIV, int OUT>
__global__ void __launch_bounds__(256) k_assemble_cheb_reduced(GeomDev g, ChebTables t, const cxd* __restrict__ ks,
                                                               int nk, int kchunk, void* const* __restrict__ outs,
                                                               void* const* __restrict__ los, long long ld) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  const int bcol = blockIdx.y * blockDim.y + threadIdx.y;
  if (a >= g.m || bcol >= g.m) return;
  const int q0 = blockIdx.z * kchunk, q1 = min(nk, q0 + kchunk);
  const int i = g.fund[a], j = g.fund[bcol];
  const size_t off = (size_t)a + (size_t)bcol * (size_t)ld;
  const double xi = g.x[i], yi = g.y[i];
  PairGeom p;
  int pj = 0;
  double tj = 0.0;
  if (i != j) {
    p = pair_geom(g, i, j);
    panel_of(p.r, 0.0, t.rmax, t.dr_j, t.invdr_j, t.nj, pj, tj);
  }
  for (int q = q0; q < q1; ++q) {
    const cxd k = ks[q];
    cxd F, F1(0.0, 0.0), F2(0.0, 0.0);
    if (i == j) {
      F = cxd(1.0 - g.ws[i] * g.kappa[i], 0.0);
    } else {
      cxd h0, h1, j0, j1;
      cheb_h01(t, q, p.r, k, h0, h1);
      clenshaw2(t.J + (((size_t)q * t.nj + pj) * (t.Mj + 1)) * 2, t.Mj, tj, j0, j1);
      entry_vals<0, DERIV>(p, k, h0, h1, j0, j1, &F, &F1, &F2);
    }
    for (int l = 0; l < g.norb; ++l) {
      const int qn = g.orb[bcol * g.norb + l];
      if (qn == j) continue;
      const double dxq = xi - g.x[qn], dyq = yi - g.y[qn];
      const double r = hypot(dxq, dyq);
      if (r < 2.220446049250313e-16) continue;
      const double c = (g.nx[qn] * dxq + g.ny[qn] * dyq) / r;
      const cxd sc(g.orb_scale[2 * (bcol * g.norb + l)], g.orb_scale[2 * (bcol * g.norb + l) + 1]);
      cxd h0, h1;
      cheb_h01(t, q, r, k, h0, h1);
      image_terms<DERIV>(c, g.speed[qn] * g.ws[qn], sc, r, k, h0, h1, F, F1, F2);
    }
    store_entry<OUT>(outs, los, q, off, F);
    if (DERIV) {
      store_entry<OUT>(outs, los, nk + q, off, F1);
      store_entry<OUT>(outs, los, 2 * nk + q, off, F2);
    }
  }
}

// ---------------------------------------------------------------------------
// Symmetry-reduced CFIE (construct_matrices_reduced!, cfie_kress.jl:512-617;
// derivatives :758-892; through the panels,
// chebyshev_euclidian_helmholtz_cfie_kress.jl:698-825 and :1087-1243):
// A_red[a, b] = sum over the members j of orbit b of scale_j A_full[I_a, j],
// with A_full the Kress-split CFIE entry (the diagonal formula when j == I_a,
// the smooth cross-component kernel between components). Unlike the reduced
// DLP, every member of the orbit carries the full Kress split. CHEB: H0, H1
// from the panels (direct below r_min or the small-|z| cut-off), J0, J1
// from the panels; otherwise direct device Bessel values (J = Re H at real k).
// ---------------------------------------------------------------------------
template <int CHEB>
static __device__ __forceinline__ void hj_values(const ChebTables& t, int q, double r, cxd k, bool needj,
                                                 cxd& h0, cxd& h1, cxd& j0, cxd& j1) {
  if (CHEB) {
    cheb_h01(t, q, r, k, h0, h1);
    if (needj) {
      int pj;
      double tj;
      panel_of(r, 0.0, t.rmax, t.dr_j, t.invdr_j, t.nj, pj, tj);
      clenshaw2(t.J + (((size_t)q * t.nj + pj) * (t.Mj + 1)) * 2, t.Mj, tj, j0, j1);
    } else {
      j0 = cxd(0.0, 0.0);
      j1 = cxd(0.0, 0.0);
    }
  } else {
    Bessel01d b = bessel01(r * k);
    if (k.im == 0.0) {
      b.j0.im = 0.0;
      b.j1.im = 0.0;
    }
    h0 = b.h0();
    h1 = b.h1();
    j0 = b.j0;
    j1 = b.j1;
  }
}

template <int DERIV, int OUT, int CHEB>
__global__ void __launch_bounds__(256) k_assemble_cfie_reduced(GeomDev g, ChebTables t, const cxd* __restrict__ ks,
                                                               int nk, int kchunk, void* const* __restrict__ outs,
                                                               void* const* __restrict__ los, long long ld) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  const int bcol = blockIdx.y * blockDim.y + threadIdx.y;
  if (a >= g.m || bcol >= g.m) return;
  const int q0 = blockIdx.z * kchunk, q1 = min(nk, q0 + kchunk);
  const int i = g.fund[a];
  const size_t off = (size_t)a + (size_t)bcol * (size_t)ld;
  for (int q = q0; q < q1; ++q) {
    const cxd k = ks[q];
    cxd F(0.0, 0.0), F1(0.0, 0.0), F2(0.0, 0.0);
    for (int l = 0; l < g.norb; ++l) {
      const int j = g.orb[bcol * g.norb + l];
      const cxd sc(g.orb_scale[2 * (bcol * g.norb + l)], g.orb_scale[2 * (bcol * g.norb + l) + 1]);
      cxd e, e1(0.0, 0.0), e2(0.0, 0.0);
      if (j == i) {
        e = diag_fp64<1>(g, i, k);
        if (DERIV) diag_derivs<1>(g, i, k, &e1, &e2);
      } else {
        const PairGeom p = pair_geom(g, i, j);
        if (!CHEB && !p.same && p.r * p.r <= 4.93038065763132e-32) continue;  // eps(T)^2 guard, cfie_kress.jl:569
        cxd h0, h1, j0, j1;
        hj_values<CHEB>(t, q, p.r, k, p.same, h0, h1, j0, j1);
        entry_vals<1, DERIV>(p, k, h0, h1, j0, j1, &e, &e1, &e2);
      }
      F += sc * e;
      if (DERIV) {
        F1 += sc * e1;
        F2 += sc * e2;
      }
    }
    store_entry<OUT>(outs, los, q, off, F);
    if (DERIV) {
      store_entry<OUT>(outs, los, nk + q, off, F1);
      store_entry<OUT>(outs, los, 2 * nk + q, off, F2);
    }
  }
}

// reduced CFIE launcher: cheb == nullptr evaluates the kernels directly;
// prec QBG_PREC_FP32 writes complex64 values without low words
static int launch_cfie_reduced(const GeomDev& g, const ChebTables* cheb, const cxd* ks, int nk, int deriv, int prec,
                               void* const* outs_dev, void* const* lo_outs_dev, long long ld, cudaStream_t st) {
  const int kchunk = 8;
  dim3 blk(32, 8), grd((g.m + 31) / 32, (g.m + 7) / 8, (nk + kchunk - 1) / kchunk);
  const ChebTables t0 = cheb ? *cheb : ChebTables();
  void* const* lo = prec == QBG_PREC_MIXED ? lo_outs_dev : nullptr;
#define QBG_CFR(D, O, C) k_assemble_cfie_reduced<D, O, C><<<grd, blk, 0, st>>>(g, t0, ks, nk, kchunk, outs_dev, lo, ld)
  if (prec == QBG_PREC_FP64) {
    if (cheb) {
      if (deriv) QBG_CFR(1, 0, 1); else QBG_CFR(0, 0, 1);
    } else {
      if (deriv) QBG_CFR(1, 0, 0); else QBG_CFR(0, 0, 0);
    }
  } else {
    if (deriv) {
      set_error("derivative assembly is available in FP64");
      return QBG_ENOTSUP;
    }
    if (cheb) QBG_CFR(0, 1, 1); else QBG_CFR(0, 1, 0);
  }
#undef QBG_CFR
  QBG_LAUNCH_CHECK("k_assemble_cfie_reduced");
  return QBG_OK;
}

// ---------------------------------------------------------------------------
// Symmetric-pair Chebyshev assembly (value only, no derivatives).
// The kernel values of (i, j) and (j, i) depend on the pair only through r, so
// one panel evaluation serves both entries. With the pair coefficients folded,
//   F_ij = -(alpha J1 + beta H1 + gamma J0 + delta H0),
//   alpha = (cD1 - cD3) (-k/2pi), beta = cD2 (ik/2),
//   gamma = (cS1 - cS3) (-ik/2pi), delta = cS2 (-k/2),
// which is dval + ik sval of entry_vals regrouped (cross-component CFIE
// pairs keep only beta = w inner/r and delta = w s). CTA = one 32 x 32 tile
// pair (bi <= bj); the mirrored tile is written through shared memory so both
// stores are coalesced.
// ---------------------------------------------------------------------------
struct Fold {
  double A, B, C, D;  // real pair coefficients of J1, H1, J0, H0
};

template <int FORM>
static __device__ __forceinline__ Fold fold_of(const PairGeom& p) {
  Fold f;
  if (FORM == 1 && !p.same) {
    f.A = 0.0; f.B = p.wj * p.inn * p.invr; f.C = 0.0; f.D = p.wj * p.sj;
    return f;
  }
  const double cD1 = p.Rk * p.inn * p.invr, cD2 = p.wj * p.inn * p.invr, cD3 = p.wj * p.lt * p.inn * p.invr;
  f.A = cD1 - cD3;
  f.B = cD2;
  if (FORM == 1) {
    const double cS1 = p.Rk * p.sj, cS2 = p.wj * p.sj, cS3 = p.wj * p.sj * p.lt;
    f.C = cS1 - cS3;
    f.D = cS2;
  } else {
    f.C = 0.0;
    f.D = 0.0;
  }
  return f;
}

static __device__ __forceinline__ cxd folded_entry(const Fold& f, cxd kaL1, cxd kaL2, cxd kg, cxd kd, cxd h0,
                                                   cxd h1, cxd j0, cxd j1) {
  cxd s = (f.A * kaL1) * j1;
  cfma(s, f.B * kaL2, h1);
  cfma(s, f.C * kg, j0);
  cfma(s, f.D * kd, h0);
  return -s;
}

static __device__ __forceinline__ int2 tile_pair(int t) {
  int bj = (int)((sqrt(8.0 * (double)t + 1.0) - 1.0) * 0.5);
  while ((bj + 1) * (bj + 2) / 2 <= t) ++bj;
  while (bj * (bj + 1) / 2 > t) --bj;
  return make_int2(t - bj * (bj + 1) / 2, bj);
}

template <int FORM, int OUT>
__global__ void __launch_bounds__(512) k_assemble_cheb_sym(GeomDev g, ChebTables t, const cxd* __restrict__ ks,
                                                           int nk, int kchunk, void* const* __restrict__ outs,
                                                           void* const* __restrict__ los, long long ld) {
  __shared__ cxd sm[32][33];
  const int2 bp = tile_pair(blockIdx.x);
  const int bi = bp.x, bj = bp.y;
  const bool dtile = (bi == bj);
  const int tx = threadIdx.x, ty = threadIdx.y;  // 32 x 16
  const int i = bi * 32 + tx;
  const int q0 = blockIdx.z * kchunk, q1 = min(nk, q0 + kchunk);
  auto store = [&](int slot, size_t off, cxd v) {
    if (OUT == 0) {
      reinterpret_cast<cxd*>(outs[slot])[off] = v;
    } else {
      const cxf hi(v);
      reinterpret_cast<cxf*>(outs[slot])[off] = hi;
      if (los) reinterpret_cast<cxf*>(los[slot])[off] = cxf((float)(v.re - (double)hi.re), (float)(v.im - (double)hi.im));
    }
  };
  // pair data for the two column slots s = 0, 1 (j = bj*32 + ty + 16 s)
  bool act[2], isdiag[2], zero[2], direct[2];
  Fold fij[2], fji[2];
  int ph[2], pj[2];
  double th[2], tj[2], rr[2];
#pragma unroll
  for (int s = 0; s < 2; ++s) {
    const int j = bj * 32 + ty + 16 * s;
    const bool inb = (i < g.n) && (j < g.n);
    isdiag[s] = inb && (i == j);
    act[s] = inb && !isdiag[s] && (!dtile || i < j);
    zero[s] = false;
    direct[s] = false;
    rr[s] = 0.0;
    ph[s] = pj[s] = 0;
    th[s] = tj[s] = 0.0;
    if (act[s]) {
      const PairGeom pa = pair_geom(g, i, j);
      const PairGeom pb = pair_geom(g, j, i);
      fij[s] = fold_of<FORM>(pa);
      fji[s] = fold_of<FORM>(pb);
      rr[s] = pa.r;
      zero[s] = (FORM == 1 && !pa.same && pa.r * pa.r <= 4.93038065763132e-32);
      panel_of(pa.r, t.rmin, t.rmax, t.dr_h, t.invdr_h, t.nh, ph[s], th[s]);
      panel_of(pa.r, 0.0, t.rmax, t.dr_j, t.invdr_j, t.nj, pj[s], tj[s]);
      direct[s] = pa.r < t.rmin;
    }
  }
  const double inv2pi = 0.15915494309189533577;
  for (int q = q0; q < q1; ++q) {
    const cxd k = ks[q];
    const double ak = hypot(k.re, k.im);
    const cxd kaL1 = (-inv2pi) * k, kaL2 = 0.5 * cmul_i(k), kg = (-inv2pi) * cmul_i(k), kd = -0.5 * k;
#pragma unroll
    for (int s = 0; s < 2; ++s) {
      const int j = bj * 32 + ty + 16 * s;
      cxd vij(0.0, 0.0), vji(0.0, 0.0);
      if (isdiag[s]) {
        store(q, (size_t)i + (size_t)j * ld, diag_fp64<FORM>(g, i, k));
      } else if (act[s]) {
        if (!zero[s]) {
          cxd h0, h1, j0(0.0, 0.0), j1(0.0, 0.0);
          if (direct[s] || rr[s] * ak < t.small_cut) {
            const Bessel01d b = bessel01(rr[s] * k);
            h0 = b.h0();
            h1 = b.h1();
          } else {
            clenshaw2(t.H + (((size_t)q * t.nh + ph[s]) * (t.Mh + 1)) * 2, t.Mh, th[s], h0, h1);
          }
          if (fij[s].A != 0.0 || fij[s].C != 0.0 || fji[s].A != 0.0 || fji[s].C != 0.0)
            clenshaw2(t.J + (((size_t)q * t.nj + pj[s]) * (t.Mj + 1)) * 2, t.Mj, tj[s], j0, j1);
          vij = folded_entry(fij[s], kaL1, kaL2, kg, kd, h0, h1, j0, j1);
          vji = folded_entry(fji[s], kaL1, kaL2, kg, kd, h0, h1, j0, j1);
        }
        store(q, (size_t)i + (size_t)j * ld, vij);
      }
      sm[ty + 16 * s][tx] = vji;  // row = j - bj*32, column = i - bi*32
    }
    __syncthreads();
#pragma unroll
    for (int s = 0; s < 2; ++s) {
      const int jl = tx, il = ty + 16 * s;  // output (row j, column i)
      const int j = bj * 32 + jl, ii = bi * 32 + il;
      const bool ok = (j < g.n) && (ii < g.n) && (dtile ? (jl > il) : true);
      if (ok) store(q, (size_t)j + (size_t)ii * ld, sm[jl][il]);
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// Double-float evaluation for the complex64 forms (QBG_PREC_MIXED / FP32)
// ---------------------------------------------------------------------------
// The FP64 pipe of this part runs at 1/64 of the FP32 rate, and the FP64
// symmetric kernel above spends nearly all its time there (two degree-M
// Clenshaw sums and the fold per pair and node). Here every per-node step runs
// on FP32 pairs (hi + lo, ~2^-48 relative): the Chebyshev polynomials T_m(t)
// by their recurrence, the four premultiplied series of each table as
// error-free FMA dot products, and the fold with the pair's real coefficients.
// Per pair and tile the geometry, the fold coefficients and the panel
// arguments are computed once in FP64 for all nodes. The result is the mixed
// form's (hi, lo) pair directly. Pairs below the direct-evaluation cut and the
// diagonal keep the FP64 route.
namespace {

struct dfl {
  float hi, lo;
};

__device__ __forceinline__ dfl df_of(double x) {
  dfl r;
  r.hi = (float)x;
  r.lo = (float)(x - (double)r.hi);
  return r;
}

__device__ __forceinline__ dfl df_two_sum(float a, float b) {
  const float s = a + b;
  const float bb = s - a;
  return {s, (a - (s - bb)) + (b - bb)};
}

__device__ __forceinline__ dfl df_fast_sum(float a, float b) {  // |a| >= |b|
  const float s = a + b;
  return {s, b - (s - a)};
}

__device__ __forceinline__ dfl df_mul(dfl a, dfl b) {
  const float p = a.hi * b.hi;
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, e);
  e = fmaf(a.lo, b.hi, e);
  return df_fast_sum(p, e);
}

__device__ __forceinline__ dfl df_sub(dfl a, dfl b) {
  dfl s = df_two_sum(a.hi, -b.hi);
  s.lo += a.lo - b.lo;
  return df_fast_sum(s.hi, s.lo);
}

// acc += c t, acc kept unnormalised (hi exact partial sums, lo the errors)
__device__ __forceinline__ void df_acc(dfl& acc, dfl c, dfl t) {
  const float p = c.hi * t.hi;
  float e = fmaf(c.hi, t.hi, -p);
  e = fmaf(c.hi, t.lo, e);
  e = fmaf(c.lo, t.hi, e);
  const dfl s = df_two_sum(acc.hi, p);
  acc.hi = s.hi;
  acc.lo += s.lo + e;
}

__device__ __forceinline__ dfl df_norm(dfl a) { return df_two_sum(a.hi, a.lo); }

// Compile-time degree MT: every coefficient of the row is loaded before the
// recurrence, so a thread waits for one cache latency per series instead of
// one per degree (the loop over a runtime degree keeps each load in its own
// iteration).
template <bool S0, int MT>
__device__ __forceinline__ void df_series_m(const float4* __restrict__ c, dfl t, dfl* v0r, dfl* v0i, dfl* v1r,
                                            dfl* v1i) {
  float4 k1[MT + 1], k0[S0 ? MT + 1 : 1];
#pragma unroll
  for (int m = 0; m <= MT; ++m) {
    k1[m] = __ldg(c + 2 * m + 1);
    if (S0) k0[m] = __ldg(c + 2 * m);
  }
  dfl a0r{0.f, 0.f}, a0i{0.f, 0.f}, a1r{0.f, 0.f}, a1i{0.f, 0.f};
  dfl tp{1.f, 0.f}, tc = t;
  const dfl t2{2.f * t.hi, 2.f * t.lo};
#pragma unroll
  for (int m = 0; m <= MT; ++m) {
    dfl tm;
    if (m == 0) {
      tm = tp;
    } else if (m == 1) {
      tm = tc;
    } else {
      tm = df_sub(df_mul(t2, tc), tp);
      tp = tc;
      tc = tm;
    }
    df_acc(a1r, dfl{k1[m].x, k1[m].y}, tm);
    df_acc(a1i, dfl{k1[m].z, k1[m].w}, tm);
    if (S0) {
      df_acc(a0r, dfl{k0[m].x, k0[m].y}, tm);
      df_acc(a0i, dfl{k0[m].z, k0[m].w}, tm);
    }
  }
  *v1r = a1r;
  *v1i = a1i;
  if (S0) {
    *v0r = a0r;
    *v0i = a0i;
  }
}

// sum_m c_m T_m(t) for the two complex series of one table row (float4 pairs
// per degree: {series 0, series 1}); S0 skips series 0 (DLP needs only J1, H1)
template <bool S0>
__device__ __forceinline__ void df_series(const float4* __restrict__ c, int M, dfl t, dfl* v0r, dfl* v0i, dfl* v1r,
                                          dfl* v1i) {
  dfl a0r{0.f, 0.f}, a0i{0.f, 0.f}, a1r{0.f, 0.f}, a1i{0.f, 0.f};
  dfl tp{1.f, 0.f}, tc = t;  // T_{m-1}, T_m
  const dfl t2{2.f * t.hi, 2.f * t.lo};
  for (int m = 0; m <= M; ++m) {
    dfl tm;
    if (m == 0) {
      tm = tp;
    } else if (m == 1) {
      tm = tc;
    } else {
      tm = df_sub(df_mul(t2, tc), tp);
      tp = tc;
      tc = tm;
    }
    const float4 c1 = __ldg(c + 2 * m + 1);
    df_acc(a1r, dfl{c1.x, c1.y}, tm);
    df_acc(a1i, dfl{c1.z, c1.w}, tm);
    if (S0) {
      const float4 c0 = __ldg(c + 2 * m);
      df_acc(a0r, dfl{c0.x, c0.y}, tm);
      df_acc(a0i, dfl{c0.z, c0.w}, tm);
    }
  }
  *v1r = a1r;
  *v1i = a1i;
  if (S0) {
    *v0r = a0r;
    *v0i = a0i;
  }
}

template <bool S0, int DM>
__device__ __forceinline__ void df_series_d(const float4* __restrict__ c, int M, dfl t, dfl* v0r, dfl* v0i, dfl* v1r,
                                            dfl* v1i) {
  if (DM > 0) df_series_m<S0, (DM > 0 ? DM : 1)>(c, t, v0r, v0i, v1r, v1i);
  else df_series<S0>(c, M, t, v0r, v0i, v1r, v1i);
}


__device__ __forceinline__ float4 pack_split(cxd v) {
  const float hr = (float)v.re, hi = (float)v.im;
  return make_float4(hr, hi, (float)(v.re - (double)hr), (float)(v.im - (double)hi));
}

}  // namespace

__global__ void k_node_consts(const cxd* __restrict__ ks, int nk, NodeConst* out) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nk) return;
  const cxd k = ks[q];
  const double inv2pi = 0.15915494309189533577;
  NodeConst c;
  c.kaL1 = (-inv2pi) * k;
  c.kaL2 = 0.5 * cmul_i(k);
  c.kg = (-inv2pi) * cmul_i(k);
  c.kd = -0.5 * k;
  c.ak = hypot(k.re, k.im);
  out[q] = c;
}

// grid (rows / 256, nk, 2 tables); rows = panels x (M + 1)
__global__ void k_cheb_df_tables(ChebTables t) {
  const int tab = blockIdx.z, q = blockIdx.y;
  const long long rows = (long long)(tab ? t.nj : t.nh) * ((tab ? t.Mj : t.Mh) + 1);
  const long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= rows) return;
  const NodeConst nc = t.nkc[q];
  const cxd* src = (tab ? t.J : t.H) + ((size_t)q * rows + r) * 2;
  const cxd s0 = tab ? nc.kg * src[0] : nc.kd * src[0];
  const cxd s1 = tab ? nc.kaL1 * src[1] : nc.kaL2 * src[1];
  float4* dst = (tab ? t.JD : t.HD) + ((size_t)q * rows + r) * 2;
  const dfl a = df_of(s0.re), b = df_of(s0.im), c = df_of(s1.re), d = df_of(s1.im);
  dst[0] = make_float4(a.hi, a.lo, b.hi, b.lo);
  dst[1] = make_float4(c.hi, c.lo, d.hi, d.lo);
}

// ---------------------------------------------------------------------------
// J/E tables and the sorted-tile double-float assembly of full operators.
//
// With z = k r, l = (2/pi) ln r and the ascending series of A&S 9.1.11 and
// 9.1.13, Y0 = (2/pi)(ln(z/2) + gamma) J0 + ..., Y1 = -2/(pi z) +
// (2/pi)(ln(z/2) + gamma) J1 + ..., the functions
//   G0 = Y0 - l J0 = (2/pi) [(ln(k/2) + gamma) J0 - s0],
//   G1 = Y1 - l J1 + 2/(pi z) = (2/pi)(ln(k/2) + gamma) J1 - s1 / pi
// (s0 = sum H_m t0_m, s1 = sum (H_m + H_{m+1}) t1_m over the series terms)
// are entire in r: the logarithm and the pole of the Hankel functions are
// exact per-pair factors, ln r and 1/r, while the panels only resolve the
// oscillation e^{+-ikr}. One table on the J grid of [0, rmax] therefore
// replaces the H table on [rmin, rmax], whose panels also had to resolve
// 1/r near rmin (7695 against 863 J panels at N = 2048, k = 200, 1e-13),
// and one Chebyshev recurrence per pair serves all four series.
// ---------------------------------------------------------------------------
// J0, J1, G0, G1 at r for the node k; lkg = ln(k/2) + gamma
static __device__ void je_values(cxd k, cxd lkg, double r, cxd& j0, cxd& j1, cxd& g0, cxd& g1) {
  const double inv_pi = 0.31830988618379067154, two_over_pi = 0.63661977236758134308;
  if (r == 0.0) {
    j0 = cxd(1.0, 0.0);
    j1 = cxd(0.0, 0.0);
    g0 = two_over_pi * lkg;
    g1 = cxd(0.0, 0.0);
    return;
  }
  const cxd z = r * k;
  if (cabs_d(z) < 4.0) {
    // terms t0_m = (-z^2/4)^m / (m!)^2, t1_m = (z/2)(-z^2/4)^m / (m!(m+1)!); at
    // |z| < 4 the largest term is below 5, so the sums lose no digits
    const cxd h = 0.5 * z, q = -(h * h);
    cxd t0(1.0, 0.0), t1 = h, a0(0.0, 0.0), a1(0.0, 0.0), s0(0.0, 0.0), s1(0.0, 0.0);
    double hm = 0.0;  // harmonic number H_m
    for (int m = 0; m < 48; ++m) {
      if (m > 0) {
        t0 = t0 * q * (1.0 / ((double)m * m));
        t1 = t1 * q * (1.0 / ((double)m * (m + 1)));
        hm += 1.0 / m;
      }
      a0 += t0;
      a1 += t1;
      s0 += hm * t0;
      s1 += (2.0 * hm + 1.0 / (m + 1)) * t1;
      if (cabs_d(t0) < 1e-18 && cabs_d(t1) < 1e-18) break;
    }
    j0 = a0;
    j1 = a1;
    g0 = two_over_pi * (lkg * a0 - s0);
    g1 = two_over_pi * (lkg * a1) - inv_pi * s1;
  } else {
    const Bessel01d b = bessel01(z);
    const double l = two_over_pi * log(r);
    j0 = b.j0;
    j1 = b.j1;
    g0 = b.y0 - l * b.j0;
    g1 = b.y1 - l * b.j1 + two_over_pi * cinv(z);
  }
}

// CTA = (JE_BUILD_THREADS / (M + 1)) panels of one node, one thread per
// Chebyshev-Lobatto point (the FP64 Bessel evaluation is the cost: one
// thread per panel left the FP64 pipe idle on latency); then one thread per
// (panel, degree) forms the DCT-I coefficients (as k_cheb_build) from the
// values in shared memory and stores their double-float split; last, one
// thread per panel folds the panel's FP32-tail degree into JEm by atomicMax
// (the largest over the nodes, so the assembly reads it once per pair).
constexpr int JE_BUILD_THREADS = 128;

template <int NS>
__global__ void __launch_bounds__(JE_BUILD_THREADS) k_cheb_build_je(ChebTables t, const cxd* __restrict__ ks) {
  constexpr int MMAX = QBG_CHEB_MAX_DEGREE;
  __shared__ cxd fv[JE_BUILD_THREADS][NS];
  __shared__ double mag[JE_BUILD_THREADS][NS];
  __shared__ double dct[(MMAX + 1) * (MMAX + 1)];
  const int M = t.Mje, P = M + 1, ppb = JE_BUILD_THREADS / P;
  const int q = blockIdx.y;
  const int tid = threadIdx.x;
  for (int x = tid; x < P * P; x += JE_BUILD_THREADS) {
    const int jn = x / P, m = x % P;
    dct[x] = cospi((double)(jn * m) / (double)M);  // cos(pi jn m / M)
  }
  const int lp = tid / P, n = tid % P;
  const int p = blockIdx.x * ppb + lp;
  const bool live = lp < ppb && p < t.nje;
  const cxd k = ks[q];
  if (live) {
    const double a = (double)p * t.dr_je;
    const double b = (p + 1 == t.nje) ? t.rmax : (double)(p + 1) * t.dr_je;
    const bool realk = (k.im == 0.0);
    const cxd kaL2 = 0.5 * cmul_i(k), kd = -0.5 * k;
    const cxd lkg = clog_d(0.5 * k) + cxd(0.57721566490153286061, 0.0);
    const double tn = cospi((double)n / (double)M);
    const double r = 0.5 * ((b + a) + (b - a) * tn);
    cxd j0, j1, g0, g1;
    je_values(k, lkg, r, j0, j1, g0, g1);
    if (realk) { j0.im = 0.0; j1.im = 0.0; g0.im = 0.0; g1.im = 0.0; }
    fv[tid][0] = kaL2 * j1;
    fv[tid][1] = kaL2 * (j1 + cmul_i(g1));
    if (NS == 4) {
      fv[tid][2] = kd * j0;
      fv[tid][3] = kd * (j0 + cmul_i(g0));
    }
  }
  __syncthreads();
  if (live) {
    const int m = n, base = lp * P;  // this thread: degree m of panel p
    const double sg = (m & 1) ? -1.0 : 1.0;
    double sc = 2.0 / (double)M;
    if (m == 0) sc *= 0.5;
    float4* out = t.JE + ((size_t)q * t.nje + p) * (size_t)P * NS;
#pragma unroll
    for (int s = 0; s < NS; ++s) {
      cxd acc = 0.5 * fv[base][s] + (0.5 * sg) * fv[base + M][s];
      for (int jn = 1; jn < M; ++jn) acc += dct[jn * P + m] * fv[base + jn][s];
      acc = sc * acc;
      const dfl re = df_of(acc.re), im = df_of(acc.im);
      out[m * NS + s] = make_float4(re.hi, re.lo, im.hi, im.lo);
      mag[tid][s] = fabs(acc.re) + fabs(acc.im);
    }
  }
  __syncthreads();
  if (live && n == 0) {
    // FP32 tail: terms from degree m0 on, in every series, sum to at most
    // 2^-26 of the series' coefficient magnitudes; FP32 products of those
    // terms (|T_m| <= 1, error <= 2^-23 each) then stay below 2^-49 of that
    // sum, the order of the double-float rounding of the head (m0 >= 2: the
    // recurrence of the head supplies T_{m0-1} and T_{m0-2})
    const int base = lp * P;
    int m0 = 2;
#pragma unroll
    for (int s = 0; s < NS; ++s) {
      double tot = 0.0;
      for (int m = 0; m <= M; ++m) tot += mag[base + m][s];
      double tail = 0.0;
      int ms = M + 1;
      while (ms > 2 && tail + mag[base + ms - 1][s] <= 0x1p-26 * tot) tail += mag[base + --ms][s];
      m0 = ms > m0 ? ms : m0;
    }
    atomicMax(t.JEm + p, m0);
  }
}

namespace {
// pair coefficients of one entry on the J/E series (negated as stored):
//   entry.re = b U.re + a P.im + d W.re + c R.im + kk
//   entry.im = b U.im - a P.re + d W.im - c R.re
// with b = -B, a = A/pi + B l, d = -D, c = C/pi + D l, kk = -B/(pi r)
struct JeCoef {
  dfl b, a, d, c, kk;
};

template <int FORM>
__device__ __forceinline__ JeCoef je_coef(const Fold& f, double l, double invr) {
  const double inv_pi = 0.31830988618379067154;
  JeCoef e;
  e.b = df_of(-f.B);
  e.a = df_of(f.A * inv_pi + f.B * l);
  e.kk = df_of(-f.B * inv_pi * invr);
  if (FORM == 1) {
    e.d = df_of(-f.D);
    e.c = df_of(f.C * inv_pi + f.D * l);
  } else {
    e.d = dfl{0.f, 0.f};
    e.c = dfl{0.f, 0.f};
  }
  return e;
}

// shared-memory layout of the two entries' coefficients of a slot: NC float4
// rows of 1024 slots, {b, a} (ij), {b, a} (ji), {kk_ij, kk_ji}, then for the
// CFIE {d, c} (ij), {d, c} (ji)
template <int FORM>
__host__ __device__ constexpr int je_coef_words() {
  return FORM == 1 ? 5 : 3;
}

template <int FORM>
__device__ __forceinline__ void je_coef_store(float4* sm, int slot, const JeCoef& x, const JeCoef& y) {
  sm[0 * 1024 + slot] = make_float4(x.b.hi, x.b.lo, x.a.hi, x.a.lo);
  sm[1 * 1024 + slot] = make_float4(y.b.hi, y.b.lo, y.a.hi, y.a.lo);
  sm[2 * 1024 + slot] = make_float4(x.kk.hi, x.kk.lo, y.kk.hi, y.kk.lo);
  if (FORM == 1) {
    sm[3 * 1024 + slot] = make_float4(x.d.hi, x.d.lo, x.c.hi, x.c.lo);
    sm[4 * 1024 + slot] = make_float4(y.d.hi, y.d.lo, y.c.hi, y.c.lo);
  }
}

template <int FORM>
__device__ __forceinline__ void je_coef_load(const float4* sm, int slot, JeCoef& x, JeCoef& y) {
  float4 u = sm[0 * 1024 + slot];
  x.b = dfl{u.x, u.y};
  x.a = dfl{u.z, u.w};
  u = sm[1 * 1024 + slot];
  y.b = dfl{u.x, u.y};
  y.a = dfl{u.z, u.w};
  u = sm[2 * 1024 + slot];
  x.kk = dfl{u.x, u.y};
  y.kk = dfl{u.z, u.w};
  if (FORM == 1) {
    u = sm[3 * 1024 + slot];
    x.d = dfl{u.x, u.y};
    x.c = dfl{u.z, u.w};
    u = sm[4 * 1024 + slot];
    y.d = dfl{u.x, u.y};
    y.c = dfl{u.z, u.w};
  } else {
    x.d = x.c = y.d = y.c = dfl{0.f, 0.f};
  }
}

template <int FORM>
__device__ __forceinline__ float4 je_fold(const JeCoef& e, const dfl* v) {
  // v: P.re, P.im, U.re, U.im, R.re, R.im, W.re, W.im
  dfl re = e.kk, im{0.f, 0.f};
  const dfl na{-e.a.hi, -e.a.lo};
  df_acc(re, e.b, v[2]);
  df_acc(re, e.a, v[1]);
  df_acc(im, e.b, v[3]);
  df_acc(im, na, v[0]);
  if (FORM == 1) {
    const dfl nc{-e.c.hi, -e.c.lo};
    df_acc(re, e.d, v[6]);
    df_acc(re, e.c, v[5]);
    df_acc(im, e.d, v[7]);
    df_acc(im, nc, v[4]);
  }
  re = df_norm(re);
  im = df_norm(im);
  return make_float4(re.hi, im.hi, re.lo, im.lo);
}

// the FP64 routes of the J/E kernel, out of line so that their registers do
// not weigh on the series loop: the diagonal, and coincident nodes of different
// components (r below every table radius; the CFIE's vanish before this)
template <int FORM>
__device__ __noinline__ float4 je_diag(const GeomDev& g, int i, cxd k) {
  return pack_split(diag_fp64<FORM>(g, i, k));
}

template <int FORM>
__device__ __noinline__ void je_direct_pair(const GeomDev& g, int i, int j, cxd k, float4* vij, float4* vji) {
  const PairGeom pa = pair_geom(g, i, j);
  const PairGeom pb = pair_geom(g, j, i);
  const double inv2pi = 0.15915494309189533577;
  const cxd kaL1 = (-inv2pi) * k, kaL2 = 0.5 * cmul_i(k), kg = (-inv2pi) * cmul_i(k), kd = -0.5 * k;
  const Bessel01d bz = bessel01(pa.r * k);
  *vij = pack_split(folded_entry(fold_of<FORM>(pa), kaL1, kaL2, kg, kd, bz.h0(), bz.h1(), bz.j0, bz.j1));
  *vji = pack_split(folded_entry(fold_of<FORM>(pb), kaL1, kaL2, kg, kd, bz.h0(), bz.h1(), bz.j0, bz.j1));
}

// sum_m c_m T_m(t) of the NS complex series of one table row: degrees below
// m0 in double-float, the tail (m0 <= m <= M) as FP32 products added to the
// low words (the accumulators are unnormalised: hi exact partial sums)
template <int NS>
__device__ __forceinline__ void je_series(const float4* __restrict__ c, int M, int m0, dfl t, dfl* v) {
#pragma unroll
  for (int s = 0; s < 2 * NS; ++s) v[s] = dfl{0.f, 0.f};
  dfl tp{1.f, 0.f}, tc = t;
  const dfl t2{2.f * t.hi, 2.f * t.lo};
#pragma unroll 2
  for (int m = 0; m < m0; ++m) {
    dfl tm;
    if (m == 0) {
      tm = tp;
    } else if (m == 1) {
      tm = tc;
    } else {
      tm = df_sub(df_mul(t2, tc), tp);
      tp = tc;
      tc = tm;
    }
#pragma unroll
    for (int s = 0; s < NS; ++s) {
      const float4 cc = __ldg(c + m * NS + s);
      df_acc(v[2 * s], dfl{cc.x, cc.y}, tm);
      df_acc(v[2 * s + 1], dfl{cc.z, cc.w}, tm);
    }
  }
  // m0 >= 2: tc = T_{m0-1}, tp = T_{m0-2}
  float fp = tp.hi, fc = tc.hi;
  const float f2 = t2.hi;
#pragma unroll 2
  for (int m = m0; m <= M; ++m) {
    const float fm = fmaf(f2, fc, -fp);
    fp = fc;
    fc = fm;
#pragma unroll
    for (int s = 0; s < NS; ++s) {
      const float4 cc = __ldg(c + m * NS + s);
      v[2 * s].lo = fmaf(cc.x, fm, v[2 * s].lo);
      v[2 * s + 1].lo = fmaf(cc.z, fm, v[2 * s + 1].lo);
    }
  }
}
}  // namespace

// Full symmetric operator on the J/E tables, every node of ks in one pass.
// CTA = one 32 x 32 tile pair (bi <= bj) as k_assemble_cheb_sym, but the
// tile's pairs are sorted by table panel before the node loop (bitonic sort of
// 1024 keys in shared memory), so the 32 pairs of a warp read a few table rows
// instead of 32 (the row loads were the bound of the per-pair order: 23
// sectors per request, half the issue slots lost to long-scoreboard stalls).
// Both mirrored entries of a pair are staged in shared memory per node and
// written as coalesced columns.
template <int FORM, int OCC>
__global__ void __launch_bounds__(512, OCC) k_assemble_je_df(GeomDev g, ChebTables t, const cxd* __restrict__ ks,
                                                             int nk, void* const* __restrict__ outs,
                                                             void* const* __restrict__ los, long long ld) {
  constexpr int NS = FORM == 1 ? 4 : 2;
  // dynamic shared memory: tA [32][32] float4 = entries (i, j) at [j - 32 bj][i - 32 bi] (the whole
  // tile when bi == bj); tB [32][32] = entries (j, i) at [i - 32 bi][j - 32 bj], its first 4 KB
  // holding the sort keys before the node loop; coef [NC][1024], the pair coefficients of every
  // sorted slot (registers would spill). Column reads of tA / tB are contiguous per warp, so the
  // tiles need no padding.
  extern __shared__ float4 smem_je[];
  float4(*tA)[32] = reinterpret_cast<float4(*)[32]>(smem_je);
  float4(*tB)[32] = reinterpret_cast<float4(*)[32]>(smem_je + 1024);
  unsigned* keys = reinterpret_cast<unsigned*>(smem_je + 1024);
  float4* coef = smem_je + 2048;
  const int2 bp = tile_pair(blockIdx.x);
  const int bi = bp.x, bj = bp.y;
  const bool dtile = (bi == bj);
  const int tid = threadIdx.y * 32 + threadIdx.x;
  const unsigned NOPANEL = (1u << 22) - 1;
  // keys: panel << 10 | pair index e = il + 32 jl; inactive pairs last
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    const int e = tid + 512 * h;
    const int i = bi * 32 + (e & 31), j = bj * 32 + (e >> 5);
    unsigned pk = NOPANEL;
    if (i < g.n && j < g.n && i != j && (!dtile || i < j)) {
      // FP32 distance: the key only groups pairs by panel (the slot's panel is FP64)
      const float dx = (float)(g.x[i] - g.x[j]), dy = (float)(g.y[i] - g.y[j]);
      int qp = (int)(sqrtf(fmaf(dx, dx, dy * dy)) * (float)t.invdr_je);
      qp = qp < 0 ? 0 : (qp >= t.nje ? t.nje - 1 : qp);
      pk = (unsigned)qp;
    }
    keys[e] = (pk << 10) | (unsigned)e;
  }
  __syncthreads();
  for (int kk = 2; kk <= 1024; kk <<= 1) {
    for (int jj = kk >> 1; jj > 0; jj >>= 1) {
      const int lo = 2 * tid - (tid & (jj - 1)), hi = lo + jj;
      const bool up = (lo & kk) == 0;
      const unsigned x = keys[lo], y = keys[hi];
      if ((x > y) == up) {
        keys[lo] = y;
        keys[hi] = x;
      }
      __syncthreads();
    }
  }
  // per slot (sorted positions tid and tid + 512): meta = e | m0 << 10 | flags, panel, argument
  constexpr unsigned ACT = 1u << 16, ZERO = 1u << 17, DIRECT = 1u << 18;
  unsigned meta[2];
  int ppan[2];
  dfl tt[2];
#pragma unroll
  for (int s = 0; s < 2; ++s) {
    const unsigned key = keys[tid + 512 * s];
    const int e = (int)(key & 1023u);
    unsigned mt = (unsigned)e;
    ppan[s] = 0;
    double td = 0.0;
    Fold fij{0.0, 0.0, 0.0, 0.0}, fji{0.0, 0.0, 0.0, 0.0};
    double l = 0.0, invr = 0.0;
    if ((key >> 10) != NOPANEL) {
      const int i = bi * 32 + (e & 31), j = bj * 32 + (e >> 5);
      PairGeom pa, pb;
      pair_geom_sym(g, i, j, pa, pb);
      fij = fold_of<FORM>(pa);
      fji = fold_of<FORM>(pb);
      const bool zero = (FORM == 1 && !pa.same && pa.r * pa.r <= 4.93038065763132e-32);
      mt |= ACT | (zero ? ZERO : 0u) | ((!zero && pa.r < t.rmin) ? DIRECT : 0u);
      panel_of(pa.r, 0.0, t.rmax, t.dr_je, t.invdr_je, t.nje, ppan[s], td);
      mt |= (unsigned)t.JEm[ppan[s]] << 10;
      l = 0.63661977236758134308 * log(pa.r);
      invr = pa.invr;
    }
    meta[s] = mt;
    tt[s] = df_of(td);
    je_coef_store<FORM>(coef, tid + 512 * s, je_coef<FORM>(fij, l, invr), je_coef<FORM>(fji, l, invr));
  }
  __syncthreads();  // every key is read before the node loop writes tB
  const int Mt = t.Mje;
  for (int q = 0; q < nk; ++q) {
#pragma unroll
    for (int s = 0; s < 2; ++s) {
      const unsigned mt = meta[s];
      if (!(mt & ACT)) continue;
      const int il = mt & 31, jl = (mt >> 5) & 31;
      float4 vij = make_float4(0.f, 0.f, 0.f, 0.f), vji = vij;
      if (mt & ZERO) {
        // both entries vanish
      } else if (mt & DIRECT) {
        je_direct_pair<FORM>(g, bi * 32 + il, bj * 32 + jl, ks[q], &vij, &vji);
      } else {
        dfl v[8];
        je_series<NS>(t.JE + ((size_t)q * t.nje + ppan[s]) * (size_t)(Mt + 1) * NS, Mt, (int)((mt >> 10) & 31u),
                      tt[s], v);
        JeCoef cij, cji;
        je_coef_load<FORM>(coef, tid + 512 * s, cij, cji);
        vij = je_fold<FORM>(cij, v);
        vji = je_fold<FORM>(cji, v);
      }
      tA[jl][il] = vij;
      if (dtile) tA[il][jl] = vji;
      else tB[il][jl] = vji;
    }
    if (dtile && tid < 32 && bi * 32 + tid < g.n) tA[tid][tid] = je_diag<FORM>(g, bi * 32 + tid, ks[q]);
    __syncthreads();
    const int row = threadIdx.x;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int c = threadIdx.y + 16 * h;
      const int i = bi * 32 + row, j = bj * 32 + c;  // tile A: row i, column j
      if (i < g.n && j < g.n) {
        const float4 v = tA[c][row];
        const size_t off = (size_t)i + (size_t)j * ld;
        reinterpret_cast<cxf*>(outs[q])[off] = cxf(v.x, v.y);
        if (los) reinterpret_cast<cxf*>(los[q])[off] = cxf(v.z, v.w);
      }
      if (!dtile) {
        const int jr = bj * 32 + row, ic = bi * 32 + c;  // tile B: row j, column i
        if (jr < g.n && ic < g.n) {
          const float4 v = tB[c][row];
          const size_t off = (size_t)jr + (size_t)ic * ld;
          reinterpret_cast<cxf*>(outs[q])[off] = cxf(v.x, v.y);
          if (los) reinterpret_cast<cxf*>(los[q])[off] = cxf(v.z, v.w);
        }
      }
    }
    __syncthreads();
  }
}

// Symmetry-reduced DLP (value, complex64 forms) on double-float arithmetic:
// one thread per reduced entry (a, b), every node of ks in one pass. Per
// entry the FP64 geometry, the fold coefficients of the main pair, and for
// each other orbit member the image coefficient c w_q sc and its panel
// argument are formed once; per node the premultiplied series (kaL2 H1 on the
// H table, kaL1 J1 on the J table) are evaluated in FP32 pairs:
//   F_ab = [1 - w kappa]_(a=b) - (A kaL1 J1 + B kaL2 H1)(r_ij) - sum_images c w_q sc kaL2 H1(r_iq)
// (dlp_kress.jl:1151-1189 with the images of :1081-1100). Entries with a
// distance below the panels' r_min take the FP64 route.
template <int MAXIMG, int DM>
__global__ void __launch_bounds__(256, 1) k_assemble_cheb_reduced_df(GeomDev g, ChebTables t, const cxd* __restrict__ ks,
                                                                  int nk, void* const* __restrict__ outs,
                                                                  void* const* __restrict__ los, long long ld) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  const int bcol = blockIdx.y * blockDim.y + threadIdx.y;
  if (a >= g.m || bcol >= g.m) return;
  const int i = g.fund[a], j = g.fund[bcol];
  const size_t off = (size_t)a + (size_t)bcol * (size_t)ld;
  const double xi = g.x[i], yi = g.y[i];
  const bool diag = (i == j);
  bool fp64 = false;
  dfl nA{0.f, 0.f}, nB{0.f, 0.f}, th{0.f, 0.f}, tj{0.f, 0.f}, dc{0.f, 0.f};
  int ph = 0, pj = 0;
  if (diag) {
    dc = df_of(1.0 - g.ws[i] * g.kappa[i]);
  } else {
    const PairGeom p = pair_geom(g, i, j);
    const Fold f = fold_of<0>(p);
    nA = df_of(-f.A);
    nB = df_of(-f.B);
    double thd = 0.0, tjd = 0.0;
    panel_of(p.r, t.rmin, t.rmax, t.dr_h, t.invdr_h, t.nh, ph, thd);
    panel_of(p.r, 0.0, t.rmax, t.dr_j, t.invdr_j, t.nj, pj, tjd);
    th = df_of(thd);
    tj = df_of(tjd);
    fp64 |= p.r < t.rmin;
  }
  // image slots filled through compile-time indices (registers, not local memory)
  int nim = 0;
  int iph[MAXIMG];
  dfl ith[MAXIMG], ere[MAXIMG], eim[MAXIMG];
#pragma unroll
  for (int sl = 0; sl < MAXIMG; ++sl) {
    iph[sl] = 0;
    ith[sl] = dfl{0.f, 0.f};
    ere[sl] = dfl{0.f, 0.f};
    eim[sl] = dfl{0.f, 0.f};
  }
  if (g.norb > MAXIMG + 1) fp64 = true;
#pragma unroll
  for (int l = 0; l < MAXIMG + 1; ++l) {
    if (l >= g.norb) break;
    const int qn = g.orb[bcol * g.norb + l];
    if (qn == j) continue;
    const double dxq = xi - g.x[qn], dyq = yi - g.y[qn];
    const double r = hypot(dxq, dyq);
    if (r < 2.220446049250313e-16) continue;
    if (r < t.rmin) {
      fp64 = true;
      continue;
    }
    const double c = (g.nx[qn] * dxq + g.ny[qn] * dyq) / r;
    const double e = c * g.speed[qn] * g.ws[qn];
    const double scr = g.orb_scale[2 * (bcol * g.norb + l)], sci = g.orb_scale[2 * (bcol * g.norb + l) + 1];
    int php = 0;
    double thd = 0.0;
    panel_of(r, t.rmin, t.rmax, t.dr_h, t.invdr_h, t.nh, php, thd);
#pragma unroll
    for (int sl = 0; sl < MAXIMG; ++sl)
      if (sl == nim) {
        iph[sl] = php;
        ith[sl] = df_of(thd);
        ere[sl] = df_of(-e * scr);  // F -= (e sc) H1': accumulate (-e sc) H1'
        eim[sl] = df_of(-e * sci);
      }
    if (nim < MAXIMG) ++nim;
    else fp64 = true;
  }
  for (int q = 0; q < nk; ++q) {
    float4 v;
    if (fp64) {
      const cxd k = ks[q];
      cxd F;
      if (diag) {
        F = cxd(1.0 - g.ws[i] * g.kappa[i], 0.0);
      } else {
        const PairGeom p = pair_geom(g, i, j);
        int pjj = 0;
        double tjd = 0.0;
        panel_of(p.r, 0.0, t.rmax, t.dr_j, t.invdr_j, t.nj, pjj, tjd);
        cxd h0, h1, j0, j1, F1, F2;
        cheb_h01(t, q, p.r, k, h0, h1);
        clenshaw2(t.J + (((size_t)q * t.nj + pjj) * (t.Mj + 1)) * 2, t.Mj, tjd, j0, j1);
        entry_vals<0, 0>(p, k, h0, h1, j0, j1, &F, &F1, &F2);
      }
      for (int l = 0; l < g.norb; ++l) {
        const int qn = g.orb[bcol * g.norb + l];
        if (qn == j) continue;
        const double dxq = xi - g.x[qn], dyq = yi - g.y[qn];
        const double r = hypot(dxq, dyq);
        if (r < 2.220446049250313e-16) continue;
        const double c = (g.nx[qn] * dxq + g.ny[qn] * dyq) / r;
        const cxd sc(g.orb_scale[2 * (bcol * g.norb + l)], g.orb_scale[2 * (bcol * g.norb + l) + 1]);
        cxd h0, h1, F1, F2;
        cheb_h01(t, q, r, k, h0, h1);
        image_terms<0>(c, g.speed[qn] * g.ws[qn], sc, r, k, h0, h1, F, F1, F2);
      }
      v = pack_split(F);
    } else {
      dfl re = dc, im{0.f, 0.f};
      dfl hr, hi_, jr, ji;
      if (!diag) {
        df_series_d<false, DM>(t.HD + ((size_t)q * t.nh + ph) * (t.Mh + 1) * 2, t.Mh, th, nullptr, nullptr, &hr,
                               &hi_);
        df_series_d<false, DM>(t.JD + ((size_t)q * t.nj + pj) * (t.Mj + 1) * 2, t.Mj, tj, nullptr, nullptr, &jr,
                               &ji);
        df_acc(re, nB, hr);
        df_acc(im, nB, hi_);
        df_acc(re, nA, jr);
        df_acc(im, nA, ji);
      }
#pragma unroll
      for (int l = 0; l < MAXIMG; ++l) {
        if (l >= nim) break;
        df_series_d<false, DM>(t.HD + ((size_t)q * t.nh + iph[l]) * (t.Mh + 1) * 2, t.Mh, ith[l], nullptr, nullptr,
                               &hr, &hi_);
        // (ere + i eim)(hr + i hi_)
        df_acc(re, ere[l], hr);
        df_acc(re, dfl{-eim[l].hi, -eim[l].lo}, hi_);
        df_acc(im, ere[l], hi_);
        df_acc(im, eim[l], hr);
      }
      re = df_norm(re);
      im = df_norm(im);
      v = make_float4(re.hi, im.hi, re.lo, im.lo);
    }
    reinterpret_cast<cxf*>(outs[q])[off] = cxf(v.x, v.y);
    if (los) reinterpret_cast<cxf*>(los[q])[off] = cxf(v.z, v.w);
  }
}

bool cheb_je_applies(const GeomDev& g, int deriv, int prec) {
  return prec == QBG_PREC_MIXED && !deriv && g.m == g.n && g.quad != 1;
}

size_t cheb_je_bytes(const ChebTables& t) {
  return sizeof(float4) * (size_t)t.nse * t.nk * t.nje * (size_t)(t.Mje + 1) + sizeof(int) * (size_t)t.nje;
}

int cheb_je_build(ChebTables& t, const cxd* ks, cudaStream_t st) {
  if (!t.JE || t.nje < 1 || t.nje >= (1 << 21) || t.Mje < 1 || t.Mje > QBG_CHEB_MAX_DEGREE ||
      (t.nse != 2 && t.nse != 4)) {
    set_error("cheb_je_build: invalid table parameters");
    return QBG_EINVAL;
  }
  t.JEm = reinterpret_cast<int*>(t.JE + (size_t)t.nse * t.nk * t.nje * (size_t)(t.Mje + 1));
  QBG_CUDA(cudaMemsetAsync(t.JEm, 0, sizeof(int) * (size_t)t.nje, st));
  const int ppb = JE_BUILD_THREADS / (t.Mje + 1);
  dim3 grd((t.nje + ppb - 1) / ppb, t.nk);
  if (t.nse == 4) k_cheb_build_je<4><<<grd, JE_BUILD_THREADS, 0, st>>>(t, ks);
  else k_cheb_build_je<2><<<grd, JE_BUILD_THREADS, 0, st>>>(t, ks);
  QBG_LAUNCH_CHECK("k_cheb_build_je");
  return QBG_OK;
}

bool cheb_df_applies(const GeomDev& g, int deriv) {
  // full operators take the J/E tables (cheb_je_applies)
  return !deriv && g.m != g.n && g.form == 0 && g.norb <= 4;
}

void cheb_df_bytes(const ChebTables& t, size_t* hd, size_t* jd, size_t* nkc) {
  *hd = sizeof(float4) * 2 * (size_t)t.nk * t.nh * (t.Mh + 1);
  *jd = sizeof(float4) * 2 * (size_t)t.nk * t.nj * (t.Mj + 1);
  *nkc = sizeof(NodeConst) * (size_t)t.nk;
}

int cheb_df_tables(ChebTables& t, const cxd* ks, cudaStream_t st) {
  if (!t.HD || !t.JD || !t.nkc) {
    set_error("cheb_df_tables: buffers not set");
    return QBG_EINVAL;
  }
  k_node_consts<<<(t.nk + 127) / 128, 128, 0, st>>>(ks, t.nk, t.nkc);
  QBG_LAUNCH_CHECK("k_node_consts");
  const long long rows = std::max((long long)t.nh * (t.Mh + 1), (long long)t.nj * (t.Mj + 1));
  dim3 grd((unsigned)((rows + 255) / 256), t.nk, 2);
  k_cheb_df_tables<<<grd, 256, 0, st>>>(t);
  QBG_LAUNCH_CHECK("k_cheb_df_tables");
  return QBG_OK;
}

int cheb_r_range(const GeomDev& g, unsigned long long* dscratch2, double* rmin, double* rmax, cudaStream_t st) {
  unsigned long long init[2] = {0ull, 0ull};
  const double big = 1e300;
  memcpy(&init[0], &big, sizeof(double));
  QBG_CUDA(cudaMemcpyAsync(dscratch2, init, sizeof(init), cudaMemcpyHostToDevice, st));
  dim3 blk(32, 8), grd((g.n + 31) / 32, (g.n + 7) / 8);
  k_pair_rminmax<<<grd, blk, 0, st>>>(g, dscratch2);
  QBG_LAUNCH_CHECK("k_pair_rminmax");
  unsigned long long res[2];
  QBG_CUDA(cudaMemcpyAsync(res, dscratch2, sizeof(res), cudaMemcpyDeviceToHost, st));
  QBG_CUDA(cudaStreamSynchronize(st));
  double lo, hi;
  memcpy(&lo, &res[0], sizeof(double));
  memcpy(&hi, &res[1], sizeof(double));
  *rmin = lo;
  *rmax = hi;
  return QBG_OK;
}

// Panel error check of the autotuner (chebyshev_optimal_panelization.jl:221-307):
// max |interpolated - direct| of H0, H1 at ns radii uniform on [t.rmin, t.rmax]
// and of J0, J1 at ns radii uniform on [0, t.rmax], per wavenumber;
// err[4 q + f] (f = H0, H1, J0, J1) holds the bits of non-negative doubles.
__global__ void k_cheb_errors(ChebTables t, const cxd* __restrict__ ks, int ns, unsigned long long* err) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  const int q = blockIdx.y;
  const cxd k = ks[q];
  const bool realk = (k.im == 0.0);
  double e[4] = {0.0, 0.0, 0.0, 0.0};
  if (s < ns) {
    const double u = ns > 1 ? (double)s / (double)(ns - 1) : 0.0;
    const double rh = t.rmin + (t.rmax - t.rmin) * u;
    int p;
    double tt;
    cxd v0, v1;
    panel_of(rh, t.rmin, t.rmax, t.dr_h, t.invdr_h, t.nh, p, tt);
    clenshaw2(t.H + (((size_t)q * t.nh + p) * (t.Mh + 1)) * 2, t.Mh, tt, v0, v1);
    const Bessel01d bh = bessel01(rh * k);
    e[0] = cabs_d(v0 - bh.h0());
    e[1] = cabs_d(v1 - bh.h1());
    const double rj = t.rmax * u;
    panel_of(rj, 0.0, t.rmax, t.dr_j, t.invdr_j, t.nj, p, tt);
    clenshaw2(t.J + (((size_t)q * t.nj + p) * (t.Mj + 1)) * 2, t.Mj, tt, v0, v1);
    cxd j0(1.0, 0.0), j1(0.0, 0.0);
    if (rj > 0.0) {
      Bessel01d bj = bessel01(rj * k);
      if (realk) { bj.j0.im = 0.0; bj.j1.im = 0.0; }
      j0 = bj.j0;
      j1 = bj.j1;
    }
    e[2] = cabs_d(v0 - j0);
    e[3] = cabs_d(v1 - j1);
  }
#pragma unroll
  for (int f = 0; f < 4; ++f) {
    double m = e[f];
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(&err[4 * q + f], (unsigned long long)__double_as_longlong(m));
  }
}

int cheb_errors(const ChebTables& t, const cxd* ks, int ns, unsigned long long* err, cudaStream_t st) {
  dim3 grd((ns + 255) / 256, t.nk);
  k_cheb_errors<<<grd, 256, 0, st>>>(t, ks, ns, err);
  QBG_LAUNCH_CHECK("k_cheb_errors");
  return QBG_OK;
}

int cheb_build(ChebTables& t, const cxd* ks, cudaStream_t st) {
  const int npmax = t.nh > t.nj ? t.nh : t.nj;
  dim3 grd((npmax + 127) / 128, t.nk, 2);
  k_cheb_build<<<grd, 128, 0, st>>>(t, ks);
  QBG_LAUNCH_CHECK("k_cheb_build");
  return QBG_OK;
}

// blocks per SM of k_assemble_je_df: 2 (64 registers, 2 x 112 KB of shared
// memory for the CFIE; default) or 1 (128 registers, QBG_JE_OCC=1). On C2 the
// assembly phase took 8.2 ms at 2 and 9.2 ms at 1.
static int je_occupancy() {
  static const int occ = [] {
    const char* e = getenv("QBG_JE_OCC");
    return (e && atoi(e) == 1) ? 1 : 2;
  }();
  return occ;
}

template <int FORM>
static int launch_je_df(const GeomDev& g, const ChebTables& t, const cxd* ks, int nk, void* const* outs,
                        void* const* los, long long ld, dim3 grd, dim3 blk, cudaStream_t st) {
  const size_t dyn = sizeof(float4) * (2048 + 1024 * (size_t)je_coef_words<FORM>());
  if (je_occupancy() == 2) {
    QBG_CUDA(cudaFuncSetAttribute(k_assemble_je_df<FORM, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn));
    QBG_CUDA(cudaFuncSetAttribute(k_assemble_je_df<FORM, 2>, cudaFuncAttributePreferredSharedMemoryCarveout,
                                  (int)cudaSharedmemCarveoutMaxShared));
    k_assemble_je_df<FORM, 2><<<grd, blk, dyn, st>>>(g, t, ks, nk, outs, los, ld);
  } else {
    QBG_CUDA(cudaFuncSetAttribute(k_assemble_je_df<FORM, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn));
    k_assemble_je_df<FORM, 1><<<grd, blk, dyn, st>>>(g, t, ks, nk, outs, los, ld);
  }
  return QBG_OK;
}

int launch_assemble_cheb(const GeomDev& g, const ChebTables& t, const cxd* ks, int nk, int deriv, int prec,
                         void* const* outs_dev, void* const* lo_outs_dev, long long ld, cudaStream_t st) {
  if (g.quad == 1) return launch_alpert(g, &t, ks, nk, deriv, prec, outs_dev, ld, st, lo_outs_dev);
  if (prec == QBG_PREC_FP32) {
    set_error("the FP32 form evaluates its kernel values directly (no Chebyshev panels)");
    return QBG_ENOTSUP;
  }
  if (deriv && prec != QBG_PREC_FP64) {
    set_error("Chebyshev derivative assembly is available in FP64");
    return QBG_ENOTSUP;
  }
  const int kchunk = 8;
  if (g.m != g.n) {
    if (g.form != 0) return launch_cfie_reduced(g, &t, ks, nk, deriv, prec, outs_dev, lo_outs_dev, ld, st);
    dim3 blk(32, 8), grd((g.m + 31) / 32, (g.m + 7) / 8, (nk + kchunk - 1) / kchunk);
    if (prec == QBG_PREC_FP64) {
      if (deriv)
        k_assemble_cheb_reduced<1, 0><<<grd, blk, 0, st>>>(g, t, ks, nk, kchunk, outs_dev, nullptr, ld);
      else
        k_assemble_cheb_reduced<0, 0><<<grd, blk, 0, st>>>(g, t, ks, nk, kchunk, outs_dev, nullptr, ld);
    } else if (t.HD && t.JD && t.nkc && g.norb <= 4) {
      dim3 dgrd((g.m + 31) / 32, (g.m + 7) / 8, 1);
      const int dm = (t.Mh == t.Mj) ? t.Mh : 0;
#define QBG_RED_DF(D) k_assemble_cheb_reduced_df<3, D><<<dgrd, blk, 0, st>>>(g, t, ks, nk, outs_dev, lo_outs_dev, ld)
      switch (dm) {
        case 5: QBG_RED_DF(5); break;
        case 7: QBG_RED_DF(7); break;
        case 9: QBG_RED_DF(9); break;
        case 11: QBG_RED_DF(11); break;
        case 13: QBG_RED_DF(13); break;
        default: QBG_RED_DF(0); break;
      }
#undef QBG_RED_DF
    } else {
      k_assemble_cheb_reduced<0, 1><<<grd, blk, 0, st>>>(g, t, ks, nk, kchunk, outs_dev, lo_outs_dev, ld);
    }
    QBG_LAUNCH_CHECK("k_assemble_cheb_reduced");
    return QBG_OK;
  }
  if (!deriv) {
    const int nt = (g.n + 31) / 32;
    dim3 sblk(32, 16), sgrd((unsigned)(nt * (nt + 1) / 2), 1, (nk + kchunk - 1) / kchunk);
    if (prec == QBG_PREC_FP64) {
      if (g.form == 0)
        k_assemble_cheb_sym<0, 0><<<sgrd, sblk, 0, st>>>(g, t, ks, nk, kchunk, outs_dev, nullptr, ld);
      else
        k_assemble_cheb_sym<1, 0><<<sgrd, sblk, 0, st>>>(g, t, ks, nk, kchunk, outs_dev, nullptr, ld);
    } else if (t.JE && prec == QBG_PREC_MIXED) {
      dim3 dgrd((unsigned)(nt * (nt + 1) / 2), 1, 1);
      if (g.form == 0) QBG_TRY(launch_je_df<0>(g, t, ks, nk, outs_dev, lo_outs_dev, ld, dgrd, sblk, st));
      else QBG_TRY(launch_je_df<1>(g, t, ks, nk, outs_dev, lo_outs_dev, ld, dgrd, sblk, st));
    } else {
      if (g.form == 0)
        k_assemble_cheb_sym<0, 1><<<sgrd, sblk, 0, st>>>(g, t, ks, nk, kchunk, outs_dev, lo_outs_dev, ld);
      else
        k_assemble_cheb_sym<1, 1><<<sgrd, sblk, 0, st>>>(g, t, ks, nk, kchunk, outs_dev, lo_outs_dev, ld);
    }
    QBG_LAUNCH_CHECK("k_assemble_cheb_sym");
    return QBG_OK;
  }
  dim3 blk(32, 8), grd((g.n + 31) / 32, (g.n + 7) / 8, (nk + kchunk - 1) / kchunk);
  if (prec == QBG_PREC_FP64) {
    if (g.form == 0) {
      if (deriv)
        k_assemble_cheb<0, 1, 0><<<grd, blk, 0, st>>>(g, t, ks, nk, kchunk, outs_dev, nullptr, ld);
      else
        k_assemble_cheb<0, 0, 0><<<grd, blk, 0, st>>>(g, t, ks, nk, kchunk, outs_dev, nullptr, ld);
    } else {
      if (deriv)
        k_assemble_cheb<1, 1, 0><<<grd, blk, 0, st>>>(g, t, ks, nk, kchunk, outs_dev, nullptr, ld);
      else
        k_assemble_cheb<1, 0, 0><<<grd, blk, 0, st>>>(g, t, ks, nk, kchunk, outs_dev, nullptr, ld);
    }
  } else {
    if (g.form == 0)
      k_assemble_cheb<0, 0, 1><<<grd, blk, 0, st>>>(g, t, ks, nk, kchunk, outs_dev, lo_outs_dev, ld);
    else
      k_assemble_cheb<1, 0, 1><<<grd, blk, 0, st>>>(g, t, ks, nk, kchunk, outs_dev, lo_outs_dev, ld);
  }
  QBG_LAUNCH_CHECK("k_assemble_cheb");
  return QBG_OK;
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
  if (g.quad == 1) return launch_alpert(g, nullptr, ks, nk, deriv, prec, outs_dev, ld, st, lo_outs_dev);
  if (reduced) {
    if (g.form != 0) return launch_cfie_reduced(g, nullptr, ks, nk, deriv, prec, outs_dev, lo_outs_dev, ld, st);
    if (deriv && prec != QBG_PREC_FP64) {
      set_error("derivative assembly is available in FP64");
      return QBG_ENOTSUP;
    }
    if (prec == QBG_PREC_FP64) {
      if (deriv)
        k_assemble_dlp_reduced<1, 0><<<grd, blk, 0, st>>>(g, ks, nk, outs_dev, nullptr, ld);
      else
        k_assemble_dlp_reduced<0, 0><<<grd, blk, 0, st>>>(g, ks, nk, outs_dev, nullptr, ld);
    } else {
      k_assemble_dlp_reduced<0, 1><<<grd, blk, 0, st>>>(g, ks, nk, outs_dev,
                                                         prec == QBG_PREC_MIXED ? lo_outs_dev : nullptr, ld);
    }
    QBG_LAUNCH_CHECK("k_assemble_dlp_reduced");
    return QBG_OK;
  }
  if (prec == QBG_PREC_FP64) {
    if (g.form == 0) {
      if (deriv)
        k_assemble_fp64<0, 1><<<grd, blk, 0, st>>>(g, ks, nk, (cxd* const*)outs_dev, ld);
      else
        k_assemble_fp64<0, 0><<<grd, blk, 0, st>>>(g, ks, nk, (cxd* const*)outs_dev, ld);
    } else {
      if (deriv)
        k_assemble_fp64<1, 1><<<grd, blk, 0, st>>>(g, ks, nk, (cxd* const*)outs_dev, ld);
      else
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
