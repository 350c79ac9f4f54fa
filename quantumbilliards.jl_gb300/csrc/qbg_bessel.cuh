// Device Bessel/Hankel functions of order 0 and 1 for complex argument.
//
// The reference evaluates H0^(1), H1^(1), J0, J1 with Bessels.jl (real
// argument) or AMOS through SpecialFunctions.jl (complex argument),
// src/utils/special_functions_calls.jl:3-7. AMOS is not restated here; these
// routines are written from the published mathematics:
//
//  * |z| < 14.5: Miller's backward recurrence for J_n(z) (Abramowitz & Stegun
//    9.1.27 recurrence run downward from n0 ~ |z| + 26), normalised with the
//    generating-function identity exp(-/+ i z) = J0 + 2 sum_{n>=1} (-/+ i)^n J_n
//    (sign chosen so that no cancellation occurs for Im z != 0), and the
//    Neumann series (A&S 9.1.88 for Y0; its derivative for Y1):
//        Y0 = (2/pi) [ (log(z/2)+gamma) J0 - 2 sum_{k>=1} (-1)^k J_{2k}/k ]
//        Y1 = (2/pi) [ (log(z/2)+gamma) J1 - J0/z - J1
//                      + sum_{m>=1} (-1)^{m+1} (2m+1)/(m(m+1)) J_{2m+1} ]
//  * |z| >= 14.5: Hankel's asymptotic expansion (A&S 9.2.5-9.2.10,
//    DLMF 10.17.1-10.17.4), summed until the terms stop decreasing:
//        J_nu = sqrt(2/(pi z)) (P cos w - Q sin w),
//        Y_nu = sqrt(2/(pi z)) (P sin w + Q cos w),   w = z - nu pi/2 - pi/4,
//        a_k(nu) = a_{k-1}(nu) (4 nu^2 - (2k-1)^2) / (8k).
//
// Accuracy (checked against mpmath in tests/test_gpu_bessel.py): max error
// relative to max(|J|,|Y|) below 1e-14 for Re z > 0, |Im z| <= 3.
//
// The FP32 variant used by the mixed form takes z in FP64, reduces Re z modulo
// 2*pi in FP64 (k*r reaches several thousand radians) and evaluates the
// asymptotic series in FP32; callers use it only for |z| >= 12, where the
// FP32-truncated series is accurate to FP32 rounding.
#pragma once
#include "qbg_common.cuh"

namespace qbg {

struct Bessel01d {
  cxd j0, j1, y0, y1;
  __device__ __forceinline__ cxd h0() const { return j0 + cmul_i(y0); }
  __device__ __forceinline__ cxd h1() const { return j1 + cmul_i(y1); }
};

__device__ __forceinline__ cxd cexp_d(cxd z) {
  double e = exp(z.re), s, c;
  sincos(z.im, &s, &c);
  return {e * c, e * s};
}

__device__ __forceinline__ cxd clog_d(cxd z) { return {log(hypot(z.re, z.im)), atan2(z.im, z.re)}; }

__device__ __forceinline__ cxd csqrt_d(cxd z) {
  double m = hypot(z.re, z.im);
  if (m == 0.0) return {0.0, 0.0};
  double t = sqrt(0.5 * (m + fabs(z.re)));
  if (z.re >= 0.0) return {t, 0.5 * z.im / t};
  return {0.5 * fabs(z.im) / t, copysign(t, z.im)};
}

__device__ __noinline__ Bessel01d bessel01_miller(cxd z) {
  const double az = hypot(z.re, z.im);
  const int n0 = 2 * (int)((az + 26.0) * 0.5);
  const cxd iz = cinv(z);
  const bool upper = z.im >= 0.0;  // normalise with exp(-iz) (upper) or exp(+iz)
  cxd fp1(0.0, 0.0), f(1e-30, 0.0);
  cxd snorm(0.0, 0.0), sy0(0.0, 0.0), sy1(0.0, 0.0);
  for (int n = n0; n >= 1; --n) {
    // (-i)^n for upper, (+i)^n for lower, n mod 4
    cxd fn2 = 2.0 * f;
    switch (n & 3) {
      case 0: snorm += fn2; break;
      case 1: snorm += upper ? cxd(fn2.im, -fn2.re) : cxd(-fn2.im, fn2.re); break;
      case 2: snorm -= fn2; break;
      default: snorm += upper ? cxd(-fn2.im, fn2.re) : cxd(fn2.im, -fn2.re); break;
    }
    if ((n & 1) == 0) {
      int k = n >> 1;
      double c = ((k & 1) ? -1.0 : 1.0) / (double)k;
      sy0 += c * f;
    } else {
      int m = (n - 1) >> 1;
      if (m >= 1) {
        double c = ((m & 1) ? 1.0 : -1.0) * (double)(2 * m + 1) / ((double)m * (double)(m + 1));
        sy1 += c * f;
      }
    }
    cxd fm1 = (2.0 * (double)n) * (iz * f) - fp1;
    fp1 = f;
    f = fm1;
    if (fabs(f.re) + fabs(f.im) > 1e200) {
      f = 1e-200 * f; fp1 = 1e-200 * fp1;
      snorm = 1e-200 * snorm; sy0 = 1e-200 * sy0; sy1 = 1e-200 * sy1;
    }
  }
  cxd f0 = f, f1 = fp1;
  cxd e = upper ? cexp_d(cxd(z.im, -z.re)) : cexp_d(cxd(-z.im, z.re));  // exp(-iz) or exp(iz)
  cxd sc = e * cinv(f0 + snorm);
  Bessel01d r;
  r.j0 = f0 * sc;
  r.j1 = f1 * sc;
  sy0 = sy0 * sc;
  sy1 = sy1 * sc;
  const double twopi_inv = 0.63661977236758134308;  // 2/pi
  cxd L = clog_d(0.5 * z) + cxd(0.57721566490153286061, 0.0);
  r.y0 = twopi_inv * (L * r.j0 - 2.0 * sy0);
  r.y1 = twopi_inv * (L * r.j1 - r.j0 * iz - r.j1 + sy1);
  return r;
}

__device__ __noinline__ Bessel01d bessel01_asym(cxd z) {
  const cxd w = cinv(z);
  const double aw = hypot(w.re, w.im);
  cxd wk(1.0, 0.0);
  double rk = 1.0, a0 = 1.0, a1 = 1.0, prev = 1e300;
  cxd P0(0, 0), Q0(0, 0), P1(0, 0), Q1(0, 0);
  for (int k = 0; k < 64; ++k) {
    double t = fmax(fabs(a0), fabs(a1)) * rk;
    if (t > prev) break;
    double sg = ((k >> 1) & 1) ? -1.0 : 1.0;
    if ((k & 1) == 0) { P0 += (sg * a0) * wk; P1 += (sg * a1) * wk; }
    else              { Q0 += (sg * a0) * wk; Q1 += (sg * a1) * wk; }
    if (t < 1e-17) break;
    prev = t;
    wk = wk * w;
    rk *= aw;
    double m = (double)(2 * k + 1);
    double d = 8.0 * (double)(k + 1);
    a0 *= (-m * m) / d;
    a1 *= (4.0 - m * m) / d;
  }
  // sqrt(2/(pi z))
  cxd pref = 0.79788456080286535588 * cinv(csqrt_d(z));
  double s, c;
  sincos(z.re, &s, &c);
  const double r2 = 0.70710678118654752440;
  double ca = (c + s) * r2, sa = (s - c) * r2;  // cos, sin of (Re z - pi/4)
  double ch = cosh(z.im), sh = sinh(z.im);
  cxd cw(ca * ch, -sa * sh), sw(sa * ch, ca * sh);  // cos w0, sin w0 (complex)
  Bessel01d r;
  r.j0 = pref * (P0 * cw - Q0 * sw);
  r.y0 = pref * (P0 * sw + Q0 * cw);
  // nu = 1: w1 = w0 - pi/2, cos w1 = sin w0, sin w1 = -cos w0
  r.j1 = pref * (P1 * sw + Q1 * cw);
  r.y1 = pref * (Q1 * sw - P1 * cw);
  return r;
}

__device__ __forceinline__ Bessel01d bessel01(cxd z) {
  return (hypot(z.re, z.im) < 14.5) ? bessel01_miller(z) : bessel01_asym(z);
}

// ---------------------------------------------------------------------------
// FP32 asymptotic evaluation with FP64 phase reduction (mixed form).
// ---------------------------------------------------------------------------
struct Bessel01f {
  cxf j0, j1, y0, y1;
  __device__ __forceinline__ cxf h0() const { return j0 + cmul_i(y0); }
  __device__ __forceinline__ cxf h1() const { return j1 + cmul_i(y1); }
};

__device__ __forceinline__ Bessel01f bessel01_asym_f32(cxd z64) {
  // phase: x - 2*pi*round(x/(2*pi)) in FP64 (2*pi split in two parts)
  const double x = z64.re;
  const double q = rint(x * 0.15915494309189533577);
  const double xr = fma(-q, 6.2831853071795862320, x) - q * 2.4492935982947064e-16;
  const float xf = (float)xr;
  const cxf z((float)z64.re, (float)z64.im);
  const cxf w = cinv(z);
  const float aw = sqrtf(w.re * w.re + w.im * w.im);
  cxf wk(1.f, 0.f);
  float rk = 1.f, a0 = 1.f, a1 = 1.f, prev = 1e30f;
  cxf P0(0, 0), Q0(0, 0), P1(0, 0), Q1(0, 0);
#pragma unroll 1
  for (int k = 0; k < 16; ++k) {
    float t = fmaxf(fabsf(a0), fabsf(a1)) * rk;
    if (t > prev) break;
    float sg = ((k >> 1) & 1) ? -1.f : 1.f;
    if ((k & 1) == 0) { P0 += (sg * a0) * wk; P1 += (sg * a1) * wk; }
    else              { Q0 += (sg * a0) * wk; Q1 += (sg * a1) * wk; }
    if (t < 3e-9f) break;
    prev = t;
    wk = wk * w;
    rk *= aw;
    float m = (float)(2 * k + 1);
    float d = 8.f * (float)(k + 1);
    a0 *= (-m * m) / d;
    a1 *= (4.f - m * m) / d;
  }
  // sqrt(2/(pi z)) = sqrt(2/pi) / sqrt(z)
  const float mz = sqrtf(z.re * z.re + z.im * z.im);
  float t = sqrtf(0.5f * (mz + fabsf(z.re)));
  cxf sz = (z.re >= 0.f) ? cxf(t, 0.5f * z.im / t) : cxf(0.5f * fabsf(z.im) / t, copysignf(t, z.im));
  cxf pref = 0.797884560802865f * cinv(sz);
  float s, c;
  sincosf(xf, &s, &c);
  const float r2 = 0.70710678118654752f;
  float ca = (c + s) * r2, sa = (s - c) * r2;
  float ch = coshf(z.im), sh = sinhf(z.im);
  cxf cw(ca * ch, -sa * sh), sw(sa * ch, ca * sh);
  Bessel01f r;
  r.j0 = pref * (P0 * cw - Q0 * sw);
  r.y0 = pref * (P0 * sw + Q0 * cw);
  r.j1 = pref * (P1 * sw + Q1 * cw);
  r.y1 = pref * (Q1 * sw - P1 * cw);
  return r;
}

}  // namespace qbg
