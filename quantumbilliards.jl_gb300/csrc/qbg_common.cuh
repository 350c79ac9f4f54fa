// Shared device/host helpers for libqbgpu: a small complex type templated on
// the real type (double for the plain FP64 form, float for the mixed form),
// status plumbing and launch checks.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <cmath>

#define QBG_HD __host__ __device__ __forceinline__

template <class T>
struct cx {
  T re, im;
  cx() = default;  // trivial, so cx<T> may live in __shared__ arrays
  QBG_HD cx(T r) : re(r), im(0) {}
  QBG_HD cx(T r, T i) : re(r), im(i) {}
  template <class U>
  QBG_HD explicit cx(const cx<U>& o) : re((T)o.re), im((T)o.im) {}
};

template <class T> QBG_HD cx<T> operator+(cx<T> a, cx<T> b) { return {a.re + b.re, a.im + b.im}; }
template <class T> QBG_HD cx<T> operator-(cx<T> a, cx<T> b) { return {a.re - b.re, a.im - b.im}; }
template <class T> QBG_HD cx<T> operator-(cx<T> a) { return {-a.re, -a.im}; }
template <class T> QBG_HD cx<T> operator*(cx<T> a, cx<T> b) {
  return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
}
template <class T> QBG_HD cx<T> operator*(T s, cx<T> a) { return {s * a.re, s * a.im}; }
template <class T> QBG_HD cx<T> operator*(cx<T> a, T s) { return {s * a.re, s * a.im}; }
// complex quotient by Smith's scaling (avoids overflow of |b|^2)
template <class T> QBG_HD cx<T> operator/(cx<T> a, cx<T> b) {
  if ((b.re < 0 ? -b.re : b.re) >= (b.im < 0 ? -b.im : b.im)) {
    const T r = b.im / b.re, d = b.re + b.im * r;
    return {(a.re + a.im * r) / d, (a.im - a.re * r) / d};
  }
  const T r = b.re / b.im, d = b.re * r + b.im;
  return {(a.re * r + a.im) / d, (a.im * r - a.re) / d};
}
template <class T> QBG_HD cx<T>& operator+=(cx<T>& a, cx<T> b) { a.re += b.re; a.im += b.im; return a; }
template <class T> QBG_HD cx<T>& operator-=(cx<T>& a, cx<T> b) { a.re -= b.re; a.im -= b.im; return a; }
template <class T> QBG_HD cx<T> cmul_i(cx<T> a) { return {-a.im, a.re}; }          // i*a
template <class T> QBG_HD T cabs2(cx<T> a) { return a.re * a.re + a.im * a.im; }
template <class T> QBG_HD T cabs1(cx<T> a) { return fabs(a.re) + fabs(a.im); }  // LAPACK izamax measure
QBG_HD double cabs_d(cx<double> a) { return hypot(a.re, a.im); }
template <class T> QBG_HD cx<T> conj(cx<T> a) { return {a.re, -a.im}; }
template <class T> QBG_HD cx<T> cinv(cx<T> a) {
  // 1/a with Smith's scaling to avoid overflow in |a|^2
  if (fabs(a.re) >= fabs(a.im)) {
    T r = a.im / a.re, d = a.re + a.im * r;
    return {T(1) / d, -r / d};
  } else {
    T r = a.re / a.im, d = a.im + a.re * r;
    return {r / d, T(-1) / d};
  }
}
template <class T> QBG_HD cx<T> cdiv(cx<T> a, cx<T> b) { return a * cinv(b); }
// a += b*c  (4 real FMAs)
template <class T> QBG_HD void cfma(cx<T>& a, cx<T> b, cx<T> c) {
  a.re = fma(b.re, c.re, a.re);
  a.re = fma(-b.im, c.im, a.re);
  a.im = fma(b.re, c.im, a.im);
  a.im = fma(b.im, c.re, a.im);
}
// a -= b*c
template <class T> QBG_HD void cfms(cx<T>& a, cx<T> b, cx<T> c) {
  a.re = fma(-b.re, c.re, a.re);
  a.re = fma(b.im, c.im, a.re);
  a.im = fma(-b.re, c.im, a.im);
  a.im = fma(-b.im, c.re, a.im);
}

typedef cx<double> cxd;
typedef cx<float> cxf;

// Status codes come from the public header.
#include "qbgpu.h"

namespace qbg {
void set_error(const char* fmt, ...);
void note_launch();
int cuda_status(cudaError_t e, const char* what);

// Streams of the library: request work (assembly, Beyn, QR) one step above
// the device's least priority, background sweeps at the least, so that the
// block scheduler dispatches a latency-bound request's blocks ahead of a
// sweep's FP64 factorisations. Streams at higher priorities stay above both.
inline cudaError_t stream_create(cudaStream_t* st, bool background = false) {
  int least = 0, greatest = 0;
  cudaError_t e = cudaDeviceGetStreamPriorityRange(&least, &greatest);
  if (e != cudaSuccess) return e;
  const int prio = background ? least : (greatest < least ? least - 1 : least);
  return cudaStreamCreateWithPriority(st, cudaStreamNonBlocking, prio);
}
}  // namespace qbg

#define QBG_CUDA(call)                                          \
  do {                                                          \
    cudaError_t _e = (call);                                    \
    if (_e != cudaSuccess) return qbg::cuda_status(_e, #call);  \
  } while (0)

#define QBG_TRY(x)          \
  do {                      \
    int _s = (x);           \
    if (_s) return _s;      \
  } while (0)

// Every kernel launch of the library is followed by exactly one
// QBG_LAUNCH_CHECK, which also counts it (qbg_launch_count).
#define QBG_LAUNCH_CHECK(what)                                              \
  do {                                                                      \
    qbg::note_launch();                                                     \
    cudaError_t _e = cudaGetLastError();                                    \
    if (_e != cudaSuccess) return qbg::cuda_status(_e, what);               \
  } while (0)
