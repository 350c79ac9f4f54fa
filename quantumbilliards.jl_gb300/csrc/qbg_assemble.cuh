#pragma once
#include "qbg_common.cuh"
#include "qbg_geom.cuh"

namespace qbg {
// prec: QBG_PREC_FP64 (complex128 outputs), QBG_PREC_MIXED (FP64 values split into complex64 hi in
// outs_dev and complex64 lo in lo_outs_dev when non-null), QBG_PREC_FP32 (FP32 values, complex64)
// outs_dev: device array of nk*(1+2*deriv) device pointers, each an ld x dim column-major matrix
int launch_assemble(const GeomDev& g, const cxd* ks, int nk, int deriv, int prec, void* const* outs_dev,
                    long long ld, cudaStream_t st, void* const* lo_outs_dev = nullptr);
int launch_kress_column(double* out, int N, cudaStream_t st);
int launch_bessel_eval(const cxd* z, int n, cxd* out, int f32, cudaStream_t st);
}  // namespace qbg
