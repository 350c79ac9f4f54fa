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

// Chebyshev panel tables for nk wavenumbers (layout [k][panel][m][2], the pair
// (H0, H1) on [rmin, rmax] in H and (J0, J1) on [0, rmax] in J).
#define QBG_CHEB_MAX_DEGREE 16
// per-wavenumber factors of the folded kernel entry (k_assemble_cheb_sym):
// the J1, H1, J0, H0 terms carry kaL1 = -k/2pi, kaL2 = ik/2, kg = -ik/2pi, kd = -k/2
struct NodeConst {
  cxd kaL1, kaL2, kg, kd;
  double ak;  // |k|
};
struct ChebTables {
  int nk = 0, nh = 0, Mh = 0, nj = 0, Mj = 0;
  double rmin = 0, rmax = 0, dr_h = 0, invdr_h = 0, dr_j = 0, invdr_j = 0;
  double small_cut = 0.2;  // |k r| below which Hankel values are evaluated directly
  cxd* H = nullptr;
  cxd* J = nullptr;
  // double-float copies of the coefficients, each series premultiplied by its
  // node factor: per (node, panel, degree) two float4 (re.hi, re.lo, im.hi, im.lo)
  // = {kd H0, kaL2 H1} and {kg J0, kaL1 J1}; built by cheb_df_tables
  float4* HD = nullptr;
  float4* JD = nullptr;
  NodeConst* nkc = nullptr;
  // J/E form for the double-float assembly of full operators (k_cheb_build_je):
  // on nje uniform panels of [0, rmax], degree Mje, per (node, panel, degree)
  // nse float4 (re.hi, re.lo, im.hi, im.lo) = {P, U, R, W} (DLP: {P, U}) with
  //   P = kaL2 J1,  U = kaL2 (J1 + i G1),  R = kd J0,  W = kd (J0 + i G0),
  //   G0 = Y0 - l J0,  G1 = Y1 - l J1 + 2/(pi k r),  l = (2/pi) ln r,
  // all entire in r, so that kaL2 H1 = U + i l P + 1/(pi r), kd H0 = W + i l R,
  // kaL1 J1 = (i/pi) P and kg J0 = (i/pi) R
  float4* JE = nullptr;
  // per panel: the first degree whose terms, and all higher ones, sum to at
  // most 2^-26 of the row's coefficient magnitudes in every series and at
  // every node; the assembly adds those terms in FP32 (stored after the
  // coefficients in JE)
  int* JEm = nullptr;
  int nje = 0, Mje = 0, nse = 0;
  double dr_je = 0, invdr_je = 0;
};
// min / max pair distance over all off-diagonal pairs (host values; dscratch2 = 2 device words)
int cheb_r_range(const GeomDev& g, unsigned long long* dscratch2, double* rmin, double* rmax, cudaStream_t st);
int cheb_build(ChebTables& t, const cxd* ks, cudaStream_t st);
// double-float tables for the complex64 forms (HD, JD, nkc: device buffers of the
// sizes cheb_df_bytes reports, owned by the caller); after cheb_build
void cheb_df_bytes(const ChebTables& t, size_t* hd, size_t* jd, size_t* nkc);
int cheb_df_tables(ChebTables& t, const cxd* ks, cudaStream_t st);
// the J/E tables of the mixed form's full symmetric assembly: whether they
// apply, their bytes (t.nk, nje, Mje, nse set), and their build (t.JE set)
bool cheb_je_applies(const GeomDev& g, int deriv, int prec);
size_t cheb_je_bytes(const ChebTables& t);
int cheb_je_build(ChebTables& t, const cxd* ks, cudaStream_t st);
// whether the complex64 Chebyshev assembly of g runs on double-float tables
// (symmetric full operators; the reduced DLP with orbits of at most 4 nodes)
bool cheb_df_applies(const GeomDev& g, int deriv);
// max interpolation errors of H0, H1, J0, J1 per wavenumber at ns sampled radii (err: 4 nk zeroed words)
int cheb_errors(const ChebTables& t, const cxd* ks, int ns, unsigned long long* err, cudaStream_t st);
int launch_assemble_cheb(const GeomDev& g, const ChebTables& t, const cxd* ks, int nk, int deriv, int prec,
                         void* const* outs_dev, void* const* lo_outs_dev, long long ld, cudaStream_t st);
int launch_bessel_eval(const cxd* z, int n, cxd* out, int f32, cudaStream_t st);
}  // namespace qbg
