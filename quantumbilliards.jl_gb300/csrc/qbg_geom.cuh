// Device-resident boundary geometry (structure of arrays, FP64).
//
// One node per boundary point, all components concatenated in the order the
// reference uses for its global matrix (component offsets, cfie_kress.jl:212-316).
// Everything pairwise (distances, inner products, log terms, the circulant
// Kress weights) is recomputed in registers by the assembly kernels from
// these O(N) arrays instead of being stored as N x N caches
// (the reference's CFIEGeomCache, boundarypoints.jl:823-880).
#pragma once
#include "qbg_common.cuh"

namespace qbg {

struct GeomDev {
  int n = 0;        // total nodes (matrix dimension of the full operator)
  int ncomp = 0;    // boundary components
  int form = 0;     // 0 = DLP (F = I - D), 1 = CFIE (A = I - (D + ik S))
  const double* x = nullptr;
  const double* y = nullptr;
  const double* dx = nullptr;   // d gamma / d sigma
  const double* dy = nullptr;
  const double* ts = nullptr;   // computational parameter sigma (Kress log term)
  const double* ws = nullptr;   // quadrature weights
  const double* speed = nullptr;
  const double* kappa = nullptr;  // (1/2pi) * signed curvature term
  const int* comp = nullptr;      // component of each node
  const int* lidx = nullptr;      // index within its component
  const int* coff = nullptr;      // ncomp+1 component offsets
  const double* kcol = nullptr;   // per-component Kress first columns, concatenated
  // symmetry reduction (DLP image assembly, dlp_kress.jl:1151-1189)
  int m = 0;                      // reduced dimension (== n when not reduced)
  int norb = 0;                   // images per fundamental node
  const int* fund = nullptr;      // m: full index of fundamental node a
  const int* orb = nullptr;       // m*norb: images q of fundamental node b
  const double* orb_scale = nullptr;  // m*norb complex (re, im) scale factors
  const double* nx = nullptr;     // unit normals (ty, -tx)/|t| for image terms
  const double* ny = nullptr;
  // Alpert quadrature (quad == 1)
  int quad = 0;
  int aa = 0, aj = 0, ani = 0;    // near band, correction nodes per side, stencil
  const double* aw = nullptr;     // aj rule weights
  const int* aoff = nullptr;      // [2][aj][ani]
  const double* awt = nullptr;    // [2][aj][ani]
  const double* anodes = nullptr; // [6][aj][n]
};

}  // namespace qbg
