// C ABI of libqbgpu (declarations and reference citations in include/qbgpu.h).
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <vector>
#include <algorithm>
#include <atomic>

#include "qbg_assemble.cuh"
#include "qbg_handles.cuh"
#include "qbg_dense.cuh"
#include "qbg_linalg.cuh"

namespace qbg {
static thread_local std::string g_err;
static std::atomic<unsigned long long> g_launches{0};
void note_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

void set_error(const char* fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_err = buf;
}
int cuda_status(cudaError_t e, const char* what) {
  set_error("%s: %s", what, cudaGetErrorString(e));
  return (e == cudaErrorMemoryAllocation) ? QBG_ENOMEM : QBG_ECUDA;
}

}  // namespace qbg

using namespace qbg;


extern "C" {

qbg_status qbg_version(int32_t* major, int32_t* minor) {
  if (major) *major = 0;
  if (minor) *minor = 1;
  return QBG_OK;
}

size_t qbg_last_error(char* buf, size_t len) {
  const std::string& e = qbg::g_err;
  if (buf && len) {
    size_t n = std::min(len - 1, e.size());
    memcpy(buf, e.data(), n);
    buf[n] = 0;
  }
  return e.size();
}

qbg_status qbg_device_sync(void) {
  QBG_CUDA(cudaDeviceSynchronize());
  return QBG_OK;
}

qbg_status qbg_geom_create(const qbg_geom_desc* desc, qbg_geom** out) {
  if (!desc || !out) { set_error("qbg_geom_create: null argument"); return QBG_EINVAL; }
  *out = nullptr;
  if (desc->ncomp < 1 || !desc->comp_offsets || !desc->x || !desc->y || !desc->dx || !desc->dy || !desc->ddx ||
      !desc->ddy || !desc->ts || !desc->ws) {
    set_error("qbg_geom_create: missing geometry arrays");
    return QBG_EINVAL;
  }
  if (desc->form != QBG_FORM_DLP && desc->form != QBG_FORM_CFIE) {
    set_error("qbg_geom_create: unknown form %d", desc->form);
    return QBG_EINVAL;
  }
  if (desc->form == QBG_FORM_DLP && desc->ncomp != 1) {
    set_error("DLP_kress supports exactly one closed boundary component; use a CFIE form");
    return QBG_EINVAL;
  }
  const int64_t n = desc->comp_offsets[desc->ncomp];
  if (desc->comp_offsets[0] != 0 || n < 2 || n > (1ll << 30)) {
    set_error("qbg_geom_create: bad component offsets (n = %lld)", (long long)n);
    return QBG_EINVAL;
  }
  for (int c = 0; c < desc->ncomp; ++c)
    if (desc->comp_offsets[c + 1] - desc->comp_offsets[c] < 2) {
      set_error("qbg_geom_create: component %d has fewer than 2 nodes", c);
      return QBG_EINVAL;
    }
  qbg_geom* g = new (std::nothrow) qbg_geom();
  if (!g) { set_error("host allocation failed"); return QBG_ENOMEM; }
  auto fail = [&](int s) { delete g; return s; };
  cudaError_t e = stream_create(&g->stream);
  if (e != cudaSuccess) return fail(cuda_status(e, "cudaStreamCreate"));
  std::vector<double> speed(n), kappa(n), nx(n), ny(n);
  std::vector<int> comp(n), lidx(n), coff(desc->ncomp + 1);
  for (int c = 0; c <= desc->ncomp; ++c) coff[c] = (int)desc->comp_offsets[c];
  for (int c = 0; c < desc->ncomp; ++c)
    for (int64_t i = coff[c]; i < coff[c + 1]; ++i) { comp[i] = c; lidx[i] = (int)(i - coff[c]); }
  for (int64_t i = 0; i < n; ++i) {
    const double dx = desc->dx[i], dy = desc->dy[i], ddx = desc->ddx[i], ddy = desc->ddy[i];
    const double s2 = dx * dx + dy * dy;
    if (!(s2 > 0.0) || !std::isfinite(desc->x[i]) || !std::isfinite(desc->y[i])) {
      delete g;
      set_error("qbg_geom_create: degenerate or non-finite node %lld", (long long)i);
      return QBG_EINVAL;
    }
    speed[i] = std::sqrt(s2);
    kappa[i] = (1.0 / (2.0 * M_PI)) * (-(dx * ddy - dy * ddx)) / s2;  // boundarypoints.jl:876-878
    nx[i] = dy / speed[i];                                               // dlp_kress.jl:686-699
    ny[i] = -dx / speed[i];
  }
  GeomDev& d = g->d;
  d.n = (int)n;
  d.ncomp = desc->ncomp;
  d.form = desc->form;
  int s = QBG_OK;
  if ((s = g->upload(desc->x, n, &d.x)) || (s = g->upload(desc->y, n, &d.y)) || (s = g->upload(desc->dx, n, &d.dx)) ||
      (s = g->upload(desc->dy, n, &d.dy)) || (s = g->upload(desc->ts, n, &d.ts)) ||
      (s = g->upload(desc->ws, n, &d.ws)) || (s = g->upload(speed.data(), n, &d.speed)) ||
      (s = g->upload(kappa.data(), n, &d.kappa)) || (s = g->upload(comp.data(), n, &d.comp)) ||
      (s = g->upload(lidx.data(), n, &d.lidx)) || (s = g->upload(coff.data(), coff.size(), &d.coff)) ||
      (s = g->upload(nx.data(), n, &d.nx)) || (s = g->upload(ny.data(), n, &d.ny)))
    return fail(s);
  double* kcol = nullptr;
  if ((s = dmalloc(&kcol, sizeof(double) * n))) return fail(s);
  g->allocs.push_back(kcol);
  for (int c = 0; c < desc->ncomp; ++c)
    if ((s = launch_kress_column(kcol + coff[c], coff[c + 1] - coff[c], g->stream))) return fail(s);
  d.kcol = kcol;
  d.m = (int)n;
  if (desc->m > 0) {
    if ((desc->form != QBG_FORM_DLP && desc->form != QBG_FORM_CFIE) || desc->norb < 1 || !desc->fund ||
        !desc->orbit || !desc->orbit_scale || desc->m > n) {
      delete g;
      set_error("qbg_geom_create: invalid symmetry reduction arguments");
      return QBG_EINVAL;
    }
    std::vector<int> fund(desc->m), orb((size_t)desc->m * desc->norb);
    for (int64_t a = 0; a < desc->m; ++a) {
      if (desc->fund[a] < 0 || desc->fund[a] >= n) { delete g; set_error("fund index out of range"); return QBG_EINVAL; }
      fund[a] = (int)desc->fund[a];
    }
    for (size_t q = 0; q < orb.size(); ++q) {
      if (desc->orbit[q] < 0 || desc->orbit[q] >= n) { delete g; set_error("orbit index out of range"); return QBG_EINVAL; }
      orb[q] = (int)desc->orbit[q];
    }
    d.m = (int)desc->m;
    d.norb = desc->norb;
    if ((s = g->upload(fund.data(), fund.size(), &d.fund)) || (s = g->upload(orb.data(), orb.size(), &d.orb)) ||
        (s = g->upload(desc->orbit_scale, orb.size() * 2, &d.orb_scale)))
      return fail(s);
  }
  if (desc->quad == 1) {
    const int aj = desc->alpert_j, ani = desc->alpert_ninterp;
    if (desc->form != QBG_FORM_CFIE || desc->m > 0 || desc->alpert_a < 1 || aj < 1 || ani < 2 || ani > 64 ||
        !desc->alpert_w || !desc->alpert_off || !desc->alpert_wt || !desc->alpert_nodes) {
      delete g;
      set_error("qbg_geom_create: invalid Alpert arguments (CFIE only, no symmetry reduction)");
      return QBG_EINVAL;
    }
    std::vector<int> off((size_t)2 * aj * ani);
    for (size_t q = 0; q < off.size(); ++q) {
      if (std::llabs(desc->alpert_off[q]) > n) { delete g; set_error("Alpert offset out of range"); return QBG_EINVAL; }
      off[q] = (int)desc->alpert_off[q];
    }
    d.quad = 1;
    d.aa = desc->alpert_a;
    d.aj = aj;
    d.ani = ani;
    if ((s = g->upload(desc->alpert_w, (size_t)aj, &d.aw)) || (s = g->upload(off.data(), off.size(), &d.aoff)) ||
        (s = g->upload(desc->alpert_wt, off.size(), &d.awt)) ||
        (s = g->upload(desc->alpert_nodes, (size_t)6 * aj * n, &d.anodes)))
      return fail(s);
  } else if (desc->quad != 0) {
    delete g;
    set_error("qbg_geom_create: unknown quadrature %d", desc->quad);
    return QBG_EINVAL;
  }
  g->dim = d.m;
  e = cudaStreamSynchronize(g->stream);
  if (e != cudaSuccess) return fail(cuda_status(e, "qbg_geom_create sync"));
  *out = g;
  return QBG_OK;
}

qbg_status qbg_geom_destroy(qbg_geom* g) {
  delete g;
  return QBG_OK;
}

qbg_status qbg_geom_dim(const qbg_geom* g, int64_t* dim) {
  if (!g || !dim) { set_error("qbg_geom_dim: null argument"); return QBG_EINVAL; }
  *dim = g->dim;
  return QBG_OK;
}

}  // extern "C"
namespace qbg {
int check_ks(const double* ks, int64_t nk) {
  for (int64_t q = 0; q < 2 * nk; ++q)
    if (!std::isfinite(ks[q])) { set_error("non-finite wavenumber at index %lld", (long long)(q / 2)); return QBG_EINVAL; }
  for (int64_t q = 0; q < nk; ++q)
    if (ks[2 * q] == 0.0 && ks[2 * q + 1] == 0.0) { set_error("wavenumber k = 0 is not allowed"); return QBG_EINVAL; }
  return QBG_OK;
}
}  // namespace qbg

// Chebyshev tables for nk device wavenumbers; rmin/rmax padded by 0.95/1.05
// exactly as build_cfie_kress_block_caches (chebyshev_euclidian_helmholtz_cfie_kress.jl:396-456).
namespace qbg {
int cheb_params_check(const qbg_cheb_params* prm) {
  if (prm->n_panels_h < 1 || prm->n_panels_j < 1 || prm->M_h < 2 || prm->M_j < 2 ||
      prm->M_h > QBG_CHEB_MAX_DEGREE || prm->M_j > QBG_CHEB_MAX_DEGREE || prm->n_panels_h > (1 << 24) ||
      prm->n_panels_j > (1 << 24)) {
    set_error("Chebyshev parameters out of range (panels >= 1, 2 <= degree <= %d)", QBG_CHEB_MAX_DEGREE);
    return QBG_EINVAL;
  }
  return QBG_OK;
}

qbg_cheb_params cheb_defaults(const qbg_cheb_params* prm) {
  // the reference's defaults: n_panels_h = 15000, M_h = 5, n_panels_j = 3000, M_j = 5
  qbg_cheb_params p{15000, 5, 3000, 5};
  if (prm) {
    if (prm->n_panels_h > 0) p.n_panels_h = prm->n_panels_h;
    if (prm->M_h > 0) p.M_h = prm->M_h;
    if (prm->n_panels_j > 0) p.n_panels_j = prm->n_panels_j;
    if (prm->M_j > 0) p.M_j = prm->M_j;
  }
  return p;
}

static int cheb_range(qbg_geom* g, std::vector<void*>& tmp, cudaStream_t st, double* lo, double* hi) {
  unsigned long long* red = nullptr;
  QBG_TRY(dmalloc(&red, 2 * sizeof(unsigned long long)));
  tmp.push_back(red);
  QBG_TRY(cheb_r_range(g->d, red, lo, hi, st));
  if (!(*hi > 0.0) || !(*lo < 1e299)) {
    set_error("Chebyshev range: no pair distance above eps");
    return QBG_EINVAL;
  }
  return QBG_OK;
}

int make_cheb(qbg_geom* g, const cxd* dks, int nk, const qbg_cheb_params& prm, ChebTables& t,
              std::vector<void*>& tmp, cudaStream_t st) {
  double lo = 0, hi = 0;
  QBG_TRY(cheb_range(g, tmp, st, &lo, &hi));
  t.nk = nk;
  t.nh = prm.n_panels_h; t.Mh = prm.M_h;
  t.nj = prm.n_panels_j; t.Mj = prm.M_j;
  t.rmin = 0.95 * lo;
  t.rmax = 1.05 * hi;
  t.dr_h = (t.rmax - t.rmin) / t.nh;
  t.invdr_h = 1.0 / t.dr_h;
  t.dr_j = t.rmax / t.nj;
  t.invdr_j = 1.0 / t.dr_j;
  // CFIE route: direct Hankel values below |k r| = 0.2 (chebyshev_bessels.jl:1190-1207);
  // DLP route: panels everywhere above rmin (chebyshev_bessels.jl:1051-1073)
  t.small_cut = (g->d.form == QBG_FORM_CFIE) ? 0.2 : 0.0;
  QBG_TRY(dmalloc(&t.H, sizeof(cxd) * (size_t)nk * t.nh * (t.Mh + 1) * 2));
  tmp.push_back(t.H);
  QBG_TRY(dmalloc(&t.J, sizeof(cxd) * (size_t)nk * t.nj * (t.Mj + 1) * 2));
  tmp.push_back(t.J);
  return cheb_build(t, dks, st);
}

// J/E tables on the J grid of the parameters refined 1.5x: their G series
// carry up to ~2.4x the interpolation error of J0, J1 on the same panels, and
// 1.5x more panels lower it by 1.5^(M+1) (11x at M = 5, 58x at M = 9), so the
// tables are at least as accurate as the reference's J tables
int make_cheb_je(qbg_geom* g, const cxd* dks, int nk, const qbg_cheb_params& prm, ChebTables& t,
                 std::vector<void*>& tmp, cudaStream_t st) {
  double lo = 0, hi = 0;
  QBG_TRY(cheb_range(g, tmp, st, &lo, &hi));
  t.nk = nk;
  t.nh = prm.n_panels_h; t.Mh = prm.M_h;
  t.nj = prm.n_panels_j; t.Mj = prm.M_j;
  t.rmin = 0.95 * lo;
  t.rmax = 1.05 * hi;
  t.small_cut = 0.0;
  t.nje = (int)std::min<long long>((3LL * prm.n_panels_j + 1) / 2, (1LL << 21) - 1);
  t.Mje = prm.M_j;
  t.dr_je = t.rmax / t.nje;
  t.invdr_je = 1.0 / t.dr_je;
  t.nse = (g->d.form == QBG_FORM_CFIE) ? 4 : 2;
  QBG_TRY(dmalloc(&t.JE, cheb_je_bytes(t)));
  tmp.push_back(t.JE);
  return cheb_je_build(t, dks, st);
}

int make_cheb_df(ChebTables& t, const cxd* dks, std::vector<void*>& tmp, cudaStream_t st) {
  size_t hd = 0, jd = 0, nc = 0;
  cheb_df_bytes(t, &hd, &jd, &nc);
  QBG_TRY(dmalloc(&t.HD, hd));
  tmp.push_back(t.HD);
  QBG_TRY(dmalloc(&t.JD, jd));
  tmp.push_back(t.JD);
  QBG_TRY(dmalloc(&t.nkc, nc));
  tmp.push_back(t.nkc);
  return cheb_df_tables(t, dks, st);
}
}  // namespace qbg

extern "C" {

static int assemble_impl(qbg_geom* g, const double* ks, int64_t nk, int32_t deriv, int32_t prec, int32_t flags,
                         const qbg_cheb_params* cheb, void* const* outs) {
  if (!g || !ks || !outs || nk < 1 || (deriv != 0 && deriv != 1) || prec < 0 || prec > 2) {
    set_error("qbg_assemble: invalid arguments");
    return QBG_EINVAL;
  }
  QBG_TRY(check_ks(ks, nk));
  std::lock_guard<std::mutex> lk(g->mu);
  const int64_t dim = g->dim;
  const size_t esz = prec ? sizeof(cxf) : sizeof(cxd);
  const size_t mat_bytes = (size_t)dim * dim * esz;
  // QBG_SPLIT_LO: the mixed form's low words as a second block of nk outputs
  const bool split = (flags & QBG_SPLIT_LO) != 0;
  if (split && (prec != QBG_PREC_MIXED || deriv)) {
    set_error("qbg_assemble: QBG_SPLIT_LO needs prec QBG_PREC_MIXED and deriv = 0");
    return QBG_EINVAL;
  }
  const int nout = split ? 2 : 1 + 2 * deriv;
  const bool dev = (flags & QBG_PTR_DEVICE) != 0;
  // chunk the k list so that device staging stays below 8 GiB for host outputs
  int64_t chunk = nk;
  if (!dev) chunk = std::max<int64_t>(1, std::min<int64_t>(nk, (int64_t)((8ull << 30) / (mat_bytes * nout))));
  cxd* dks = nullptr;
  void** dptrs = nullptr;
  char* stage = nullptr;
  int s = QBG_OK;
  if ((s = dmalloc(&dks, sizeof(cxd) * nk))) return s;
  if ((s = dmalloc(&dptrs, sizeof(void*) * chunk * nout))) { dfree(dks); return s; }
  if (!dev && (s = dmalloc(&stage, mat_bytes * chunk * nout))) { dfree(dks); dfree(dptrs); return s; }
  cudaStream_t st = g->stream;
  std::vector<void*> hp(chunk * nout);
  auto cleanup = [&]() { dfree(dks, st); dfree(dptrs, st); if (stage) dfree(stage, st); };
  cudaError_t e = cudaMemcpyAsync(dks, ks, sizeof(cxd) * nk, cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) { cleanup(); return cuda_status(e, "qbg_assemble H2D"); }
  for (int64_t k0 = 0; k0 < nk; k0 += chunk) {
    const int64_t c = std::min(chunk, nk - k0);
    for (int o = 0; o < nout; ++o)
      for (int64_t q = 0; q < c; ++q)
        hp[o * c + q] = dev ? outs[o * nk + k0 + q] : (void*)(stage + (size_t)(o * c + q) * mat_bytes);
    e = cudaMemcpyAsync(dptrs, hp.data(), sizeof(void*) * c * nout, cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) { cleanup(); return cuda_status(e, "qbg_assemble ptrs"); }
    if (cheb) {
      std::vector<void*> ctmp;
      ChebTables t;
      if (cheb_je_applies(g->d, deriv, prec)) {
        s = make_cheb_je(g, dks + k0, (int)c, *cheb, t, ctmp, st);
      } else {
        s = make_cheb(g, dks + k0, (int)c, *cheb, t, ctmp, st);
        if (!s && prec != QBG_PREC_FP64 && cheb_df_applies(g->d, deriv)) s = make_cheb_df(t, dks + k0, ctmp, st);
      }
      if (!s)
        s = launch_assemble_cheb(g->d, t, dks + k0, (int)c, deriv, prec, dptrs, split ? dptrs + c : nullptr, dim,
                                 st);
      cudaError_t e2 = cudaStreamSynchronize(st);
      for (void* p : ctmp) dfree(p, st);
      if (!s && e2 != cudaSuccess) s = cuda_status(e2, "qbg_assemble_cheb");
    } else {
      s = launch_assemble(g->d, dks + k0, (int)c, deriv, prec, dptrs, dim, st, split ? dptrs + c : nullptr);
    }
    if (s) { cleanup(); return s; }
    if (!dev) {
      for (int o = 0; o < nout; ++o)
        for (int64_t q = 0; q < c; ++q) {
          e = cudaMemcpyAsync(outs[o * nk + k0 + q], stage + (size_t)(o * c + q) * mat_bytes, mat_bytes,
                              cudaMemcpyDeviceToHost, st);
          if (e != cudaSuccess) { cleanup(); return cuda_status(e, "qbg_assemble D2H"); }
        }
    }
    e = cudaStreamSynchronize(st);  // also keeps hp/dptrs valid for the next chunk
    if (e != cudaSuccess) { cleanup(); return cuda_status(e, "qbg_assemble"); }
  }
  cleanup();
  return QBG_OK;
}

qbg_status qbg_assemble(qbg_geom* g, const double* ks, int64_t nk, int32_t deriv, int32_t prec, int32_t flags,
                        void* const* outs) {
  return assemble_impl(g, ks, nk, deriv, prec, flags, nullptr, outs);
}

qbg_status qbg_assemble_cheb(qbg_geom* g, const double* ks, int64_t nk, int32_t deriv, int32_t prec, int32_t flags,
                             const qbg_cheb_params* cheb, void* const* outs) {
  const qbg_cheb_params p = cheb_defaults(cheb);
  QBG_TRY(cheb_params_check(&p));
  return assemble_impl(g, ks, nk, deriv, prec, flags, &p, outs);
}

}  // extern "C"


extern "C" {

// ---------------------------------------------------------------------------
// sigma_min (svdvals(A)[end], macros.jl:159-161) for every k: the k are taken
// in chunks; a chunk's A(k) are assembled in FP64 straight into one LU batch,
// factored by the library's batched LU and inverted (LU solves with the
// identity), and the subspace iteration on the inverses runs on the device
// until 1/sqrt(lambda_max) changes by less than 1e-13 relative (at most
// SM_ITERS steps): for many operators of n <= 1024 one CTA per k runs the
// whole iteration and one host synchronisation per chunk reads the results;
// otherwise each k's products are split over the whole GPU (sigma_single).
// An exactly singular U gives sigma_min = 0.
// ---------------------------------------------------------------------------
qbg_status qbg_sigma_min(qbg_geom* g, const double* ks, int64_t nk, double* sig) {
  if (!g || !ks || !sig || nk < 1) { set_error("qbg_sigma_min: invalid arguments"); return QBG_EINVAL; }
  constexpr int SM_ITERS = 40;
  std::vector<double> kc(2 * nk);
  for (int64_t q = 0; q < nk; ++q) { kc[2 * q] = ks[q]; kc[2 * q + 1] = 0.0; }
  QBG_TRY(check_ks(kc.data(), nk));
  std::lock_guard<std::mutex> lk(g->mu);
  const int n = (int)g->dim;
  // a sweep runs on a background stream (after the geometry stream's earlier
  // work): its FP64 factorisations fill every SM for milliseconds, and the
  // blocks of latency-bound requests on the library's other streams go first
  cudaStream_t st = nullptr;
  cudaEvent_t ev_in = nullptr;
  {
    cudaError_t e0 = stream_create(&st, true);
    if (e0 == cudaSuccess) e0 = cudaEventCreateWithFlags(&ev_in, cudaEventDisableTiming);
    if (e0 == cudaSuccess) e0 = cudaEventRecord(ev_in, g->stream);
    if (e0 == cudaSuccess) e0 = cudaStreamWaitEvent(st, ev_in, 0);
    if (e0 != cudaSuccess) {
      if (st) cudaStreamDestroy(st);
      if (ev_in) cudaEventDestroy(ev_in);
      return cuda_status(e0, "sigma_min stream");
    }
  }
  struct StreamGuard {
    cudaStream_t s;
    cudaEvent_t e;
    ~StreamGuard() {
      cudaStreamSynchronize(s);
      cudaStreamDestroy(s);
      cudaEventDestroy(e);
    }
  } sguard{st, ev_in};
  // chunk: the operators and their inverses within about 1 GB
  const size_t per_k = sizeof(cxd) * (size_t)n * n * 2;
  const int chunk = (int)std::max<int64_t>(1, std::min<int64_t>(std::min<int64_t>(nk, 256),
                                                                (int64_t)((1ull << 30) / per_k)));
  int s = QBG_OK;
  {
    Dense64 D;
    cxd *Cinv = nullptr, *dks = nullptr, *work = nullptr, *X0 = nullptr, *CH = nullptr, *P = nullptr;
    double *dsig = nullptr, *state = nullptr;
    void** dptrs = nullptr;
    // many small operators: one CTA per k runs the whole iteration (sigma_iterate);
    // otherwise each k's products are spread over the GPU (sigma_single)
    const bool per_cta = n <= 1024 && chunk >= 16;
    if ((s = D.create(n, chunk, st)) || (s = D.alloc(&Cinv, sizeof(cxd) * (size_t)n * n * chunk)) ||
        (s = D.alloc(&dks, sizeof(cxd) * nk)) || (s = D.alloc(&work, sizeof(cxd) * (size_t)3 * n * DENSE_P * chunk)) ||
        (s = D.alloc(&X0, sizeof(cxd) * (size_t)n * DENSE_P)) || (s = D.alloc(&dsig, sizeof(double) * chunk)) ||
        (s = D.alloc(&dptrs, sizeof(void*) * chunk)) ||
        (!per_cta && ((s = D.alloc(&CH, sizeof(cxd) * (size_t)n * n)) ||
                      (s = D.alloc(&P, sizeof(cxd) * std::max<size_t>(gemm_tall_scratch(n, DENSE_P), 1))) ||
                      (s = D.alloc(&state, sizeof(double) * (2 + 2 * DENSE_P))))))
      return s;
    std::vector<cxd> hx;
    dense_start_block(n, hx);
    std::vector<void*> hp(chunk);
    for (int q = 0; q < chunk; ++q) hp[q] = D.A(q);
    QBG_CUDA(cudaMemcpyAsync(X0, hx.data(), sizeof(cxd) * hx.size(), cudaMemcpyHostToDevice, st));
    QBG_CUDA(cudaMemcpyAsync(dks, kc.data(), sizeof(cxd) * nk, cudaMemcpyHostToDevice, st));
    QBG_CUDA(cudaMemcpyAsync(dptrs, hp.data(), sizeof(void*) * chunk, cudaMemcpyHostToDevice, st));
    std::vector<int> info;
    std::vector<double> hs(chunk);
    for (int64_t k0 = 0; k0 < nk; k0 += chunk) {
      const int c = (int)std::min<int64_t>(chunk, nk - k0);
      D.f.batch = c;
      QBG_TRY(launch_assemble(g->d, dks + k0, c, 0, QBG_PREC_FP64, dptrs, n, st));
      QBG_TRY(lu_factor<double>(D.f, st));
      QBG_TRY(D.inverse(Cinv));
      info.assign(c, 0);
      QBG_CUDA(cudaMemcpyAsync(info.data(), D.f.info, sizeof(int) * c, cudaMemcpyDeviceToHost, st));
      if (per_cta) {
        QBG_TRY(sigma_iterate(Cinv, n, c, X0, work, SM_ITERS, 1e-13, dsig, nullptr, nullptr, st));
        QBG_CUDA(cudaMemcpyAsync(hs.data(), dsig, sizeof(double) * c, cudaMemcpyDeviceToHost, st));
        QBG_CUDA(cudaStreamSynchronize(st));
      } else {
        QBG_CUDA(cudaStreamSynchronize(st));
        for (int q = 0; q < c; ++q) {
          hs[q] = 0.0;
          if (info[q] > 0) continue;
          cxd* W3 = work;
          QBG_TRY(sigma_single(Cinv + (size_t)q * n * n, CH, n, X0, W3, W3 + (size_t)n * DENSE_P,
                               W3 + 2 * (size_t)n * DENSE_P, P, state, SM_ITERS, 1e-13, &hs[q], nullptr, st));
        }
      }
      for (int q = 0; q < c; ++q) sig[k0 + q] = info[q] > 0 ? 0.0 : hs[q];
    }
    D.f.batch = chunk;
  }
  return s;
}

// chebyshev_params (chebyshev_optimal_panelization.jl:221-307): grow the panel
// counts by 1.5 (every 5th iteration the degrees by 2 instead) until the max
// absolute error of every interpolated H0, H1, J0, J1 over all wavenumbers is
// below tol at nsample radii.
qbg_status qbg_cheb_autotune(qbg_geom* g, const double* ks, int64_t nk, double tol, int32_t nsample,
                             int32_t max_iter, int32_t grow_M, qbg_cheb_params* io, double* err4) {
  if (!g || !ks || !io || nk < 1 || nk > 65535 || !(tol > 0.0) || nsample < 2 || max_iter < 1 || grow_M < 0) {
    set_error("qbg_cheb_autotune: invalid arguments");
    return QBG_EINVAL;
  }
  QBG_TRY(check_ks(ks, nk));
  qbg_cheb_params p = cheb_defaults(io);
  QBG_TRY(cheb_params_check(&p));
  std::lock_guard<std::mutex> lk(g->mu);
  cudaStream_t st = g->stream;
  cxd* dks = nullptr;
  unsigned long long* derr = nullptr;
  QBG_TRY(dmalloc(&dks, sizeof(cxd) * nk));
  int s = dmalloc(&derr, sizeof(unsigned long long) * 4 * nk);
  if (s) { dfree(dks, st); return s; }
  std::vector<unsigned long long> herr(4 * nk);
  double worst[4] = {0, 0, 0, 0};
  cudaError_t e = cudaMemcpyAsync(dks, ks, sizeof(cxd) * nk, cudaMemcpyHostToDevice, st);
  bool ok = false;
  for (int it = 1; e == cudaSuccess && !s && it <= max_iter; ++it) {
    std::vector<void*> ctmp;
    ChebTables t;
    s = make_cheb(g, dks, (int)nk, p, t, ctmp, st);
    if (!s) e = cudaMemsetAsync(derr, 0, sizeof(unsigned long long) * 4 * nk, st);
    if (!s && e == cudaSuccess) s = cheb_errors(t, dks, nsample, derr, st);
    if (!s && e == cudaSuccess)
      e = cudaMemcpyAsync(herr.data(), derr, sizeof(unsigned long long) * 4 * nk, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    for (void* q : ctmp) dfree(q, st);
    if (s || e != cudaSuccess) break;
    for (int f = 0; f < 4; ++f) worst[f] = 0.0;
    for (int64_t q = 0; q < nk; ++q)
      for (int f = 0; f < 4; ++f) {
        double v;
        memcpy(&v, &herr[4 * q + f], sizeof(double));
        worst[f] = std::max(worst[f], v);
      }
    const bool okH = worst[0] < tol && worst[1] < tol, okJ = worst[2] < tol && worst[3] < tol;
    if (okH && okJ) { ok = true; break; }
    if (it == max_iter) break;
    auto grow = [&](int& npan, int& M) {
      if (grow_M > 0 && it % 5 == 0 && M + grow_M <= QBG_CHEB_MAX_DEGREE) M += grow_M;
      else npan = (int)std::ceil(1.5 * (double)npan);
    };
    if (!okH) grow(p.n_panels_h, p.M_h);
    if (!okJ) grow(p.n_panels_j, p.M_j);
    if (p.n_panels_h > (1 << 24) || p.n_panels_j > (1 << 24)) break;
  }
  dfree(dks, st);
  dfree(derr, st);
  if (s) return s;
  if (e != cudaSuccess) return cuda_status(e, "qbg_cheb_autotune");
  *io = p;
  if (err4)
    for (int f = 0; f < 4; ++f) err4[f] = worst[f];
  if (!ok) {
    set_error("Chebyshev tuning did not reach tol = %g after %d iterations (best effort returned)", tol, max_iter);
    return QBG_ETIMEOUT;
  }
  return QBG_OK;
}

// residual_and_norm_select's device part (beyn.jl:557-593): T(lambda_j) at
// each candidate, y = T phi_j, and the norms the selection uses
qbg_status qbg_candidate_residuals(qbg_geom* g, const double* lambdas, int64_t n, const double* Phi,
                                   const qbg_cheb_params* cheb, double* out) {
  if (!g || !lambdas || !Phi || !out || n < 1) {
    set_error("qbg_candidate_residuals: invalid arguments");
    return QBG_EINVAL;
  }
  QBG_TRY(check_ks(lambdas, n));
  qbg_cheb_params cp{};
  if (cheb) {
    cp = cheb_defaults(cheb);
    QBG_TRY(cheb_params_check(&cp));
  }
  std::lock_guard<std::mutex> lk(g->mu);
  const int N = (int)g->dim;
  cudaStream_t st = g->stream;
  const int chunk = (int)std::min<int64_t>(n, 8);
  const size_t NN = (size_t)N * N;
  cxd *T = nullptr, *dl = nullptr, *phi = nullptr, *y = nullptr;
  double *nrm = nullptr, *an = nullptr;
  void** dptrs = nullptr;
  std::vector<void*> tmp;
  auto cleanup = [&]() { for (void* p : tmp) dfree(p, st); };
  auto talloc = [&](auto** p, size_t bytes) {
    int s = dmalloc(p, bytes);
    if (!s) tmp.push_back(*p);
    return s;
  };
  int s = QBG_OK;
  if ((s = talloc(&T, sizeof(cxd) * NN * chunk)) || (s = talloc(&dl, sizeof(cxd) * n)) ||
      (s = talloc(&phi, sizeof(cxd) * (size_t)N * chunk)) || (s = talloc(&y, sizeof(cxd) * (size_t)N * chunk)) ||
      (s = talloc(&nrm, sizeof(double) * 4 * chunk)) || (s = talloc(&an, sizeof(double) * chunk)) ||
      (s = talloc(&dptrs, sizeof(void*) * chunk))) {
    cleanup();
    return s;
  }
  std::vector<void*> hp(chunk);
  for (int q = 0; q < chunk; ++q) hp[q] = T + (size_t)q * NN;
  cudaError_t e = cudaMemcpyAsync(dl, lambdas, sizeof(cxd) * n, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dptrs, hp.data(), sizeof(void*) * chunk, cudaMemcpyHostToDevice, st);
  std::vector<double> hn(4 * chunk), ha(chunk);
  for (int64_t q0 = 0; e == cudaSuccess && !s && q0 < n; q0 += chunk) {
    const int c = (int)std::min<int64_t>(chunk, n - q0);
    e = cudaMemcpyAsync(phi, Phi + 2 * (size_t)N * q0, sizeof(cxd) * (size_t)N * c, cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) break;
    std::vector<void*> ctmp;
    if (cheb) {
      ChebTables t;
      s = make_cheb(g, dl + q0, c, cp, t, ctmp, st);
      if (!s) s = launch_assemble_cheb(g->d, t, dl + q0, c, 0, QBG_PREC_FP64, dptrs, nullptr, N, st);
    } else {
      s = launch_assemble(g->d, dl + q0, c, 0, QBG_PREC_FP64, dptrs, N, st);
    }
    if (!s) s = gemm_batched<double>(N, 1, N, cxd(1.0, 0.0), T, N, (long long)NN, phi, N, N, cxd(0.0, 0.0), y, N, N,
                                     c, st);
    if (!s) e = cudaMemsetAsync(an, 0, sizeof(double) * c, st);
    if (!s && e == cudaSuccess) s = opnorm1_batched(T, N, (long long)NN, c, an, st);
    if (!s && e == cudaSuccess) s = vec_norms(y, phi, N, c, nrm, st);
    if (!s && e == cudaSuccess) e = cudaMemcpyAsync(hn.data(), nrm, sizeof(double) * 4 * c, cudaMemcpyDeviceToHost, st);
    if (!s && e == cudaSuccess) e = cudaMemcpyAsync(ha.data(), an, sizeof(double) * c, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    for (void* p : ctmp) dfree(p, st);
    if (s || e != cudaSuccess) break;
    for (int q = 0; q < c; ++q) {
      double* o = out + 5 * (q0 + q);
      o[0] = std::sqrt(hn[4 * q + 0]);  // ||T phi||_2
      o[1] = hn[4 * q + 1];             // ||T phi||_1
      o[2] = ha[q];                     // opnorm(T, 1)
      o[3] = hn[4 * q + 2];             // ||phi||_1
      o[4] = std::sqrt(hn[4 * q + 3]);  // ||phi||_2
    }
  }
  cleanup();
  if (s) return s;
  if (e != cudaSuccess) return cuda_status(e, "qbg_candidate_residuals");
  return QBG_OK;
}

qbg_status qbg_bessel01(const double* z, int64_t n, int32_t f32, double* out) {
  if (!z || !out || n < 1) { set_error("qbg_bessel01: invalid arguments"); return QBG_EINVAL; }
  cxd *dz = nullptr, *dout = nullptr;
  int s = dmalloc(&dz, sizeof(cxd) * n);
  if (s) return s;
  if ((s = dmalloc(&dout, sizeof(cxd) * 4 * n))) { dfree(dz); return s; }
  cudaError_t e = cudaMemcpy(dz, z, sizeof(cxd) * n, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) {
    s = launch_bessel_eval(dz, (int)n, dout, f32, 0);
    if (!s) e = cudaMemcpy(out, dout, sizeof(cxd) * 4 * n, cudaMemcpyDeviceToHost);
  }
  dfree(dz);
  dfree(dout);
  if (s) return s;
  if (e != cudaSuccess) return cuda_status(e, "qbg_bessel01");
  return QBG_OK;
}

qbg_status qbg_cgemm_c64(int32_t engine, int32_t M, int32_t N, int32_t K, const float* alpha, const float* A,
                         int64_t lda, const float* B, int64_t ldb, const float* beta, float* C, int64_t ldc,
                         int32_t batch) {
  if (!alpha || !beta || !A || !B || !C || M < 1 || N < 1 || K < 1 || batch < 1 || batch > 65535 || lda < M ||
      ldb < K || ldc < M || engine < GEMM_ENGINE_SIMT || engine > GEMM_ENGINE_TCGEN05_STAGED) {
    set_error("qbg_cgemm_c64: invalid arguments");
    return QBG_EINVAL;
  }
  const long long sA = lda * (long long)K, sB = ldb * (long long)N, sC = ldc * (long long)N;
  cxf *dA = nullptr, *dB = nullptr, *dC = nullptr;
  int s = dmalloc(&dA, sizeof(cxf) * sA * batch);
  if (!s) s = dmalloc(&dB, sizeof(cxf) * sB * batch);
  if (!s) s = dmalloc(&dC, sizeof(cxf) * sC * batch);
  cudaError_t e = cudaSuccess;
  if (!s) {
    e = cudaMemcpy(dA, A, sizeof(cxf) * sA * batch, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(dB, B, sizeof(cxf) * sB * batch, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(dC, C, sizeof(cxf) * sC * batch, cudaMemcpyHostToDevice);
  }
  if (!s && e == cudaSuccess) {
    const cxf al(alpha[0], alpha[1]), be(beta[0], beta[1]);
    if (engine != GEMM_ENGINE_SIMT)
      s = tc_gemm_c64(M, N, K, al, dA, lda, sA, dB, ldb, sB, be, dC, ldc, sC, batch, 0, 1, 0, 0, 0,
                      engine == GEMM_ENGINE_TCGEN05);
    else
      s = gemm_batched_simt<float>(M, N, K, al, dA, lda, sA, dB, ldb, sB, be, dC, ldc, sC, batch, 0);
    if (!s && engine != GEMM_ENGINE_SIMT) s = tc_check(0);
    if (!s) e = cudaMemcpy(C, dC, sizeof(cxf) * sC * batch, cudaMemcpyDeviceToHost);
  }
  dfree(dA);
  dfree(dB);
  dfree(dC);
  if (s) return s;
  if (e != cudaSuccess) return cuda_status(e, "qbg_cgemm_c64");
  return QBG_OK;
}

qbg_status qbg_dense_inverse(int32_t n, int32_t batch, int32_t prec, const double* A, double* X, double* sig,
                             double* work_out) {
  if (n < 1 || batch < 1 || batch > 65535 || !A || !X || (prec != QBG_PREC_FP64 && prec != QBG_PREC_FP32) ||
      (prec == QBG_PREC_FP32 && (sig || work_out))) {
    set_error("qbg_dense_inverse: invalid arguments");
    return QBG_EINVAL;
  }
  cudaStream_t st = nullptr;
  QBG_CUDA(stream_create(&st));
  int s = QBG_OK;
  const size_t nn = (size_t)n * n;
  if (prec == QBG_PREC_FP32) {
    LUBatch<float> f;
    f.n = n;
    f.batch = batch;
    f.stride = (long long)nn;
    f.nb = std::min(64, n);
    f.nblk = (n + f.nb - 1) / f.nb;
    std::vector<void*> mem;
    auto alloc = [&](auto** p, size_t bytes) {
      int r = dmalloc(p, bytes);
      if (!r) mem.push_back(*p);
      return r;
    };
    cxd* Ad = nullptr;
    cxf* Xf = nullptr;
    if (!(s = alloc(&Ad, sizeof(cxd) * nn * batch)) && !(s = alloc(&f.A, sizeof(cxf) * nn * batch)) &&
        !(s = alloc(&Xf, sizeof(cxf) * nn * batch)) && !(s = alloc(&f.ipiv, sizeof(int) * (size_t)n * batch)) &&
        !(s = alloc(&f.perm, sizeof(int) * (size_t)n * batch)) && !(s = alloc(&f.info, sizeof(int) * batch)) &&
        !(s = alloc(&f.Linv, sizeof(cxf) * (size_t)f.nblk * f.nb * f.nb * batch)) &&
        !(s = alloc(&f.Uinv, sizeof(cxf) * (size_t)f.nblk * f.nb * f.nb * batch))) {
      cudaError_t e = cudaMemcpyAsync(Ad, A, sizeof(cxd) * nn * batch, cudaMemcpyHostToDevice, st);
      s = e == cudaSuccess ? QBG_OK : cuda_status(e, "qbg_dense_inverse");
      if (!s) s = convert_d2f(Ad, f.A, (long long)(nn * batch), st);
      if (!s) s = lu_factor<float>(f, st);
      if (!s) s = lu_inverse<float>(f, Xf, st);
      if (!s) s = tc_check(st);
      if (!s) {
        e = cudaMemsetAsync(Ad, 0, sizeof(cxd) * nn * batch, st);
        s = e == cudaSuccess ? axpy_f2d(Xf, Ad, (long long)(nn * batch), st) : cuda_status(e, "qbg_dense_inverse");
      }
      if (!s) {
        e = cudaMemcpyAsync(X, Ad, sizeof(cxd) * nn * batch, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) s = cuda_status(e, "qbg_dense_inverse");
      }
    }
    cudaStreamSynchronize(st);
    for (void* p : mem) dfree(p);
    cudaStreamDestroy(st);
    return s;
  }
  {
    Dense64 D;
    cxd *Cinv = nullptr, *work = nullptr, *X0 = nullptr;
    double* dsig = nullptr;
    if (!(s = D.create(n, batch, st)) && !(s = D.alloc(&Cinv, sizeof(cxd) * nn * batch)) &&
        !(s = D.alloc(&work, sizeof(cxd) * (size_t)3 * n * DENSE_P * batch)) &&
        !(s = D.alloc(&X0, sizeof(cxd) * (size_t)n * DENSE_P)) && !(s = D.alloc(&dsig, sizeof(double) * batch))) {
      std::vector<cxd> hx;
      dense_start_block(n, hx);
      cudaError_t e = cudaMemcpyAsync(D.f.A, A, sizeof(cxd) * nn * batch, cudaMemcpyHostToDevice, st);
      if (e == cudaSuccess) e = cudaMemcpyAsync(X0, hx.data(), sizeof(cxd) * hx.size(), cudaMemcpyHostToDevice, st);
      s = e == cudaSuccess ? QBG_OK : cuda_status(e, "qbg_dense_inverse");
      if (!s) s = lu_factor<double>(D.f, st);
      if (!s) s = D.inverse(Cinv);
      if (!s && sig) s = sigma_iterate(Cinv, n, batch, X0, work, 40, 1e-13, dsig, nullptr, nullptr, st);
      if (!s) {
        e = cudaMemcpyAsync(X, Cinv, sizeof(cxd) * nn * batch, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess && sig)
          e = cudaMemcpyAsync(sig, dsig, sizeof(double) * batch, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess && work_out)
          e = cudaMemcpyAsync(work_out, work, sizeof(cxd) * (size_t)3 * n * DENSE_P * batch, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) s = cuda_status(e, "qbg_dense_inverse");
      }
    }
  }
  cudaStreamDestroy(st);
  return s;
}

qbg_status qbg_set_lu_plan(int32_t outer, int32_t cluster, int32_t parts) {
  if (outer > 16 || cluster > 1 || cluster < -1 || parts > LUBatch<float>::MAX_SPLIT) {
    set_error("qbg_set_lu_plan: outer must be <= 16, cluster -1, 0 or 1 and parts <= %d", LUBatch<float>::MAX_SPLIT);
    return QBG_EINVAL;
  }
  set_lu_plan(outer, cluster, parts);
  return QBG_OK;
}

qbg_status qbg_get_lu_plan(int32_t* outer, int32_t* cluster, int32_t* parts) {
  int o = 0, c = 0, q = 0;
  get_lu_plan(&o, &c, &q);
  if (outer) *outer = o;
  if (cluster) *cluster = c;
  if (parts) *parts = q;
  return QBG_OK;
}

qbg_status qbg_set_tc_wait_limit(int64_t polls) { return tc_set_wait_limit(polls); }

qbg_status qbg_clear_tc_error(void) { return tc_clear_error(); }

qbg_status qbg_launch_count(uint64_t* count) {
  if (!count) { set_error("qbg_launch_count: null pointer"); return QBG_EINVAL; }
  *count = g_launches.load(std::memory_order_relaxed);
  return QBG_OK;
}

qbg_status qbg_zgemm_sub_tc(int32_t M, int32_t N, int32_t K, const double* A, int64_t lda, const double* B,
                            int64_t ldb, double* C, int64_t ldc, int32_t batch) {
  if (!A || !B || !C || M < 1 || N < 1 || K < 1 || batch < 1 || batch > 65535 || lda < M || ldb < K || ldc < M) {
    set_error("qbg_zgemm_sub_tc: invalid arguments");
    return QBG_EINVAL;
  }
  const size_t na = (size_t)lda * K, nbm = (size_t)ldb * N, nc = (size_t)ldc * N;
  cxd *dA = nullptr, *dB = nullptr, *dC = nullptr;
  int s = QBG_OK;
  if ((s = dmalloc(&dA, sizeof(cxd) * na * batch))) return s;
  if ((s = dmalloc(&dB, sizeof(cxd) * nbm * batch))) { dfree(dA); return s; }
  if ((s = dmalloc(&dC, sizeof(cxd) * nc * batch))) { dfree(dA); dfree(dB); return s; }
  cudaError_t e = cudaMemcpy(dA, A, sizeof(cxd) * na * batch, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(dB, B, sizeof(cxd) * nbm * batch, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(dC, C, sizeof(cxd) * nc * batch, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) s = cuda_status(e, "qbg_zgemm_sub_tc staging");
  if (!s) s = tc_gemm_sub_f64(M, N, K, dA, lda, (long long)na, dB, ldb, (long long)nbm, dC, ldc, (long long)nc, batch, 0);
  if (!s) s = tc_check(0);
  if (!s) {
    e = cudaMemcpy(C, dC, sizeof(cxd) * nc * batch, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) s = cuda_status(e, "qbg_zgemm_sub_tc D2H");
  }
  dfree(dA);
  dfree(dB);
  dfree(dC);
  return s;
}

qbg_status qbg_residual_c64(int32_t engine, int32_t n, int32_t L, int32_t batch, const float* Th, const float* Tl,
                            const double* X, const double* V, double* R, double* rmax) {
  if (!Th || !X || !V || !R || !rmax || n < 1 || L < 1 || batch < 1 || batch > 65535 || engine < 0 || engine > 2) {
    set_error("qbg_residual_c64: invalid arguments");
    return QBG_EINVAL;
  }
  const size_t nn = (size_t)n * n, nl = (size_t)n * L;
  std::vector<void*> tmp;
  auto cleanup = [&]() { for (void* p : tmp) dfree(p); };
  auto talloc = [&](auto** p, size_t bytes) {
    int s = dmalloc(p, bytes);
    if (!s) tmp.push_back(*p);
    return s;
  };
  cxf *dTh = nullptr, *dTl = nullptr;
  cxd *dX = nullptr, *dV = nullptr, *dR = nullptr;
  double* dmax = nullptr;
  void *tmem = nullptr, *xmem = nullptr;
  int s = QBG_OK;
  if ((s = talloc(&dTh, sizeof(cxf) * nn * batch)) || (Tl && (s = talloc(&dTl, sizeof(cxf) * nn * batch))) ||
      (s = talloc(&dX, sizeof(cxd) * nl * batch)) || (s = talloc(&dV, sizeof(cxd) * nl * batch)) ||
      (s = talloc(&dR, sizeof(cxd) * nl * batch)) || (s = talloc(&dmax, sizeof(double)))) {
    cleanup();
    return s;
  }
  cudaError_t e = cudaMemcpy(dTh, Th, sizeof(cxf) * nn * batch, cudaMemcpyHostToDevice);
  if (e == cudaSuccess && Tl) e = cudaMemcpy(dTl, Tl, sizeof(cxf) * nn * batch, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(dX, X, sizeof(cxd) * nl * batch, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(dV, V, sizeof(cxd) * nl * batch, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset(dmax, 0, sizeof(double));
  if (e != cudaSuccess) { cleanup(); return cuda_status(e, "qbg_residual_c64 staging"); }
  if (engine == 1) {
    s = residual_df32(dTh, dTl, (long long)nn, dX, (long long)nl, dV, (long long)nl, dR, (long long)nl, n, L, batch,
                      dmax, 0);
  } else {
    TcResidT t;
    if (!(s = talloc(&tmem, tc_resid_T_bytes(n, batch))) && !(s = talloc(&xmem, tc_resid_X_bytes(n, L, batch)))) {
      e = cudaMemset(xmem, 0, tc_resid_X_bytes(n, L, batch));
      if (e != cudaSuccess) s = cuda_status(e, "memset");
    }
    if (!s) s = tc_resid_bind_T(t, n, batch, tmem, 0);
    if (!s) s = tc_resid_prepare_T(t, dTh, dTl, (long long)nn, batch, 0);
    if (!s)
      s = tc_residual(t, dX, (long long)nl, dV, (long long)nl, dR, (long long)nl, L, batch, dmax, xmem, 0,
                      engine == 2 ? 6 : 7);
    if (!s) s = tc_check(0);
  }
  if (!s) {
    e = cudaMemcpy(R, dR, sizeof(cxd) * nl * batch, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(rmax, dmax, sizeof(double), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) s = cuda_status(e, "qbg_residual_c64 D2H");
  }
  cleanup();
  return s;
}

qbg_status qbg_set_gemm_engine(int32_t engine) {
  if (engine < GEMM_ENGINE_SIMT || engine > GEMM_ENGINE_TCGEN05_STAGED) {
    set_error("qbg_set_gemm_engine: engine must be 0, 1 or 2");
    return QBG_EINVAL;
  }
  set_gemm_engine(engine);
  return QBG_OK;
}

}  // extern "C"
