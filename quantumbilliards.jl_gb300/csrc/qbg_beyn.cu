// Beyn contour step on the device (construct_B_matrix, beyn.jl:257-322): the
// contour nodes of one or more disks, T(z_j) at every node, the LU of every
// node, X_j = T(z_j)^{-1} V and the moment sums A0 = sum w_j X_j,
// A1 = sum w_j z_j X_j per disk.
//
// Residency. By default every node's operator stays factored in HBM between
// qbg_beyn_create and the moments calls (the reference keeps its nq LU
// factors the same way, beyn.jl:270-277). With opts.node_chunk > 0 the handle
// keeps only node_chunk operators resident: each moments call streams the
// nodes through them in groups (assemble, factor, solve, accumulate), which
// bounds the memory at large N at the price of re-assembling per call.
#include <algorithm>
#include <complex>
#include <cstdlib>
#include <cusolverDn.h>
#include <limits>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>
#include <vector>

#include "qbg_assemble.cuh"
#include "qbg_handles.cuh"
#include "qbg_linalg.cuh"

using namespace qbg;

struct qbg_beyn {
  qbg_geom* g = nullptr;
  int n = 0;        // operator dimension
  int nq = 0;       // contour nodes per disk
  int ndisk = 1;
  int nn = 0;       // nq * ndisk contour nodes, disk-major
  int cap = 0;      // operators resident at once
  int prec = 0;
  qbg_beyn_opts opts{};
  cxd* zj = nullptr;  // device contour nodes (nn)
  cxd* wj = nullptr;  // device contour weights (nn)
  LUBatch<double> fd;  // FP64 form: cap operators
  LUBatch<float> ff;   // complex64 forms: cap operators
  cxf* Tcopy = nullptr;  // complex64 forms: unfactored hi words for the refinement residual
  cxf* Tlo = nullptr;    // mixed form: lo words, T = hi + lo to ~2^-48
  bool tc_resid = false;  // complex64 forms: residual on the tensor cores from digit planes of T
  TcResidT tr;
  void** dptrs = nullptr;  // device array of the cap operator slots
  void** dlo = nullptr;    // device array of the cap lo slots (mixed form)
  int res0 = -1, resn = 0;  // nodes [res0, res0 + resn) are factored in the slots
  std::vector<void*> allocs;
  cudaStream_t st = nullptr;
  // extra streams of the LU and the triangular solves: nsplit parts of the
  // operator batch run concurrently. QBG_LU_SPLIT in the environment sets the
  // number of parts (default 4, at most 4; 0 or 1 keeps everything on st);
  // the results are the same either way
  int nsplit = 1;
  cudaStream_t stx[LUBatch<float>::MAX_SPLIT - 1] = {};
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  // helper streams of the per-disk QR of the moments (created on first use)
  static constexpr int QR_STREAMS = 8;
  cudaStream_t qst[QR_STREAMS] = {};
  cudaEvent_t qev[QR_STREAMS] = {};
  cudaEvent_t qfork = nullptr;
  cudaEvent_t ev[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
  double ms_assemble = 0, ms_factor = 0;  // device time of the last load(s)
  int singular = 0;
  // moment blocks kept on the device for qbg_beyn_moments_qr: per disk N x mcap,
  // column-major, the first mcols columns filled
  cxd* macc0 = nullptr;
  cxd* macc1 = nullptr;
  int mcap = 0, mcols = 0;
  std::mutex mu;
  ~qbg_beyn() {
    if (st) cudaStreamSynchronize(st);
    for (void* p : allocs) dfree(p, st);
    dfree(macc0, st);
    dfree(macc1, st);
    for (auto& e : ev)
      if (e) cudaEventDestroy(e);
    for (cudaStream_t x : stx)
      if (x) {
        cudaStreamSynchronize(x);
        tc_release_scratch(x);
        cudaStreamDestroy(x);
      }
    if (ev_fork) cudaEventDestroy(ev_fork);
    if (ev_join) cudaEventDestroy(ev_join);
    for (int i = 0; i < QR_STREAMS; ++i) {
      if (qst[i]) {
        cudaStreamSynchronize(qst[i]);
        cudaStreamDestroy(qst[i]);
      }
      if (qev[i]) cudaEventDestroy(qev[i]);
    }
    if (qfork) cudaEventDestroy(qfork);
    if (st) {
      tc_release_scratch(st);
      cudaStreamDestroy(st);
    }
  }
  template <class P>
  int alloc(P** p, size_t bytes) {
    int s = dmalloc(p, bytes);
    if (!s) allocs.push_back(*p);
    return s;
  }
};

namespace {

template <class T>
int setup_lu(qbg_beyn* b, LUBatch<T>& f, int nb, int solve_levels) {
  f.n = b->n;
  f.batch = b->cap;
  f.nb = nb;
  f.nblk = (b->n + nb - 1) / nb;
  f.stride = (long long)b->n * b->n;
  QBG_TRY(b->alloc(&f.A, sizeof(cx<T>) * (size_t)f.stride * f.batch));
  QBG_TRY(b->alloc(&f.ipiv, sizeof(int) * (size_t)b->n * f.batch));
  QBG_TRY(b->alloc(&f.perm, sizeof(int) * (size_t)b->n * f.batch));
  QBG_TRY(b->alloc(&f.info, sizeof(int) * f.batch));
  QBG_TRY(b->alloc(&f.Linv, sizeof(cx<T>) * (size_t)f.nblk * nb * nb * f.batch));
  QBG_TRY(b->alloc(&f.Uinv, sizeof(cx<T>) * (size_t)f.nblk * nb * nb * f.batch));
  // the FP64 LU is bound by the FP64 pipe: a second stream only adds contention
  if (sizeof(T) == sizeof(float)) {
    f.nsplit = b->nsplit;
    for (int i = 0; i + 1 < b->nsplit; ++i) f.stx[i] = b->stx[i];
    f.ev_fork = b->ev_fork;
    f.ev_join = b->ev_join;
  }
  if (solve_levels > 0) {
    void* mem = nullptr;
    QBG_TRY(b->alloc(&mem, lu_solve_blocks_bytes<T>(f, solve_levels, 128)));
    lu_solve_blocks_bind<T>(f, mem);
  }
  return QBG_OK;
}

// contour (beyn.jl:258-261): theta_j = 2 pi j / nq, z_j = k0 + R e^{i theta_j}, w_j = (R / nq) e^{i theta_j}
int setup(qbg_beyn* b, const double* k0s, const double* Rs) {
  const int n = b->n, nq = b->nq, nn = b->nn;
  cudaStream_t st = b->st;
  std::vector<cxd> z(nn), w(nn);
  for (int d = 0; d < b->ndisk; ++d) {
    const double k0r = k0s[2 * d], k0i = k0s[2 * d + 1], R = Rs[d];
    for (int j = 0; j < nq; ++j) {
      const double th = 2.0 * M_PI * (double)j / (double)nq;
      const double c = std::cos(th), s = std::sin(th);
      z[d * nq + j] = cxd(k0r + R * c, k0i + R * s);
      w[d * nq + j] = cxd((R / nq) * c, (R / nq) * s);
    }
  }
  QBG_TRY(b->alloc(&b->zj, sizeof(cxd) * nn));
  QBG_TRY(b->alloc(&b->wj, sizeof(cxd) * nn));
  QBG_CUDA(cudaMemcpyAsync(b->zj, z.data(), sizeof(cxd) * nn, cudaMemcpyHostToDevice, st));
  QBG_CUDA(cudaMemcpyAsync(b->wj, w.data(), sizeof(cxd) * nn, cudaMemcpyHostToDevice, st));
  for (auto& e : b->ev) QBG_CUDA(cudaEventCreate(&e));
  const int nb = b->opts.nb > 0 ? b->opts.nb : (b->prec ? 64 : 32);
  if (nb != 32 && nb != 64) {
    set_error("LU block size must be 32 or 64");
    return QBG_EINVAL;
  }
  const int cap = b->cap;
  std::vector<void*> ptrs(cap), lp(cap);
  QBG_TRY(b->alloc(&b->dptrs, sizeof(void*) * cap));
  if (b->prec == QBG_PREC_FP64) {
    QBG_TRY(setup_lu(b, b->fd, nb, 0));
    for (int j = 0; j < cap; ++j) ptrs[j] = b->fd.A + (size_t)j * b->fd.stride;
  } else {
    int levels = n >= 8 * nb ? 2 : (n >= 4 * nb ? 1 : 0);
    if (b->opts.solve_block != 0) {
      const int sb = b->opts.solve_block;
      if (sb != nb && sb != 2 * nb && sb != 4 * nb) {
        set_error("solve_block must be nb, 2 nb or 4 nb (nb = %d)", nb);
        return QBG_EINVAL;
      }
      levels = sb == nb ? 0 : (sb == 2 * nb ? 1 : 2);
    }
    QBG_TRY(setup_lu(b, b->ff, nb, levels));
    for (int j = 0; j < cap; ++j) ptrs[j] = b->ff.A + (size_t)j * b->ff.stride;
    QBG_TRY(b->alloc(&b->Tcopy, sizeof(cxf) * (size_t)b->ff.stride * cap));
  }
  QBG_CUDA(cudaMemcpyAsync(b->dptrs, ptrs.data(), sizeof(void*) * cap, cudaMemcpyHostToDevice, st));
  if (b->prec == QBG_PREC_MIXED) {
    QBG_TRY(b->alloc(&b->Tlo, sizeof(cxf) * (size_t)b->ff.stride * cap));
    QBG_TRY(b->alloc(&b->dlo, sizeof(void*) * cap));
    for (int j = 0; j < cap; ++j) lp[j] = b->Tlo + (size_t)j * b->ff.stride;
    QBG_CUDA(cudaMemcpyAsync(b->dlo, lp.data(), sizeof(void*) * cap, cudaMemcpyHostToDevice, st));
  }
  if (b->prec != QBG_PREC_FP64 && b->opts.resid_engine == 0) {
    void* mem = nullptr;
    QBG_TRY(b->alloc(&mem, tc_resid_T_bytes(n, cap)));
    QBG_TRY(tc_resid_bind_T(b->tr, n, cap, mem, st));
    b->tc_resid = true;
  } else if (b->opts.resid_engine != 0 && b->opts.resid_engine != 1) {
    set_error("resid_engine must be 0 (tensor cores) or 1 (compensated FP32)");
    return QBG_EINVAL;
  }
  QBG_CUDA(cudaStreamSynchronize(st));  // the host pointer tables must outlive their copies
  return QBG_OK;
}

// assemble and factor nodes [n0, n0 + c) into slots 0 .. c-1
int load(qbg_beyn* b, int n0, int c) {
  const int n = b->n;
  cudaStream_t st = b->st;
  b->res0 = -1;
  b->resn = 0;
  QBG_CUDA(cudaEventRecord(b->ev[0], st));
  // the FP32 form evaluates its kernels directly
  const bool use_cheb = b->opts.eval_mode == 0 && b->prec != QBG_PREC_FP32;
  if (use_cheb) {
    const qbg_cheb_params cp = cheb_defaults(&b->opts.cheb);
    QBG_TRY(cheb_params_check(&cp));
    std::vector<void*> ctmp;
    ChebTables t;
    int s = QBG_OK;
    if (cheb_je_applies(b->g->d, 0, b->prec)) {
      s = make_cheb_je(b->g, b->zj + n0, c, cp, t, ctmp, st);
    } else {
      s = make_cheb(b->g, b->zj + n0, c, cp, t, ctmp, st);
      if (!s && b->prec != QBG_PREC_FP64 && cheb_df_applies(b->g->d, 0)) s = make_cheb_df(t, b->zj + n0, ctmp, st);
    }
    if (!s) s = launch_assemble_cheb(b->g->d, t, b->zj + n0, c, 0, b->prec, b->dptrs, b->dlo, n, st);
    if (!s) {
      cudaEventRecord(b->ev[1], st);
      cudaError_t e = cudaStreamSynchronize(st);  // the tables are freed below
      if (e != cudaSuccess) s = cuda_status(e, "Chebyshev assembly");
    }
    for (void* p : ctmp) dfree(p, st);
    if (s) return s;
  } else {
    QBG_TRY(launch_assemble(b->g->d, b->zj + n0, c, 0, b->prec, b->dptrs, n, st, b->dlo));
    QBG_CUDA(cudaEventRecord(b->ev[1], st));
  }
  int* info = nullptr;
  if (b->prec == QBG_PREC_FP64) {
    b->fd.batch = c;
    QBG_TRY(lu_factor<double>(b->fd, st));
    info = b->fd.info;
  } else {
    QBG_CUDA(cudaMemcpyAsync(b->Tcopy, b->ff.A, sizeof(cxf) * (size_t)b->ff.stride * c, cudaMemcpyDeviceToDevice,
                             st));
    if (b->tc_resid) QBG_TRY(tc_resid_prepare_T(b->tr, b->Tcopy, b->Tlo, b->ff.stride, c, st));
    b->ff.batch = c;
    QBG_TRY(lu_factor<float>(b->ff, st));
    info = b->ff.info;
  }
  QBG_CUDA(cudaEventRecord(b->ev[2], st));
  std::vector<int> hinfo(c);
  QBG_CUDA(cudaMemcpyAsync(hinfo.data(), info, sizeof(int) * c, cudaMemcpyDeviceToHost, st));
  QBG_CUDA(cudaStreamSynchronize(st));
  if (b->prec != QBG_PREC_FP64) QBG_TRY(tc_check(st));
  for (int v : hinfo) b->singular += (v != 0);
  float ma = 0.f, mf = 0.f;
  QBG_CUDA(cudaEventElapsedTime(&ma, b->ev[0], b->ev[1]));
  QBG_CUDA(cudaEventElapsedTime(&mf, b->ev[1], b->ev[2]));
  b->ms_assemble += ma;
  b->ms_factor += mf;
  b->res0 = n0;
  b->resn = c;
  return QBG_OK;
}

}  // namespace

namespace {

// state of one moments call
struct Call {
  qbg_beyn* b = nullptr;
  int L = 0;
  size_t nl = 0;
  cxd *dV = nullptr, *dA0 = nullptr, *dA1 = nullptr;
  bool per_disk = false;  // V holds one N x L block per disk
  cxd* Vn = nullptr;      // per-disk V: the resident nodes' blocks, node-major
  cxf* Vn32 = nullptr;
  double vmax = 1.0;
  cxd *X64 = nullptr, *R64 = nullptr;
  cxf *V32 = nullptr, *X32 = nullptr, *R32 = nullptr;
  double* dmax = nullptr;
  void* xmem = nullptr;  // digit planes of X for the tensor-core residual
  std::vector<void*> tmp;
  std::vector<cudaEvent_t> sev;  // start/stop pairs around the solve passes
  // statistics (the history is the last node group's)
  int sweeps = 0, nhist = 0, n_resid = 0, nf32 = 0;
  double rel = 0.0, ms_resid = 0.0;
  double hist[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  double f32hist[4] = {0, 0, 0, 0};
  ~Call() {
    for (void* p : tmp) dfree(p, b ? b->st : nullptr);
    for (cudaEvent_t e : sev) cudaEventDestroy(e);
  }
  template <class P>
  int talloc(P** p, size_t bytes) {
    int s = dmalloc(p, bytes);
    if (!s) tmp.push_back(*p);
    return s;
  }
  int timed_solve(const cxf* rhs, long long srhs) {
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (sev.size() < 64 && cudaEventCreate(&e0) == cudaSuccess && cudaEventCreate(&e1) == cudaSuccess) {
      sev.push_back(e0);
      sev.push_back(e1);
      cudaEventRecord(e0, b->st);
    } else {
      if (e0) cudaEventDestroy(e0);
      e0 = e1 = nullptr;
    }
    int r = lu_solve_shared<float>(b->ff, rhs, L, X32, srhs, b->st);
    if (e1) cudaEventRecord(e1, b->st);
    return r;
  }
};

// digits of the first tensor-core residual of a refinement: 6, or 7 with
// QBG_RESID_DIGITS=7. The error of a residual survives into the solution as
// ~cond x (its relative error) and is contracted by the next sweep by the
// FP32 factors' ~5e-4 (C2), so the first residual needs ~2^-40 where the last
// needs the full ~2^-47 (five digits, ~2^-33, left the C2 eigenvalues at
// 1.9e-12 of the oracle instead of 1.8e-13)
static int first_resid_digits() {
  static const int nd = [] {
    const char* e = getenv("QBG_RESID_DIGITS");
    return (e && atoi(e) == 7) ? 7 : 6;
  }();
  return nd;
}

// complex64 forms: X32 = LU32 \ V32; corrections from plain FP32 residuals;
// then compensated residuals R = V - (hi + lo) X64 and corrections until
// max|R| <= refine_tol max|V| (the correction from that residual is applied)
int refine_resident(Call& c) {
  qbg_beyn* b = c.b;
  cudaStream_t st = b->st;
  const int n = b->n, nr = b->resn, L = c.L;
  const size_t nl = c.nl;
  const long long tot = (long long)(nl * nr);
  int s = QBG_OK;
  QBG_CUDA(cudaMemsetAsync(c.X64, 0, sizeof(cxd) * tot, st));
  const cxd* V64 = c.per_disk ? c.Vn : c.dV;
  const cxf* V32 = c.per_disk ? c.Vn32 : c.V32;
  const long long sV = c.per_disk ? (long long)nl : 0;
  if ((s = c.timed_solve(V32, sV)) || (s = axpy_f2d(c.X32, c.X64, tot, st))) return s;
  int sweeps = 0;
  c.nhist = 0;
  c.nf32 = 0;
  const int nf = std::min(b->opts.fp32_sweeps > 0 ? b->opts.fp32_sweeps : 1, 4);
  for (int q = 0; q < nf; ++q) {
    // X32 holds the first solve's result for q == 0, a correction afterwards
    if (q > 0 && (s = convert_d2f(c.X64, c.X32, tot, st))) return s;
    QBG_CUDA(cudaMemsetAsync(c.dmax, 0, sizeof(double), st));
    if (c.per_disk)
      QBG_CUDA(cudaMemcpyAsync(c.R32, c.Vn32, sizeof(cxf) * tot, cudaMemcpyDeviceToDevice, st));
    else if ((s = broadcast_f(c.V32, (long long)nl, nr, c.R32, st)))
      return s;
    if (
        (s = gemm_batched<float>(n, L, n, cxf(-1.f, 0.f), b->Tcopy, n, b->ff.stride, c.X32, n, (long long)nl,
                                 cxf(1.f, 0.f), c.R32, n, (long long)nl, nr, st)) ||
        (s = maxabs_c64(c.R32, tot, c.dmax, st)) || (s = c.timed_solve(c.R32, (long long)nl)) ||
        (s = axpy_f2d(c.X32, c.X64, tot, st)))
      return s;
    double fmax = 0.0;
    QBG_CUDA(cudaMemcpyAsync(&fmax, c.dmax, sizeof(double), cudaMemcpyDeviceToHost, st));
    QBG_CUDA(cudaStreamSynchronize(st));
    if (c.nf32 < 4) c.f32hist[c.nf32++] = fmax / c.vmax;
    ++sweeps;
  }
  double rel = 0.0;
  for (int it = 0; it < b->opts.max_refine; ++it) {
    // the first tensor-core residual from six digits of T and X (~2^-40 of
    // the scales); when it already meets the tolerance its correction may be
    // the last, and it is recomputed from all seven
    int nd = (it == 0 && b->tc_resid) ? first_resid_digits() : 7;
    double rmax = 0.0;
    for (;;) {
      QBG_CUDA(cudaMemsetAsync(c.dmax, 0, sizeof(double), st));
      cudaEventRecord(b->ev[4], st);
      if (b->tc_resid)
        s = tc_residual(b->tr, c.X64, (long long)nl, V64, sV, c.R64, (long long)nl, L, nr, c.dmax, c.xmem, st, nd);
      else
        s = residual_df32(b->Tcopy, b->Tlo, b->ff.stride, c.X64, (long long)nl, V64, sV, c.R64, (long long)nl, n,
                          L, nr, c.dmax, st);
      if (s) return s;
      cudaEventRecord(b->ev[5], st);
      QBG_CUDA(cudaMemcpyAsync(&rmax, c.dmax, sizeof(double), cudaMemcpyDeviceToHost, st));
      QBG_CUDA(cudaStreamSynchronize(st));
      float ms_r = 0.f;
      if (cudaEventElapsedTime(&ms_r, b->ev[4], b->ev[5]) == cudaSuccess) {
        c.ms_resid += ms_r;
        ++c.n_resid;
      }
      if (nd < 7 && rmax <= 16.0 * b->opts.refine_tol * c.vmax) {
        nd = 7;
        continue;
      }
      break;
    }
    rel = rmax / c.vmax;
    if (c.nhist < 8) c.hist[c.nhist++] = rel;
    ++sweeps;
    if (!(rel == rel)) break;  // Inf or NaN in T or X: no correction can help; NaN is reported
    // correction from this residual; when it already meets the tolerance this
    // is the final correction (the residual is in hand, the solve costs one FP32 pass)
    if ((s = convert_d2f(c.R64, c.R32, tot, st)) || (s = c.timed_solve(c.R32, (long long)nl)) ||
        (s = axpy_f2d(c.X32, c.X64, tot, st)))
      return s;
    if (rel <= b->opts.refine_tol) break;
    // no progress (the FP32 factors contract the residual by less than 2 per
    // sweep): further sweeps cannot converge; the caller sees refine_residual
    if (c.nhist >= 2 && rel > 0.5 * c.hist[c.nhist - 2]) break;
  }
  c.sweeps = std::max(c.sweeps, sweeps);
  c.rel = (c.rel != c.rel || rel != rel) ? std::numeric_limits<double>::quiet_NaN() : std::max(c.rel, rel);
  return QBG_OK;
}

// solves for the resident nodes and adds their moments to the disks' A0, A1
int solve_and_accumulate(Call& c) {
  qbg_beyn* b = c.b;
  cudaStream_t st = b->st;
  const int n = b->n, nr = b->resn, r0 = b->res0;
  if (c.per_disk) {
    // node j's right-hand side is its disk's probe block
    for (int j = 0; j < nr; ++j) {
      const int d = (r0 + j) / b->nq;
      QBG_CUDA(cudaMemcpyAsync(c.Vn + (size_t)j * c.nl, c.dV + (size_t)d * c.nl, sizeof(cxd) * c.nl,
                               cudaMemcpyDeviceToDevice, st));
    }
    if (b->prec != QBG_PREC_FP64) QBG_TRY(convert_d2f(c.Vn, c.Vn32, (long long)(c.nl * nr), st));
  }
  if (b->prec == QBG_PREC_FP64) {
    QBG_TRY(lu_solve_shared<double>(b->fd, c.per_disk ? c.Vn : c.dV, c.L, c.X64, c.per_disk ? (long long)c.nl : 0,
                                    st));
  } else {
    QBG_TRY(refine_resident(c));
  }
  for (int node = r0; node < r0 + nr;) {
    const int d = node / b->nq;
    const int end = std::min((d + 1) * b->nq, r0 + nr);
    QBG_TRY(moments<double>(c.X64 + (size_t)(node - r0) * c.nl, (long long)c.nl, end - node, n, c.L, b->wj + node,
                            b->zj + node, c.dA0 + (size_t)d * c.nl, c.dA1 + (size_t)d * c.nl, 1, st));
    node = end;
  }
  return QBG_OK;
}

qbg_status create_impl(qbg_geom* g, const double* k0s, const double* Rs, int ndisk, int nq, int prec,
                       const qbg_beyn_opts* opts, qbg_beyn** out) {
  if (!g || !out || !k0s || !Rs || ndisk < 1 || nq < 2 || prec < 0 || prec > 2 ||
      (long long)ndisk * nq > 65535) {
    set_error("qbg_beyn_create: invalid arguments");
    return QBG_EINVAL;
  }
  for (int d = 0; d < ndisk; ++d)
    if (!(Rs[d] > 0.0) || !std::isfinite(Rs[d]) || !std::isfinite(k0s[2 * d]) || !std::isfinite(k0s[2 * d + 1])) {
      set_error("qbg_beyn_create: disk %d has a non-finite centre or a radius <= 0", d);
      return QBG_EINVAL;
    }
  *out = nullptr;
  qbg_beyn* b = new (std::nothrow) qbg_beyn();
  if (!b) {
    set_error("host allocation failed");
    return QBG_ENOMEM;
  }
  b->g = g;
  b->n = (int)g->dim;
  b->nq = nq;
  b->ndisk = ndisk;
  b->nn = nq * ndisk;
  b->prec = prec;
  b->opts = qbg_beyn_opts{};
  b->opts.max_refine = 10;
  b->opts.refine_tol = 1e-6;
  if (opts) {
    b->opts = *opts;
    if (b->opts.max_refine <= 0) b->opts.max_refine = 10;
    if (!(b->opts.refine_tol > 0.0)) b->opts.refine_tol = 1e-6;
  }
  b->cap = (b->opts.node_chunk > 0 && b->opts.node_chunk < b->nn) ? b->opts.node_chunk : b->nn;
  int s = QBG_OK;
  {
    // the geometry was uploaded on its own stream
    std::lock_guard<std::mutex> lk(g->mu);
    cudaError_t e = cudaStreamSynchronize(g->stream);
    if (e != cudaSuccess) s = cuda_status(e, "geometry stream");
  }
  if (!s) {
    cudaError_t e = stream_create(&b->st);
    if (e != cudaSuccess) s = cuda_status(e, "cudaStreamCreate");
  }
  int parts = 1;
  get_lu_plan(nullptr, nullptr, &parts);  // stream parts of the operator batch (qbg_set_lu_plan)
  parts = std::max(1, std::min(parts, LUBatch<float>::MAX_SPLIT));
  if (!s && parts > 1) {
    cudaError_t e = cudaEventCreateWithFlags(&b->ev_fork, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->ev_join, cudaEventDisableTiming);
    for (int i = 0; i + 1 < parts && e == cudaSuccess; ++i) e = stream_create(&b->stx[i]);
    if (e != cudaSuccess) s = cuda_status(e, "LU streams");
    else b->nsplit = parts;
  }
  if (!s) s = setup(b, k0s, Rs);
  if (!s && b->cap == b->nn) s = load(b, 0, b->nn);
  if (s) {
    delete b;
    return s;
  }
  *out = b;
  return QBG_OK;
}

}  // namespace

extern "C" {

qbg_status qbg_beyn_create(qbg_geom* g, double k0_re, double k0_im, double R, int32_t nq, int32_t prec,
                           const qbg_beyn_opts* opts, qbg_beyn** out) {
  const double k0[2] = {k0_re, k0_im};
  return create_impl(g, k0, &R, 1, nq, prec, opts, out);
}

qbg_status qbg_beyn_create_disks(qbg_geom* g, const double* k0s, const double* Rs, int32_t ndisk, int32_t nq,
                                 int32_t prec, const qbg_beyn_opts* opts, qbg_beyn** out) {
  return create_impl(g, k0s, Rs, ndisk, nq, prec, opts, out);
}

}  // extern "C"

namespace {

// grows the kept moment blocks to at least m columns per disk (existing columns copied)
int ensure_moment_blocks(qbg_beyn* b, int m) {
  if (m <= b->mcap) return QBG_OK;
  const size_t n = (size_t)b->n;
  const int cap = std::max(m, 2 * b->mcap);
  cxd *a0 = nullptr, *a1 = nullptr;
  QBG_TRY(dmalloc(&a0, sizeof(cxd) * n * cap * b->ndisk));
  if (int s = dmalloc(&a1, sizeof(cxd) * n * cap * b->ndisk)) {
    dfree(a0, b->st);
    return s;
  }
  for (int d = 0; d < b->ndisk && b->mcols > 0; ++d) {
    QBG_CUDA(cudaMemcpyAsync(a0 + d * n * cap, b->macc0 + d * n * b->mcap, sizeof(cxd) * n * b->mcols,
                             cudaMemcpyDeviceToDevice, b->st));
    QBG_CUDA(cudaMemcpyAsync(a1 + d * n * cap, b->macc1 + d * n * b->mcap, sizeof(cxd) * n * b->mcols,
                             cudaMemcpyDeviceToDevice, b->st));
  }
  dfree(b->macc0, b->st);
  dfree(b->macc1, b->st);
  b->macc0 = a0;
  b->macc1 = a1;
  b->mcap = cap;
  return QBG_OK;
}

// moments of V. A0/A1: outputs (host, or device with QBG_PTR_DEVICE), or both
// NULL; keep >= 0 also stores the moments in the kept blocks (0: replacing
// them, 1: behind the columns kept so far)
int moments_impl(qbg_beyn* b, const double* V, int64_t L, double* A0, double* A1, qbg_beyn_stats* stats, int keep) {
  const int n = b->n;
  const bool dev = (b->opts.flags & QBG_PTR_DEVICE) != 0;
  cudaStream_t st = b->st;
  Call c;
  c.b = b;
  c.L = (int)L;
  c.nl = (size_t)n * L;
  const size_t nl = c.nl, nA = nl * b->ndisk;
  c.per_disk = (b->opts.flags & QBG_V_PER_DISK) != 0 && b->ndisk > 1;
  const size_t nV = c.per_disk ? nA : nl;
  const bool out = A0 && A1;
  if (dev) {
    c.dV = (cxd*)V;
  } else {
    QBG_TRY(c.talloc(&c.dV, sizeof(cxd) * nV));
    QBG_CUDA(cudaMemcpyAsync(c.dV, V, sizeof(cxd) * nV, cudaMemcpyHostToDevice, st));
  }
  if (dev && out) {
    c.dA0 = (cxd*)A0;
    c.dA1 = (cxd*)A1;
  } else {
    QBG_TRY(c.talloc(&c.dA0, sizeof(cxd) * nA));
    QBG_TRY(c.talloc(&c.dA1, sizeof(cxd) * nA));
  }
  QBG_CUDA(cudaMemsetAsync(c.dA0, 0, sizeof(cxd) * nA, st));
  QBG_CUDA(cudaMemsetAsync(c.dA1, 0, sizeof(cxd) * nA, st));
  const size_t cap = (size_t)b->cap;
  QBG_TRY(c.talloc(&c.X64, sizeof(cxd) * nl * cap));
  if (c.per_disk) {
    QBG_TRY(c.talloc(&c.Vn, sizeof(cxd) * nl * cap));
    if (b->prec != QBG_PREC_FP64) QBG_TRY(c.talloc(&c.Vn32, sizeof(cxf) * nl * cap));
  }
  if (b->prec != QBG_PREC_FP64) {
    QBG_TRY(c.talloc(&c.V32, sizeof(cxf) * nl));
    QBG_TRY(c.talloc(&c.X32, sizeof(cxf) * nl * cap));
    QBG_TRY(c.talloc(&c.R32, sizeof(cxf) * nl * cap));
    QBG_TRY(c.talloc(&c.R64, sizeof(cxd) * nl * cap));
    QBG_TRY(c.talloc(&c.dmax, sizeof(double)));
    if (b->tc_resid) {
      const size_t xb = tc_resid_X_bytes(n, (int)L, b->cap);
      QBG_TRY(c.talloc(&c.xmem, xb));
      QBG_CUDA(cudaMemsetAsync(c.xmem, 0, xb, st));
    }
    QBG_TRY(convert_d2f(c.dV, c.V32, (long long)nl, st));
    // max |V| (|re| + |im|) scales the convergence test
    std::vector<cxd> hv;
    const cxd* hvp = reinterpret_cast<const cxd*>(V);
    if (dev) {
      hv.resize(nV);
      QBG_CUDA(cudaMemcpyAsync(hv.data(), c.dV, sizeof(cxd) * nV, cudaMemcpyDeviceToHost, st));
      QBG_CUDA(cudaStreamSynchronize(st));
      hvp = hv.data();
    }
    double vmax = 0.0;
    for (size_t q = 0; q < nV; ++q) vmax = std::max(vmax, std::fabs(hvp[q].re) + std::fabs(hvp[q].im));
    c.vmax = vmax > 0.0 ? vmax : 1.0;
  }
  const bool streamed = b->cap < b->nn;
  if (streamed) {
    b->ms_assemble = 0.0;
    b->ms_factor = 0.0;
    b->singular = 0;
  }
  QBG_CUDA(cudaEventRecord(b->ev[3], st));
  float ms_total = 0.f;
  if (!streamed) {
    QBG_TRY(solve_and_accumulate(c));
  } else {
    for (int n0 = 0; n0 < b->nn; n0 += b->cap) {
      QBG_TRY(load(b, n0, std::min(b->cap, b->nn - n0)));
      QBG_TRY(solve_and_accumulate(c));
    }
  }
  if (keep >= 0) {
    const int off = keep ? b->mcols : 0;
    if (!keep) b->mcols = 0;
    QBG_TRY(ensure_moment_blocks(b, off + (int)L));
    const size_t nn_ = (size_t)n;
    for (int d = 0; d < b->ndisk; ++d) {
      QBG_CUDA(cudaMemcpyAsync(b->macc0 + d * nn_ * b->mcap + (size_t)off * nn_, c.dA0 + d * nl, sizeof(cxd) * nl,
                               cudaMemcpyDeviceToDevice, st));
      QBG_CUDA(cudaMemcpyAsync(b->macc1 + d * nn_ * b->mcap + (size_t)off * nn_, c.dA1 + d * nl, sizeof(cxd) * nl,
                               cudaMemcpyDeviceToDevice, st));
    }
    b->mcols = off + (int)L;
  }
  if (!dev && out) {
    QBG_CUDA(cudaMemcpyAsync(A0, c.dA0, sizeof(cxd) * nA, cudaMemcpyDeviceToHost, st));
    QBG_CUDA(cudaMemcpyAsync(A1, c.dA1, sizeof(cxd) * nA, cudaMemcpyDeviceToHost, st));
  }
  cudaEvent_t e_end = nullptr;
  QBG_CUDA(cudaEventCreate(&e_end));
  cudaEventRecord(e_end, st);
  cudaError_t e = cudaStreamSynchronize(st);
  cudaEventElapsedTime(&ms_total, b->ev[3], e_end);
  cudaEventDestroy(e_end);
  if (e != cudaSuccess) return cuda_status(e, "qbg_beyn_moments");
  if (b->prec != QBG_PREC_FP64) QBG_TRY(tc_check(st));
  double ms_solves = 0.0;
  for (size_t q = 0; q + 1 < c.sev.size(); q += 2) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, c.sev[q], c.sev[q + 1]) == cudaSuccess) ms_solves += ms;
  }
  if (stats) {
    stats->refine_sweeps = c.sweeps;
    stats->refine_residual = c.rel;
    stats->singular = b->singular;
    stats->ms_assemble = b->ms_assemble;
    stats->ms_factor = b->ms_factor;
    // device time of this call; a streamed handle's assembly and factorisation are inside it
    stats->ms_solve = streamed ? ms_total - b->ms_assemble - b->ms_factor : ms_total;
    stats->nhist = c.nhist;
    for (int q = 0; q < 8; ++q) stats->refine_history[q] = c.hist[q];
    stats->ms_residual = c.ms_resid;
    stats->n_residual = c.n_resid;
    stats->nfp32 = c.nf32;
    for (int q = 0; q < 4; ++q) stats->fp32_history[q] = c.f32hist[q];
    stats->ms_solves = ms_solves;
    stats->n_solves = (int)c.sev.size() / 2;
  }
  return QBG_OK;
}

// thin Householder QR of every disk's kept A0 block (N x m) on the device:
// R (m x m, upper triangular) and C = Q^H A1 (m x m) to the host, column-major
// per disk. Several disks run on up to QR_STREAMS helper streams (each with its
// own cuSOLVER handle and workspace): the factorisations are latency-bound, so
// disks overlap. R and C are staged on the device and copied back at once.
std::mutex g_qr_mu;
cusolverDnHandle_t g_qr_h[64][qbg_beyn::QR_STREAMS] = {};

int qr_reduce(qbg_beyn* b, double* Rh, double* Ch) {
  const int n = b->n, m = b->mcols, nd = b->ndisk;
  cudaStream_t st = b->st;
  int dev = 0;
  QBG_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) {
    set_error("qr_reduce: device index %d", dev);
    return QBG_EINVAL;
  }
  const int S = nd > 1 ? std::min(nd, (int)qbg_beyn::QR_STREAMS) : 1;
  std::lock_guard<std::mutex> lk(g_qr_mu);
  for (int i = 0; i < S; ++i) {
    cusolverDnHandle_t& h = g_qr_h[dev][i];
    if (!h && cusolverDnCreate(&h) != CUSOLVER_STATUS_SUCCESS) {
      h = nullptr;
      set_error("cusolverDnCreate failed");
      return QBG_ECUDA;
    }
    if (S > 1 && !b->qst[i]) {
      QBG_CUDA(stream_create(&b->qst[i]));
      QBG_CUDA(cudaEventCreateWithFlags(&b->qev[i], cudaEventDisableTiming));
    }
  }
  if (S > 1 && !b->qfork) QBG_CUDA(cudaEventCreateWithFlags(&b->qfork, cudaEventDisableTiming));
  auto stream_of = [&](int slot) { return S > 1 ? b->qst[slot] : st; };
  std::vector<void*> tmp;
  auto cleanup = [&]() { for (void* p : tmp) dfree(p, st); };
  auto get = [&](auto** p, size_t bytes) {
    int s = dmalloc(p, bytes);
    if (!s) tmp.push_back(*p);
    return s;
  };
  const size_t nn_ = (size_t)n, mm = (size_t)m * m;
  const size_t per_slot = nn_ * m * 2 + (size_t)m;  // w0, w1, tau (complex words)
  cuDoubleComplex* ws = nullptr;
  cuDoubleComplex* works = nullptr;
  cxd* stage = nullptr;
  int* info = nullptr;
  int s = QBG_OK;
  if ((s = get(&ws, sizeof(cxd) * per_slot * S)) || (s = get(&stage, sizeof(cxd) * 2 * mm * nd)) ||
      (s = get(&info, sizeof(int) * nd))) {
    cleanup();
    return s;
  }
  int l1 = 0, l2 = 0;
  {
    cusolverDnHandle_t h = g_qr_h[dev][0];
    cuDoubleComplex* w0 = ws;
    if (cusolverDnZgeqrf_bufferSize(h, n, m, w0, n, &l1) != CUSOLVER_STATUS_SUCCESS ||
        cusolverDnZunmqr_bufferSize(h, CUBLAS_SIDE_LEFT, CUBLAS_OP_C, n, m, m, w0, n, w0 + 2 * nn_ * m,
                                    w0 + nn_ * m, n, &l2) != CUSOLVER_STATUS_SUCCESS) {
      cleanup();
      set_error("cuSOLVER workspace query failed");
      return QBG_ECUDA;
    }
  }
  const int lw = std::max(std::max(l1, l2), 1);
  if ((s = get(&works, sizeof(cxd) * (size_t)lw * S))) {
    cleanup();
    return s;
  }
  if (S > 1) {
    cudaError_t e = cudaEventRecord(b->qfork, st);
    for (int i = 0; i < S && e == cudaSuccess; ++i) e = cudaStreamWaitEvent(b->qst[i], b->qfork, 0);
    if (e != cudaSuccess) {
      cleanup();
      return cuda_status(e, "qr_reduce fork");
    }
  }
  for (int d = 0; d < nd && !s; ++d) {
    const int slot = d % S;
    cudaStream_t qs = stream_of(slot);
    cusolverDnHandle_t h = g_qr_h[dev][slot];
    cuDoubleComplex* w0 = ws + per_slot * slot;
    cuDoubleComplex* w1 = w0 + nn_ * m;
    cuDoubleComplex* tau = w1 + nn_ * m;
    cuDoubleComplex* work = works + (size_t)lw * slot;
    if (cusolverDnSetStream(h, qs) != CUSOLVER_STATUS_SUCCESS) {
      set_error("cusolverDnSetStream failed");
      s = QBG_ECUDA;
      break;
    }
    cudaError_t e = cudaMemcpyAsync(w0, b->macc0 + d * nn_ * b->mcap, sizeof(cxd) * nn_ * m,
                                    cudaMemcpyDeviceToDevice, qs);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(w1, b->macc1 + d * nn_ * b->mcap, sizeof(cxd) * nn_ * m, cudaMemcpyDeviceToDevice, qs);
    if (e != cudaSuccess) {
      s = cuda_status(e, "qr_reduce copy");
      break;
    }
    if (cusolverDnZgeqrf(h, n, m, w0, n, tau, work, lw, info + d) != CUSOLVER_STATUS_SUCCESS ||
        cusolverDnZunmqr(h, CUBLAS_SIDE_LEFT, CUBLAS_OP_C, n, m, m, w0, n, tau, w1, n, work, lw, info + d) !=
            CUSOLVER_STATUS_SUCCESS) {
      set_error("cusolverDnZgeqrf / Zunmqr failed");
      s = QBG_ECUDA;
      break;
    }
    e = cudaMemcpy2DAsync(stage + 2 * d * mm, sizeof(cxd) * m, w0, sizeof(cxd) * nn_, sizeof(cxd) * m, m,
                          cudaMemcpyDeviceToDevice, qs);
    if (e == cudaSuccess)
      e = cudaMemcpy2DAsync(stage + (2 * d + 1) * mm, sizeof(cxd) * m, w1, sizeof(cxd) * nn_, sizeof(cxd) * m, m,
                            cudaMemcpyDeviceToDevice, qs);
    if (e != cudaSuccess) s = cuda_status(e, "qr_reduce staging");
  }
  if (S > 1) {
    // join every helper stream back into the handle's stream (also after an error)
    for (int i = 0; i < S; ++i) {
      cudaEventRecord(b->qev[i], b->qst[i]);
      cudaStreamWaitEvent(st, b->qev[i], 0);
    }
  }
  std::vector<int> hinfo(nd, 0);
  std::vector<cxd> hstage;
  if (!s) {
    hstage.resize(2 * mm * nd);
    cudaError_t e = cudaMemcpyAsync(hstage.data(), stage, sizeof(cxd) * 2 * mm * nd, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(hinfo.data(), info, sizeof(int) * nd, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) s = cuda_status(e, "qr_reduce");
  } else {
    cudaStreamSynchronize(st);
  }
  cleanup();
  if (s) return s;
  for (int d = 0; d < nd; ++d)
    if (hinfo[d] < 0) {
      set_error("cusolverDnZgeqrf: argument %d invalid", -hinfo[d]);
      return QBG_ECUDA;
    }
  for (int d = 0; d < nd; ++d) {
    std::memcpy(Rh + 2 * d * mm, hstage.data() + 2 * d * mm, sizeof(cxd) * mm);
    std::memcpy(Ch + 2 * d * mm, hstage.data() + (2 * d + 1) * mm, sizeof(cxd) * mm);
    // R is the upper triangle; below it geqrf left the Householder vectors
    for (int j = 0; j < m; ++j)
      for (int i = j + 1; i < m; ++i) {
        Rh[2 * (d * mm + (size_t)j * m + i)] = 0.0;
        Rh[2 * (d * mm + (size_t)j * m + i) + 1] = 0.0;
      }
  }
  return QBG_OK;
}

// One-sided Jacobi SVD (Hestenes; Golub and Van Loan 8.6.4) of the m x m
// complex matrix R (column-major): columns are rotated pairwise until
// mutually orthogonal, R W = U diag(sv). On return sv holds the singular
// values in descending order and W the right singular vectors (m x m,
// column-major), ordered alike. Small singular values keep high relative
// accuracy, which the absolute rank test svd_tol relies on.
void jacobi_svd(int m, std::vector<std::complex<double>> R, std::vector<double>& sv,
                std::vector<std::complex<double>>& W) {
  using zc = std::complex<double>;
  W.assign((size_t)m * m, zc(0.0, 0.0));
  for (int i = 0; i < m; ++i) W[(size_t)i * m + i] = 1.0;
  auto col = [&](std::vector<zc>& M, int j) { return M.data() + (size_t)j * m; };
  for (int sweep = 0; sweep < 60; ++sweep) {
    bool rotated = false;
    for (int p = 0; p < m - 1; ++p)
      for (int q = p + 1; q < m; ++q) {
        zc* a = col(R, p);
        zc* b = col(R, q);
        double al = 0.0, be = 0.0;
        zc ga(0.0, 0.0);
        for (int i = 0; i < m; ++i) {
          al += std::norm(a[i]);
          be += std::norm(b[i]);
          ga += std::conj(a[i]) * b[i];
        }
        const double g = std::abs(ga);
        if (!(g > 1e-15 * std::sqrt(al * be)) || g == 0.0) continue;
        rotated = true;
        const zc ph = ga / g;  // b e^{-i phi} makes the pair's Gram entry real
        const double zeta = (be - al) / (2.0 * g);
        const double t = (zeta >= 0.0 ? 1.0 : -1.0) / (std::fabs(zeta) + std::sqrt(1.0 + zeta * zeta));
        const double c = 1.0 / std::sqrt(1.0 + t * t), sn = c * t;
        for (int i = 0; i < m; ++i) {
          const zc x = a[i], y = b[i] * std::conj(ph);
          a[i] = c * x - sn * y;
          b[i] = sn * x + c * y;
        }
        zc* wa = col(W, p);
        zc* wb = col(W, q);
        for (int i = 0; i < m; ++i) {
          const zc x = wa[i], y = wb[i] * std::conj(ph);
          wa[i] = c * x - sn * y;
          wb[i] = sn * x + c * y;
        }
      }
    if (!rotated) break;
  }
  std::vector<double> nrm(m);
  for (int j = 0; j < m; ++j) {
    double t = 0.0;
    for (int i = 0; i < m; ++i) t += std::norm(R[(size_t)j * m + i]);
    nrm[j] = std::sqrt(t);
  }
  std::vector<int> ord(m);
  for (int j = 0; j < m; ++j) ord[j] = j;
  std::stable_sort(ord.begin(), ord.end(), [&](int x, int y) { return nrm[x] > nrm[y]; });
  std::vector<zc> Wo((size_t)m * m);
  sv.resize(m);
  for (int j = 0; j < m; ++j) {
    sv[j] = nrm[ord[j]];
    std::copy(W.begin() + (size_t)ord[j] * m, W.begin() + (size_t)(ord[j] + 1) * m, Wo.begin() + (size_t)j * m);
  }
  W.swap(Wo);
}

}  // namespace

extern "C" {

qbg_status qbg_beyn_moments(qbg_beyn* b, const double* V, int64_t L, double* A0, double* A1,
                            qbg_beyn_stats* stats) {
  if (!b || !V || !A0 || !A1 || L < 1 || L > (1 << 20)) {
    set_error("qbg_beyn_moments: invalid arguments");
    return QBG_EINVAL;
  }
  std::lock_guard<std::mutex> lk(b->mu);
  return moments_impl(b, V, L, A0, A1, stats, -1);
}

qbg_status qbg_beyn_moments_qr(qbg_beyn* b, const double* V, int64_t L, int32_t append, int64_t m, double* R,
                               double* C, qbg_beyn_stats* stats) {
  if (!b || !V || !R || !C || L < 1 || L > (1 << 20)) {
    set_error("qbg_beyn_moments_qr: invalid arguments");
    return QBG_EINVAL;
  }
  std::lock_guard<std::mutex> lk(b->mu);
  const int64_t want = (append ? b->mcols : 0) + L;
  if (m != want) {
    set_error("qbg_beyn_moments_qr: m = %lld, the kept blocks will hold %lld columns", (long long)m,
              (long long)want);
    return QBG_EINVAL;
  }
  if (m > b->n) {
    set_error("qbg_beyn_moments_qr: %lld columns exceed the dimension %d", (long long)m, b->n);
    return QBG_EINVAL;
  }
  QBG_TRY(moments_impl(b, V, L, nullptr, nullptr, stats, append ? 1 : 0));
  return qr_reduce(b, R, C);
}

// construct_B_matrix (beyn.jl:257-322) in one call on a single-disk handle:
// moments of V kept on the device, A0 = Q R there, the SVD of R on the host
// (R = U_R S W^H, so A0 = (Q U_R) S W^H), the absolute rank count(S >= svd_tol),
// one regrowth r -> 2r with V2 appended when rk == r and 2r < N, then
// B = U_R,k^H (Q^H A1) W_k S_k^-1 and U_k = A0 W_k S_k^-1 (device product).
qbg_status qbg_beyn_B(qbg_beyn* b, const double* V, int64_t r, const double* V2, double svd_tol, double* B,
                      double* Uk, double* S, int64_t* rk_out, int64_t* r_used, qbg_beyn_stats* stats) {
  if (!b || !V || !B || !rk_out || !r_used || r < 1 || !(svd_tol >= 0.0)) {
    set_error("qbg_beyn_B: invalid arguments");
    return QBG_EINVAL;
  }
  if (b->ndisk != 1) {
    set_error("qbg_beyn_B: the handle holds %d disks; B is formed for single-disk handles", b->ndisk);
    return QBG_EINVAL;
  }
  if (r > b->n) {
    set_error("qbg_beyn_B: r = %lld exceeds the dimension %d", (long long)r, b->n);
    return QBG_EINVAL;
  }
  using zc = std::complex<double>;
  std::lock_guard<std::mutex> lk(b->mu);
  const int n = b->n;
  int m = (int)r;
  std::vector<double> Rh, Ch;
  std::vector<double> sv;
  std::vector<zc> W;
  auto reduce = [&]() -> int {
    Rh.assign(2 * (size_t)m * m, 0.0);
    Ch.assign(2 * (size_t)m * m, 0.0);
    QBG_TRY(qr_reduce(b, Rh.data(), Ch.data()));
    std::vector<zc> R((size_t)m * m);
    for (size_t e = 0; e < R.size(); ++e) R[e] = zc(Rh[2 * e], Rh[2 * e + 1]);
    jacobi_svd(m, R, sv, W);
    return QBG_OK;
  };
  QBG_TRY(moments_impl(b, V, r, nullptr, nullptr, stats, 0));
  QBG_TRY(reduce());
  int rk = 0;
  for (double x : sv) rk += x >= svd_tol;
  if (rk == m && 2 * r < n && V2) {  // beyn.jl:291-309: one regrowth, the loop left after it
    QBG_TRY(moments_impl(b, V2, r, nullptr, nullptr, stats, 1));
    m = 2 * (int)r;
    QBG_TRY(reduce());
    rk = 0;
    for (double x : sv) rk += x >= svd_tol;
  }
  *r_used = m;
  *rk_out = rk;
  if (S)
    for (int j = 0; j < m; ++j) S[j] = sv[j];
  if (rk == 0) return QBG_OK;
  // B = U_R,k^H C W_k S_k^-1 with R = U_R S W^H: U_R,k = R W_k S_k^-1
  std::vector<zc> C((size_t)m * m), Rz((size_t)m * m), Wk((size_t)m * rk), URk((size_t)m * rk), CW((size_t)m * rk);
  for (size_t e = 0; e < C.size(); ++e) {
    C[e] = zc(Ch[2 * e], Ch[2 * e + 1]);
    Rz[e] = zc(Rh[2 * e], Rh[2 * e + 1]);
  }
  for (int j = 0; j < rk; ++j)
    for (int i = 0; i < m; ++i) Wk[(size_t)j * m + i] = W[(size_t)j * m + i] / sv[j];  // W_k S_k^-1
  for (int j = 0; j < rk; ++j)
    for (int i = 0; i < m; ++i) {
      zc u(0.0, 0.0), c(0.0, 0.0);
      for (int l = 0; l < m; ++l) {
        u += Rz[(size_t)l * m + i] * Wk[(size_t)j * m + l];
        c += C[(size_t)l * m + i] * Wk[(size_t)j * m + l];
      }
      URk[(size_t)j * m + i] = u;
      CW[(size_t)j * m + i] = c;
    }
  for (int j = 0; j < rk; ++j)
    for (int i = 0; i < rk; ++i) {
      zc t(0.0, 0.0);
      for (int l = 0; l < m; ++l) t += std::conj(URk[(size_t)i * m + l]) * CW[(size_t)j * m + l];
      B[2 * ((size_t)j * rk + i)] = t.real();
      B[2 * ((size_t)j * rk + i) + 1] = t.imag();
    }
  if (Uk) {  // U_k = A0 W_k S_k^-1 from the kept moments
    cudaStream_t st = b->st;
    cxd *dW = nullptr, *dU = nullptr;
    QBG_TRY(dmalloc(&dW, sizeof(cxd) * (size_t)m * rk));
    const bool dev = (b->opts.flags & QBG_PTR_DEVICE) != 0;
    int s2 = dev ? QBG_OK : dmalloc(&dU, sizeof(cxd) * (size_t)n * rk);
    if (s2) { dfree(dW, st); return s2; }
    cxd* out = dev ? reinterpret_cast<cxd*>(Uk) : dU;
    cudaError_t e = cudaMemcpyAsync(dW, Wk.data(), sizeof(cxd) * Wk.size(), cudaMemcpyHostToDevice, st);
    int s = e == cudaSuccess ? QBG_OK : cuda_status(e, "qbg_beyn_B");
    if (!s)
      s = gemm_batched<double>(n, rk, m, cxd(1, 0), b->macc0, n, 0, dW, m, 0, cxd(0, 0), out, n, 0, 1, st);
    if (!s && !dev) {
      e = cudaMemcpyAsync(Uk, dU, sizeof(cxd) * (size_t)n * rk, cudaMemcpyDeviceToHost, st);
      if (e != cudaSuccess) s = cuda_status(e, "qbg_beyn_B U_k");
    }
    e = cudaStreamSynchronize(st);
    dfree(dW, st);
    if (dU) dfree(dU, st);
    if (s) return s;
    if (e != cudaSuccess) return cuda_status(e, "qbg_beyn_B");
  }
  return QBG_OK;
}

qbg_status qbg_beyn_destroy(qbg_beyn* b) {
  delete b;
  return QBG_OK;
}

}  // extern "C"
