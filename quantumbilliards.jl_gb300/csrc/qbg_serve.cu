// Request server: HBM-budget admission, worker threads with their own CUDA
// streams, and continuous batching of Beyn requests (qbg_serve_* in qbgpu.h).
//
// Scheduling. The queue is first-come first-served with a bounded look-ahead:
// a worker takes the first of the next 16 queued requests whose estimated
// device footprint fits the free budget, but once the head has been passed
// over 8 times only the head may start (no starvation of large requests).
// sigma_min sweeps are background work: at most max_sweeps of them run at
// once, and a queued sweep over that limit is passed over without counting as
// a pass of the head (it starts when the running sweep ends). Three sweeps in
// flight would hold three of four workers and every FP64 pipe of the device
// for seconds, and the Beyn and EBIM requests behind them would queue.
// A Beyn request picks up every later queued Beyn request on the same
// geometry with the same nq, precision and probe count (up to max_batch, as
// long as the merged footprint fits): their contour nodes run as one
// multi-disk device batch (qbg_beyn_create_disks) with one probe block per
// disk, so requests join a batch as they arrive instead of waiting for a
// batch to fill.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "qbg_handles.cuh"

using namespace qbg;

namespace {

using Clock = std::chrono::steady_clock;

struct Req {
  int64_t id = 0;
  qbg_request_desc d{};
  int64_t n = 0;        // operator dimension
  size_t bytes = 0;     // estimated device footprint when run alone
  bool done = false;
  int32_t status = QBG_OK;
  int32_t batched = 1;
  std::string err;
  Clock::time_point t_submit, t_start, t_end;
};

// Estimated device bytes of a Beyn batch of nn contour nodes (operators,
// LU workspaces, Chebyshev tables, the per-call solve buffers).
size_t est_beyn(int64_t n, int64_t nn, int64_t L, int prec) {
  const double N = (double)n, N2 = N * N;
  const double tables = 3.6e6;  // 15000 x 6 + 3000 x 6 panels of two complex128 series per node
  double per_node = (prec == QBG_PREC_FP64) ? 16.0 * N2 + 1024.0 * N + 16.0 * N * L + tables
                                            : 24.0 * N2 + 9216.0 * N + 56.0 * N * L + tables;
  const double per_call = 48.0 * N * L + 64.0 * N;
  return (size_t)(1.1 * (per_node * nn + per_call)) + (64u << 20);
}

size_t estimate(const qbg_request_desc& d, int64_t n) {
  const double N2 = (double)n * n;
  switch (d.kind) {
    case QBG_REQ_BEYN:
      return est_beyn(n, d.nq, d.L, d.prec);
    case QBG_REQ_EBIM:
      return (size_t)(1.1 * 3.0 * 16.0 * N2) + (64u << 20);
    default: {
      const double chunk = (double)std::min<int64_t>(d.nk, 16);
      return (size_t)(1.1 * (chunk * 16.0 * N2 + 64.0 * n)) + (64u << 20);
    }
  }
}

bool same_batch(const Req& a, const Req& b) {
  return a.d.kind == QBG_REQ_BEYN && b.d.kind == QBG_REQ_BEYN && a.d.geom == b.d.geom && a.d.nq == b.d.nq &&
         a.d.prec == b.d.prec && a.d.L == b.d.L;
}

}  // namespace

struct qbg_server {
  qbg_serve_opts opts{};
  size_t budget = 0, in_use = 0;
  int device = 0;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<std::shared_ptr<Req>> queue;
  std::unordered_map<int64_t, std::shared_ptr<Req>> all;
  std::vector<std::thread> workers;
  bool stop = false;
  int64_t next_id = 1;
  int head_skips = 0;
  int sweeps_running = 0;

  bool held_back(const Req& r) const {
    const int cap = opts.max_sweeps > 0 ? opts.max_sweeps : 1;
    return r.d.kind == QBG_REQ_SWEEP && sweeps_running >= cap;
  }

  // with mu held: the requests to run next (empty if nothing fits)
  std::vector<std::shared_ptr<Req>> pick(size_t* bytes) {
    std::vector<std::shared_ptr<Req>> out;
    size_t head = 0;  // the first request that may start now
    while (head < queue.size() && held_back(*queue[head])) ++head;
    if (head == queue.size()) return out;
    const size_t look = head_skips >= 8 ? head + 1 : std::min<size_t>(queue.size(), head + 16);
    size_t at = queue.size();
    for (size_t q = head; q < look; ++q)
      if (!held_back(*queue[q]) && in_use + queue[q]->bytes <= budget) {
        at = q;
        break;
      }
    if (at == queue.size()) return out;
    head_skips = at == head ? 0 : head_skips + 1;
    std::shared_ptr<Req> first = queue[at];
    if (first->d.kind == QBG_REQ_SWEEP) ++sweeps_running;
    out.push_back(first);
    std::vector<size_t> taken{at};
    size_t total = first->bytes;
    if (first->d.kind == QBG_REQ_BEYN) {
      const int maxb = opts.max_batch > 0 ? opts.max_batch : 8;
      for (size_t q = at + 1; q < queue.size() && (int)out.size() < maxb; ++q) {
        if (!same_batch(*first, *queue[q])) continue;
        const size_t merged = est_beyn(first->n, (int64_t)(out.size() + 1) * first->d.nq, first->d.L, first->d.prec);
        if (in_use + merged > budget) break;
        out.push_back(queue[q]);
        taken.push_back(q);
        total = merged;
      }
    }
    for (size_t q = taken.size(); q-- > 0;) queue.erase(queue.begin() + (long)taken[q]);
    *bytes = total;
    return out;
  }
};

namespace {

void finish(std::vector<std::shared_ptr<Req>>& group, int32_t status, const char* err) {
  const auto t = Clock::now();
  for (auto& r : group) {
    r->status = status;
    r->batched = (int32_t)group.size();
    r->t_end = t;
    if (status != QBG_OK && err) r->err = err;
  }
}

std::string last_error() {
  char buf[1024];
  buf[0] = 0;
  qbg_last_error(buf, sizeof(buf));
  return buf;
}

int32_t run_beyn(std::vector<std::shared_ptr<Req>>& group) {
  const qbg_request_desc& d0 = group[0]->d;
  const int nd = (int)group.size();
  const int64_t n = group[0]->n;
  const size_t nl = (size_t)n * (size_t)d0.L;
  std::vector<double> k0s(2 * nd), Rs(nd);
  for (int q = 0; q < nd; ++q) {
    k0s[2 * q] = group[q]->d.k0_re;
    k0s[2 * q + 1] = group[q]->d.k0_im;
    Rs[q] = group[q]->d.R;
  }
  qbg_beyn_opts o{};
  o.flags = nd > 1 ? QBG_V_PER_DISK : 0;
  qbg_beyn* h = nullptr;
  int32_t s = qbg_beyn_create_disks(d0.geom, k0s.data(), Rs.data(), nd, d0.nq, d0.prec, &o, &h);
  if (s) return s;
  if (nd == 1) {
    s = qbg_beyn_moments(h, d0.V, d0.L, d0.A0, d0.A1, nullptr);
  } else {
    std::vector<double> V(2 * nl * nd), A0(2 * nl * nd), A1(2 * nl * nd);
    for (int q = 0; q < nd; ++q) std::memcpy(V.data() + 2 * nl * q, group[q]->d.V, sizeof(double) * 2 * nl);
    s = qbg_beyn_moments(h, V.data(), d0.L, A0.data(), A1.data(), nullptr);
    if (!s)
      for (int q = 0; q < nd; ++q) {
        std::memcpy(group[q]->d.A0, A0.data() + 2 * nl * q, sizeof(double) * 2 * nl);
        std::memcpy(group[q]->d.A1, A1.data() + 2 * nl * q, sizeof(double) * 2 * nl);
      }
  }
  std::string err = s ? last_error() : std::string();
  qbg_beyn_destroy(h);
  if (s) set_error("%s", err.c_str());
  return s;
}

int32_t run_one(const qbg_request_desc& d) {
  if (d.kind == QBG_REQ_EBIM) {
    const double k[2] = {d.k, 0.0};
    void* outs[3] = {d.out_A, d.out_dA, d.out_ddA};
    return qbg_assemble(d.geom, k, 1, 1, QBG_PREC_FP64, 0, outs);
  }
  return qbg_sigma_min(d.geom, d.ks, d.nk, d.sig);
}

void worker(qbg_server* srv) {
  cudaSetDevice(srv->device);
  std::unique_lock<std::mutex> lk(srv->mu);
  for (;;) {
    size_t bytes = 0;
    std::vector<std::shared_ptr<Req>> group;
    srv->cv_work.wait(lk, [&] {
      if (srv->stop && srv->queue.empty()) return true;
      group = srv->pick(&bytes);
      return !group.empty();
    });
    if (group.empty()) return;  // stopping, nothing queued
    srv->in_use += bytes;
    lk.unlock();
    const auto t0 = Clock::now();
    for (auto& r : group) r->t_start = t0;
    int32_t s = group[0]->d.kind == QBG_REQ_BEYN ? run_beyn(group) : run_one(group[0]->d);
    const std::string err = s ? last_error() : std::string();
    lk.lock();
    finish(group, s, err.c_str());
    for (auto& r : group) r->done = true;
    srv->in_use -= bytes;
    if (group[0]->d.kind == QBG_REQ_SWEEP) --srv->sweeps_running;
    srv->cv_done.notify_all();
    srv->cv_work.notify_all();
  }
}

}  // namespace

extern "C" {

qbg_status qbg_serve_create(const qbg_serve_opts* opts, qbg_server** out) {
  if (!out) {
    set_error("qbg_serve_create: null output");
    return QBG_EINVAL;
  }
  *out = nullptr;
  int dev = 0;
  size_t free_b = 0, total_b = 0;
  QBG_CUDA(cudaGetDevice(&dev));
  QBG_CUDA(cudaMemGetInfo(&free_b, &total_b));
  qbg_server* srv = new (std::nothrow) qbg_server();
  if (!srv) {
    set_error("host allocation failed");
    return QBG_ENOMEM;
  }
  if (opts) srv->opts = *opts;
  srv->device = dev;
  srv->budget = srv->opts.hbm_budget > 0 ? (size_t)srv->opts.hbm_budget : (size_t)(0.8 * (double)free_b);
  const int nw = srv->opts.workers > 0 ? srv->opts.workers : 4;
  for (int q = 0; q < nw; ++q) srv->workers.emplace_back(worker, srv);
  *out = srv;
  return QBG_OK;
}

qbg_status qbg_serve_submit(qbg_server* srv, const qbg_request_desc* req, int64_t* id) {
  if (!srv || !req || !id || !req->geom) {
    set_error("qbg_serve_submit: invalid arguments");
    return QBG_EINVAL;
  }
  const qbg_request_desc& d = *req;
  int64_t n = 0;
  QBG_TRY(qbg_geom_dim(d.geom, &n));
  bool ok = true;
  switch (d.kind) {
    case QBG_REQ_BEYN:
      ok = d.V && d.A0 && d.A1 && d.L >= 1 && d.nq >= 2 && d.R > 0.0 && d.prec >= 0 && d.prec <= 2;
      break;
    case QBG_REQ_EBIM:
      ok = d.out_A && d.out_dA && d.out_ddA && d.k != 0.0;
      break;
    case QBG_REQ_SWEEP:
      ok = d.ks && d.sig && d.nk >= 1;
      break;
    default:
      ok = false;
  }
  if (!ok) {
    set_error("qbg_serve_submit: invalid request");
    return QBG_EINVAL;
  }
  auto r = std::make_shared<Req>();
  r->d = d;
  r->n = n;
  r->bytes = estimate(d, n);
  r->t_submit = Clock::now();
  std::lock_guard<std::mutex> lk(srv->mu);
  if (r->bytes > srv->budget) {
    set_error("request needs about %zu bytes of device memory, the budget is %zu", r->bytes, srv->budget);
    return QBG_EBUDGET;
  }
  if (srv->stop) {
    set_error("the server is stopping");
    return QBG_EINVAL;
  }
  r->id = srv->next_id++;
  srv->all[r->id] = r;
  srv->queue.push_back(r);
  *id = r->id;
  srv->cv_work.notify_one();
  return QBG_OK;
}

qbg_status qbg_serve_poll(qbg_server* srv, int64_t id, int32_t* done) {
  if (!srv || !done) {
    set_error("qbg_serve_poll: invalid arguments");
    return QBG_EINVAL;
  }
  std::lock_guard<std::mutex> lk(srv->mu);
  auto it = srv->all.find(id);
  if (it == srv->all.end()) {
    set_error("unknown request id %lld", (long long)id);
    return QBG_EINVAL;
  }
  *done = it->second->done ? 1 : 0;
  return QBG_OK;
}

qbg_status qbg_serve_wait(qbg_server* srv, int64_t id, double timeout_s, qbg_request_result* res) {
  if (!srv) {
    set_error("qbg_serve_wait: invalid arguments");
    return QBG_EINVAL;
  }
  std::unique_lock<std::mutex> lk(srv->mu);
  auto it = srv->all.find(id);
  if (it == srv->all.end()) {
    set_error("unknown request id %lld", (long long)id);
    return QBG_EINVAL;
  }
  std::shared_ptr<Req> r = it->second;
  auto ready = [&] { return r->done; };
  if (timeout_s < 0) {
    srv->cv_done.wait(lk, ready);
  } else if (!srv->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), ready)) {
    set_error("request %lld still running", (long long)id);
    return QBG_ETIMEOUT;
  }
  if (res) {
    res->status = r->status;
    res->batched = r->batched;
    res->queue_ms = std::chrono::duration<double, std::milli>(r->t_start - r->t_submit).count();
    res->run_ms = std::chrono::duration<double, std::milli>(r->t_end - r->t_start).count();
  }
  if (r->status != QBG_OK) set_error("%s", r->err.c_str());
  srv->all.erase(id);
  return QBG_OK;
}

qbg_status qbg_serve_destroy(qbg_server* srv) {
  if (!srv) return QBG_OK;
  {
    std::lock_guard<std::mutex> lk(srv->mu);
    srv->stop = true;
  }
  srv->cv_work.notify_all();
  for (auto& t : srv->workers) t.join();
  delete srv;
  return QBG_OK;
}

}  // extern "C"
