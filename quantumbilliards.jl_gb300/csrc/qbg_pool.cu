// Caching device allocator of the library.
//
// Every device buffer of the library (geometry uploads, Beyn operator slots,
// per-call scratch, staging) comes from here. A freed block is kept, keyed by
// its rounded size, and handed to the next request of that size class, so a
// sequence of same-shaped calls (contour after contour, request after request
// in the server) stops paying cudaMalloc/cudaFree, whose page mapping and
// implicit device synchronisation cost milliseconds per gigabyte.
//
// Stream safety: a block freed with the stream whose work last used it
// records an event there and is reused only after that event has completed;
// a block freed without a stream waits for the whole device first (the
// guarantee cudaFree gave). Sizes round up to 512 B, or to 2 MiB from 1 MiB
// on; a request takes a cached block of its class up to 1/8 larger.
//
// The cache holds at most QBG_POOL_BYTES bytes (environment, decimal; default
// a quarter of the device memory; 0 disables caching). When cudaMalloc runs
// out of memory the cache is emptied and the allocation retried once;
// qbg_pool_release() empties it on request.
#include <cstdlib>
#include <map>
#include <mutex>
#include <unordered_map>
#include <vector>
#include "qbg_common.cuh"
#include "qbg_handles.cuh"
#include "qbgpu.h"

namespace qbg {
namespace {

struct FreeBlock {
  void* p;
  int dev;
  cudaEvent_t ev;  // nullptr: reusable at once
};

struct Pool {
  std::mutex mu;
  std::unordered_map<void*, std::pair<size_t, int>> live;  // pointer -> (rounded size, device)
  std::multimap<size_t, FreeBlock> cached;
  std::vector<cudaEvent_t> spare_events;
  size_t cached_bytes = 0, live_bytes = 0;
  long long limit = -1;  // resolved on first use
  unsigned long long hits = 0, misses = 0;
};

Pool& pool() {
  static Pool* p = new Pool;  // never destroyed: no CUDA calls during static teardown
  return *p;
}

size_t round_size(size_t b) {
  if (b == 0) b = 1;
  if (b < (1u << 20)) return (b + 511) & ~(size_t)511;
  const size_t g = (size_t)2 << 20;
  return (b + g - 1) / g * g;
}

void resolve_limit(Pool& P) {
  if (P.limit >= 0) return;
  const char* env = std::getenv("QBG_POOL_BYTES");
  if (env && *env) {
    P.limit = std::strtoll(env, nullptr, 10);
    if (P.limit < 0) P.limit = 0;
    return;
  }
  size_t fr = 0, tot = 0;
  P.limit = (cudaMemGetInfo(&fr, &tot) == cudaSuccess) ? (long long)(tot / 4) : (1ll << 34);
}

// a pending event query leaves nothing behind in the runtime's last-error slot
bool event_done(cudaEvent_t ev) {
  if (!ev) return true;
  const cudaError_t e = cudaEventQuery(ev);
  if (e == cudaSuccess) return true;
  if (cudaPeekAtLastError() == cudaErrorNotReady) (void)cudaGetLastError();
  return false;
}

void drop_block(Pool& P, std::multimap<size_t, FreeBlock>::iterator it) {
  FreeBlock fb = it->second;
  if (fb.ev) {
    cudaEventSynchronize(fb.ev);
    P.spare_events.push_back(fb.ev);
  }
  int cur = 0;
  cudaGetDevice(&cur);
  if (cur != fb.dev) cudaSetDevice(fb.dev);
  cudaFree(fb.p);
  if (cur != fb.dev) cudaSetDevice(cur);
  P.cached_bytes -= it->first;
  P.cached.erase(it);
}

void release_all(Pool& P) {
  while (!P.cached.empty()) drop_block(P, P.cached.begin());
}

}  // namespace

int pool_alloc(void** out, size_t bytes) {
  Pool& P = pool();
  const size_t rs = round_size(bytes);
  int dev = 0;
  QBG_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(P.mu);
  resolve_limit(P);
  const size_t hi = rs >= ((size_t)1 << 20) ? rs + rs / 8 : rs;
  for (auto it = P.cached.lower_bound(rs); it != P.cached.end() && it->first <= hi; ++it) {
    if (it->second.dev != dev || !event_done(it->second.ev)) continue;
    *out = it->second.p;
    if (it->second.ev) P.spare_events.push_back(it->second.ev);
    P.live[*out] = {it->first, dev};
    P.cached_bytes -= it->first;
    P.live_bytes += it->first;
    P.cached.erase(it);
    ++P.hits;
    return QBG_OK;
  }
  ++P.misses;
  cudaError_t e = cudaMalloc(out, rs);
  if (e == cudaErrorMemoryAllocation && !P.cached.empty()) {
    (void)cudaGetLastError();
    release_all(P);
    e = cudaMalloc(out, rs);
  }
  if (e != cudaSuccess) {
    *out = nullptr;
    return cuda_status(e, "cudaMalloc");
  }
  P.live[*out] = {rs, dev};
  P.live_bytes += rs;
  return QBG_OK;
}

void pool_free(void* p, cudaStream_t st) {
  if (!p) return;
  Pool& P = pool();
  size_t rs = 0;
  int dev = 0;
  {
    std::lock_guard<std::mutex> lk(P.mu);
    auto it = P.live.find(p);
    if (it == P.live.end()) {  // not from the pool
      cudaFree(p);
      return;
    }
    rs = it->second.first;
    dev = it->second.second;
    P.live.erase(it);
    P.live_bytes -= rs;
    resolve_limit(P);
    if ((long long)rs > P.limit) {
      if (st) cudaStreamSynchronize(st);
      cudaFree(p);
      return;
    }
  }
  // the wait that gates reuse happens outside the lock: a device-wide wait
  // must not hold up the other threads' allocations
  cudaEvent_t ev = nullptr;
  if (st) {
    {
      std::lock_guard<std::mutex> lk(P.mu);
      if (!P.spare_events.empty()) {
        ev = P.spare_events.back();
        P.spare_events.pop_back();
      }
    }
    if (!ev && cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) != cudaSuccess) ev = nullptr;
    if (ev && cudaEventRecord(ev, st) != cudaSuccess) {
      cudaEventDestroy(ev);
      ev = nullptr;
      cudaStreamSynchronize(st);
    }
  } else {
    cudaDeviceSynchronize();
  }
  std::lock_guard<std::mutex> lk(P.mu);
  P.cached.emplace(rs, FreeBlock{p, dev, ev});
  P.cached_bytes += rs;
  // over the limit: return the largest blocks to the driver
  while ((long long)P.cached_bytes > P.limit && !P.cached.empty()) drop_block(P, std::prev(P.cached.end()));
}

}  // namespace qbg

extern "C" {

qbg_status qbg_pool_release(void) {
  qbg::Pool& P = qbg::pool();
  std::lock_guard<std::mutex> lk(P.mu);
  qbg::release_all(P);
  return QBG_OK;
}

qbg_status qbg_pool_stats(uint64_t* cached_bytes, uint64_t* live_bytes, uint64_t* hits, uint64_t* misses) {
  qbg::Pool& P = qbg::pool();
  std::lock_guard<std::mutex> lk(P.mu);
  if (cached_bytes) *cached_bytes = P.cached_bytes;
  if (live_bytes) *live_bytes = P.live_bytes;
  if (hits) *hits = P.hits;
  if (misses) *misses = P.misses;
  return QBG_OK;
}

}  // extern "C"
