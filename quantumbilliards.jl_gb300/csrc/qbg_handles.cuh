// Definitions of the opaque C-ABI handles shared by the translation units that
// implement entry points on them.
#pragma once
#include <mutex>
#include <vector>
#include "qbg_common.cuh"
#include "qbg_geom.cuh"

namespace qbg {
template <class P>
inline int dmalloc(P** p, size_t bytes) {
  cudaError_t e = cudaMalloc((void**)p, bytes ? bytes : 1);
  if (e != cudaSuccess) {
    *p = nullptr;
    return cuda_status(e, "cudaMalloc");
  }
  return QBG_OK;
}
}  // namespace qbg

struct qbg_geom {
  qbg::GeomDev d;
  int64_t dim = 0;
  std::vector<void*> allocs;
  cudaStream_t stream = nullptr;
  std::mutex mu;
  ~qbg_geom() {
    for (void* p : allocs) cudaFree(p);
    if (stream) cudaStreamDestroy(stream);
  }
  template <class P>
  int upload(const P* host, size_t count, const P** dev) {
    P* p = nullptr;
    int s = qbg::dmalloc(&p, count * sizeof(P));
    if (s) return s;
    allocs.push_back(p);
    QBG_CUDA(cudaMemcpyAsync(p, host, count * sizeof(P), cudaMemcpyHostToDevice, stream));
    *dev = p;
    return QBG_OK;
  }
};
