// qbg_assemble_noalloc: operator assembly that allocates no device memory.
//
// Who needs it: callers that own all device memory themselves and may not
// call cudaMalloc while they run — a host application that hands the library
// slices of its own pre-reserved memory arena (a Julia CuArray pool, a serving
// process that reserved its HBM budget up front), or a latency-critical loop in
// which a cudaMalloc/cudaFree (which can synchronise the device and stall the
// other streams) is not acceptable. qbg_assemble stages its wavenumber list and
// its table of output pointers in freshly allocated device buffers; this entry
// point stages both in a fixed, file-scope device array instead.
//
// Limits and sharing rules:
//  * at most QBG_NOALLOC_MAX_K wavenumbers per call (each output table holds
//    up to 3 * QBG_NOALLOC_MAX_K pointers when derivatives are requested);
//    larger requests are rejected with QBG_EINVAL;
//  * the scratch array (20 KiB) is resident on every device that loads the
//    library, until the process exits;
//  * all calls share the array, which keeps the last call's contents; nothing
//    in it needs to start at zero because every call overwrites what it reads.
//    Calls that overlap on the GPU would race on it: calls made through this
//    entry point are serialised inside the process and each returns only after
//    its kernel has finished;
//  * Alpert geometries are accepted in FP64 only: their complex64 forms stage
//    FP64 blocks of N^2 entries per wavenumber, which a fixed array cannot
//    hold, so that combination returns QBG_ENOTSUP;
//  * the first call on a device resolves the array's device address for that
//    device (cudaGetSymbolAddress with that device current); make that first
//    call before any stream capture on the device.
#include <mutex>
#include <cstring>

#include "qbg_assemble.cuh"
#include "qbg_handles.cuh"

namespace {

constexpr int kMaxK = QBG_NOALLOC_MAX_K;
constexpr size_t kKsBytes = sizeof(cxd) * kMaxK;         // wavenumbers (complex128)
constexpr size_t kPtrBytes = sizeof(void*) * 3 * kMaxK;        // output pointer table
constexpr size_t kScratchBytes = kKsBytes + kPtrBytes;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mu;                       // serialises every call of the entry point
void* g_scratch_addr[kMaxDevices] = {};  // device address of g_noalloc_scratch, per device

// Resolve (once per device, with that device current) the device address of the
// scratch array. The host-side symbol itself is only a stand-in and must never
// be handed to a kernel.
int scratch_for_current_device(void** out) {
  int dev = -1;
  QBG_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) {
    qbg::set_error("qbg_assemble_noalloc: device ordinal %d outside the supported range", dev);
    return QBG_EINVAL;
  }
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return qbg::cuda_status(e, "cudaGetSymbolAddress(noalloc scratch)");
    g_scratch_addr[dev] = p;
  }
  *out = g_scratch_addr[dev];
  return QBG_OK;
}

}  // namespace

extern "C" qbg_status qbg_assemble_noalloc(qbg_geom* g, const double* ks, int64_t nk, int32_t deriv, int32_t prec,
                                           void* const* outs_dev) {
  if (!g || !ks || !outs_dev || nk < 1 || (deriv != 0 && deriv != 1) || prec < 0 || prec > 2) {
    qbg::set_error("qbg_assemble_noalloc: invalid arguments");
    return QBG_EINVAL;
  }
  if (nk > kMaxK) {
    qbg::set_error("qbg_assemble_noalloc: %lld wavenumbers requested, the fixed scratch holds at most %d",
                   (long long)nk, kMaxK);
    return QBG_EINVAL;
  }
  for (int64_t q = 0; q < 2 * nk; ++q)
    if (!std::isfinite(ks[q])) {
      qbg::set_error("qbg_assemble_noalloc: non-finite wavenumber at index %lld", (long long)(q / 2));
      return QBG_EINVAL;
    }
  for (int64_t q = 0; q < nk; ++q)
    if (ks[2 * q] == 0.0 && ks[2 * q + 1] == 0.0) {
      qbg::set_error("qbg_assemble_noalloc: wavenumber k = 0 is not allowed");
      return QBG_EINVAL;
    }
  const int nout = (int)nk * (1 + 2 * deriv);
  for (int o = 0; o < nout; ++o)
    if (!outs_dev[o]) {
      qbg::set_error("qbg_assemble_noalloc: output pointer %d is null", o);
      return QBG_EINVAL;
    }
  if (g->d.quad == 1 && prec != QBG_PREC_FP64) {
    // the complex64 Alpert forms accumulate their corrections in FP64 staging
    // blocks of N^2 entries per wavenumber, far larger than a fixed array
    qbg::set_error("qbg_assemble_noalloc: Alpert geometries are assembled without allocation in FP64 only");
    return QBG_ENOTSUP;
  }
  std::lock_guard<std::mutex> lk_all(g_mu);
  std::lock_guard<std::mutex> lk(g->mu);
  void* base = nullptr;
  int s = scratch_for_current_device(&base);
  if (s) return s;
  cxd* dks = reinterpret_cast<cxd*>(base);
  void** dptrs = reinterpret_cast<void**>(static_cast<unsigned char*>(base) + kKsBytes);
  cudaStream_t st = g->stream;
  // From the first queued copy on, every return waits for the stream: the next
  // call (possibly on another geometry's stream) overwrites the same array.
  cudaError_t e = cudaMemcpyAsync(dks, ks, sizeof(cxd) * nk, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dptrs, outs_dev, sizeof(void*) * nout, cudaMemcpyHostToDevice, st);
  s = e == cudaSuccess ? QBG_OK : qbg::cuda_status(e, "qbg_assemble_noalloc staging copy");
  if (!s) s = qbg::launch_assemble(g->d, dks, (int)nk, deriv, prec, dptrs, g->dim, st);
  const cudaError_t es = cudaStreamSynchronize(st);
  if (s) return s;
  if (es != cudaSuccess) return qbg::cuda_status(es, "qbg_assemble_noalloc");
  return QBG_OK;
}
