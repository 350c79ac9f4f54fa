// Definitions of the opaque C-ABI handles shared by the translation units that
// implement entry points on them.
#pragma once
#include <mutex>
#include <vector>
#include "qbg_common.cuh"
#include "qbg_geom.cuh"
#include "qbg_assemble.cuh"

namespace qbg {
// caching allocator (qbg_pool.cu)
int pool_alloc(void** p, size_t bytes);
// st: the stream whose work last used p (its completion gates reuse);
// nullptr waits for the whole device before the block is cached
void pool_free(void* p, cudaStream_t st);

template <class P>
inline int dmalloc(P** p, size_t bytes) {
  void* q = nullptr;
  const int s = pool_alloc(&q, bytes);
  *p = static_cast<P*>(q);
  return s;
}
inline void dfree(void* p, cudaStream_t st = nullptr) { pool_free(p, st); }
// returns the tensor-core GEMM's packing scratch of a stream (qbg_tc_gemm.cu)
void tc_release_scratch(cudaStream_t st);
}  // namespace qbg

struct qbg_geom {
  qbg::GeomDev d;
  int64_t dim = 0;
  std::vector<void*> allocs;
  cudaStream_t stream = nullptr;
  std::mutex mu;
  ~qbg_geom() {
    for (void* p : allocs) qbg::dfree(p, stream);
    if (stream) {
      qbg::tc_release_scratch(stream);
      cudaStreamDestroy(stream);
    }
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

namespace qbg {
// host-side helpers shared by the entry-point translation units
int check_ks(const double* ks, int64_t nk);  // finite, non-zero complex wavenumbers
int cheb_params_check(const qbg_cheb_params* prm);
qbg_cheb_params cheb_defaults(const qbg_cheb_params* prm);  // zeros -> 15000, 5, 3000, 5
// Chebyshev tables for nk device wavenumbers (device buffers appended to tmp)
int make_cheb(qbg_geom* g, const cxd* dks, int nk, const qbg_cheb_params& prm, ChebTables& t,
              std::vector<void*>& tmp, cudaStream_t st);
// double-float tables of t for the complex64 forms (after make_cheb; buffers appended to tmp)
int make_cheb_df(ChebTables& t, const cxd* dks, std::vector<void*>& tmp, cudaStream_t st);
// the J/E tables alone (instead of make_cheb + make_cheb_df) where cheb_je_applies
int make_cheb_je(qbg_geom* g, const cxd* dks, int nk, const qbg_cheb_params& prm, ChebTables& t,
                 std::vector<void*>& tmp, cudaStream_t st);
}  // namespace qbg
