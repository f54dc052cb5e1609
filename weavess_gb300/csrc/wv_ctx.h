// The context behind the C ABI: device memory, stream and rand stream of one
// GPU.  Shared by the translation units that implement the entry points.
#pragma once
#include <cuda_runtime.h>

#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <map>
#include <string>
#include <vector>

#include "../../include/weavess_gpu.h"
#include "wv_host.h"
#include "wv_kdt.h"

namespace wv {

// grow-only device buffer
struct DevBuf {
  void *p = nullptr;
  size_t bytes = 0;
  cudaError_t ensure(size_t want) {
    if (want <= bytes) return cudaSuccess;
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
    cudaError_t e = cudaMalloc(&p, want);
    if (e == cudaSuccess) bytes = want;
    return e;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
  }
  template <class T>
  T *as() const {
    return reinterpret_cast<T *>(p);
  }
};

}  // namespace wv

struct wv_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;      // the stream all work is issued on
  cudaStream_t own_stream = nullptr;  // the context's own stream
  std::string err;
  wv::RandSource rnd;
  int sms = 0;

  // base vectors
  wv::DevBuf base;
  uint32_t n = 0, d = 0;
  bool base_int = false;  // every value an integer in [0, 255]
  wv::DevBuf xnorm;       // squared norm of every base row (when base_int: exact)
  // low-precision copy of the base for candidate distances
  int storage = 0;
  uint32_t rerank = 0;
  // route searches: 0 the exact traversal; E >= 1 the throughput form with
  // E parents expanded per step (wv_set_search_expansion)
  uint32_t parents = 0;
  // builds: 0 the reference's behaviour (compat); 1 clean -- the Vamana
  // link's defects fixed (wv_set_build_mode)
  int build_clean = 0;
  wv::DevBuf qbase, qscale, qnorm;  // qnorm: squared norms of the low-precision rows

  // search graph (load_graph_)
  wv::DevBuf gids, gdeg;
  uint32_t gn = 0, gw = 0, ep = 0;
  std::vector<uint32_t> ep_row;  // host copy of the entry point's row
  std::vector<uint32_t> eps;     // SSG roots (eps_) of the search graph

  // search scratch
  wv::DevBuf visited, touched;
  size_t vis_slots = 0, vis_words = 0;
  wv::DevBuf misc;  // [0] query counter (u32), [8..24) counters (u64 x2), [32] status (i32)

  // per-call staging
  wv::DevBuf q_buf, seed_buf, out_ids_buf, out_dist_buf, lq_buf, kq_buf;

  // the graph the build components pass along (final_graph_): fixed-width
  // rows of (id, distance) with a degree per node, plus the entry point
  wv::DevBuf fg_ids, fg_dist, fg_deg;
  uint32_t fg_n = 0, fg_w = 0, fg_ep = 0;
  bool fg_has_ep = false;
  std::vector<uint32_t> fg_eps;  // SSG roots of the built graph (eps_)

  // HNSW / NSW search graph (wv_hnsw.cu): layer-0 rows and the upper layers
  // in named work buffers; n = 0 while none is loaded
  struct {
    uint32_t n = 0, w0 = 0, wu = 0, ep = 0, max_level = 0, ep_layers = 0;
  } hnsw;

  // KD-trees of the last INIT_KDT on this base (wv_kdt.cu), for the KD-tree
  // search entry; T = 0 while none is built
  wv::KdtForest kdt;

  // learned entry / beam model (wv_learn.cu), or null
  void *learn = nullptr;

  // bumped whenever the base, the search graph, the candidate precision or
  // the learned model change: captured plans hold their pointers and values
  unsigned long long generation = 0;

  // named grow-only work buffers of the build kernels
  std::map<std::string, wv::DevBuf> work;
  template <class T>
  T *buf(const char *name, size_t count, cudaError_t *err) {
    cudaError_t e = work[name].ensure(count * sizeof(T) + 16);
    if (e != cudaSuccess && err) *err = e;
    return work[name].as<T>();
  }

  unsigned *d_next() { return misc.as<unsigned>(); }
  unsigned long long *d_counters() { return reinterpret_cast<unsigned long long *>(misc.as<char>() + 8); }
  int *d_status() { return reinterpret_cast<int *>(misc.as<char>() + 32); }
  void release_work() {
    for (auto &kv : work) kv.second.release();
    work.clear();
  }
};

namespace wv {

inline int fail(wv_ctx *c, int code, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  if (c) c->err = buf;
  return code;
}

#define WV_CUDA(ctx, call)                                                                         \
  do {                                                                                             \
    cudaError_t e_ = (call);                                                                       \
    if (e_ != cudaSuccess)                                                                         \
      return ::wv::fail(ctx, e_ == cudaErrorMemoryAllocation ? WV_ERR_NOMEM : WV_ERR_CUDA, "%s: %s (%s:%d)", #call, \
                        cudaGetErrorString(e_), __FILE__, __LINE__);                               \
  } while (0)

#define WV_CHECK(ctx, cond, code, ...)                      \
  do {                                                      \
    if (!(cond)) return ::wv::fail(ctx, code, __VA_ARGS__); \
  } while (0)

// reads the device status word after a launch; maps kernel-reported errors
int check_device_status(wv_ctx *c, const char *what);

}  // namespace wv

#include "wv_search.h"

namespace wv {

// visited-set scratch for `shape` at beams up to Lmax (may allocate: call it
// before a stream capture); *blocks = the persistent grid of that shape
int search_prepare(wv_ctx *c, uint32_t Lmax, SearchShape shape, int *blocks);
// the kernel arguments of a search on device-resident buffers (nq_dev: the
// query count read on the device, or null)
SearchArgs search_args(wv_ctx *c, const float *d_q, uint32_t nq, const uint32_t *nq_dev, const uint32_t *d_seeds,
                       uint32_t seed_stride, const uint32_t *d_L, const uint32_t *d_K, uint32_t L, uint32_t K,
                       uint32_t Lmax, uint32_t *d_out, float *d_dist, uint32_t out_stride);
// clears the query counter and the counters, launches; nothing synchronizes
// (capturable once search_prepare ran)
// persistent grid of a route search at beams up to Lmax in shape sh: the
// exact kernel's, or the throughput form's when the context expands E > 0
// parents per step
int route_grid(wv_ctx *c, uint32_t Lmax, SearchShape sh);
int search_enqueue(wv_ctx *c, const SearchArgs &a, SearchShape shape, int blocks);

// records `ev` on `s`; inside a stream capture as an event node of the graph
// (so that replays time it), outside as a plain record
inline cudaError_t record_event(cudaEvent_t ev, cudaStream_t s) {
  cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
  cudaError_t e = cudaStreamIsCapturing(s, &st);
  if (e != cudaSuccess) return e;
  return st == cudaStreamCaptureStatusActive ? cudaEventRecordWithFlags(ev, s, cudaEventRecordExternal)
                                             : cudaEventRecord(ev, s);
}

// visited-set scratch owned by someone other than the context (a plan)
struct SearchScratch {
  uint32_t *visited = nullptr, *touched = nullptr;
  uint32_t words = 0;
};

// the search kernel on device-resident queries / seeds / outputs (per-query
// L and K optional); counters (nullable) are read back.  shift_seeds: seed
// distances as SearchEntrySubCentroid takes them
int run_search_device(wv_ctx *c, const float *d_q, uint32_t nq, const uint32_t *d_seeds, uint32_t seed_stride,
                      const uint32_t *d_L, const uint32_t *d_K, uint32_t L, uint32_t K, uint32_t Lmax, uint32_t *d_out,
                      float *d_dist, uint32_t out_stride, wv_counters *counters, bool shift_seeds = false);

}  // namespace wv
