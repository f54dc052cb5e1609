// Allocation-free variant of the greedy beam search.
//
// Some callers cannot call cudaMalloc: a process whose GPU memory is owned
// by another allocator (a serving stack that reserves its pool up front and
// forbids driver allocations afterwards), or a latency-critical thread where
// cudaMalloc / cudaFree would implicitly synchronize the device.  For them
// wv_search_noalloc runs the same search kernel as wv_search_device, with all
// inputs and outputs supplied by the caller in device memory, and its working
// memory (the per-warp visited bitsets and their touched-word lists, the
// query counter and the status word) taken from one file-scope
// `static __device__` array instead of a context.
//
// The array is NOALLOC_SCRATCH_WORDS 32-bit words (64 MiB).  Every GPU that
// loads this library holds it until the process exits.  Every call shares
// it and it keeps the last call's contents, so each call first clears the
// part that must start at zero; two calls whose work overlaps on the GPU
// (different streams, or different host threads) race on it.
//
// Each warp slot of the launch takes a visited bitset and a touched-word
// list of n / 32 words each from the array, and a launch has at least one
// block of search_warps_per_block() = 4 slots, so n is limited to about 67
// million nodes ((16M - 64) / 8 words per bitset).
//
// Host code cannot use the array's name as a device address (it names a
// host-side stand-in), so the first call on each device looks the address up
// with cudaGetSymbolAddress while that device is current, and later calls on
// that device reuse it.  Make that first call before any stream capture.
// The kept address does not survive a cudaDeviceReset (the module is
// unloaded with the context); a process that resets a device must not call
// this entry point on it again.  Each call waits for its stream (the
// kernel's status word is read back before it returns).
#include <mutex>

#include "wv_common.cuh"
#include "wv_ctx.h"
#include "wv_search.h"

namespace {

constexpr size_t NOALLOC_SCRATCH_WORDS = (size_t)16 << 20;  // 64 MiB
constexpr size_t NOALLOC_HEADER_WORDS = 64;                // [0] query counter, [1] status

static __device__ __align__(256) uint32_t g_noalloc_scratch[NOALLOC_SCRATCH_WORDS];

constexpr int MAX_DEVICES = 64;
std::mutex g_setup_mu;
uint32_t *g_scratch_addr[MAX_DEVICES] = {nullptr};

// device address of the scratch array on the current device (set-up once)
int scratch_address(int dev, uint32_t **out) {
  if (dev < 0 || dev >= MAX_DEVICES) return WV_ERR_LIMIT;
  std::lock_guard<std::mutex> g(g_setup_mu);
  if (!g_scratch_addr[dev]) {
    void *p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return WV_ERR_CUDA;
    g_scratch_addr[dev] = static_cast<uint32_t *>(p);
  }
  *out = g_scratch_addr[dev];
  return WV_OK;
}

}  // namespace

extern "C" int wv_search_noalloc(const float *d_base, uint32_t n, uint32_t d, const uint32_t *d_graph_ids,
                                 const uint32_t *d_graph_deg, uint32_t width, const float *d_queries, uint32_t nq,
                                 const uint32_t *d_seeds, uint32_t L, uint32_t K, uint32_t *d_out_ids,
                                 float *d_out_dist, void *stream) {
  using namespace wv;
  if (!d_base || !d_graph_ids || !d_graph_deg || !d_queries || !d_seeds || !d_out_ids) return WV_ERR_ARG;
  if (n == 0 || d == 0 || width == 0) return WV_ERR_ARG;
  if (d % 4 != 0) return WV_ERR_LIMIT;
  if (K < 1 || L < K || L >= n) return WV_ERR_ARG;
  if (L > SEARCH_MAX_L || width > SEARCH_MAX_WIDTH) return WV_ERR_LIMIT;
  if (nq == 0) return WV_OK;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return WV_ERR_CUDA;
  uint32_t *scr = nullptr;
  int rc = scratch_address(dev, &scr);
  if (rc) return rc;
  // one warp slot needs a visited bitset and a touched-word list of n/32 words
  const size_t words = ((size_t)n + 31) / 32;
  const size_t slots_fit = (NOALLOC_SCRATCH_WORDS - NOALLOC_HEADER_WORDS) / (2 * words);
  const int wpb = search_warps_per_block();
  if (slots_fit < (size_t)wpb) return WV_ERR_LIMIT;  // n too large for the fixed scratch
  const uint32_t cap = width + 32;
  int blocks = search_grid(d, L, cap, dev);
  if (blocks <= 0) return WV_ERR_LIMIT;
  blocks = (int)std::min<size_t>((size_t)blocks, slots_fit / wpb);
  blocks = (int)std::min<size_t>((size_t)blocks, ((size_t)nq + wpb - 1) / wpb);
  const size_t slots = (size_t)blocks * wpb;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  uint32_t *visited = scr + NOALLOC_HEADER_WORDS;
  // header and bitsets must start at zero; the touched lists need not
  if (cudaMemsetAsync(scr, 0, (NOALLOC_HEADER_WORDS + slots * words) * 4, s) != cudaSuccess) return WV_ERR_CUDA;
  SearchArgs a{};
  a.base = d_base;
  a.n = n;
  a.d = d;
  a.gids = d_graph_ids;
  a.gdeg = d_graph_deg;
  a.gw = width;
  a.queries = d_queries;
  a.nq = nq;
  a.seeds = d_seeds;
  a.seed_stride = L;
  a.L = L;
  a.K = K;
  a.Lmax = L;
  a.out_ids = d_out_ids;
  a.out_dist = d_out_dist;
  a.out_stride = K;
  a.counters = nullptr;
  a.visited = visited;
  a.touched = visited + slots * words;
  a.words = (uint32_t)words;
  a.cap = cap;
  a.next_query = scr;
  a.status = reinterpret_cast<int *>(scr + 1);
  if (launch_search_exact(a, blocks, s) != cudaSuccess) return WV_ERR_CUDA;
  int st = 0;
  if (cudaMemcpyAsync(&st, scr + 1, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess) return WV_ERR_CUDA;
  if (cudaStreamSynchronize(s) != cudaSuccess) return WV_ERR_CUDA;
  return st ? WV_ERR_DEVICE : WV_OK;
}
