// Launch interface of the beam-search kernels (wv_search.cu).
#pragma once
#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

#include "wv_common.cuh"

namespace wv {

struct SearchArgs {
  const float *base;
  uint32_t n, d;
  const uint32_t *gids;  // graph rows, width gw
  const uint32_t *gdeg;
  uint32_t gw;
  const float *queries;  // nq x d
  uint32_t nq;
  const uint32_t *nq_dev;  // if set, the query count is read from here (captured launches)
  const uint32_t *seeds;  // nq x seed_stride
  uint32_t seed_stride;
  const uint32_t *Lq;  // per-query beam width (or null: L)
  // (nullable, nq words) dispatch order: with per-query beams the launch
  // first fills it with the query indices by beam width, widest first, and
  // the warps take queries in that order (the longest searches start first,
  // so the launch does not end on a few late wide queries); the results of
  // a query do not depend on the warp that runs it
  uint32_t *order;
  const uint32_t *Kq;  // per-query result size (or null: K)
  uint32_t L, K, Lmax;
  uint32_t *out_ids;
  float *out_dist;
  uint32_t out_stride;
  unsigned long long *counters;  // [dist_count, hop_count]
  uint32_t *visited;             // slots x words bitsets, all zero between queries
  uint32_t *touched;             // slots x words
  uint32_t words;
  uint32_t cap;   // candidate buffer entries per warp (graph width + 32)
  uint32_t hcap;  // visited-hash area per warp, 32-bit words (0: the default for Lmax); set by launch_search
  int wide_hash;  // 32-bit hash entries only (set by launch_search)
  unsigned *next_query;
  int *status;
  // candidate-search (build) mode: visit lists, vcap entries per query
  ::wv::DI *vis;
  uint32_t *vcnt;
  uint32_t vcap;    // stride between queries' visit lists
  uint32_t vlimit;  // entries recorded per query (<= vcap)
  // every base value is an integer in [0, 255]: queries that are too get
  // their distances by a warp reduction (exact in any order)
  int int_exact;
  const float *xnorm;  // squared norms of the base rows (set when int_exact)
  // SearchEntrySubCentroid: seed distances to the row shifted by one float
  // (the base carries a zero float after its last row)
  int seed_shift;
  // candidate distances from a low-precision copy of the base (0: the FP32
  // base; 1: bf16 rows; 2: fp8 e4m3 rows with a per-row FP32 scale), FP32
  // accumulation; the first `rerank` pool entries are then re-scored exactly
  // in FP32 and re-sorted before the top K are written
  int storage;
  const void *qbase;
  const float *qscale;
  const float *qnorm;  // squared norms of the low-precision rows
  uint32_t rerank;
  // 0: the exact traversal (k_search, the reference's expansion order);
  // E >= 1: the throughput form (k_beam, wv_beam.cu), E pool entries
  // expanded per step, tensor-core row distances where the layout allows
  uint32_t parents;
  // the throughput form: warps per query (1, 2 or 4; set by launch_beam
  // from the shape) -- the others join the leader's distance passes
  int query_warps;
};

constexpr uint32_t SEARCH_MAX_WIDTH = 256;  // graph row width the kernel accepts
constexpr uint32_t SEARCH_MAX_L = 1536;  // exact seed sort scratch: 2L + 256 words of stage

// the tunable launch shape of the route kernel: warps per block (1, 2, 4 or
// 8; one warp serves one query at a time) and the visited-hash area per warp
// in 32-bit words (0: the default, 2L + 256 rounded up to a power of two, at
// least 2048; a larger area keeps longer searches off the global bitset but
// costs occupancy), holding twice as many 16-bit entries unless `wide`.
// The build (candidate-search) variant runs in the default shape only.
struct SearchShape {
  int wpb = 4;
  uint32_t hcap = 0;
  bool wide = false;  // 32-bit visited-hash entries even where 16-bit ones would do
  // the throughput form only: warps per query (1, or 2 / 4 = wpb: one query
  // per block):
  // the leader warp runs the search, the others take shares of its
  // distance passes (more rows in flight per query's shared memory)
  int qw = 1;
};

// bytes of dynamic shared memory per block and warps per block
size_t search_block_smem(uint32_t d, uint32_t Lmax, uint32_t cap, SearchShape sh);
size_t search_block_smem(uint32_t d, uint32_t Lmax, uint32_t cap);
int search_warps_per_block();
uint32_t search_hash_slots(uint32_t Lmax, uint32_t want);
// the least hash area (words) a launch at beams up to Lmax may ask for; it
// needs n >= 32 * (2 Lmax + 256) (the introsort scratch then lives in the
// warp's global scratch of ceil(n / 32) words)
uint32_t search_hash_min(uint32_t Lmax, uint32_t n);
// blocks to launch for one persistent wave on this device (0 if it cannot run)
int search_grid(uint32_t d, uint32_t Lmax, uint32_t cap, int device, SearchShape sh);
int search_grid(uint32_t d, uint32_t Lmax, uint32_t cap, int device);
cudaError_t launch_search(const SearchArgs &a, SearchShape sh, int blocks, cudaStream_t stream);

// the throughput form (wv_beam.cu): candidate entries per warp for graph
// width gw and E parents per step, the persistent grid of a shape, and the
// launch (launch_search dispatches to it when a.parents > 0 and the search
// is a route search without shifted seeds)
constexpr uint32_t BEAM_MAX_PARENTS = 4;  // pool entries expanded per step, at most
uint32_t beam_cap(uint32_t gw, uint32_t parents);
int beam_grid(uint32_t d, uint32_t Lmax, uint32_t gw, uint32_t parents, int device, SearchShape sh);
cudaError_t launch_beam(const SearchArgs &a, SearchShape sh, int blocks, cudaStream_t stream);
cudaError_t launch_search_exact(const SearchArgs &a, int blocks, cudaStream_t stream);

}  // namespace wv
