// HNSW / NSW routing on GB300 over a graph in the reference's INDEX_HNSW
// file layout.
//
// Replaces ComponentSearchRouteHNSW::RouteInner / SearchAtLayer and
// ComponentSearchRouteNSW::RouteInner (src/component_route.cpp:56-260) for a
// whole query batch, over the graph IndexBuilder::load_graph(INDEX_HNSW)
// reads (src/builder.cpp:1096-1124).
//
// Layout in HBM (n nodes):
//   l0_ids  n x w0   layer-0 friends (w0 = the widest layer-0 list), l0_deg n
//   up_off  n        offset of the node's upper layers in `up` (or ~0)
//   up               per node with layers 1..t: t records of (1 + wu) words,
//                    [count, ids..., padding] (wu = the widest upper list)
//
// One warp per query (persistent).  The reference's two priority queues
// (result: FurtherFirst, a max-heap of at most L + 1; candidates:
// CloserFirst, a min-heap) are kept as libstdc++ heaps with the same
// comparators, so equal distances resolve exactly as they do there.  A
// neighbour list is handled 32 entries at a time: the lanes mark the visited
// bits and take the distances (exact reference order, a lane per row), then one lane applies
// the queue updates in list order.  The visited set is a per-warp bitset over
// the nodes, cleared through the list of words it touched (VisitedList::Reset
// gives a fresh set for every layer and every SearchAtLayer).
#include <algorithm>
#include <cstdio>
#include <vector>

#include "stl_order.cuh"
#include "wv_common.cuh"
#include "wv_ctx.h"

using namespace wv;

namespace {

constexpr int HN_WARPS = 4;
constexpr uint32_t HN_PATH = 64;       // ensure_k_path_ entries kept (the last ones)
constexpr uint32_t HN_NONE = 0xffffffffu;
constexpr int HN_CSH = 512;            // candidate-queue entries kept in shared memory

struct HEnt {
  float d;
  uint32_t id;
};
// the candidate queue's array: its first HN_CSH entries (the heap's top nine
// levels, which every push and pop walks) in shared memory, the rest in
// global memory
struct SplitHeap {
  HEnt *sh, *gl;
  __device__ __forceinline__ HEnt &operator[](int i) const { return i < HN_CSH ? sh[i] : gl[i - HN_CSH]; }
};
struct FurtherLess {  // std::less<FurtherFirst>: a max-heap by distance (index.h:435-447)
  __device__ bool operator()(const HEnt &a, const HEnt &b) const { return a.d < b.d; }
};
struct CloserLess {  // std::less<CloserFirst>: a min-heap by distance (index.h:449-459)
  __device__ bool operator()(const HEnt &a, const HEnt &b) const { return a.d > b.d; }
};

struct HnswArgs {
  const float *base;
  uint32_t n, d;
  const uint32_t *l0_ids, *l0_deg;
  uint32_t w0;
  const uint32_t *up_off, *up;
  uint32_t wu;
  uint32_t ep, max_level;
  int router;  // 0 HNSW, 1 NSW
  const float *queries;
  uint32_t nq, L, K;
  uint32_t *out_ids;
  float *out_dist;
  uint32_t *bits, *touched;  // per warp slot: words each
  uint32_t words;
  HEnt *cand;                // per warp slot: ccap entries past the shared part (candidate queue, final queue)
  uint32_t ccap;
  unsigned *next_query;
  unsigned long long *counters;
  int *status;
};

struct WarpState {
  float *qv;     // d floats
  HEnt *res;     // L + 1 entries: the result queue
  uint32_t *ids;  // 32: the current chunk's fresh ids
  float *dist;    // 32
  HEnt *path;     // HN_PATH
  HEnt *csh;      // HN_CSH: the shared part of the candidate queue
};

__host__ __device__ inline size_t hn_warp_bytes(uint32_t d, uint32_t L) {
  const size_t q = ((size_t)d * 4 + 15) & ~size_t(15);
  return q + (((size_t)(L + 1) * 8 + 15) & ~size_t(15)) + 32 * 4 + 32 * 4 +
         (size_t)HN_PATH * 8 + (size_t)HN_CSH * 8;
}

__device__ inline WarpState hn_carve(uint8_t *p, uint32_t d, uint32_t L) {
  WarpState w;
  w.qv = reinterpret_cast<float *>(p);
  p += ((size_t)d * 4 + 15) & ~size_t(15);
  w.res = reinterpret_cast<HEnt *>(p);
  p += ((size_t)(L + 1) * 8 + 15) & ~size_t(15);
  w.ids = reinterpret_cast<uint32_t *>(p);
  p += 32 * 4;
  w.dist = reinterpret_cast<float *>(p);
  p += 32 * 4;
  w.path = reinterpret_cast<HEnt *>(p);
  p += (size_t)HN_PATH * 8;
  w.csh = reinterpret_cast<HEnt *>(p);
  return w;
}

// exact-order squared L2 (Distance::compare, include/weavess/distance.h) of
// base row `id` and the query in shared memory, by one lane: a row's 16-byte
// pieces are read straight from global memory (each lane its own row)
__device__ __forceinline__ float hn_dist(const float *__restrict__ base, uint32_t d, uint32_t id, const float *qv) {
  const float4 *x = reinterpret_cast<const float4 *>(base + (size_t)id * d);
  const float4 *q = reinterpret_cast<const float4 *>(qv);
  float acc = 0.f;
  const uint32_t d4 = d >> 2;
#pragma unroll 8
  for (uint32_t g = 0; g < d4; g++) acc = __fadd_rn(acc, group4(q[g], __ldg(x + g)));
  return acc;
}

// the visited bitset of one warp: words that go from 0 to non-0 are listed
struct Bits {
  uint32_t *w, *touched;
  uint32_t nt;
  __device__ void clear(int lane) {
    for (uint32_t t = lane; t < nt; t += 32) w[touched[t]] = 0u;
    nt = 0;
    __syncwarp();
  }
  // marks `id` (want: this lane has one); true where it was not marked
  __device__ bool test_set(bool want, uint32_t id, int lane) {
    bool fresh = false, first_word = false;
    if (want) {
      const uint32_t bit = 1u << (id & 31);
      const uint32_t old = atomicOr(w + (id >> 5), bit);
      fresh = !(old & bit);
      first_word = old == 0u;
    }
    const unsigned m = __ballot_sync(FULL, first_word);
    if (first_word) touched[nt + __popc(m & ((1u << lane) - 1u))] = id >> 5;
    nt += __popc(m);
    return fresh;
  }
};

// the neighbour list of `node` at `level`
__device__ __forceinline__ void hn_row(const HnswArgs &a, uint32_t node, uint32_t level, const uint32_t *&row,
                                       uint32_t &deg) {
  if (level == 0) {
    row = a.l0_ids + (size_t)node * a.w0;
    deg = min(a.l0_deg[node], a.w0);
  } else {
    const uint32_t off = a.up_off[node];
    const uint32_t *rec = a.up + (size_t)off + (size_t)(level - 1) * (a.wu + 1);
    deg = off == HN_NONE ? 0u : min(rec[0], a.wu);
    row = rec + 1;
  }
}

// the fresh (not yet visited) entries of row[b0, b0 + 32) in list order into
// s.ids / s.dist (distances in the reference's order); returns their count
__device__ int hn_chunk(const HnswArgs &a, WarpState &s, Bits &vis, const uint32_t *row, uint32_t deg, uint32_t b0,
                        int lane) {
  const uint32_t j = b0 + lane;
  uint32_t id = j < deg ? row[j] : HN_NONE;
  if (id != HN_NONE && id >= a.n) {
    set_err(a.status, DEV_BAD_ID);
    id = HN_NONE;
  }
  const unsigned same = __match_any_sync(FULL, id);
  const bool leader = id != HN_NONE && (__ffs(same) - 1) == lane;
  const bool fresh = vis.test_set(leader, id, lane);
  const unsigned fm = __ballot_sync(FULL, fresh);
  const int cnt = __popc(fm);
  const uint32_t my = fresh ? id : 0u;
  // compact the fresh ids to lanes 0..cnt-1 (list order)
  if (fresh) s.ids[__popc(fm & ((1u << lane) - 1u))] = my;
  __syncwarp();
  const uint32_t cid = lane < cnt ? s.ids[lane] : 0u;
  const float dd = lane < cnt ? hn_dist(a.base, a.d, cid, s.qv) : 0.f;
  if (lane < cnt) s.dist[lane] = dd;
  __syncwarp();
  return cnt;
}

// SearchAtLayer (component_route.cpp:85-131 / 214-260) from `entry`,
// pushing into the result queue (size rs, lane 0's copy is authoritative)
__device__ void hn_search_layer(const HnswArgs &a, WarpState &s, Bits &vis, SplitHeap cand, uint32_t entry,
                                uint32_t &rs, unsigned long long &dc, unsigned long long &hc, int lane) {
  // the entry's distance, then both queues hold it
  {
    const float de = lane == 0 ? hn_dist(a.base, a.d, entry, s.qv) : 0.f;
    dc++;
    vis.clear(lane);
    vis.test_set(lane == 0, entry, lane);
    if (lane == 0) {
      s.res[rs] = HEnt{de, entry};
      stl::push_heap(s.res, (int)rs + 1, FurtherLess());
      cand[0] = HEnt{de, entry};
    }
    rs++;
  }
  uint32_t cs = 1;
  __syncwarp();
  while (cs > 0) {
    uint32_t node = 0;
    int stop = 0;
    if (lane == 0) {
      const HEnt c = cand[0];
      if (c.d > s.res[0].d) stop = 1;
      else {
        node = c.id;
        stl::pop_heap(cand, (int)cs, CloserLess());
      }
    }
    stop = __shfl_sync(FULL, stop, 0);
    if (stop) break;
    node = __shfl_sync(FULL, node, 0);
    cs--;
    hc++;
    const uint32_t *row;
    uint32_t deg;
    hn_row(a, node, 0, row, deg);
    for (uint32_t b0 = 0; b0 < deg; b0 += 32) {
      const int cnt = hn_chunk(a, s, vis, row, deg, b0, lane);
      dc += cnt;
      if (lane == 0) {
        for (int t = 0; t < cnt; t++) {
          const float d = s.dist[t];
          if (rs < a.L || s.res[0].d > d) {
            s.res[rs] = HEnt{d, s.ids[t]};
            stl::push_heap(s.res, (int)rs + 1, FurtherLess());
            rs++;
            if (cs >= HN_CSH + a.ccap) {
              set_err(a.status, DEV_OVERFLOW);
              cs = 0;
              break;
            }
            cand[cs] = HEnt{d, s.ids[t]};
            stl::push_heap(cand, (int)cs + 1, CloserLess());
            cs++;
            if (rs > a.L) {
              stl::pop_heap(s.res, (int)rs, FurtherLess());
              rs--;
            }
          }
        }
      }
      rs = __shfl_sync(FULL, rs, 0);
      cs = __shfl_sync(FULL, cs, 0);
      __syncwarp();
    }
  }
}

__global__ void __launch_bounds__(HN_WARPS * 32) k_hnsw(HnswArgs a) {
  extern __shared__ __align__(16) uint8_t smem[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  WarpState s = hn_carve(smem + (size_t)warp * hn_warp_bytes(a.d, a.L), a.d, a.L);
  const uint32_t slot = blockIdx.x * HN_WARPS + warp;
  Bits vis{a.bits + (size_t)slot * a.words, a.touched + (size_t)slot * a.words, 0};
  const SplitHeap cand{s.csh, a.cand + (size_t)slot * a.ccap};
  unsigned long long dc = 0, hc = 0;
  for (;;) {
    uint32_t q = 0;
    if (lane == 0) q = atomicAdd(a.next_query, 1u);
    q = __shfl_sync(FULL, q, 0);
    if (q >= a.nq) break;
    for (uint32_t k = lane; k < a.d; k += 32) s.qv[k] = a.queries[(size_t)q * a.d + k];
    __syncwarp();
    uint32_t rs = 0;
    if (a.router == 0) {
      // ---- greedy descent through every layer (component_route.cpp:144-184)
      uint32_t cur = a.ep;
      float cur_dist = lane == 0 ? hn_dist(a.base, a.d, cur, s.qv) : 0.f;
      cur_dist = __shfl_sync(FULL, cur_dist, 0);
      dc++;
      uint32_t plen = 1;  // path entries so far (the last HN_PATH kept)
      if (lane == 0) s.path[0] = HEnt{cur_dist, cur};
      for (int lv = (int)a.max_level; lv >= 0; --lv) {
        vis.clear(lane);
        vis.test_set(lane == 0, cur, lane);
        bool changed = true;
        while (changed) {
          changed = false;
          hc++;
          const uint32_t *row;
          uint32_t deg;
          hn_row(a, cur, (uint32_t)lv, row, deg);  // the list of the node the pass started from
          for (uint32_t b0 = 0; b0 < deg; b0 += 32) {
            const int cnt = hn_chunk(a, s, vis, row, deg, b0, lane);
            dc += cnt;
            // improvements in list order, each against the running minimum
            uint32_t nc = cur, np = plen;
            float nd = cur_dist;
            if (lane == 0)
              for (int t = 0; t < cnt; t++)
                if (s.dist[t] < nd) {
                  nd = s.dist[t];
                  nc = s.ids[t];
                  s.path[np % HN_PATH] = HEnt{nd, nc};
                  np++;
                }
            nc = __shfl_sync(FULL, nc, 0);
            nd = __shfl_sync(FULL, nd, 0);
            np = __shfl_sync(FULL, np, 0);
            if (np != plen) changed = true;
            cur = nc;
            cur_dist = nd;
            plen = np;
            __syncwarp();
          }
        }
      }
      // ---- layer-0 search from the path element before the last
      // (component_route.cpp:191-195); a one-element path starts from the
      // enterpoint (the reference reads before its vector's start there)
      const uint32_t ptotal = plen;  // the ring holds path entries [ptotal - HN_PATH, ptotal)
      while (rs < a.K && plen > 0) {
        plen--;
        uint32_t entry = a.ep;
        if (plen > 0) {
          if (plen - 1 + HN_PATH < ptotal) {
            if (lane == 0) set_err(a.status, DEV_OVERFLOW);  // an entry older than the ring
          } else {
            entry = s.path[(plen - 1) % HN_PATH].id;
          }
        }
        hn_search_layer(a, s, vis, cand, entry, rs, dc, hc, lane);
      }
    } else {
      hn_search_layer(a, s, vis, cand, 0u, rs, dc, hc, lane);  // ROUTER_NSW: node 0
    }
    // ---- the K nearest through the CloserFirst queue (component_route.cpp:197-210)
    if (lane == 0) {
      const SplitHeap tmp = cand;
      uint32_t ts = 0;
      while (rs > 0) {
        tmp[ts] = s.res[0];
        stl::push_heap(tmp, (int)ts + 1, CloserLess());
        ts++;
        stl::pop_heap(s.res, (int)rs, FurtherLess());
        rs--;
      }
      for (uint32_t p = 0; p < a.K; p++) {
        uint32_t id = 0;
        float d = 0.f;
        if (ts > 0) {
          id = tmp[0].id;
          d = tmp[0].d;
          stl::pop_heap(tmp, (int)ts, CloserLess());
          ts--;
        }
        a.out_ids[(size_t)q * a.K + p] = id;
        if (a.out_dist) a.out_dist[(size_t)q * a.K + p] = d;
      }
    }
    __syncwarp();
  }
  vis.clear(lane);
  if (lane == 0) {
    atomicAdd(a.counters + 0, dc);
    atomicAdd(a.counters + 1, hc);
  }
}

}  // namespace

// ================================================================ host side
extern "C" {

int wv_load_hnsw(wv_ctx *c, const uint32_t *words, size_t count) {
  if (!c) return WV_ERR_ARG;
  WV_CHECK(c, c->n > 0, WV_ERR_STATE, "upload the base first (the graph's node count must match it)");
  WV_CHECK(c, words && count >= 2, WV_ERR_ARG, "empty HNSW graph");
  const uint32_t n = c->n;
  size_t p = 2;
  const uint32_t ep = words[0], max_level = words[1];
  WV_CHECK(c, ep < n, WV_ERR_ARG, "enterpoint %u >= n=%u", ep, n);
  // first pass: record offsets, widths and layer counts
  std::vector<size_t> at(n, (size_t)-1);
  std::vector<uint32_t> layers(n, 0);
  uint32_t w0 = 1, wu = 1, total_up = 0;
  for (uint32_t r = 0; r < n; r++) {
    WV_CHECK(c, p + 2 <= count, WV_ERR_ARG, "HNSW graph truncated at record %u", r);
    const uint32_t id = words[p], t = words[p + 1];
    WV_CHECK(c, id < n && at[id] == (size_t)-1, WV_ERR_ARG, "bad or repeated node id %u in record %u", id, r);
    WV_CHECK(c, t <= 64, WV_ERR_LIMIT, "node %u has %u layers", id, t);
    at[id] = p;
    layers[id] = t;
    p += 2;
    for (uint32_t l = 0; l < t; l++) {
      WV_CHECK(c, p < count, WV_ERR_ARG, "HNSW graph truncated in node %u", id);
      const uint32_t gk = words[p++];
      WV_CHECK(c, p + gk <= count, WV_ERR_ARG, "HNSW graph truncated in node %u", id);
      for (uint32_t k = 0; k < gk; k++) WV_CHECK(c, words[p + k] < n, WV_ERR_ARG, "node %u lists id %u", id, words[p + k]);
      if (l == 0) w0 = std::max(w0, gk);
      else wu = std::max(wu, gk);
      p += gk;
    }
    if (t > 1) total_up += t - 1;
  }
  WV_CHECK(c, p == count, WV_ERR_ARG, "%zu words after the last node", count - p);
  // second pass: fixed-width layer-0 rows, upper-layer records
  std::vector<uint32_t> l0((size_t)n * w0, 0u), deg0(n, 0u), up_off(n, HN_NONE),
      up((size_t)std::max(total_up, 1u) * (wu + 1), 0u);
  uint32_t next = 0;
  for (uint32_t v = 0; v < n; v++) {
    size_t q = at[v] + 2;
    if (layers[v] > 1) up_off[v] = next * (wu + 1);
    for (uint32_t l = 0; l < layers[v]; l++) {
      const uint32_t gk = words[q++];
      if (l == 0) {
        deg0[v] = gk;
        std::copy(words + q, words + q + gk, l0.begin() + (size_t)v * w0);
      } else {
        uint32_t *rec = up.data() + (size_t)next * (wu + 1);
        rec[0] = gk;
        std::copy(words + q, words + q + gk, rec + 1);
        next++;
      }
      q += gk;
    }
  }
  WV_CUDA(c, cudaSetDevice(c->device));
  cudaError_t e = cudaSuccess;
  uint32_t *d_l0 = c->buf<uint32_t>("hn_l0", l0.size(), &e);
  uint32_t *d_deg0 = c->buf<uint32_t>("hn_deg0", n, &e);
  uint32_t *d_upoff = c->buf<uint32_t>("hn_upoff", n, &e);
  uint32_t *d_up = c->buf<uint32_t>("hn_up", up.size(), &e);
  uint32_t *d_layers = c->buf<uint32_t>("hn_layers", n, &e);
  WV_CUDA(c, e);
  WV_CUDA(c, cudaMemcpyAsync(d_layers, layers.data(), (size_t)n * 4, cudaMemcpyHostToDevice, c->stream));
  WV_CUDA(c, cudaMemcpyAsync(d_l0, l0.data(), l0.size() * 4, cudaMemcpyHostToDevice, c->stream));
  WV_CUDA(c, cudaMemcpyAsync(d_deg0, deg0.data(), (size_t)n * 4, cudaMemcpyHostToDevice, c->stream));
  WV_CUDA(c, cudaMemcpyAsync(d_upoff, up_off.data(), (size_t)n * 4, cudaMemcpyHostToDevice, c->stream));
  WV_CUDA(c, cudaMemcpyAsync(d_up, up.data(), up.size() * 4, cudaMemcpyHostToDevice, c->stream));
  WV_CUDA(c, cudaStreamSynchronize(c->stream));
  c->hnsw.n = n;
  c->hnsw.w0 = w0;
  c->hnsw.wu = wu;
  c->hnsw.ep = ep;
  c->hnsw.max_level = max_level;
  c->hnsw.ep_layers = layers[ep];
  return WV_OK;
}

int wv_search_hnsw(wv_ctx *c, const float *queries, uint32_t nq, int router, uint32_t L, uint32_t K,
                   uint32_t *out_ids, float *out_dist, wv_counters *counters) {
  if (!c) return WV_ERR_ARG;
  WV_CHECK(c, queries && out_ids, WV_ERR_ARG, "null buffer");
  WV_CHECK(c, c->hnsw.n == c->n && c->n > 0, WV_ERR_STATE, "no HNSW graph for the uploaded base");
  WV_CHECK(c, router == 0 || router == 1, WV_ERR_ARG, "router %d: 0 (HNSW) or 1 (NSW)", router);
  WV_CHECK(c, K >= 1 && L >= K, WV_ERR_ARG, "L_search=%u must be at least K_search=%u >= 1", L, K);
  WV_CHECK(c, L <= (1u << 14), WV_ERR_LIMIT, "L=%u above 16384", L);
  WV_CHECK(c, c->d % 4 == 0, WV_ERR_LIMIT, "dimension %u is not a multiple of 4", c->d);
  // the descent reads the enterpoint's list at every layer up to max_level
  WV_CHECK(c, router == 1 || c->hnsw.ep_layers > c->hnsw.max_level, WV_ERR_ARG,
           "enterpoint %u has %u layers, max level %u", c->hnsw.ep, c->hnsw.ep_layers, c->hnsw.max_level);
  if (counters) *counters = wv_counters{0, 0};
  if (nq == 0) return WV_OK;
  WV_CUDA(c, cudaSetDevice(c->device));
  const uint32_t n = c->n;
  WV_CUDA(c, c->q_buf.ensure((size_t)nq * c->d * 4));
  WV_CUDA(c, c->out_ids_buf.ensure((size_t)nq * K * 4));
  if (out_dist) WV_CUDA(c, c->out_dist_buf.ensure((size_t)nq * K * 4));
  WV_CUDA(c, cudaMemcpyAsync(c->q_buf.p, queries, (size_t)nq * c->d * 4, cudaMemcpyHostToDevice, c->stream));
  const size_t smem = (size_t)HN_WARPS * hn_warp_bytes(c->d, L);
  WV_CHECK(c, smem <= 227 * 1024, WV_ERR_LIMIT, "d=%u L=%u need %zu bytes of shared memory per block", c->d, L, smem);
  WV_CUDA(c, cudaFuncSetAttribute(k_hnsw, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int per_sm = 0;
  WV_CUDA(c, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_hnsw, HN_WARPS * 32, smem));
  WV_CHECK(c, per_sm > 0, WV_ERR_LIMIT, "the HNSW kernel does not fit an SM with d=%u L=%u", c->d, L);
  const uint32_t blocks = std::min<uint32_t>((uint32_t)c->sms * per_sm, (nq + HN_WARPS - 1) / HN_WARPS);
  const size_t slots = (size_t)blocks * HN_WARPS, words = (n + 31) / 32;
  cudaError_t e = cudaSuccess;
  uint32_t *bits = c->buf<uint32_t>("hn_bits", slots * words, &e);
  uint32_t *touched = c->buf<uint32_t>("hn_touch", slots * words, &e);
  WV_CUDA(c, e);
  WV_CUDA(c, cudaMemsetAsync(bits, 0, slots * words * 4, c->stream));
  HnswArgs a{};
  a.base = c->base.as<float>();
  a.n = n;
  a.d = c->d;
  a.l0_ids = c->work["hn_l0"].as<uint32_t>();
  a.l0_deg = c->work["hn_deg0"].as<uint32_t>();
  a.w0 = c->hnsw.w0;
  a.up_off = c->work["hn_upoff"].as<uint32_t>();
  a.up = c->work["hn_up"].as<uint32_t>();
  a.wu = c->hnsw.wu;
  a.ep = c->hnsw.ep;
  a.max_level = c->hnsw.max_level;
  a.router = router;
  a.queries = c->q_buf.as<float>();
  a.nq = nq;
  a.L = L;
  a.K = K;
  a.out_ids = c->out_ids_buf.as<uint32_t>();
  a.out_dist = out_dist ? c->out_dist_buf.as<float>() : nullptr;
  a.bits = bits;
  a.touched = touched;
  a.words = (uint32_t)words;
  a.next_query = c->d_next();
  a.counters = c->d_counters();
  a.status = c->d_status();
  // a candidate queue outgrowing its room redoes the batch with twice the room
  for (uint32_t ccap = std::max<uint32_t>(4096, 64 * L);; ccap *= 2) {
    a.ccap = ccap;
    a.cand = reinterpret_cast<HEnt *>(c->buf<unsigned long long>("hn_cand", slots * ccap, &e));
    WV_CUDA(c, e);
    WV_CUDA(c, cudaMemsetAsync(c->misc.p, 0, 32, c->stream));
    WV_CUDA(c, cudaMemsetAsync(c->d_status(), 0, 4, c->stream));
    k_hnsw<<<blocks, HN_WARPS * 32, smem, c->stream>>>(a);
    WV_CUDA(c, cudaGetLastError());
    int st = 0;
    WV_CUDA(c, cudaMemcpyAsync(&st, c->d_status(), 4, cudaMemcpyDeviceToHost, c->stream));
    WV_CUDA(c, cudaStreamSynchronize(c->stream));
    if (st == DEV_OVERFLOW && (size_t)ccap * 2 * slots * 8 <= (size_t)64 << 30) {
      WV_CUDA(c, cudaMemsetAsync(bits, 0, slots * words * 4, c->stream));
      continue;
    }
    break;
  }
  int rc = check_device_status(c, "hnsw search");
  if (rc) return rc;
  if (counters) {
    unsigned long long h[2];
    WV_CUDA(c, cudaMemcpyAsync(h, c->d_counters(), 16, cudaMemcpyDeviceToHost, c->stream));
    WV_CUDA(c, cudaStreamSynchronize(c->stream));
    counters->dist_count = h[0];
    counters->hop_count = h[1];
  }
  WV_CUDA(c, cudaMemcpyAsync(out_ids, c->out_ids_buf.p, (size_t)nq * K * 4, cudaMemcpyDeviceToHost, c->stream));
  if (out_dist)
    WV_CUDA(c, cudaMemcpyAsync(out_dist, c->out_dist_buf.p, (size_t)nq * K * 4, cudaMemcpyDeviceToHost, c->stream));
  WV_CUDA(c, cudaStreamSynchronize(c->stream));
  return WV_OK;
}

}  // extern "C"
