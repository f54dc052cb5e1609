// INIT_KDT on GB300: ComponentInitKDT::InitInner (src/component_init.cpp:500-640)
// -- nTrees randomised KD-trees whose leaves are merged into per-point
// bounded candidate sets, the graph EFANNA's refine starts from.
//
// Bit-exact with the reference run on one thread (its results with more
// threads depend on the OpenMP schedule: every split's std::mt19937 is seeded
// 1998 ^ omp_get_thread_num(), and the trees' shuffles share rand()):
//  * id lists: std::random_shuffle of 0..n-1 per tree on the context's rand()
//    stream, tree by tree (n - 1 draws each, drawn on the host in order; the
//    swaps run on the device, one thread per tree, in the inside-out form --
//    before step i the list holds i at position i);
//  * splits (meanSplit / selectDivision / planeSplit, :648-756): one warp per
//    node -- the per-dimension means and variances of the first 101 ids are
//    folded in the reference's order with round-to-nearest adds and
//    multiplies, one lane takes the top-5 variance scan, and the two Hoare
//    partitions are done in parallel from their closed form: the k-th
//    misplaced id from the left swaps with the k-th misplaced id from the
//    right (found by warp ballots, swapped all at once);
//  * level by level while fewer than 1,100 nodes are active (each split a
//    fresh rng: its first output), then one warp per remaining active node
//    walks its subtree depth-first (DFSbuild, :758-787), the k-th split in
//    preorder taking output k of mt19937(1998) from a table;
//  * merges (mergeSubGraphs, :840-912): a point's bounded set only depends on
//    the order of the offers made to it, and that order is static -- tree by
//    tree, the point's ancestors at depth >= mLevel deepest first; at an
//    ancestor whose smaller child holds the point, the ids of the leaf the
//    point descends to in the larger child, in list order; else the ids of
//    the smaller side that descend to the point's own leaf, in list order.
//    Those last lists are built for every leaf first (count, scan, scatter,
//    sort by (depth, position)); then one warp per point replays its offers
//    on a sorted (distance, id) array in shared memory with the
//    std::set<Candidate, greater> rule (offer while not full or closer than
//    the largest distance; drop the largest when over K);
//  * final rows in ascending (distance, id); a row of fewer than K is filled
//    by one thread, row by row, from mt19937(1998) outputs % n into a set
//    keyed by distance alone (equal distances kept once), as the reference.
// SEARCH_ENTRY_KDT (component_search_entry.cpp:102-170) walks the kept trees
// on the device, one warp per query; only its rand() % n fills, which share
// the rand() stream across queries, are drawn on the host in query order.
#include <algorithm>
#include <cstring>
#include <random>
#include <vector>

#include "wv_common.cuh"
#include "wv_ctx.h"
#include "wv_kdt.h"
#include "wv_nnd.h"
#include "wv_scan.h"

namespace wv {

namespace {

constexpr uint32_t KDT_TNS = 10;          // Index::TNS (index.h:257)
constexpr uint32_t KDT_SAMPLE = 100;      // Index::SAMPLE_NUM (index.h:265)
constexpr int KDT_RAND_DIM = 5;           // Index::RAND_DIM (index.h:273)
constexpr uint32_t KDT_ACTIVE_MAX = 1100;  // component_init.cpp:539
constexpr int KDT_MAX_DEPTH = 200;        // deeper trees are refused (records keep 8 bits of depth)
constexpr int KW = 4;                     // warps per block
constexpr uint32_t KDT_MAX_K = 1024;

// ---------------------------------------------------------------- shuffle
// std::random_shuffle of 0..n-1 (libstdc++: step i swaps positions i and
// j = rand() % (i + 1)); before step i position i still holds i, so a step is
// a[i] = a[j]; a[j] = i.  The steps run in blocks of SH_W: the SH_W reads of
// a block are issued together (they see every store of earlier blocks), and
// a read of a position an earlier step of the same block wrote takes that
// step's value from registers instead.
constexpr int SH_W = 16;

__device__ __forceinline__ void shuffle_steps(uint32_t *a, const int *rt, uint32_t n) {
  a[0] = 0;
  uint32_t i0 = 1;
  for (; i0 + SH_W <= n; i0 += SH_W) {
    uint32_t j[SH_W], v[SH_W];
#pragma unroll
    for (int k = 0; k < SH_W; k++) {
      j[k] = (uint32_t)((long long)rt[i0 + k - 1] % (long long)(i0 + k + 1));
      v[k] = a[j[k]];
    }
#pragma unroll
    for (int k = 0; k < SH_W; k++) {
#pragma unroll
      for (int m = 0; m < k; m++) {
        if (j[k] == i0 + m) v[k] = v[m];  // step m wrote a[i_m] = (its read)
        if (j[k] == j[m]) v[k] = i0 + m;  // ... then a[j_m] = i_m (a[i_m] when j_m == i_m)
      }
    }
#pragma unroll
    for (int k = 0; k < SH_W; k++) {
      const uint32_t i = i0 + k;
      if (j[k] == i) {
        a[i] = i;
      } else {
        a[i] = v[k];
        a[j[k]] = i;
      }
    }
  }
  for (uint32_t i = i0; i < n; i++) {
    const uint32_t jj = (uint32_t)((long long)rt[i - 1] % (long long)(i + 1));
    if (jj == i) {
      a[i] = i;
    } else {
      a[i] = a[jj];
      a[jj] = i;
    }
  }
}

__global__ void k_kdt_shuffle(uint32_t n, const int *r, uint32_t *leaf, int in_smem) {
  extern __shared__ uint32_t sh[];
  if (threadIdx.x != 0) return;
  const uint32_t t = blockIdx.x;
  uint32_t *a = in_smem ? sh : leaf + (size_t)t * n;
  shuffle_steps(a, r + (size_t)t * (n - 1), n);
  if (in_smem)
    for (uint32_t i = 0; i < n; i++) leaf[(size_t)t * n + i] = a[i];
}

// ---------------------------------------------------------------- split
__device__ __forceinline__ float coord(const float *__restrict__ base, uint32_t d, uint32_t id, int dim) {
  return base[(size_t)id * d + dim];
}

// Hoare partition of ids[lo, hi) (planeSplit's loops): "left" ids (< cut, or
// <= cut when le) first.  Returns the boundary.  scr: hi - lo words.
__device__ uint32_t warp_hoare(const float *__restrict__ base, uint32_t d, int dim, uint32_t *ids, uint32_t lo,
                               uint32_t hi, float cut, bool le, uint32_t *scr, int lane) {
  const unsigned lt = (1u << lane) - 1u;
  auto left_of = [&](uint32_t p) {
    const float v = coord(base, d, ids[p], dim);
    return le ? v <= cut : v < cut;
  };
  uint32_t m = lo;
  for (uint32_t p0 = lo; p0 < hi; p0 += 32) {
    const uint32_t p = p0 + lane;
    m += __popc(__ballot_sync(FULL, p < hi && left_of(p)));
  }
  uint32_t *A = scr, *B = scr + (hi - lo) / 2;
  uint32_t s = 0;
  for (uint32_t p0 = lo; p0 < m; p0 += 32) {
    const uint32_t p = p0 + lane;
    const bool f = p < m && !left_of(p);
    const unsigned b = __ballot_sync(FULL, f);
    if (f) A[s + __popc(b & lt)] = p;
    s += __popc(b);
  }
  uint32_t r = 0;
  for (uint32_t p0 = m; p0 < hi; p0 += 32) {
    const uint32_t p = p0 + lane;
    const bool f = p < hi && left_of(p);
    const unsigned b = __ballot_sync(FULL, f);
    if (f) B[s - 1 - (r + __popc(b & lt))] = p;
    r += __popc(b);
  }
  __syncwarp();
  for (uint32_t k = lane; k < s; k += 32) {
    const uint32_t a = A[k], b = B[k];
    const uint32_t x = ids[a];
    ids[a] = ids[b];
    ids[b] = x;
  }
  __syncwarp();
  return m;
}

struct Split {
  uint32_t mid;
  int dim;
  float val;
};

// meanSplit (component_init.cpp:648-696) of ids[0, count) with the rng
// output rv; mean / var: d floats of the warp's shared memory
__device__ Split warp_split(const float *__restrict__ base, uint32_t d, uint32_t *ids, uint32_t count, uint32_t rv,
                            float *mean, float *var, uint32_t *scr, int lane) {
  const uint32_t cnt = min(KDT_SAMPLE + 1, count);
  const float div = __fdiv_rn(1.f, (float)cnt);
  for (uint32_t k = lane; k < d; k += 32) {
    float m = 0.f;
    for (uint32_t j = 0; j < cnt; j++) m = __fadd_rn(m, coord(base, d, ids[j], k));
    m = __fmul_rn(m, div);
    float v = 0.f;
    for (uint32_t j = 0; j < cnt; j++) {
      const float dd = __fsub_rn(coord(base, d, ids[j], k), m);
      v = __fadd_rn(v, __fmul_rn(dd, dd));
    }
    mean[k] = m;
    var[k] = v;
  }
  __syncwarp();
  int dim = 0;
  if (lane == 0) {
    // selectDivision (component_init.cpp:732-756)
    int num = 0;
    uint32_t top[KDT_RAND_DIM];
    for (uint32_t i = 0; i < d; i++) {
      if (num < KDT_RAND_DIM || var[i] > var[top[num - 1]]) {
        if (num < KDT_RAND_DIM) top[num++] = i;
        else top[num - 1] = i;
        int j = num - 1;
        while (j > 0 && var[top[j]] > var[top[j - 1]]) {
          const uint32_t x = top[j];
          top[j] = top[j - 1];
          top[j - 1] = x;
          --j;
        }
      }
    }
    dim = (int)top[rv % (uint32_t)num];
  }
  dim = __shfl_sync(FULL, dim, 0);
  const float cut = mean[dim];
  const uint32_t lim1 = warp_hoare(base, d, dim, ids, 0, count, cut, false, scr, lane);
  const uint32_t lim2 = warp_hoare(base, d, dim, ids, lim1, count, cut, true, scr, lane);
  uint32_t idx;
  if (lim1 > count / 2) idx = lim1;
  else if (lim2 < count / 2) idx = lim2;
  else idx = count / 2;
  if (lim1 == count || lim2 == 0) idx = count / 2;
  __syncwarp();
  return Split{idx, dim, cut};
}

__device__ __forceinline__ KNode child_node(uint32_t start, uint32_t end, int parent, int depth, int tree) {
  KNode x;
  x.dim = -1;
  x.val = 0.f;
  x.start = start;
  x.end = end;
  x.left = x.right = -1;
  x.parent = parent;
  x.depth = depth;
  x.tree = tree;
  return x;
}

// one level of the active set: warp i splits node act[i], its children go to
// nodes child_base + 2i, + 2i + 1
__global__ void __launch_bounds__(KW * 32)
    k_kdt_level(const float *__restrict__ base, uint32_t d, uint32_t n, uint32_t *leaf, uint32_t *scr, KNode *nodes,
                const int *act, uint32_t nact, uint32_t child_base, uint32_t rv0) {
  extern __shared__ float ksm[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  float *mean = ksm + (size_t)warp * 2 * d, *var = mean + d;
  for (uint32_t i = blockIdx.x * KW + warp; i < nact; i += gridDim.x * KW) {
    const int nd = act[i];
    const KNode x = nodes[nd];
    const size_t off = (size_t)x.tree * n + x.start;
    const Split sp = warp_split(base, d, leaf + off, x.end - x.start, rv0, mean, var, scr + off, lane);
    if (lane == 0) {
      const int l = (int)(child_base + 2 * i), r = l + 1;
      nodes[l] = child_node(x.start, x.start + sp.mid, nd, x.depth + 1, x.tree);
      nodes[r] = child_node(x.start + sp.mid, x.end, nd, x.depth + 1, x.tree);
      nodes[nd].dim = sp.dim;
      nodes[nd].val = sp.val;
      nodes[nd].left = l;
      nodes[nd].right = r;
    }
    __syncwarp();
  }
}

// DFSbuild below each remaining active node (one warp each): nodes of more
// than TNS ids split with the next output of the table in preorder
__global__ void __launch_bounds__(KW * 32)
    k_kdt_dfs(const float *__restrict__ base, uint32_t d, uint32_t n, uint32_t *leaf, uint32_t *scr, KNode *nodes,
              const int *act, uint32_t nact, uint32_t *node_count, uint32_t ncap, const uint32_t *mt, uint32_t nmt,
              int *stacks, int *status) {
  extern __shared__ float ksm[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  float *mean = ksm + (size_t)warp * 2 * d, *var = mean + d;
  int *stack = stacks + (size_t)(blockIdx.x * KW + warp) * KDT_MAX_DEPTH;
  for (uint32_t i = blockIdx.x * KW + warp; i < nact; i += gridDim.x * KW) {
    int cur = act[i], sp = 0;
    uint32_t k = 0;
    while (true) {
      const KNode x = nodes[cur];
      const uint32_t count = x.end - x.start;
      if (count > KDT_TNS) {
        if (k >= nmt || x.depth + 1 >= KDT_MAX_DEPTH) {
          if (lane == 0) set_err(status, DEV_OVERFLOW);
          break;
        }
        const size_t off = (size_t)x.tree * n + x.start;
        const Split s = warp_split(base, d, leaf + off, count, mt[k++], mean, var, scr + off, lane);
        int l = 0;
        if (lane == 0) {
          l = (int)atomicAdd(node_count, 2u);
          if ((uint32_t)l + 2 > ncap) {
            set_err(status, DEV_OVERFLOW);
            l = -1;
          } else {
            nodes[l] = child_node(x.start, x.start + s.mid, cur, x.depth + 1, x.tree);
            nodes[l + 1] = child_node(x.start + s.mid, x.end, cur, x.depth + 1, x.tree);
            nodes[cur].dim = s.dim;
            nodes[cur].val = s.val;
            nodes[cur].left = l;
            nodes[cur].right = l + 1;
          }
        }
        l = __shfl_sync(FULL, l, 0);
        __syncwarp();
        if (l < 0) break;
        if (lane == 0) stack[sp] = l + 1;
        sp++;
        cur = l;
        __syncwarp();
        continue;
      }
      if (sp == 0) break;
      __syncwarp();
      cur = stack[--sp];
      __syncwarp();
    }
  }
}

// ---------------------------------------------------------------- merges
__global__ void k_kdt_leafmap(const KNode *nodes, const uint32_t *node_count, uint32_t n, int *leaf_of) {
  const uint32_t cnt = *node_count;
  for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < cnt; j += gridDim.x * blockDim.x) {
    const KNode x = nodes[j];
    if (x.left >= 0) continue;
    for (uint32_t p = x.start; p < x.end; p++) leaf_of[(size_t)x.tree * n + p] = (int)j;
  }
}

__global__ void k_kdt_pos(const uint32_t *leaf, size_t total, uint32_t n, uint32_t *pos_of) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
    const size_t t = i / n;
    pos_of[t * n + leaf[i]] = (uint32_t)(i - t * n);
  }
}

// SearchToLeaf (component_init.cpp:828-838) from node nd by the point's values
__device__ __forceinline__ int to_leaf(const float *__restrict__ base, uint32_t d, const KNode *nodes, int nd,
                                       uint32_t id) {
  while (nodes[nd].left >= 0 && nodes[nd].right >= 0)
    nd = coord(base, d, id, nodes[nd].dim) < nodes[nd].val ? nodes[nd].left : nodes[nd].right;
  return nd;
}

__device__ __forceinline__ bool smaller_is_left(const KNode *nodes, const KNode &a) {
  const KNode &l = nodes[a.left], &r = nodes[a.right];
  return (l.end - l.start) < (r.end - r.start);
}

// the offers a point on the smaller side of an ancestor makes to the leaf it
// reaches in the larger side: counted (rec == null) or written as
// (255 - depth) << 32 | position at the leaf's cursor
__global__ void k_kdt_records(const float *__restrict__ base, uint32_t d, uint32_t n, size_t total,
                              const uint32_t *leaf, const KNode *nodes, const int *leaf_of, int mlevel, uint32_t *cnt,
                              const uint32_t *off, unsigned long long *rec) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
    const uint32_t p = (uint32_t)(i % n), y = leaf[i];
    int child = leaf_of[i];
    int a = nodes[child].parent;
    while (a >= 0 && nodes[a].depth >= mlevel) {
      const KNode an = nodes[a];
      const bool sl = smaller_is_left(nodes, an);
      const int small = sl ? an.left : an.right, large = sl ? an.right : an.left;
      if (child == small) {
        const int lf = to_leaf(base, d, nodes, large, y);
        const uint32_t slot = atomicAdd(cnt + lf, 1u);
        if (rec) rec[off[lf] + slot] = ((unsigned long long)(255 - an.depth) << 32) | p;
      }
      child = a;
      a = an.parent;
    }
  }
}

// sorts each leaf's records ascending (depth descending, position ascending)
__global__ void k_kdt_sort_records(const uint32_t *node_count, const uint32_t *off, const uint32_t *cnt,
                                   const unsigned long long *rec, unsigned long long *out) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t nn = *node_count;
  for (uint32_t j = blockIdx.x * (blockDim.x >> 5) + warp; j < nn; j += gridDim.x * (blockDim.x >> 5)) {
    const uint32_t o = off[j], m = cnt[j];
    for (uint32_t a = lane; a < m; a += 32) {
      const unsigned long long key = rec[o + a];
      uint32_t rank = 0;
      for (uint32_t b = 0; b < m; b++) rank += rec[o + b] < key;
      out[o + rank] = key;
    }
  }
}

// std::set<Candidate, greater> offer (component_init.cpp:886-908) on the
// ascending (distance, id) array sd / si of sz entries, cap K
__device__ void set_offer(float *sd, uint32_t *si, uint32_t &sz, uint32_t K, float dist, uint32_t id, int lane) {
  if (sz == K && !(dist < sd[K - 1])) return;
  uint32_t less = 0;
  bool eq = false;
  for (uint32_t j0 = 0; j0 < sz; j0 += 32) {
    const uint32_t j = j0 + lane;
    bool l = false, e = false;
    if (j < sz) {
      const float x = sd[j];
      l = x < dist || (x == dist && si[j] < id);
      e = x == dist && si[j] == id;
    }
    less += __popc(__ballot_sync(FULL, l));
    eq |= __any_sync(FULL, e);
  }
  if (eq) return;
  for (int hi = (int)sz; hi > (int)less; hi -= 32) {
    const int lo = max((int)less, hi - 32), j = lo + lane;
    float v = 0.f;
    uint32_t w = 0;
    if (j < hi) {
      v = sd[j];
      w = si[j];
    }
    __syncwarp();
    if (j < hi && j + 1 < (int)K) {
      sd[j + 1] = v;
      si[j + 1] = w;
    }
    __syncwarp();
  }
  if (lane == 0) {
    sd[less] = dist;
    si[less] = id;
  }
  __syncwarp();
  sz = min(sz + 1, K);
}

// squared L2 of row `id` against xr (shared memory), the reference's order
__device__ __forceinline__ float row_l2(const float *__restrict__ base, uint32_t d, uint32_t id, const float *xr) {
  const float4 *r = reinterpret_cast<const float4 *>(base + (size_t)id * d);
  const float4 *x = reinterpret_cast<const float4 *>(xr);
  float acc = 0.f;
  for (uint32_t g = 0; g < (d >> 2); g++) acc = __fadd_rn(acc, group4(__ldg(r + g), x[g]));
  return acc;
}

__device__ void offer_batch(const float *__restrict__ base, uint32_t d, const float *xr, uint32_t my, int cnt,
                            float *sd, uint32_t *si, uint32_t &sz, uint32_t K, int lane) {
  const float dist = lane < cnt ? row_l2(base, d, my, xr) : 0.f;
  for (int b = 0; b < cnt; b++) {
    const float db = __shfl_sync(FULL, dist, b);
    const uint32_t ib = __shfl_sync(FULL, my, b);
    set_offer(sd, si, sz, K, db, ib, lane);
  }
}

// floats of a warp's merge area: the point's row, then K distances and K ids
// (rounded up so that every warp's row starts on 16 bytes)
__host__ __device__ inline uint32_t merge_stride(uint32_t d, uint32_t K) { return d + ((2 * K + 3) & ~3u); }

// one warp per point: its offers in the reference's order; the sorted set
// is written to kn (n x K) with its size
__global__ void __launch_bounds__(KW * 32)
    k_kdt_merge(const float *__restrict__ base, uint32_t d, uint32_t n, uint32_t T, uint32_t K, int mlevel,
                const uint32_t *leaf, const KNode *nodes, const int *leaf_of, const uint32_t *pos_of,
                const uint32_t *off, const uint32_t *cnt, const unsigned long long *rec, uint32_t *kn_ids,
                float *kn_dist, uint32_t *kn_sz) {
  extern __shared__ __align__(16) float msm[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  float *xr = msm + (size_t)warp * merge_stride(d, K);
  float *sd = xr + d;
  uint32_t *si = reinterpret_cast<uint32_t *>(sd + K);
  for (uint32_t x = blockIdx.x * KW + warp; x < n; x += gridDim.x * KW) {
    for (uint32_t k = lane; k < d; k += 32) xr[k] = base[(size_t)x * d + k];
    __syncwarp();
    uint32_t sz = 0;
    for (uint32_t t = 0; t < T; t++) {
      const uint32_t *lt = leaf + (size_t)t * n;
      const uint32_t p = pos_of[(size_t)t * n + x];
      const int lf = leaf_of[(size_t)t * n + p];
      uint32_t ri = off[lf];
      const uint32_t rend = ri + cnt[lf];
      int child = lf, a = nodes[lf].parent;
      while (a >= 0 && nodes[a].depth >= mlevel) {
        const KNode an = nodes[a];
        const bool sl = smaller_is_left(nodes, an);
        const int small = sl ? an.left : an.right, large = sl ? an.right : an.left;
        if (child == small) {
          const KNode tl = nodes[to_leaf(base, d, nodes, large, x)];
          for (uint32_t q0 = tl.start; q0 < tl.end; q0 += 32) {
            const int c = (int)min(32u, tl.end - q0);
            const uint32_t my = lane < c ? lt[q0 + lane] : 0u;
            offer_batch(base, d, xr, my, c, sd, si, sz, K, lane);
          }
        } else {
          const unsigned long long tag = (unsigned long long)(255 - an.depth) << 32;
          while (ri < rend && (rec[ri] & 0xffffffff00000000ull) < tag) ri++;  // (none expected)
          uint32_t re = ri;
          while (re < rend && (rec[re] & 0xffffffff00000000ull) == tag) re++;
          for (uint32_t q0 = ri; q0 < re; q0 += 32) {
            const int c = (int)min(32u, re - q0);
            const uint32_t my = lane < c ? lt[(uint32_t)rec[q0 + lane]] : 0u;
            offer_batch(base, d, xr, my, c, sd, si, sz, K, lane);
          }
          ri = re;
        }
        child = a;
        a = an.parent;
      }
    }
    for (uint32_t j = lane; j < sz; j += 32) {
      kn_ids[(size_t)x * K + j] = si[j];
      kn_dist[(size_t)x * K + j] = sd[j];
    }
    if (lane == 0) kn_sz[x] = sz;
    __syncwarp();
  }
}

// rows of K into the graph; rows short of K counted
__global__ void k_kdt_rows(uint32_t n, uint32_t K, const uint32_t *kn_ids, const float *kn_dist, const uint32_t *kn_sz,
                           uint32_t *g_ids, float *g_dist, uint32_t *g_deg, uint32_t *short_rows) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < (size_t)n * K;
       i += (size_t)gridDim.x * blockDim.x) {
    const uint32_t x = (uint32_t)(i / K), j = (uint32_t)(i % K);
    if (j < kn_sz[x]) {
      g_ids[i] = kn_ids[i];
      g_dist[i] = kn_dist[i];
    }
    if (j == 0) {
      g_deg[x] = kn_sz[x];
      if (kn_sz[x] < K) atomicAdd(short_rows, 1u);
    }
  }
}

// the rows short of K, in row order, on one thread (component_init.cpp:614-634):
// a set keyed by distance alone, filled from mt[0..) % n.  more[0] = 1 when
// the table ran out (the host grows it and runs this again), 2 when a row
// cannot reach K distinct distances.
__global__ void k_kdt_fill(const float *__restrict__ base, uint32_t d, uint32_t n, uint32_t K, const uint32_t *kn_ids,
                           const float *kn_dist, const uint32_t *kn_sz, const uint32_t *mt, size_t nmt,
                           uint32_t *g_ids, float *g_dist, uint32_t *g_deg, int *more) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  size_t k = 0;
  for (uint32_t x = 0; x < n; x++) {
    const uint32_t sz = kn_sz[x];
    if (sz >= K) continue;
    uint32_t *ri = g_ids + (size_t)x * K;
    float *rd = g_dist + (size_t)x * K;
    uint32_t m = 0;
    for (uint32_t j = 0; j < sz; j++) {  // ascending: equal distances are adjacent, the first is kept
      const float dj = kn_dist[(size_t)x * K + j];
      if (m > 0 && rd[m - 1] == dj) continue;
      ri[m] = kn_ids[(size_t)x * K + j];
      rd[m++] = dj;
    }
    const float *xr = base + (size_t)x * d;
    const size_t cap = 64ull * n + 1000000ull;
    size_t tries = 0;
    while (m < K) {
      if (k >= nmt) {
        more[0] = 1;
        return;
      }
      if (++tries > cap) {
        more[0] = 2;
        return;
      }
      const uint32_t id = mt[k++] % n;
      const float4 *a = reinterpret_cast<const float4 *>(xr);
      const float4 *b = reinterpret_cast<const float4 *>(base + (size_t)id * d);
      float dist = 0.f;
      for (uint32_t g = 0; g < (d >> 2); g++) dist = __fadd_rn(dist, group4(a[g], b[g]));
      uint32_t pos = 0;
      while (pos < m && rd[pos] < dist) pos++;
      if (pos < m && rd[pos] == dist) continue;
      for (uint32_t j = m; j > pos; j--) {
        ri[j] = ri[j - 1];
        rd[j] = rd[j - 1];
      }
      ri[pos] = id;
      rd[pos] = dist;
      m++;
    }
    g_deg[x] = K;
  }
  more[0] = 0;
}

// SEARCH_ENTRY_KDT's leaf part (component_search_entry.cpp:115-134), one
// query per warp: lane 0 walks each tree for its first lsize leaves in
// getSearchNodeList's order (the query's side of a cut first), then the
// warp takes their ids leaf-major across the trees without repeats (the base
// id equal to the query's number excluded); taken[q] = how many
__global__ void k_kdt_entry(const KNode *nodes, uint32_t nnodes, const uint32_t *leaf, uint32_t n, uint32_t T,
                            const float *queries, uint32_t nq, uint32_t d, uint32_t L, uint32_t lsize, int *vn,
                            uint32_t *seeds, uint32_t stride, uint32_t *taken, int *status) {
  const int lane = threadIdx.x & 31;
  const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
  for (uint32_t q = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; q < nq; q += nw) {
    const float *qv = queries + (size_t)q * d;
    int *vq = vn + (size_t)q * T * lsize;
    if (lane == 0) {
      int stack[KDT_MAX_DEPTH + 2];
      for (uint32_t t = 0; t < T; t++) {
        uint32_t cnt = 0;
        int sp = 0;
        stack[sp++] = (int)t;
        while (sp > 0 && cnt < lsize) {
          const int nd = stack[--sp];
          // a forest is walked only as the init left it; a node or a split
          // dimension out of range is reported, never followed
          if (nd < 0 || (uint32_t)nd >= nnodes) {
            set_err(status, DEV_BAD_ID);
            break;
          }
          const KNode x = nodes[nd];
          if (x.left >= 0 && x.right >= 0 && (x.dim < 0 || (uint32_t)x.dim >= d)) {
            set_err(status, DEV_BAD_ID);
            break;
          }
          if (x.left >= 0 && x.right >= 0) {
            if (sp + 2 > KDT_MAX_DEPTH + 2) {
              set_err(status, DEV_OVERFLOW);
              break;
            }
            const bool lt = qv[x.dim] < x.val;
            stack[sp++] = lt ? x.right : x.left;
            stack[sp++] = lt ? x.left : x.right;
          } else {
            vq[t * lsize + cnt++] = nd;
          }
        }
        for (; cnt < lsize; cnt++) vq[t * lsize + cnt] = -1;
      }
    }
    __syncwarp();
    uint32_t *s = seeds + (size_t)q * stride;
    uint32_t p = 0;
    for (uint32_t ni = 0; ni < lsize && p < L; ni++) {
      for (uint32_t t = 0; t < T && p < L; t++) {
        const int nd = vq[t * lsize + ni];
        if (nd < 0) continue;
        const KNode lf = nodes[nd];
        if (lf.start > lf.end || lf.end > n) {
          if (lane == 0) set_err(status, DEV_BAD_ID);
          continue;
        }
        for (uint32_t j = lf.start; j < lf.end && p < L; j++) {
          const uint32_t id = leaf[(size_t)t * n + j];
          bool hit = false;
          for (uint32_t u = lane; u < p; u += 32) hit |= s[u] == id;
          if (id == q || __any_sync(FULL, hit)) continue;
          if (lane == 0) s[p] = id;
          p++;
          __syncwarp();
        }
      }
    }
    if (lane == 0) taken[q] = p;
    __syncwarp();
  }
}

int nblocks(size_t items, int per_block, int cap) {
  return (int)std::max<size_t>(1, std::min<size_t>((items + per_block - 1) / per_block, (size_t)cap));
}

}  // namespace

int init_kdt_gpu(wv_ctx *c, uint32_t T, uint32_t K, uint32_t mlevel) {
  WV_CHECK(c, c->n >= 2, WV_ERR_STATE, "INIT_KDT needs an uploaded base of at least 2 points");
  WV_CHECK(c, c->d % 4 == 0, WV_ERR_LIMIT, "dimension %u is not a multiple of 4", c->d);
  WV_CHECK(c, T >= 1 && T <= 4096, WV_ERR_ARG, "nTrees=%u (1..4096)", T);
  WV_CHECK(c, K >= 1 && K <= KDT_MAX_K, WV_ERR_ARG, "K=%u (1..%u)", K, KDT_MAX_K);
  WV_CHECK(c, mlevel < (uint32_t)KDT_MAX_DEPTH, WV_ERR_ARG, "mLevel=%u", mlevel);
  // the work buffers are rewritten from here on: the old forest is gone
  // whether or not this init completes
  c->kdt = KdtForest{};
  const uint32_t n = c->n, d = c->d;
  const size_t total = (size_t)T * n;
  const uint32_t ncap = (uint32_t)std::min<size_t>(2 * total, 0x7fffffffu);
  WV_CHECK(c, 2 * total < 0x7fffffffu, WV_ERR_LIMIT, "nTrees x n too large");
  const size_t smem_split = (size_t)KW * 2 * d * 4;
  const size_t smem_merge = (size_t)KW * merge_stride(d, K) * 4;
  WV_CHECK(c, smem_split <= 200 * 1024 && smem_merge <= 200 * 1024, WV_ERR_LIMIT, "d=%u K=%u need too much shared memory",
           d, K);
  cudaError_t e = cudaSuccess;
  uint32_t *leaf = c->buf<uint32_t>("kd_leaf", total, &e);
  uint32_t *scr = c->buf<uint32_t>("kd_scr", total, &e);
  KNode *nodes = c->buf<KNode>("kd_nodes", ncap, &e);
  uint32_t *ncount = c->buf<uint32_t>("kd_ncount", 4, &e);
  int *act_d = c->buf<int>("kd_act", std::max<size_t>(2 * KDT_ACTIVE_MAX + T, 16), &e);
  int *rnd_d = c->buf<int>("kd_rand", (size_t)T * (n - 1), &e);
  WV_CUDA(c, e);
  // id lists: n - 1 rand() values per tree, tree by tree
  {
    std::vector<int> r((size_t)T * (n - 1));
    for (auto &v : r) v = c->rnd.next();
    WV_CUDA(c, cudaMemcpyAsync(rnd_d, r.data(), r.size() * 4, cudaMemcpyHostToDevice, c->stream));
    const size_t sm = (size_t)n * 4;
    const bool in_smem = sm <= 200 * 1024;
    if (in_smem) WV_CUDA(c, cudaFuncSetAttribute(k_kdt_shuffle, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    k_kdt_shuffle<<<T, 32, in_smem ? sm : 0, c->stream>>>(n, rnd_d, leaf, in_smem ? 1 : 0);
    WV_CUDA(c, cudaGetLastError());
    WV_CUDA(c, cudaStreamSynchronize(c->stream));
  }
  // roots, then the active levels
  std::vector<KNode> roots(T);
  for (uint32_t t = 0; t < T; t++) roots[t] = KNode{-1, 0.f, 0, n, -1, -1, -1, 0, (int)t};
  WV_CUDA(c, cudaMemcpyAsync(nodes, roots.data(), T * sizeof(KNode), cudaMemcpyHostToDevice, c->stream));
  uint32_t count = T;
  std::vector<int> act(T);
  for (uint32_t t = 0; t < T; t++) act[t] = (int)t;
  std::mt19937 first(1998);
  const uint32_t rv0 = (uint32_t)first();
  WV_CUDA(c, cudaFuncSetAttribute(k_kdt_level, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_split));
  WV_CUDA(c, cudaFuncSetAttribute(k_kdt_dfs, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_split));
  std::vector<KNode> kids;
  while (!act.empty() && act.size() < KDT_ACTIVE_MAX) {
    const uint32_t na = (uint32_t)act.size();
    WV_CHECK(c, count + 2 * (size_t)na <= ncap, WV_ERR_LIMIT, "KD-tree node capacity");
    WV_CUDA(c, cudaMemcpyAsync(act_d, act.data(), na * 4, cudaMemcpyHostToDevice, c->stream));
    k_kdt_level<<<nblocks(na, KW, c->sms * 8), KW * 32, smem_split, c->stream>>>(c->base.as<float>(), d, n, leaf,
                                                                                   scr, nodes, act_d, na, count, rv0);
    WV_CUDA(c, cudaGetLastError());
    kids.resize(2 * (size_t)na);
    WV_CUDA(c, cudaMemcpyAsync(kids.data(), nodes + count, kids.size() * sizeof(KNode), cudaMemcpyDeviceToHost,
                               c->stream));
    WV_CUDA(c, cudaStreamSynchronize(c->stream));
    std::vector<int> next;
    for (uint32_t i = 0; i < na; i++) {
      if (kids[2 * i].end - kids[2 * i].start > K) next.push_back((int)(count + 2 * i));
      if (kids[2 * i + 1].end - kids[2 * i + 1].start > K) next.push_back((int)(count + 2 * i + 1));
    }
    count += 2 * na;
    act.swap(next);
  }
  WV_CUDA(c, cudaMemcpyAsync(ncount, &count, 4, cudaMemcpyHostToDevice, c->stream));
  if (!act.empty()) {
    const uint32_t na = (uint32_t)act.size();
    uint32_t nmt = 0;  // splits below one active node: fewer than its ids
    std::vector<KNode> an(na);
    for (uint32_t i = 0; i < na; i++) {
      WV_CUDA(c, cudaMemcpyAsync(&an[i], nodes + act[i], sizeof(KNode), cudaMemcpyDeviceToHost, c->stream));
    }
    WV_CUDA(c, cudaStreamSynchronize(c->stream));
    for (auto &x : an) nmt = std::max(nmt, x.end - x.start);
    uint32_t *mt = c->buf<uint32_t>("kd_mt", nmt + 1, &e);
    const int blocks = nblocks(na, KW, c->sms * 4);
    int *stacks = c->buf<int>("kd_stack", (size_t)blocks * KW * KDT_MAX_DEPTH, &e);
    WV_CUDA(c, e);
    int rc = mt19937_gpu(c, 1998, mt, nmt + 1);
    if (rc) return rc;
    WV_CUDA(c, cudaMemcpyAsync(act_d, act.data(), na * 4, cudaMemcpyHostToDevice, c->stream));
    k_kdt_dfs<<<blocks, KW * 32, smem_split, c->stream>>>(c->base.as<float>(), d, n, leaf, scr, nodes, act_d, na,
                                                            ncount, ncap, mt, nmt + 1, stacks, c->d_status());
    WV_CUDA(c, cudaGetLastError());
  }
  int rc = check_device_status(c, "KD-tree build");
  if (rc) return rc;
  WV_CUDA(c, cudaMemcpyAsync(&count, ncount, 4, cudaMemcpyDeviceToHost, c->stream));
  WV_CUDA(c, cudaStreamSynchronize(c->stream));
  // merges
  int *leaf_of = c->buf<int>("kd_leafof", total, &e);
  uint32_t *pos_of = c->buf<uint32_t>("kd_posof", total, &e);
  uint32_t *rcnt = c->buf<uint32_t>("kd_rcnt", (size_t)count + 1, &e);
  uint32_t *roff = c->buf<uint32_t>("kd_roff", (size_t)count + 1, &e);
  uint32_t *scan_tmp = c->buf<uint32_t>("kd_scan", scan_scratch_words((size_t)count + 1), &e);
  WV_CUDA(c, e);
  const int gb = c->sms * 8;
  k_kdt_leafmap<<<nblocks(count, 256, gb), 256, 0, c->stream>>>(nodes, ncount, n, leaf_of);
  k_kdt_pos<<<nblocks(total, 256, gb), 256, 0, c->stream>>>(leaf, total, n, pos_of);
  WV_CUDA(c, cudaMemsetAsync(rcnt, 0, ((size_t)count + 1) * 4, c->stream));
  k_kdt_records<<<nblocks(total, 256, gb), 256, 0, c->stream>>>(c->base.as<float>(), d, n, total, leaf, nodes,
                                                                  leaf_of, (int)mlevel, rcnt, nullptr, nullptr);
  WV_CUDA(c, cudaGetLastError());
  {
    // the offsets are 32-bit: refuse forests whose records would not fit
    std::vector<uint32_t> hc((size_t)count + 1);
    WV_CUDA(c, cudaMemcpyAsync(hc.data(), rcnt, hc.size() * 4, cudaMemcpyDeviceToHost, c->stream));
    WV_CUDA(c, cudaStreamSynchronize(c->stream));
    unsigned long long sum = 0;
    for (uint32_t v : hc) sum += v;
    WV_CHECK(c, sum < 0xffffffffull, WV_ERR_LIMIT, "INIT_KDT: %llu merge records exceed 32-bit offsets", sum);
  }
  WV_CUDA(c, exclusive_scan_u32(rcnt, roff, (size_t)count + 1, scan_tmp, c->stream));
  uint32_t nrec = 0;
  WV_CUDA(c, cudaMemcpyAsync(&nrec, roff + count, 4, cudaMemcpyDeviceToHost, c->stream));
  WV_CUDA(c, cudaStreamSynchronize(c->stream));
  unsigned long long *rec = c->buf<unsigned long long>("kd_rec", (size_t)nrec + 1, &e);
  unsigned long long *rec2 = c->buf<unsigned long long>("kd_rec2", (size_t)nrec + 1, &e);
  WV_CUDA(c, e);
  WV_CUDA(c, cudaMemsetAsync(rcnt, 0, ((size_t)count + 1) * 4, c->stream));
  k_kdt_records<<<nblocks(total, 256, gb), 256, 0, c->stream>>>(c->base.as<float>(), d, n, total, leaf, nodes,
                                                                  leaf_of, (int)mlevel, rcnt, roff, rec);
  k_kdt_sort_records<<<nblocks(count, 8, gb), 256, 0, c->stream>>>(ncount, roff, rcnt, rec, rec2);
  WV_CUDA(c, cudaGetLastError());
  uint32_t *kn_ids = c->buf<uint32_t>("kd_knids", (size_t)n * K, &e);
  float *kn_dist = c->buf<float>("kd_kndist", (size_t)n * K, &e);
  uint32_t *kn_sz = c->buf<uint32_t>("kd_knsz", n, &e);
  uint32_t *short_rows = c->buf<uint32_t>("kd_short", 4, &e);
  WV_CUDA(c, e);
  WV_CUDA(c, cudaFuncSetAttribute(k_kdt_merge, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_merge));
  k_kdt_merge<<<nblocks(n, KW, c->sms * 16), KW * 32, smem_merge, c->stream>>>(
      c->base.as<float>(), d, n, T, K, (int)mlevel, leaf, nodes, leaf_of, pos_of, roff, rcnt, rec2, kn_ids, kn_dist,
      kn_sz);
  WV_CUDA(c, cudaGetLastError());
  // the graph
  WV_CUDA(c, c->fg_ids.ensure((size_t)n * K * 4));
  WV_CUDA(c, c->fg_dist.ensure((size_t)n * K * 4));
  WV_CUDA(c, c->fg_deg.ensure((size_t)n * 4));
  WV_CUDA(c, cudaMemsetAsync(short_rows, 0, 4, c->stream));
  k_kdt_rows<<<nblocks((size_t)n * K, 256, gb), 256, 0, c->stream>>>(
      n, K, kn_ids, kn_dist, kn_sz, c->fg_ids.as<uint32_t>(), c->fg_dist.as<float>(), c->fg_deg.as<uint32_t>(),
      short_rows);
  uint32_t nshort = 0;
  WV_CUDA(c, cudaMemcpyAsync(&nshort, short_rows, 4, cudaMemcpyDeviceToHost, c->stream));
  WV_CUDA(c, cudaStreamSynchronize(c->stream));
  if (nshort > 0) {
    int *more = c->buf<int>("kd_more", 4, &e);
    WV_CUDA(c, e);
    size_t nmt = std::max<size_t>(4096, (size_t)nshort * K * 4);
    for (int attempt = 0;; attempt++) {
      uint32_t *mt = c->buf<uint32_t>("kd_fillmt", nmt, &e);
      WV_CUDA(c, e);
      rc = mt19937_gpu(c, 1998, mt, nmt);
      if (rc) return rc;
      k_kdt_fill<<<1, 32, 0, c->stream>>>(c->base.as<float>(), d, n, K, kn_ids, kn_dist, kn_sz, mt, nmt,
                                          c->fg_ids.as<uint32_t>(), c->fg_dist.as<float>(), c->fg_deg.as<uint32_t>(),
                                          more);
      WV_CUDA(c, cudaGetLastError());
      int h = 0;
      WV_CUDA(c, cudaMemcpyAsync(&h, more, 4, cudaMemcpyDeviceToHost, c->stream));
      WV_CUDA(c, cudaStreamSynchronize(c->stream));
      if (h == 0) break;
      WV_CHECK(c, h == 1 && attempt < 8, WV_ERR_ARG,
               "INIT_KDT: a row cannot reach K=%u distinct distances (the reference would not terminate)", K);
      nmt *= 8;
    }
  }
  c->fg_n = n;
  c->fg_w = K;
  c->fg_has_ep = false;
  c->fg_eps.clear();
  rc = check_device_status(c, "INIT_KDT");
  if (rc) return rc;
  // the forest stays in the work buffers for SEARCH_ENTRY_KDT
  c->kdt.n = n;
  c->kdt.T = T;
  c->kdt.nodes = count;
  return WV_OK;
}

int draw_seeds_kdt(wv_ctx *c, const float *queries, uint32_t nq, uint32_t L, uint32_t *seeds, uint32_t stride) {
  const KdtForest &F = c->kdt;
  WV_CHECK(c, F.T > 0 && F.n == c->n && F.nodes >= F.T, WV_ERR_STATE,
           "the KD-tree entry needs the trees of a completed wv_init_kdt on this base");
  if (nq == 0) return WV_OK;
  const uint32_t n = F.n, d = c->d, lsize = L / (F.T * KDT_TNS) + 1;
  cudaError_t e = cudaSuccess;
  const KNode *nodes = c->buf<KNode>("kd_nodes", 1, &e);
  const uint32_t *leaf = c->buf<uint32_t>("kd_leaf", 1, &e);
  float *dq = c->buf<float>("kd_q", (size_t)nq * d, &e);
  int *vn = c->buf<int>("kd_vn", (size_t)nq * F.T * lsize, &e);
  uint32_t *ds = c->buf<uint32_t>("kd_seeds", (size_t)nq * L, &e);
  uint32_t *dt = c->buf<uint32_t>("kd_taken", nq, &e);
  WV_CUDA(c, e);
  WV_CUDA(c, cudaMemcpyAsync(dq, queries, (size_t)nq * d * 4, cudaMemcpyHostToDevice, c->stream));
  k_kdt_entry<<<nblocks(nq, 8, c->sms * 16), 256, 0, c->stream>>>(nodes, F.nodes, leaf, n, F.T, dq, nq, d, L, lsize,
                                                                   vn, ds, L, dt, c->d_status());
  WV_CUDA(c, cudaGetLastError());
  std::vector<uint32_t> taken(nq), hs((size_t)nq * L);
  WV_CUDA(c, cudaMemcpyAsync(hs.data(), ds, hs.size() * 4, cudaMemcpyDeviceToHost, c->stream));
  WV_CUDA(c, cudaMemcpyAsync(taken.data(), dt, (size_t)nq * 4, cudaMemcpyDeviceToHost, c->stream));
  int rc = check_device_status(c, "KD-tree entry");
  if (rc) return rc;
  // rand() % n fills, in query order (they share the rand() stream)
  std::vector<char> flags(n, 0);
  for (uint32_t q = 0; q < nq; q++) {
    const uint32_t *g = hs.data() + (size_t)q * L;
    uint32_t *s = seeds + (size_t)q * stride;
    uint32_t p = taken[q];
    std::copy(g, g + p, s);
    if (p >= L) continue;
    for (uint32_t i = 0; i < p; i++) flags[s[i]] = 1;
    if (q < n) flags[q] = 1;
    while (p < L) {
      const uint32_t id = (uint32_t)c->rnd.next() % n;
      if (flags[id]) continue;
      flags[id] = 1;
      s[p++] = id;
    }
    for (uint32_t i = 0; i < L; i++) flags[s[i]] = 0;
    if (q < n) flags[q] = 0;
  }
  return WV_OK;
}

}  // namespace wv
