// K1/K2: INIT_RANDOM and REFINE_NN_DESCENT on GB300.
//
// Replaces ComponentInitRandom::InitInner (src/component_init.cpp:11-45) and
// ComponentRefineNNDescent::RefineInner (src/component_refine.cpp:12-239,
// with nhood::insert / nhood::join, include/weavess/index.h:86-150).
//
// Layout in HBM (n nodes):
//   pool   n x L  {float dist, u32 id|FLAG}  the per-node bounded max-heap, kept
//                 in libstdc++'s heap arrangement between join and update
//   psz, M n      pool sizes, sampled-prefix lengths
//   nnew   n x (S+R), nold n x min(L+R, 2R)  join lists, lnew/lold lengths
//
// The plain form reproduces the single-threaded reference bit for bit:
//  * join: every local-join pair is evaluated once (exact-order FP32) and its
//    two offers ("insert j into i", "insert i into j") are keyed by the
//    reference's sequential position (node n, pair position in
//    nhood::join's loops, side).  Offers that cannot pass nhood::insert's
//    first test (dist > pool max at that time; the max only falls during a
//    join) are dropped at the source.  The rest are grouped per target, sorted
//    by key, and applied by one warp per target with libstdc++'s
//    push_heap/pop_heap, so ties resolve exactly as they do sequentially.
//    Nodes are processed in chunks in node order, so a later chunk sees the
//    pools the earlier chunks left.
//  * update: per node std::sort (stl_order.cuh), the sampled prefix M, the
//    new/old split and make_heap run as in the reference.  The reverse
//    condition reads pool.back() of the other node as the reference's
//    sequential order sees it: the last slot of its make_heap'd pool if the
//    other node was processed earlier, its maximum otherwise.  Reverse lists
//    are capped at R; each push beyond R overwrites slot rand() % R, the
//    rand() values being drawn on the host, in global (n, l) order, from the
//    context's stream.
//  * the first join is skipped: nhood(L, S) leaves nn_new as 2S zeros
//    (index.h:98-103), which join pairs with nothing.
#include <cuda_bf16.h>

#include <algorithm>
#include <cstdlib>
#include <string>
#include <vector>

#include "wv_common.cuh"
#include "wv_mt.cuh"
#include "wv_nnd.h"
#include "wv_scan.h"
#include "wv_umma.cuh"

namespace wv {
namespace {

struct Ent {
  float d;
  uint32_t idf;  // id | FLAG when flag (Neighbor::flag) is true
};
struct EntLess {
  __host__ __device__ bool operator()(const Ent &a, const Ent &b) const { return a.d < b.d; }
};

// ---------------------------------------------------------------- mt19937
// std::mt19937 stream of one seed (wv_mt.cuh), twisted by a block.
__global__ void __launch_bounds__(256) k_mt19937(uint32_t seed, uint32_t *out, size_t count) {
  __shared__ uint32_t mt[624];
  const int t = threadIdx.x;
  if (t == 0) {
    mt[0] = seed;
    for (int i = 1; i < 624; i++) mt[i] = mt_seed_next(mt[i - 1], (uint32_t)i);
  }
  __syncthreads();
  for (size_t base = 0; base < count; base += 624) {
    // phase A: i in [0, 227) reads only old words
    uint32_t v = 0;
    if (t < 227) v = mt_mix(mt[t], mt[t + 1], mt[t + 397]);
    __syncthreads();
    if (t < 227) mt[t] = v;
    __syncthreads();
    // phase B: i in [227, 454) reads new word i - 227
    if (t < 227) v = mt_mix(mt[t + 227], mt[t + 228], mt[t]);
    __syncthreads();
    if (t < 227) mt[t + 227] = v;
    __syncthreads();
    // phase C: i in [454, 623)
    if (t < 169) v = mt_mix(mt[t + 454], mt[t + 455], mt[t + 227]);
    __syncthreads();
    if (t < 169) mt[t + 454] = v;
    __syncthreads();
    // phase D: i = 623 wraps to the new word 0
    if (t == 0) mt[623] = mt_mix(mt[623], mt[0], mt[396]);
    __syncthreads();
    for (int i = t; i < 624; i += blockDim.x)
      if (base + i < count) out[base + i] = mt_temper(mt[i]);
    __syncthreads();
  }
}

// ---------------------------------------------------------------- INIT_RANDOM
// One warp per node: GenRandom from the node's S+1 consecutive mt19937
// outputs, distances (self hits dropped), std::sort of the row.
constexpr int INIT_WARPS = 4;

__global__ void __launch_bounds__(INIT_WARPS * 32)
    k_init_random(const float *__restrict__ base, uint32_t n, uint32_t d, uint32_t S, const uint32_t *__restrict__ mt,
                  uint32_t *ids, float *dist, uint32_t *deg) {
  extern __shared__ __align__(16) uint8_t smem[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const size_t per_warp = (size_t)STAGE_FLOATS * 4 + ((d + 3) & ~3u) * 4 + 64 * sizeof(DI);
  uint8_t *p = smem + warp * per_warp;
  float *stage = (float *)p;
  float *qv = (float *)(p + (size_t)STAGE_FLOATS * 4);
  DI *row = (DI *)(p + (size_t)STAGE_FLOATS * 4 + ((d + 3) & ~3u) * 4);
  const uint32_t gw = gridDim.x * INIT_WARPS;
  for (uint32_t i = blockIdx.x * INIT_WARPS + warp; i < n; i += gw) {
    const uint32_t *r = mt + (size_t)i * (S + 1);
    // addr[j] = rng() % (N - size), sorted (ints: any correct sort agrees)
    uint32_t v = lane < (int)S ? r[lane] % (n - S) : 0xffffffffu;
    for (int k = 2; k <= 32; k <<= 1)
      for (int j = k >> 1; j > 0; j >>= 1) {
        uint32_t o = __shfl_xor_sync(FULL, v, j);
        bool up = (lane & k) == 0, lower = (lane & j) == 0;
        uint32_t lo = min(v, o), hi = max(v, o);
        v = (lower == up) ? lo : hi;
      }
    // bump duplicates: a_j = max(v_j, a_{j-1} + 1) = j + max_{j'<=j}(v_j' - j')
    long long m = (long long)v - lane;
    for (int o = 1; o < 32; o <<= 1) {
      long long y = __shfl_up_sync(FULL, m, o);
      if (lane >= o) m = max(m, y);
    }
    uint32_t a = (uint32_t)(m + lane);
    uint32_t off = r[S] % n;
    uint32_t id = (a + off) % n;
    bool keep = lane < (int)S && id != i;
    unsigned km = __ballot_sync(FULL, keep);
    int cnt = __popc(km);
    // compact kept ids (draw order) to lanes 0..cnt-1
    uint32_t *xch = (uint32_t *)row;
    if (keep) xch[__popc(km & ((1u << lane) - 1))] = id;
    for (uint32_t k = lane; k < d; k += 32) qv[k] = base[(size_t)i * d + k];
    __syncwarp();
    uint32_t my = lane < cnt ? xch[lane] : 0u;
    __syncwarp();
    float dd = warp_l2_rows(base, d, my, cnt, qv, stage, lane);
    // std::sort of the row: stable order unless ties with cnt > 16
    float dv = lane < cnt ? dd : __int_as_float(0x7f800000);
    int rank = 0;
    bool tie = false;
    for (int t = 0; t < cnt; t++) {
      float o = __shfl_sync(FULL, dv, t);
      rank += (o < dv) || (o == dv && t < lane);
      tie |= (o == dv && t != lane && lane < cnt);
    }
    tie = __any_sync(FULL, tie);
    if (!tie || cnt <= 16) {
      if (lane < cnt) row[rank] = DI{dd, my};
    } else {
      if (lane < cnt) row[lane] = DI{dd, my};
      __syncwarp();
      if (lane == 0) stl::sort(row, cnt, DILess());
    }
    __syncwarp();
    if (lane < cnt) {
      ids[(size_t)i * S + lane] = row[lane].i;
      dist[(size_t)i * S + lane] = row[lane].d;
    }
    if (lane == 0) deg[i] = cnt;
    __syncwarp();
  }
}

// ---------------------------------------------------------------- INIT_RAND
// ComponentInitRand::InitInner (component_init.cpp:979-1025): node i draws L
// ids by GenRandom from the shared mt19937 stream (outputs [i (L + 1),
// (i + 1)(L + 1))), skips itself, takes the distances (exact reference order,
// a lane per row), and its pool goes through make_heap then std::sort (the
// heap arrangement is where the sort starts, which settles equal
// distances); one warp per node, the two sequential steps on one lane.
constexpr int IR_WARPS = 4;
__host__ __device__ inline size_t init_rand_warp_bytes(uint32_t L, uint32_t d) {
  // a multiple of 16 bytes, so that every warp's query copy starts 16-byte aligned
  const size_t b = (size_t)pow2_ge(L) * 4 + (size_t)L * 4 + (size_t)L * sizeof(DI) + (((size_t)d * 4 + 15) & ~size_t(15));
  return (b + 15) & ~size_t(15);
}
__global__ void __launch_bounds__(IR_WARPS * 32)
    k_init_rand(const float *__restrict__ base, uint32_t n, uint32_t d, uint32_t L, const uint32_t *__restrict__ mt,
                uint32_t *ids, float *dist, uint32_t *deg) {
  extern __shared__ __align__(16) uint8_t smem[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  uint8_t *p = smem + (size_t)warp * init_rand_warp_bytes(L, d);
  float *qv = reinterpret_cast<float *>(p);
  p += ((size_t)d * 4 + 15) & ~size_t(15);
  DI *pool = reinterpret_cast<DI *>(p);
  p += (size_t)L * sizeof(DI);
  uint32_t *gen = reinterpret_cast<uint32_t *>(p);
  p += (size_t)L * 4;
  uint32_t *key = reinterpret_cast<uint32_t *>(p);
  const unsigned lt = (1u << lane) - 1u;
  for (uint32_t i = blockIdx.x * IR_WARPS + warp; i < n; i += gridDim.x * IR_WARPS) {
    const uint32_t *r = mt + (size_t)i * (L + 1);
    for (uint32_t j = lane; j < L; j += 32) key[j] = r[j] % (n - L);
    for (uint32_t k = lane; k < d; k += 32) qv[k] = base[(size_t)i * d + k];
    __syncwarp();
    warp_gen_random_tail(key, L, r[L] % n, n, gen, lane);
    // the pool in draw order without the node itself
    uint32_t cnt = 0;
    for (uint32_t b = 0; b < L; b += 32) {
      const uint32_t j = b + lane;
      const uint32_t id = j < L ? gen[j] : i;
      const bool keep = j < L && id != i;
      const unsigned km = __ballot_sync(FULL, keep);
      if (keep) {
        const float4 *x = reinterpret_cast<const float4 *>(qv);
        const float4 *y = reinterpret_cast<const float4 *>(base + (size_t)id * d);
        float acc = 0.f;
        for (uint32_t g = 0; g < (d >> 2); g++) acc = __fadd_rn(acc, group4(x[g], __ldg(y + g)));
        pool[cnt + __popc(km & lt)] = DI{acc, id};
      }
      cnt += __popc(km);
    }
    __syncwarp();
    if (lane == 0) {
      stl::make_heap(pool, (int)cnt, DILess());
      stl::sort(pool, (int)cnt, DILess());
    }
    __syncwarp();
    for (uint32_t j = lane; j < cnt; j += 32) {
      ids[(size_t)i * L + j] = pool[j].i;
      dist[(size_t)i * L + j] = pool[j].d;
    }
    if (lane == 0) deg[i] = cnt;
    __syncwarp();
  }
}

// ---------------------------------------------------------------- NN-Descent state
struct Nnd {
  uint32_t n, d, S, K, L, R, capn, capo;
  const float *base;
  const float *xnorm;  // squared row norms (integer data; the tensor-core join)
  Ent *pool;
  uint32_t *psz, *M;
  uint32_t *nnew, *nold, *lnew, *lold, *pnew, *pold;
  Ent *pre;  // sorted sampled prefix of the last update (n x L)
  float *maxd, *hback;
};

// init(): pools <- init rows (flag true), make_heap; M = S.
// efanna: ComponentRefineEFANNA::init (component_refine.cpp:1044-1057) sorts
// the row by distance (std::sort) and skips the node itself and an id equal
// to its predecessor in that order
__global__ void k_nnd_init(Nnd s, const uint32_t *ids, const float *dist, const uint32_t *deg, uint32_t w,
                           int efanna) {
  extern __shared__ __align__(16) uint8_t smem[];
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  Ent *P = (Ent *)smem + (size_t)threadIdx.x * (s.L + 1);
  if (i >= s.n) return;
  uint32_t sz = min(deg[i], s.L);
  for (uint32_t j = 0; j < sz; j++) P[j] = Ent{dist[(size_t)i * w + j], ids[(size_t)i * w + j] | FLAG};
  if (efanna) {
    stl::sort(P, (int)sz, EntLess());
    uint32_t k = 0, prev = 0;
    for (uint32_t t = 0; t < sz; t++) {
      const uint32_t id = P[t].idf & ID_MASK;
      const bool skip = id == i || (t > 0 && id == prev);
      prev = id;
      if (!skip) P[k++] = P[t];
    }
    sz = k;
  }
  stl::make_heap(P, (int)sz, EntLess());
  for (uint32_t j = 0; j < sz; j++) s.pool[(size_t)i * s.L + j] = P[j];
  s.psz[i] = sz;
  s.M[i] = s.S;
}

// nhood(L, S, rng, N) (index.h:105-111) for every node: nn_new = GenRandom of
// 2S ids from the shared mt19937 stream (node i reads outputs
// [i (2S + 1), (i + 1)(2S + 1))), nn_old empty.  A warp per node.
constexpr int EF_WARPS = 4;
__global__ void __launch_bounds__(EF_WARPS * 32) k_efanna_nnew(Nnd s, const uint32_t *mtv) {
  extern __shared__ uint32_t ef_key[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t L2 = 2 * s.S;
  uint32_t *key = ef_key + (size_t)warp * pow2_ge(L2);
  for (uint32_t i = blockIdx.x * EF_WARPS + warp; i < s.n; i += gridDim.x * EF_WARPS) {
    const uint32_t *r = mtv + (size_t)i * (L2 + 1);
    for (uint32_t j = lane; j < L2; j += 32) key[j] = r[j] % (s.n - L2);
    __syncwarp();
    warp_gen_random_tail(key, L2, r[L2] % s.n, s.n, s.nnew + (size_t)i * s.capn, lane);
    if (lane == 0) {
      s.lnew[i] = L2;
      s.lold[i] = 0;
    }
  }
}

// update() passes 1-3 for node i: sort, sampled prefix M, new/old lists from
// the pool, flags cleared, make_heap; records the prefix, the sorted maximum
// and the back slot of the heap for the reverse condition.
__global__ void k_upd_sort(Nnd s) {
  extern __shared__ __align__(16) uint8_t smem[];
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  Ent *P = (Ent *)smem + (size_t)threadIdx.x * (s.L + 1);
  if (i >= s.n) return;
  const uint32_t sz = s.psz[i];
  for (uint32_t j = 0; j < sz; j++) P[j] = s.pool[(size_t)i * s.L + j];
  stl::sort(P, (int)sz, EntLess());
  const uint32_t maxl = min(s.M[i] + s.S, sz);
  uint32_t c = 0, l = 0;
  while (l < maxl && c < s.S) {
    if (P[l].idf & FLAG) ++c;
    ++l;
  }
  s.M[i] = l;
  uint32_t pn = 0, po = 0;
  for (uint32_t j = 0; j < l; j++) {
    s.pre[(size_t)i * s.L + j] = P[j];
    uint32_t id = P[j].idf & ID_MASK;
    if (P[j].idf & FLAG) {
      s.nnew[(size_t)i * s.capn + pn++] = id;
    } else {
      // nn_old is truncated to 2R at the end of the update (refine.cpp:231-234)
      if (po < s.capo) s.nold[(size_t)i * s.capo + po] = id;
      po++;
    }
    P[j].idf = id;
  }
  s.pnew[i] = pn;
  s.pold[i] = po;
  s.maxd[i] = sz ? P[sz - 1].d : 0.f;
  stl::make_heap(P, (int)sz, EntLess());
  s.hback[i] = sz ? P[sz - 1].d : 0.f;
  for (uint32_t j = 0; j < sz; j++) s.pool[(size_t)i * s.L + j] = P[j];
}

constexpr int BK_WARPS = 4;
constexpr int BK_CAP = 1024;

// reverse condition of update() pass 3 (component_refine.cpp:191, 202)
__device__ __forceinline__ bool rev_cond(const Nnd &s, uint32_t n, uint32_t o, float dist) {
  float back = o < n ? s.hback[o] : s.maxd[o];
  return dist > back;
}

// events per node and per (target, list) bucket
__global__ void k_upd_count(Nnd s, uint32_t *ecount, uint32_t *bcnt, uint32_t *bmax) {
  const uint32_t n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= s.n) return;
  uint32_t cnt = 0;
  for (uint32_t l = 0; l < s.M[n]; l++) {
    Ent e = s.pre[(size_t)n * s.L + l];
    uint32_t o = e.idf & ID_MASK;
    if (rev_cond(s, n, o, e.d)) {
      cnt++;
      uint32_t prev = atomicAdd(&bcnt[2 * o + ((e.idf & FLAG) ? 0 : 1)], 1u);
      if (prev + 1 > BK_CAP) atomicMax(bmax, prev + 1);
    }
  }
  ecount[n] = cnt;
}

__global__ void k_upd_scatter(Nnd s, const uint32_t *eoff, const uint32_t *boff, uint32_t *bcur, uint32_t *bsrc,
                              uint32_t *bflat) {
  const uint32_t n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= s.n) return;
  uint32_t f = eoff[n];
  for (uint32_t l = 0; l < s.M[n]; l++) {
    Ent e = s.pre[(size_t)n * s.L + l];
    uint32_t o = e.idf & ID_MASK;
    if (rev_cond(s, n, o, e.d)) {
      uint32_t b = 2 * o + ((e.idf & FLAG) ? 0 : 1);
      uint32_t slot = boff[b] + atomicAdd(&bcur[b], 1u);
      bsrc[slot] = n;
      bflat[slot] = f;
      f++;
    }
  }
}

// sorts one bucket's (src, flat) pairs by src (srcs are distinct) in shared
// memory with a warp bitonic sort; marks events ranked >= R as overflow

__device__ void warp_bitonic_u64(unsigned long long *k, int P, int lane) {
  for (int sz = 2; sz <= P; sz <<= 1)
    for (int j = sz >> 1; j > 0; j >>= 1) {
      for (int i = lane; i < P; i += 32) {
        int l = i ^ j;
        if (l > i) {
          bool up = (i & sz) == 0;
          unsigned long long a = k[i], b = k[l];
          if ((a > b) == up) {
            k[i] = b;
            k[l] = a;
          }
        }
      }
      __syncwarp();
    }
}

__global__ void __launch_bounds__(BK_WARPS * 32)
    k_bucket_sort(uint32_t nb, const uint32_t *boff, const uint32_t *bcnt, uint32_t *bsrc, uint32_t *bflat,
                  uint32_t R, uint32_t *ovf, uint32_t *bigb, uint32_t *nbig) {
  __shared__ unsigned long long keys[BK_WARPS][BK_CAP];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t b = blockIdx.x * BK_WARPS + warp;
  if (b >= nb) return;
  const uint32_t cnt = bcnt[b], off = boff[b];
  if (cnt <= 1) return;
  if (cnt > BK_CAP) {  // left to the block path
    if (lane == 0) bigb[atomicAdd(nbig, 1u)] = b;
    return;
  }
  int P = 1;
  while (P < (int)cnt) P <<= 1;
  unsigned long long *k = keys[warp];
  for (int i = lane; i < P; i += 32)
    k[i] = i < (int)cnt ? ((unsigned long long)bsrc[off + i] << 32) | bflat[off + i] : ~0ull;
  __syncwarp();
  warp_bitonic_u64(k, P, lane);
  for (int i = lane; i < (int)cnt; i += 32) {
    bsrc[off + i] = (uint32_t)(k[i] >> 32);
    bflat[off + i] = (uint32_t)k[i];
    if ((uint32_t)i >= R) ovf[(uint32_t)k[i]] = 1u;
  }
}

// buckets longer than BK_CAP: one block each, bitonic sort in a global
// scratch region of P (power of 2 >= the longest bucket) keys per block
__global__ void __launch_bounds__(1024)
    k_bucket_sort_big(const uint32_t *bigb, const uint32_t *boff, const uint32_t *bcnt, uint32_t *bsrc,
                      uint32_t *bflat, uint32_t R, uint32_t *ovf, unsigned long long *scratch, uint32_t P) {
  const uint32_t b = bigb[blockIdx.x], cnt = bcnt[b], off = boff[b];
  unsigned long long *k = scratch + (size_t)blockIdx.x * P;
  for (uint32_t i = threadIdx.x; i < P; i += blockDim.x)
    k[i] = i < cnt ? ((unsigned long long)bsrc[off + i] << 32) | bflat[off + i] : ~0ull;
  __syncthreads();
  for (uint32_t sz = 2; sz <= P; sz <<= 1)
    for (uint32_t j = sz >> 1; j > 0; j >>= 1) {
      for (uint32_t i = threadIdx.x; i < P; i += blockDim.x) {
        uint32_t l = i ^ j;
        if (l > i) {
          bool up = (i & sz) == 0;
          unsigned long long x = k[i], y = k[l];
          if ((x > y) == up) {
            k[i] = y;
            k[l] = x;
          }
        }
      }
      __syncthreads();
    }
  for (uint32_t i = threadIdx.x; i < cnt; i += blockDim.x) {
    bsrc[off + i] = (uint32_t)(k[i] >> 32);
    bflat[off + i] = (uint32_t)k[i];
    if (i >= R) ovf[(uint32_t)k[i]] = 1u;
  }
}

// update() pass 4: node o's lists = pool part ++ reverse list (first R
// pushes, then the overflow overwrites in order); nn_old truncated to 2R
__global__ void k_bucket_apply(Nnd s, const uint32_t *boff, const uint32_t *bcnt, const uint32_t *bsrc,
                               const uint32_t *bflat, const uint32_t *ovf_ord, const int *rv) {
  const uint32_t o = blockIdx.x * blockDim.x + threadIdx.x;
  if (o >= s.n) return;
  for (int type = 0; type < 2; type++) {
    const uint32_t b = 2 * o + type, cnt = bcnt[b], off = boff[b];
    uint32_t *list = type == 0 ? s.nnew + (size_t)o * s.capn + s.pnew[o] : s.nold + (size_t)o * s.capo + s.pold[o];
    const uint32_t keep = min(cnt, s.R);
    // the part of the reverse list that fits the (truncated) list
    const uint32_t room = type == 0 ? s.capn - s.pnew[o] : (s.pold[o] < 2 * s.R ? 2 * s.R - s.pold[o] : 0u);
    for (uint32_t j = 0; j < keep && j < room; j++) list[j] = bsrc[off + j];
    for (uint32_t j = s.R; j < cnt; j++) {
      uint32_t pos = (uint32_t)rv[ovf_ord[bflat[off + j]]] % s.R;
      if (pos < room) list[pos] = bsrc[off + j];
    }
    if (type == 0) s.lnew[o] = s.pnew[o] + keep;
    else s.lold[o] = min(s.pold[o] + keep, 2 * s.R);
  }
}

// ---------------------------------------------------------------- join
struct Offers {
  uint32_t *tgt;
  unsigned long long *key;
  uint32_t *cand;
  float *dist;
  uint32_t *cursor;
  uint32_t cap;
  uint32_t *tcnt;
};

constexpr int J_THREADS = 256;
constexpr int J_TI = 16;  // new rows per i tile
constexpr int J_TJ = 64;  // rows per j tile (new ++ old); fewer for long rows (the tile must fit shared memory)

__device__ __forceinline__ void emit(const Offers &o, bool ok, uint32_t t, unsigned long long key, uint32_t c,
                                     float d, int lane, int *status) {
  unsigned m = __ballot_sync(FULL, ok);
  if (!m) return;
  uint32_t base = 0;
  int leader = __ffs(m) - 1;
  if (lane == leader) base = atomicAdd(o.cursor, (uint32_t)__popc(m));
  base = __shfl_sync(FULL, base, leader);
  if (ok) {
    uint32_t pos = base + __popc(m & ((1u << lane) - 1));
    if (pos < o.cap) {
      o.tgt[pos] = t;
      o.key[pos] = key;
      o.cand[pos] = c;
      o.dist[pos] = d;
      atomicAdd(&o.tcnt[t], 1u);
    } else {
      set_err(status, DEV_OVERFLOW);
    }
  }
}

// local join of nodes [n0, n1): one block per node
__global__ void __launch_bounds__(J_THREADS) k_join(Nnd s, uint32_t n0, Offers of, unsigned long long *pairs,
                                                     int *status, uint32_t tjc) {
  extern __shared__ __align__(16) uint8_t smem[];
  const uint32_t n = n0 + blockIdx.x;
  const uint32_t a = s.lnew[n], b = s.lold[n];
  if (a == 0) return;
  const uint32_t tot = a + b;
  const uint32_t stride = ((s.d + 3) & ~3u) + 4;
  float *ri = (float *)smem;                     // J_TI rows
  float *rj = ri + (size_t)J_TI * stride;        // J_TJ rows
  uint32_t *ids = (uint32_t *)(rj + (size_t)tjc * stride);  // tot ids: new ++ old
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (uint32_t t = threadIdx.x; t < tot; t += J_THREADS)
    ids[t] = t < a ? s.nnew[(size_t)n * s.capn + t] : s.nold[(size_t)n * s.capo + (t - a)];
  __syncthreads();
  const uint32_t d4 = s.d >> 2;
  unsigned long long npairs = 0;
  for (uint32_t i0 = 0; i0 < a; i0 += J_TI) {
    const uint32_t ti = min((uint32_t)J_TI, a - i0);
    for (uint32_t j0 = 0; j0 < tot; j0 += tjc) {
      const uint32_t tj = min(tjc, tot - j0);
      __syncthreads();
      // stage rows (coalesced 16-byte copies, one row per warp step)
      for (uint32_t r = warp; r < ti + tj; r += J_THREADS / 32) {
        const uint32_t id = r < ti ? ids[i0 + r] : ids[j0 + (r - ti)];
        float *dst = r < ti ? ri + (size_t)r * stride : rj + (size_t)(r - ti) * stride;
        const float *src = s.base + (size_t)id * s.d;
        for (uint32_t k = lane; k < d4; k += 32) cp_async16(dst + 4 * k, src + 4 * k);
      }
      cp_async_wait_all();
      __syncthreads();
      // warps take i rows, lanes take j rows
      for (uint32_t pa = warp; pa < ti; pa += J_THREADS / 32) {
        const uint32_t gi = i0 + pa, iid = ids[gi];
        for (uint32_t pj0 = 0; pj0 < tj; pj0 += 32) {
          const uint32_t pj = pj0 + lane, gj = j0 + pj;
          bool valid = false;
          uint32_t jid = 0;
          if (pj < tj) {
            jid = ids[gj];
            valid = gj < a ? (iid < jid) : (iid != jid);
          }
          float dist = 0.f;
          if (valid) {
            const float4 *x = reinterpret_cast<const float4 *>(ri + (size_t)pa * stride);
            const float4 *y = reinterpret_cast<const float4 *>(rj + (size_t)pj * stride);
            for (uint32_t g = 0; g < d4; g++) dist = __fadd_rn(dist, group4(x[g], y[g]));
            npairs++;
          }
          const unsigned long long kbase = ((unsigned long long)n << 32) | ((gi * tot + gj) << 1);
          // offer 1: insert(i <- j); offer 2: insert(j <- i)
          bool ok1 = valid && s.psz[iid] > 0 && dist <= s.pool[(size_t)iid * s.L].d;
          emit(of, ok1, iid, kbase, jid, dist, lane, status);
          bool ok2 = valid && s.psz[jid] > 0 && dist <= s.pool[(size_t)jid * s.L].d;
          emit(of, ok2, jid, kbase | 1ull, iid, dist, lane, status);
        }
      }
    }
  }
  if (pairs) {
    for (int o = 16; o > 0; o >>= 1) npairs += __shfl_xor_sync(FULL, npairs, o);
    if (lane == 0 && npairs) atomicAdd(pairs, npairs);
  }
}

// ---------------------------------------------------------------- join on the tensor cores
// The same local join for integer data in [0, 255] with d a multiple of 16,
// d <= 128 and new lists of at most 128 ids: every pair distance is the
// norm form |x|^2 + |y|^2 - 2 x.y with the dot products of a Gram tile
// computed by tcgen05.mma, BF16 operands (the integer values are exact in
// BF16, their products in FP32) and FP32 accumulation in tensor memory --
// every partial sum an integer below 2^24, so the distances are the exact
// FP32 values the reference's sequential sum gives, and the offers (targets,
// keys, candidates, distances) are those of k_join.
//
// One CTA of 8 warps per node.  The node's rows (new ++ old) are converted to
// BF16 into the canonical no-swizzle K-major layout (8 x 8 core matrices of
// 16-byte rows, K-adjacent core matrices 128 bytes apart, 8-row groups d * 16
// bytes apart).  The first 128 rows (the new rows, then old ones) are the B
// operand (N = the new rows rounded up to 16) and also the first A tile;
// later A tiles of 128 rows take the second buffer.  Per tile one thread
// issues d / 16 MMAs (M = 128, N, K = 16) into up to 128 columns of tensor
// memory and commits to an mbarrier; warp w reads accumulator lanes
// 32(w % 4).. (rows j of new ++ old) 16 columns (new rows i) at a time with
// tcgen05.ld and emits the two offers of each valid pair (i, j) -- warps w
// and w + 4 share lanes 32w.. and split the columns; all warps hold rows,
// the columns run over the short new list.  The targets'
// pool maxima are read once per node into shared memory (pools do not change
// during a join chunk).  The wait on the MMAs is bounded: on time-out the CTA
// reports DEV_TIMEOUT, waits (bounded) once more for its MMAs and frees its
// tensor memory.
constexpr int JT_THREADS = 256;  // 8 warps: warps w and w + 4 share TMEM lanes 32w.. (column halves)
constexpr uint32_t JT_ROWS = 128;  // rows per operand buffer (M of A, the N chunk of B)
constexpr uint32_t JT_LBO = 128;
constexpr uint32_t JT_TMEM_COLS = 128;

__device__ __forceinline__ uint32_t jt_pack(float lo, float hi) {
  const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<const uint32_t *>(&v);
}

// rows [r0, r0 + 128) of the node's list as BF16 in the K-major core layout
// (zeros past tot).  Item e is the 16-byte core row at byte offset 16 e of
// the layout (8-row group e / (8 kc), core matrix (e / 8) % kc, row e % 8):
// consecutive threads store consecutive 16 bytes (no bank conflicts) and
// each loads 32 bytes of one row.
__device__ void jt_stage(uint8_t *dst, const float *__restrict__ base, uint32_t d, const uint32_t *ids, uint32_t tot,
                         uint32_t r0, int tid) {
  const uint32_t kc = d / 8;
  for (uint32_t e = tid; e < JT_ROWS * kc; e += JT_THREADS) {
    const uint32_t r = (e / (8 * kc)) * 8 + (e & 7), k = ((e >> 3) % kc) * 8;
    uint4 v = make_uint4(0, 0, 0, 0);
    if (r0 + r < tot) {
      const float4 *src = reinterpret_cast<const float4 *>(base + (size_t)ids[r0 + r] * d + k);
      const float4 x0 = __ldg(src), x1 = __ldg(src + 1);
      v = make_uint4(jt_pack(x0.x, x0.y), jt_pack(x0.z, x0.w), jt_pack(x1.x, x1.y), jt_pack(x1.z, x1.w));
    }
    reinterpret_cast<uint4 *>(dst)[e] = v;
  }
}

size_t join_tc_smem(uint32_t d, uint32_t capn, uint32_t capo) {
  return 2 * (size_t)JT_ROWS * d * 2 + 3 * (size_t)(capn + capo) * 4 + 16;
}

__global__ void __launch_bounds__(JT_THREADS) k_join_tc(Nnd s, uint32_t n0, Offers of, unsigned long long *pairs,
                                                        int *status) {
  extern __shared__ __align__(16) uint8_t smem[];  // (the no-swizzle layout needs 16-byte alignment)
  __shared__ __align__(8) uint64_t bar;
  __shared__ uint32_t tmem_base;
  const uint32_t n = n0 + blockIdx.x;
  const uint32_t a = s.lnew[n], b = s.lold[n];
  if (a == 0) return;  // (block-uniform, before any tensor memory is taken)
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t tot = a + b, d = s.d;
  const uint32_t sbo = (d / 8) * 128;
  uint8_t *tA = smem, *tB = smem + (size_t)JT_ROWS * d * 2;
  uint32_t *ids = reinterpret_cast<uint32_t *>(tB + (size_t)JT_ROWS * d * 2);
  float *nrm = reinterpret_cast<float *>(ids + s.capn + s.capo);
  float *mx = nrm + s.capn + s.capo;
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(umma::smem_u32(&tmem_base)),
                 "r"(JT_TMEM_COLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 0) {
    umma::mbar_init(&bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;");
  }
  for (uint32_t t = tid; t < tot; t += JT_THREADS) {
    const uint32_t id = t < a ? s.nnew[(size_t)n * s.capn + t] : s.nold[(size_t)n * s.capo + (t - a)];
    ids[t] = id;
    nrm[t] = s.xnorm[id];
    // nhood::insert's first test against the pool's current maximum (an
    // empty pool takes nothing here, as k_join's psz test)
    mx[t] = s.psz[id] > 0 ? s.pool[(size_t)id * s.L].d : __int_as_float(0xff800000);
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = tmem_base;
  jt_stage(tA, s.base, d, ids, tot, 0, tid);
  unsigned long long npairs = 0;
  uint32_t phase = 0;
  bool ok = true;
  const uint32_t acols = (a + 15) & ~15u;  // N: the new rows, rounded up to 16
  for (uint32_t m0 = 0; m0 < tot && ok; m0 += JT_ROWS) {
    const uint8_t *at = m0 == 0 ? tA : tB;
    if (m0 > 0) jt_stage(tB, s.base, d, ids, tot, m0, tid);
    asm volatile("fence.proxy.async.shared::cta;");  // generic stores -> tensor core reads
    __syncthreads();
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;");
      const uint32_t a0 = umma::smem_u32(at), b0 = umma::smem_u32(tA);
      const uint32_t idesc = umma::idesc(128, (int)acols);
      for (uint32_t kk = 0; kk < d / 16; kk++) {
        const uint64_t ad = umma::desc(a0 + kk * 2 * JT_LBO, JT_LBO, sbo);
        const uint64_t bd = umma::desc(b0 + kk * 2 * JT_LBO, JT_LBO, sbo);
        const uint32_t acc = kk > 0 ? 1u : 0u;
        asm volatile(
            "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
            " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
            "l"(ad), "l"(bd), "r"(idesc), "r"(acc));
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          umma::smem_u32(&bar)));
    }
    ok = __syncthreads_and(umma::mbar_wait(&bar, phase)) != 0;
    phase ^= 1;
    asm volatile("tcgen05.fence::after_thread_sync;");
    if (!ok) break;
    // warp w: TMEM lanes 32 (w % 4).. (rows of new ++ old), columns (new
    // rows) of half w / 4
    const uint32_t quad = warp & 3, chalf = (uint32_t)(warp >> 2) * 64;
    if (m0 + quad * 32 < tot) {
      const uint32_t gj = m0 + quad * 32 + lane;  // this lane's row of new ++ old
      const bool rowok = gj < tot;
      const uint32_t jid = rowok ? ids[gj] : 0u;
      const float nj = rowok ? nrm[gj] : 0.f, mj = rowok ? mx[gj] : __int_as_float(0xff800000);
      for (uint32_t c0 = chalf; c0 < a && c0 < chalf + 64; c0 += 16) {
        uint32_t v[16];
        const uint32_t addr = tmem + ((quad * 32) << 16) + c0;
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
            : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
              "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
            : "r"(addr));
        asm volatile("tcgen05.wait::ld.sync.aligned;");
#pragma unroll
        for (int ii = 0; ii < 16; ii++) {
          const uint32_t gi = c0 + ii;  // a new row (warp-uniform)
          if (gi >= a) continue;
          const uint32_t iid = ids[gi];
          const bool valid = rowok && (gj < a ? (iid < jid) : (iid != jid));
          // integers below 2^24 throughout: the exact FP32 distance
          const float dist = (nrm[gi] + nj) - 2.f * __uint_as_float(v[ii]);
          npairs += valid;
          const unsigned long long kbase = ((unsigned long long)n << 32) | ((gi * tot + gj) << 1);
          emit(of, valid && dist <= mx[gi], iid, kbase, jid, dist, lane, status);
          emit(of, valid && dist <= mj, jid, kbase | 1ull, iid, dist, lane, status);
        }
      }
    }
    // the accumulator is read and the A buffer free before the next tile
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
  }
  if (!ok) {
    if (tid == 0) set_err(status, DEV_TIMEOUT);
    // the MMAs of the chunk that timed out may still run: wait for them
    // (bounded) before the tensor memory is freed
    umma::mbar_wait(&bar, phase ^ 1);
  }
  if (pairs) {
    for (int o = 16; o > 0; o >>= 1) npairs += __shfl_xor_sync(FULL, npairs, o);
    if (lane == 0 && npairs) atomicAdd(pairs, npairs);
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(JT_TMEM_COLS));
}

// targets with offers, and the largest segment
__global__ void k_active(uint32_t n, const uint32_t *tcnt, uint32_t *act, uint32_t *nact, uint32_t *big,
                         uint32_t *nbig, uint32_t warp_cap, uint32_t *maxseg) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  uint32_t c = tcnt[t];
  if (c == 0) return;
  atomicMax(maxseg, c);
  if (c <= warp_cap) act[atomicAdd(nact, 1u)] = t;
  else big[atomicAdd(nbig, 1u)] = t;
}

struct WarpSync {
  __device__ void operator()() const { __syncwarp(); }
};
struct BlockSync {
  __device__ void operator()() const { __syncthreads(); }
};

struct Grouped {
  unsigned long long key;
  uint32_t cand;
  float dist;
};

__global__ void k_group(uint32_t count, Offers of, const uint32_t *toff, uint32_t *tcur, Grouped *g) {
  const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= count) return;
  uint32_t t = of.tgt[r];
  uint32_t pos = toff[t] + atomicAdd(&tcur[t], 1u);
  g[pos] = Grouped{of.key[r], of.cand[r], of.dist[r]};
}

// sorts `cnt` grouped offers by key in shared memory (P = pow2 >= cnt),
// threads [0, nthr) of the calling group cooperate; `sync` orders steps
template <class Sync>
__device__ void bitonic_grouped(Grouped *k, int P, int tid, int nthr, Sync sync) {
  for (int sz = 2; sz <= P; sz <<= 1)
    for (int j = sz >> 1; j > 0; j >>= 1) {
      for (int i = tid; i < P; i += nthr) {
        int l = i ^ j;
        if (l > i) {
          bool up = (i & sz) == 0;
          Grouped a = k[i], b = k[l];
          if ((a.key > b.key) == up) {
            k[i] = b;
            k[l] = a;
          }
        }
      }
      sync();
    }
}

// nhood::insert (index.h:120-135) applied to one target's offers in key order
// by one warp; pool P (heap) in shared memory.  Lane 0 runs the heap steps.
__device__ void apply_offers(Ent *P, uint32_t &sz, uint32_t L, const Grouped *off, uint32_t cnt, int lane) {
  uint32_t i = 0;
  while (i < cnt) {
    const float front = P[0].d;
    const uint32_t j = i + lane;
    bool pass = j < cnt && !(off[j].dist > front);
    unsigned m = __ballot_sync(FULL, pass);
    if (!m) {
      i += 32;
      continue;
    }
    const uint32_t f = i + __ffs(m) - 1;
    const uint32_t cid = off[f].cand;
    bool dup = false;
    for (uint32_t x = lane; x < sz; x += 32) dup |= (P[x].idf & ID_MASK) == cid;
    dup = __any_sync(FULL, dup);
    if (!dup && lane == 0) {
      if (sz < L) {
        P[sz] = Ent{off[f].dist, cid | FLAG};
        sz++;
        stl::push_heap(P, (int)sz, EntLess());
      } else {
        stl::pop_heap(P, (int)sz, EntLess());
        P[sz - 1] = Ent{off[f].dist, cid | FLAG};
        stl::push_heap(P, (int)sz, EntLess());
      }
    }
    sz = __shfl_sync(FULL, sz, 0);
    __syncwarp();
    i = f + 1;
  }
}

constexpr int AP_WARPS = 4;
constexpr uint32_t AP_WARP_CAP = 1024;   // offers per target for the warp path
constexpr uint32_t AP_BIG_CAP = 8192;    // offers per target for the block path (power of 2)

__global__ void __launch_bounds__(AP_WARPS * 32)
    k_apply_warp(Nnd s, const uint32_t *act, const uint32_t *nact, const uint32_t *toff, const uint32_t *tcnt,
                 Grouped *g) {
  extern __shared__ __align__(16) uint8_t smem[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t w = blockIdx.x * AP_WARPS + warp;
  if (w >= *nact) return;
  Grouped *k = (Grouped *)smem + (size_t)warp * AP_WARP_CAP;
  Ent *P = (Ent *)((Grouped *)smem + (size_t)AP_WARPS * AP_WARP_CAP) + (size_t)warp * (s.L + 1);
  const uint32_t t = act[w], cnt = tcnt[t], off = toff[t];
  int Pn = 1;
  while (Pn < (int)cnt) Pn <<= 1;
  for (int i = lane; i < Pn; i += 32) k[i] = i < (int)cnt ? g[off + i] : Grouped{~0ull, 0u, 0.f};
  uint32_t sz = s.psz[t];
  for (uint32_t i = lane; i < sz; i += 32) P[i] = s.pool[(size_t)t * s.L + i];
  __syncwarp();
  bitonic_grouped(k, Pn, lane, 32, WarpSync());
  apply_offers(P, sz, s.L, k, cnt, lane);
  for (uint32_t i = lane; i < sz; i += 32) s.pool[(size_t)t * s.L + i] = P[i];
  if (lane == 0) s.psz[t] = sz;
}

__global__ void __launch_bounds__(512)
    k_apply_block(Nnd s, const uint32_t *big, const uint32_t *toff, const uint32_t *tcnt, Grouped *g) {
  extern __shared__ __align__(16) uint8_t smem[];
  const uint32_t t = big[blockIdx.x], cnt = tcnt[t], off = toff[t];
  Grouped *k = (Grouped *)smem;
  Ent *P = (Ent *)(k + AP_BIG_CAP);
  __shared__ uint32_t szs;
  int Pn = 1;
  while (Pn < (int)cnt) Pn <<= 1;
  for (int i = threadIdx.x; i < Pn; i += blockDim.x) k[i] = i < (int)cnt ? g[off + i] : Grouped{~0ull, 0u, 0.f};
  const uint32_t sz0 = s.psz[t];
  for (uint32_t i = threadIdx.x; i < sz0; i += blockDim.x) P[i] = s.pool[(size_t)t * s.L + i];
  __syncthreads();
  bitonic_grouped(k, Pn, threadIdx.x, blockDim.x, BlockSync());
  if (threadIdx.x < 32) {
    uint32_t sz = sz0;
    apply_offers(P, sz, s.L, k, cnt, threadIdx.x);
    if (threadIdx.x == 0) szs = sz;
  }
  __syncthreads();
  for (uint32_t i = threadIdx.x; i < szs; i += blockDim.x) s.pool[(size_t)t * s.L + i] = P[i];
  if (threadIdx.x == 0) s.psz[t] = szs;
}

// RefineInner tail: sort each pool, keep the first K (PruneNaive)
__global__ void k_nnd_final(Nnd s, uint32_t *ids, float *dist, uint32_t *deg) {
  extern __shared__ __align__(16) uint8_t smem[];
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  Ent *P = (Ent *)smem + (size_t)threadIdx.x * (s.L + 1);
  if (i >= s.n) return;
  const uint32_t sz = s.psz[i];
  for (uint32_t j = 0; j < sz; j++) P[j] = s.pool[(size_t)i * s.L + j];
  stl::sort(P, (int)sz, EntLess());
  const uint32_t k = min(sz, s.K);
  for (uint32_t j = 0; j < k; j++) {
    ids[(size_t)i * s.K + j] = P[j].idf & ID_MASK;
    dist[(size_t)i * s.K + j] = P[j].d;
  }
  deg[i] = k;
}

constexpr int NODE_THREADS = 64;  // threads per block of the per-node sort kernels

}  // namespace

// ================================================================ host side
int mt19937_gpu(wv_ctx *c, uint32_t seed, uint32_t *d_out, size_t count) {
  k_mt19937<<<1, 256, 0, c->stream>>>(seed, d_out, count);
  WV_CUDA(c, cudaGetLastError());
  return WV_OK;
}

int init_random_gpu(wv_ctx *c, uint32_t S) {
  WV_CHECK(c, c->n > 0, WV_ERR_STATE, "no base uploaded");
  WV_CHECK(c, S >= 1 && S <= 32, WV_ERR_LIMIT, "S=%u: this build supports 1 <= S <= 32", S);
  WV_CHECK(c, S < c->n, WV_ERR_ARG, "S=%u must be smaller than n=%u", S, c->n);
  WV_CHECK(c, c->d % 4 == 0, WV_ERR_LIMIT, "dimension %u is not a multiple of 4", c->d);
  cudaError_t e = cudaSuccess;
  const size_t count = (size_t)c->n * (S + 1);
  uint32_t *mt = c->buf<uint32_t>("mt", count, &e);
  WV_CUDA(c, e);
  // `std::mt19937 rng(rand())`: one draw from the process rand() stream
  const uint32_t seed = (uint32_t)c->rnd.next();
  int rc = mt19937_gpu(c, seed, mt, count);
  if (rc) return rc;
  WV_CUDA(c, c->fg_ids.ensure((size_t)c->n * S * 4));
  WV_CUDA(c, c->fg_dist.ensure((size_t)c->n * S * 4));
  WV_CUDA(c, c->fg_deg.ensure((size_t)c->n * 4));
  const size_t smem = INIT_WARPS * ((size_t)STAGE_FLOATS * 4 + ((c->d + 3) & ~3u) * 4 + 64 * sizeof(DI));
  WV_CUDA(c, cudaFuncSetAttribute(k_init_random, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const int blocks = (int)std::min<size_t>((c->n + INIT_WARPS - 1) / INIT_WARPS, (size_t)c->sms * 16);
  k_init_random<<<blocks, INIT_WARPS * 32, smem, c->stream>>>(c->base.as<float>(), c->n, c->d, S, mt,
                                                               c->fg_ids.as<uint32_t>(), c->fg_dist.as<float>(),
                                                               c->fg_deg.as<uint32_t>());
  WV_CUDA(c, cudaGetLastError());
  c->fg_n = c->n;
  c->fg_w = S;
  c->fg_has_ep = false;
  c->fg_eps.clear();
  return check_device_status(c, "init_random");
}

int init_rand_gpu(wv_ctx *c, uint32_t L) {
  WV_CHECK(c, c->n > 0, WV_ERR_STATE, "no base uploaded");
  WV_CHECK(c, L >= 1 && L <= 1024, WV_ERR_LIMIT, "L=%u: this build supports 1 <= L <= 1024", L);
  WV_CHECK(c, L < c->n, WV_ERR_ARG, "L=%u must be smaller than n=%u", L, c->n);
  WV_CHECK(c, c->d % 4 == 0, WV_ERR_LIMIT, "dimension %u is not a multiple of 4", c->d);
  cudaError_t e = cudaSuccess;
  const size_t count = (size_t)c->n * (L + 1);
  uint32_t *mt = c->buf<uint32_t>("mt", count, &e);
  WV_CUDA(c, e);
  // `std::mt19937 rng(rand())`: one draw from the process rand() stream
  const uint32_t seed = (uint32_t)c->rnd.next();
  int rc = mt19937_gpu(c, seed, mt, count);
  if (rc) return rc;
  WV_CUDA(c, c->fg_ids.ensure((size_t)c->n * L * 4));
  WV_CUDA(c, c->fg_dist.ensure((size_t)c->n * L * 4));
  WV_CUDA(c, c->fg_deg.ensure((size_t)c->n * 4));
  const size_t smem = IR_WARPS * init_rand_warp_bytes(L, c->d);
  WV_CHECK(c, smem <= 227 * 1024, WV_ERR_LIMIT, "L=%u d=%u need %zu bytes of shared memory", L, c->d, smem);
  WV_CUDA(c, cudaFuncSetAttribute(k_init_rand, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const int blocks = (int)std::min<size_t>((c->n + IR_WARPS - 1) / IR_WARPS, (size_t)c->sms * 16);
  k_init_rand<<<blocks, IR_WARPS * 32, smem, c->stream>>>(c->base.as<float>(), c->n, c->d, L, mt,
                                                           c->fg_ids.as<uint32_t>(), c->fg_dist.as<float>(),
                                                           c->fg_deg.as<uint32_t>());
  WV_CUDA(c, cudaGetLastError());
  c->fg_n = c->n;
  c->fg_w = L;
  c->fg_has_ep = false;
  c->fg_eps.clear();
  return check_device_status(c, "init_rand");
}

int nndescent_gpu(wv_ctx *c, const NndParams &p, NndStats *st) {
  WV_CHECK(c, c->n > 0 && c->fg_n == c->n, WV_ERR_STATE, "NN-Descent needs the base and an initial graph");
  WV_CHECK(c, p.L >= 1 && p.K >= 1 && p.S >= 1 && p.R >= 1, WV_ERR_ARG, "S, K, L, R must be positive");
  WV_CHECK(c, p.L <= 256, WV_ERR_LIMIT, "L=%u above the supported 256", p.L);
  WV_CHECK(c, c->d % 4 == 0, WV_ERR_LIMIT, "dimension %u is not a multiple of 4", c->d);
  // the join key packs (pair position << 1 | side) into 32 bits
  WV_CHECK(c, 2ull * (p.S + p.R) * (p.S + 3ull * p.R) < (1ull << 31), WV_ERR_LIMIT, "S=%u R=%u too large", p.S, p.R);
  NndStats local;
  NndStats &S = st ? *st : local;
  S = NndStats();
  cudaError_t e = cudaSuccess;
  const uint32_t n = c->n;
  Nnd s{};
  s.n = n;
  s.d = c->d;
  s.S = p.S;
  s.K = p.K;
  s.L = p.L;
  s.R = p.R;
  s.capn = std::max(p.S + p.R, 2 * p.S);  // EFANNA's first nn_new holds 2S ids
  s.capo = std::min(p.L + p.R, 2 * p.R);
  s.base = c->base.as<float>();
  s.xnorm = c->base_int ? c->xnorm.as<float>() : nullptr;
  s.pool = c->buf<Ent>("pool", (size_t)n * p.L, &e);
  s.psz = c->buf<uint32_t>("psz", n, &e);
  s.M = c->buf<uint32_t>("M", n, &e);
  s.nnew = c->buf<uint32_t>("nnew", (size_t)n * s.capn, &e);
  s.nold = c->buf<uint32_t>("nold", (size_t)n * s.capo, &e);
  s.lnew = c->buf<uint32_t>("lnew", n, &e);
  s.lold = c->buf<uint32_t>("lold", n, &e);
  s.pnew = c->buf<uint32_t>("pnew", n, &e);
  s.pold = c->buf<uint32_t>("pold", n, &e);
  s.pre = c->buf<Ent>("pre", (size_t)n * p.L, &e);
  s.maxd = c->buf<float>("maxd", n, &e);
  s.hback = c->buf<float>("hback", n, &e);
  uint32_t *ecount = c->buf<uint32_t>("ecount", n, &e);
  uint32_t *eoff = c->buf<uint32_t>("eoff", n + 1, &e);
  uint32_t *bcnt = c->buf<uint32_t>("bcnt", 2 * (size_t)n, &e);
  uint32_t *boff = c->buf<uint32_t>("boff", 2 * (size_t)n + 1, &e);
  uint32_t *bcur = c->buf<uint32_t>("bcur", 2 * (size_t)n, &e);
  uint32_t *scan_tmp = c->buf<uint32_t>("scan", scan_scratch_words((size_t)n * p.L + 2 * (size_t)n), &e);
  uint32_t *tcnt = c->buf<uint32_t>("tcnt", n, &e);
  uint32_t *toff = c->buf<uint32_t>("toff", n + 1, &e);
  uint32_t *tcur = c->buf<uint32_t>("tcur", n, &e);
  uint32_t *act = c->buf<uint32_t>("act", n, &e);
  uint32_t *big = c->buf<uint32_t>("big", n, &e);
  uint32_t *small = c->buf<uint32_t>("small", 16, &e);  // [0] nact [1] nbig [2] maxseg [3] cursor
  uint32_t *usmall = c->buf<uint32_t>("usmall", 8, &e);  // [0] longest big bucket [1] big buckets
  uint32_t *bigb = c->buf<uint32_t>("bigb", 2 * (size_t)n, &e);
  unsigned long long *pairs = (unsigned long long *)c->buf<uint64_t>("pairs", 2, &e);
  WV_CUDA(c, e);

  // offer buffers: the largest chunk holds at most `cap` offers
  size_t free_b = 0, total_b = 0;
  WV_CUDA(c, cudaMemGetInfo(&free_b, &total_b));
  const size_t rec_bytes = 4 + 8 + 4 + 4 + sizeof(Grouped);
  uint32_t cap = (uint32_t)std::min<size_t>((size_t)1 << 28, std::max<size_t>(free_b / 3 / rec_bytes, 1u << 20));
  // WV_NND_OFFER_CAP lowers the per-chunk offer capacity (more, smaller
  // join chunks); results do not depend on it
  if (const char *env = getenv("WV_NND_OFFER_CAP")) cap = std::max<uint32_t>(1024u, std::min<uint32_t>(cap, (uint32_t)atol(env)));
  Offers of{};
  of.tgt = c->buf<uint32_t>("of_t", cap, &e);
  of.key = c->buf<unsigned long long>("of_k", cap, &e);
  of.cand = c->buf<uint32_t>("of_c", cap, &e);
  of.dist = c->buf<float>("of_d", cap, &e);
  Grouped *grp = c->buf<Grouped>("of_g", cap, &e);
  WV_CUDA(c, e);
  of.cap = cap;
  of.tcnt = tcnt;
  of.cursor = small + 3;

  cudaEvent_t ev0, ev1;
  cudaEventCreate(&ev0);
  cudaEventCreate(&ev1);

  const int nb = (int)((n + NODE_THREADS - 1) / NODE_THREADS);
  const size_t node_smem = (size_t)NODE_THREADS * (p.L + 1) * sizeof(Ent);
  WV_CUDA(c, cudaFuncSetAttribute(k_nnd_init, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)node_smem));
  WV_CUDA(c, cudaFuncSetAttribute(k_upd_sort, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)node_smem));
  WV_CUDA(c, cudaFuncSetAttribute(k_nnd_final, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)node_smem));
  if (p.efanna) {
    // one rand() seeds the mt19937 the nhoods draw their first nn_new from
    WV_CHECK(c, 2ull * p.S < n, WV_ERR_ARG, "EFANNA needs 2S < n (S=%u, n=%u)", p.S, n);
    std::vector<uint32_t> hdeg(n);
    WV_CUDA(c, cudaMemcpyAsync(hdeg.data(), c->fg_deg.p, (size_t)n * 4, cudaMemcpyDeviceToHost, c->stream));
    WV_CUDA(c, cudaStreamSynchronize(c->stream));
    for (uint32_t i = 0; i < n; i++)
      WV_CHECK(c, hdeg[i] <= p.L, WV_ERR_LIMIT, "init row %u has %u entries > L=%u (the pool would outgrow L)", i,
               hdeg[i], p.L);
    const uint32_t seed = (uint32_t)c->rnd.next();
    const size_t count = (size_t)n * (2 * p.S + 1);
    uint32_t *mtv = c->buf<uint32_t>("ef_mt", count, &e);
    WV_CUDA(c, e);
    int rc = mt19937_gpu(c, seed, mtv, count);
    if (rc) return rc;
    const size_t ef_smem = (size_t)EF_WARPS * pow2_ge(2 * p.S) * 4;
    WV_CUDA(c, cudaFuncSetAttribute(k_efanna_nnew, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ef_smem));
    k_efanna_nnew<<<c->sms * 8, EF_WARPS * 32, ef_smem, c->stream>>>(s, mtv);
    WV_CUDA(c, cudaGetLastError());
  }
  k_nnd_init<<<nb, NODE_THREADS, node_smem, c->stream>>>(s, c->fg_ids.as<uint32_t>(), c->fg_dist.as<float>(),
                                                          c->fg_deg.as<uint32_t>(), c->fg_w, p.efanna ? 1 : 0);
  WV_CUDA(c, cudaGetLastError());

  // the local join's pair distances: on the tensor cores where they are exact
  // (integer data, d a multiple of 16 up to 128, new lists of at most 128
  // ids; WV_NND_JOIN=fp32 keeps the FP32 pair kernel), else in FP32 in the
  // reference's order.  Both give the same offers.
  const char *join_env = getenv("WV_NND_JOIN");
  const bool join_tc = c->base_int && c->d % 16 == 0 && c->d <= 128 && s.capn <= JT_ROWS &&
                       !(join_env && std::string(join_env) == "fp32");
  const size_t jtc_smem = join_tc_smem(c->d, s.capn, s.capo);
  if (join_tc) WV_CUDA(c, cudaFuncSetAttribute(k_join_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)jtc_smem));
  const uint32_t stride = ((c->d + 3) & ~3u) + 4;
  uint32_t tjc = J_TJ;
  while (tjc > 32 && (size_t)(J_TI + tjc) * stride * 4 > 200 * 1024) tjc -= 32;
  const size_t join_smem = (size_t)(J_TI + tjc) * stride * 4 + (size_t)(s.capn + s.capo) * 4 + 16;
  WV_CHECK(c, join_smem <= 227 * 1024, WV_ERR_LIMIT, "dimension %u too large for the local-join tile", c->d);
  WV_CUDA(c, cudaFuncSetAttribute(k_join, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)join_smem));
  const size_t apw_smem = (size_t)AP_WARPS * AP_WARP_CAP * sizeof(Grouped) + (size_t)AP_WARPS * (p.L + 1) * sizeof(Ent);
  WV_CUDA(c, cudaFuncSetAttribute(k_apply_warp, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)apw_smem));
  const size_t apb_smem = (size_t)AP_BIG_CAP * sizeof(Grouped) + (size_t)(p.L + 1) * sizeof(Ent);
  WV_CUDA(c, cudaFuncSetAttribute(k_apply_block, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)apb_smem));
  WV_CUDA(c, cudaMemsetAsync(pairs, 0, 8, c->stream));

  std::vector<uint32_t> h_lnew(n), h_lold(n);
  for (uint32_t it = 0; it < p.ITER; it++) {
    // ------------------------------------------------------------ join
    // (NN_DESCENT's first join pairs 2S zero ids -- nothing; EFANNA's is live)
    if (it > 0 || p.efanna) {
      cudaEventRecord(ev0, c->stream);
      WV_CUDA(c, cudaMemcpyAsync(h_lnew.data(), s.lnew, (size_t)n * 4, cudaMemcpyDeviceToHost, c->stream));
      WV_CUDA(c, cudaMemcpyAsync(h_lold.data(), s.lold, (size_t)n * 4, cudaMemcpyDeviceToHost, c->stream));
      WV_CUDA(c, cudaStreamSynchronize(c->stream));
      uint32_t n0 = 0;
      while (n0 < n) {
        // chunk: the most nodes whose offer upper bound fits `cap`
        uint64_t acc = 0;
        uint32_t n1 = n0;
        while (n1 < n) {
          uint64_t a = h_lnew[n1], b = h_lold[n1];
          uint64_t ub = a * (a - (a > 0)) + 2 * a * b;  // 2 offers per pair
          if (n1 > n0 && acc + ub > cap) break;
          acc += ub;
          n1++;
        }
        WV_CHECK(c, acc <= cap, WV_ERR_LIMIT, "node %u alone may produce %llu offers (> %u)", n0,
                 (unsigned long long)acc, cap);
        while (true) {
          WV_CUDA(c, cudaMemsetAsync(tcnt, 0, (size_t)n * 4, c->stream));
          WV_CUDA(c, cudaMemsetAsync(small, 0, 16, c->stream));
          if (join_tc)
            k_join_tc<<<n1 - n0, JT_THREADS, jtc_smem, c->stream>>>(s, n0, of, pairs, c->d_status());
          else
            k_join<<<n1 - n0, J_THREADS, join_smem, c->stream>>>(s, n0, of, pairs, c->d_status(), tjc);
          WV_CUDA(c, cudaGetLastError());
          k_active<<<nb, NODE_THREADS, 0, c->stream>>>(n, tcnt, act, small, big, small + 1, AP_WARP_CAP, small + 2);
          uint32_t hs[4];
          WV_CUDA(c, cudaMemcpyAsync(hs, small, 16, cudaMemcpyDeviceToHost, c->stream));
          WV_CUDA(c, cudaStreamSynchronize(c->stream));
          if (hs[2] > AP_BIG_CAP && n1 - n0 > 1) {
            n1 = n0 + (n1 - n0) / 2;  // a target gets too many offers: smaller chunk
            continue;
          }
          WV_CHECK(c, hs[2] <= AP_BIG_CAP, WV_ERR_LIMIT, "one node sends %u offers to one target", hs[2]);
          const uint32_t count = hs[3];
          S.offers += count;
          S.chunks++;
          WV_CUDA(c, exclusive_scan_u32(tcnt, toff, n, scan_tmp, c->stream));
          WV_CUDA(c, cudaMemsetAsync(tcur, 0, (size_t)n * 4, c->stream));
          if (count) {
            k_group<<<(count + 255) / 256, 256, 0, c->stream>>>(count, of, toff, tcur, grp);
            if (hs[0])
              k_apply_warp<<<(hs[0] + AP_WARPS - 1) / AP_WARPS, AP_WARPS * 32, apw_smem, c->stream>>>(
                  s, act, small, toff, tcnt, grp);
            if (hs[1]) k_apply_block<<<hs[1], 512, apb_smem, c->stream>>>(s, big, toff, tcnt, grp);
            WV_CUDA(c, cudaGetLastError());
          }
          break;
        }
        n0 = n1;
      }
      cudaEventRecord(ev1, c->stream);
      cudaEventSynchronize(ev1);
      float ms = 0;
      cudaEventElapsedTime(&ms, ev0, ev1);
      S.ms_join += ms;
    }
    // ------------------------------------------------------------ update
    cudaEventRecord(ev0, c->stream);
    k_upd_sort<<<nb, NODE_THREADS, node_smem, c->stream>>>(s);
    WV_CUDA(c, cudaMemsetAsync(bcnt, 0, 2 * (size_t)n * 4, c->stream));
    WV_CUDA(c, cudaMemsetAsync(usmall, 0, 8, c->stream));
    k_upd_count<<<nb, NODE_THREADS, 0, c->stream>>>(s, ecount, bcnt, usmall);
    WV_CUDA(c, exclusive_scan_u32(ecount, eoff, n, scan_tmp, c->stream));
    WV_CUDA(c, exclusive_scan_u32(bcnt, boff, 2 * (size_t)n, scan_tmp, c->stream));
    uint32_t tail[2];
    WV_CUDA(c, cudaMemcpyAsync(&tail[0], eoff + n - 1, 4, cudaMemcpyDeviceToHost, c->stream));
    WV_CUDA(c, cudaMemcpyAsync(&tail[1], ecount + n - 1, 4, cudaMemcpyDeviceToHost, c->stream));
    WV_CUDA(c, cudaStreamSynchronize(c->stream));
    const uint32_t E = tail[0] + tail[1];
    uint32_t *bsrc = c->buf<uint32_t>("bsrc", E + 1, &e);
    uint32_t *bflat = c->buf<uint32_t>("bflat", E + 1, &e);
    uint32_t *ovf = c->buf<uint32_t>("ovf", E + 1, &e);
    uint32_t *ovf_ord = c->buf<uint32_t>("ovf_ord", E + 1, &e);
    uint32_t *scan_e = c->buf<uint32_t>("scan_e", scan_scratch_words(E + 1), &e);
    WV_CUDA(c, e);
    WV_CUDA(c, cudaMemsetAsync(bcur, 0, 2 * (size_t)n * 4, c->stream));
    WV_CUDA(c, cudaMemsetAsync(ovf, 0, (size_t)(E + 1) * 4, c->stream));
    k_upd_scatter<<<nb, NODE_THREADS, 0, c->stream>>>(s, eoff, boff, bcur, bsrc, bflat);
    const uint32_t nbk = 2 * n;
    k_bucket_sort<<<(nbk + BK_WARPS - 1) / BK_WARPS, BK_WARPS * 32, 0, c->stream>>>(nbk, boff, bcnt, bsrc, bflat,
                                                                                    p.R, ovf, bigb, usmall + 1);
    WV_CUDA(c, cudaGetLastError());
    uint32_t hb[2];
    WV_CUDA(c, cudaMemcpyAsync(hb, usmall, 8, cudaMemcpyDeviceToHost, c->stream));
    WV_CUDA(c, cudaStreamSynchronize(c->stream));
    if (hb[1]) {
      uint32_t P = 1;
      while (P < hb[0]) P <<= 1;
      unsigned long long *bscr = c->buf<unsigned long long>("bscr", (size_t)hb[1] * P, &e);
      WV_CUDA(c, e);
      k_bucket_sort_big<<<hb[1], 1024, 0, c->stream>>>(bigb, boff, bcnt, bsrc, bflat, p.R, ovf, bscr, P);
      WV_CUDA(c, cudaGetLastError());
    }
    WV_CUDA(c, exclusive_scan_u32(ovf, ovf_ord, (size_t)E + 1, scan_e, c->stream));
    uint32_t nov = 0;
    WV_CUDA(c, cudaMemcpyAsync(&nov, ovf_ord + E, 4, cudaMemcpyDeviceToHost, c->stream));
    WV_CUDA(c, cudaStreamSynchronize(c->stream));
    int rc = check_device_status(c, "nndescent update");
    if (rc) return rc;
    // the overflow overwrites consume rand() in (n, l) order
    std::vector<int> hrv(nov + 1);
    for (uint32_t k = 0; k < nov; k++) hrv[k] = c->rnd.next();
    int *rv = c->buf<int>("rv", nov + 1, &e);
    WV_CUDA(c, e);
    WV_CUDA(c, cudaMemcpyAsync(rv, hrv.data(), (size_t)(nov + 1) * 4, cudaMemcpyHostToDevice, c->stream));
    k_bucket_apply<<<nb, NODE_THREADS, 0, c->stream>>>(s, boff, bcnt, bsrc, bflat, ovf_ord, rv);
    WV_CUDA(c, cudaGetLastError());
    S.overflow_events += nov;
    cudaEventRecord(ev1, c->stream);
    WV_CUDA(c, cudaEventSynchronize(ev1));
    float ms = 0;
    cudaEventElapsedTime(&ms, ev0, ev1);
    S.ms_update += ms;
  }
  // ------------------------------------------------------------ tail
  WV_CUDA(c, c->fg_ids.ensure((size_t)n * p.K * 4));
  WV_CUDA(c, c->fg_dist.ensure((size_t)n * p.K * 4));
  WV_CUDA(c, c->fg_deg.ensure((size_t)n * 4));
  k_nnd_final<<<nb, NODE_THREADS, node_smem, c->stream>>>(s, c->fg_ids.as<uint32_t>(), c->fg_dist.as<float>(),
                                                           c->fg_deg.as<uint32_t>());
  WV_CUDA(c, cudaGetLastError());
  unsigned long long hp = 0;
  WV_CUDA(c, cudaMemcpyAsync(&hp, pairs, 8, cudaMemcpyDeviceToHost, c->stream));
  WV_CUDA(c, cudaStreamSynchronize(c->stream));
  S.pairs = hp;
  cudaEventDestroy(ev0);
  cudaEventDestroy(ev1);
  c->fg_w = p.K;
  c->fg_has_ep = false;
  c->fg_eps.clear();
  return check_device_status(c, "nndescent");
}

}  // namespace wv
