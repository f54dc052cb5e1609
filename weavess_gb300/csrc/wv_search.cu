// K6 / K3: batched greedy beam search on GB300.
//
// ROUTER_GREEDY: replaces the per-query loop of IndexBuilder::search
// (src/builder.cpp:445-454) over ComponentSearchEntry*::SearchEntryInner +
// ComponentSearchRouteGreedy::RouteInner (src/component_route.cpp:9-53).
// Build mode: ComponentCandidateNSG::CandidateInner
// (src/component_candidate.cpp:10-85) for base points.
//
// One warp owns one query at a time; persistent warps pull query indices
// from a global counter, so queries of different beam widths L and result
// sizes K share one launch.  Per expansion the warp reads the node's row once
// (coalesced), tests every neighbour against its visited set, computes the
// distances of the fresh ones with all their row loads in flight together,
// and merges the accepted ones into the pool.
//
// Exactness (the plain FP32 form): result ids, pool order and the
// DistCount/HopCount counters equal the reference's, because
//  * distances are folded in the reference's order (one lane per row,
//    wv_common.cuh), or -- when base and query are integers in [0, 255] and
//    d <= 256, so every partial sum is an integer below 2^24 and any order
//    gives the same FP32 value -- summed by a coalesced warp reduction;
//  * the seed pool is ordered as std::sort orders it: a bitonic sort on
//    (dist, seed position) gives the stable order, which is std::sort's
//    whenever L <= 16 or no two seed distances tie; otherwise the warp replays
//    libstdc++'s introsort (warp_sort.cuh) on the seeds in their drawn order;
//  * one expansion's sequential InsertIntoPool calls (index.h:152-180) equal a
//    stable merge of the pool with the accepted candidates sorted by
//    (distance, adjacency position), pool entries before equal candidates,
//    truncated to L; candidates whose id is already pooled (unvisited seeds)
//    are rejected; and the restart index nk is the smallest final position of
//    an accepted candidate (positions before it never move);
//  * the visited set (flags, route.cpp:14) is exact: an open-addressing hash
//    in shared memory while it is at most half full, then the warp's global
//    bitset for the rest of the query.  Route mode does not mark seeds, build
//    mode does, as the reference.
#include <cuda_bf16.h>
#include <cuda_fp8.h>

#include <cstdio>

#include "warp_sort.cuh"
#include "wv_common.cuh"
#include "wv_lowp.cuh"
#include "wv_search.h"

namespace wv {

namespace {

constexpr int WARPS = 4;  // warps per block
constexpr uint32_t EMPTY = 0xffffffffu;

__host__ __device__ inline size_t align16(size_t x) { return (x + 15) & ~size_t(15); }
__host__ __device__ inline uint32_t pow2_at_least(uint32_t x) {
  uint32_t p = 1;
  while (p < x) p <<= 1;
  return p;
}
// pool arrays: room for L + 1 entries and for the bitonic sort of nextpow2(L)
__host__ __device__ inline uint32_t pool_cap(uint32_t Lmax) { return max(pow2_at_least(Lmax), Lmax + 1); }
// hash slots: >= 2048, and room for the seed sort's partition scratch
__host__ __device__ inline uint32_t hash_cap(uint32_t Lmax) { return pow2_at_least(max(2048u, 2 * Lmax + 256)); }

struct WarpSmem {
  uint32_t *hash;  // hcap
  float *qv;       // dpad
  float *pa_d;     // pool A (pcap)
  uint32_t *pa_i;
  float *pb_d;     // pool B (pcap)
  uint32_t *pb_i;
  float *cd;       // accepted candidates (cap)
  uint32_t *ci;
  uint32_t *fi;    // fresh ids of one expansion (cap)
};

__host__ __device__ inline size_t warp_smem_bytes(uint32_t d, uint32_t Lmax, uint32_t cap) {
  size_t b = 0;
  b += align16((size_t)hash_cap(Lmax) * 4);
  b += align16(((d + 3) & ~3u) * 4);
  b += 4 * align16((size_t)pool_cap(Lmax) * 4);
  b += 3 * align16(cap * 4);
  return b;
}

__device__ inline WarpSmem carve(uint8_t *p, uint32_t d, uint32_t Lmax, uint32_t cap) {
  WarpSmem s;
  const uint32_t pc = pool_cap(Lmax);
  s.hash = (uint32_t *)p;
  p += align16((size_t)hash_cap(Lmax) * 4);
  s.qv = (float *)p;
  p += align16(((d + 3) & ~3u) * 4);
  s.pa_d = (float *)p;
  p += align16((size_t)pc * 4);
  s.pa_i = (uint32_t *)p;
  p += align16((size_t)pc * 4);
  s.pb_d = (float *)p;
  p += align16((size_t)pc * 4);
  s.pb_i = (uint32_t *)p;
  p += align16((size_t)pc * 4);
  s.cd = (float *)p;
  p += align16(cap * 4);
  s.ci = (uint32_t *)p;
  p += align16(cap * 4);
  s.fi = (uint32_t *)p;
  return s;
}

// first index >= from with the FLAG bit set, or L
__device__ inline int first_flag(const uint32_t *pi, int from, int L, int lane) {
  for (int b = from; b < L; b += 32) {
    int i = b + lane;
    unsigned m = __ballot_sync(FULL, i < L && (pi[i] & FLAG));
    if (m) return b + __ffs(m) - 1;
  }
  return L;
}

// number of entries of the sorted array a[0..n) with a[i] <= x (upper bound)
__device__ inline int upper_bound_f(const float *a, int n, float x) {
  int lo = 0, hi = n;
  while (lo < hi) {
    int mid = (lo + hi) >> 1;
    if (a[mid] <= x) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}
// number of entries with a[i] < x (lower bound)
__device__ inline int lower_bound_f(const float *a, int n, float x) {
  int lo = 0, hi = n;
  while (lo < hi) {
    int mid = (lo + hi) >> 1;
    if (a[mid] < x) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

__device__ __forceinline__ uint32_t hslot(uint32_t id, uint32_t mask) { return (id * 2654435761u) & mask; }

// visited test-and-set over a shared-memory hash that spills to a bitset
struct Visited {
  uint32_t *hash, mask, inserted, limit;
  bool spill;  // the hash reached its limit: new ids go to the global bitset
  uint32_t *bits, *touched, ntouch;

  __device__ void clear(int lane) {
    for (uint32_t i = lane; i <= mask; i += 32) hash[i] = EMPTY;
    __syncwarp();
    for (uint32_t i = lane; i < ntouch; i += 32) bits[touched[i]] = 0u;
    __syncwarp();
    inserted = 0;
    spill = false;
    ntouch = 0;
  }
  // warp-uniform call; `want` lanes test `id` (ids distinct among lanes);
  // returns true for lanes whose id was not visited before
  __device__ bool test_and_set(bool want, uint32_t id, int lane) {
    const unsigned wm = __ballot_sync(FULL, want);
    if (!spill && inserted + __popc(wm) > limit) spill = true;
    bool fresh = false, newword = false;
    if (want) {
      uint32_t h = hslot(id, mask);
      if (!spill) {
        while (true) {
          const uint32_t old = atomicCAS(&hash[h], EMPTY, id);
          if (old == EMPTY) {
            fresh = true;
            break;
          }
          if (old == id) break;
          h = (h + 1) & mask;
        }
      } else {
        bool in_hash = false;
        while (true) {
          const uint32_t v = hash[h];
          if (v == id) {
            in_hash = true;
            break;
          }
          if (v == EMPTY) break;
          h = (h + 1) & mask;
        }
        if (!in_hash) {
          const uint32_t bit = 1u << (id & 31);
          const uint32_t old = atomicOr(bits + (id >> 5), bit);
          fresh = (old & bit) == 0;
          newword = old == 0;
        }
      }
    }
    const unsigned fm = __ballot_sync(FULL, fresh);
    if (!spill) inserted += __popc(fm);
    const unsigned nwm = __ballot_sync(FULL, newword);
    if (newword) touched[ntouch + __popc(nwm & ((1u << lane) - 1u))] = id >> 5;
    ntouch += __popc(nwm);
    return fresh;
  }
};

// Orders the L seeds (pa_*, in drawn order) into pb_* exactly as std::sort
// would, flags set.  A bitonic sort on (dist, seed position) gives the stable
// order, which is std::sort's whenever L <= 16 or no two seed distances tie;
// otherwise the warp replays libstdc++'s introsort (warp_sort.cuh).  Uses the
// hash area as scratch (the caller clears it afterwards).
__device__ void sort_seeds(WarpSmem &s, int L, int lane) {
  const int P = (int)pow2_at_least((uint32_t)L);
  float *kd = s.pb_d;
  uint32_t *kx = s.pb_i;
  for (int i = lane; i < P; i += 32) {
    kd[i] = i < L ? s.pa_d[i] : __int_as_float(0x7f800000);
    kx[i] = i;
  }
  __syncwarp();
  for (int k = 2; k <= P; k <<= 1) {
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int i = lane; i < P; i += 32) {
        int l = i ^ j;
        if (l > i) {
          bool up = (i & k) == 0;
          float di = kd[i], dl = kd[l];
          uint32_t xi = kx[i], xl = kx[l];
          bool gt = di > dl || (di == dl && xi > xl);
          if (gt == up) {
            kd[i] = dl;
            kd[l] = di;
            kx[i] = xl;
            kx[l] = xi;
          }
        }
      }
      __syncwarp();
    }
  }
  bool tie = false;
  for (int i = lane + 1; i < L; i += 32) tie |= kd[i] == kd[i - 1];
  tie = __any_sync(FULL, tie);
  if (!tie || L <= 16) {
    // kd already holds the sorted distances; each lane rewrites its own slots
    for (int i = lane; i < L; i += 32) s.pb_i[i] = s.pa_i[kx[i]] | FLAG;
  } else {
    // ties and L > 16: replay libstdc++ introsort on the drawn order; the
    // pairs sort in the B pool region (pb_d and pb_i are contiguous,
    // 2 * pcap >= 2L words), the partition scratch sits in the hash area
    __syncwarp();
    DI *tmp = reinterpret_cast<DI *>(s.pb_d);
    for (int i = lane; i < L; i += 32) tmp[i] = DI{s.pa_d[i], s.pa_i[i]};
    int *scr = reinterpret_cast<int *>(s.hash);
    __syncwarp();
    warp_std_sort(tmp, L, DILess(), WarpSortScratch{scr, scr + L, scr + 2 * L, scr + 2 * L + 192}, lane);
    // unpack through pool A (the drawn order is no longer needed)
    for (int i = lane; i < L; i += 32) {
      const DI x = tmp[i];
      s.pa_d[i] = x.d;
      s.pa_i[i] = x.i;
    }
    __syncwarp();
    for (int i = lane; i < L; i += 32) {
      s.pb_d[i] = s.pa_d[i];
      s.pb_i[i] = s.pa_i[i] | FLAG;
    }
  }
  __syncwarp();
}

// distances of `cnt` rows (ids in lanes 0..cnt-1 of `my`) to the query.
// INTS: warp-cooperative coalesced rows (any summation order is exact);
// else one lane per row in the reference's order.
template <bool INTS>
__device__ __forceinline__ float batch_dist(const float *__restrict__ base, uint32_t d, uint32_t my, int cnt,
                                            const float *qv, int lane) {
  float out = 0.f;
  const uint32_t d4 = d >> 2;
  if (INTS) {
    const float4 *q4 = reinterpret_cast<const float4 *>(qv);
    constexpr int G = 8;
    for (int c0 = 0; c0 < cnt; c0 += G) {
      float part[G];
      const float4 *row[G];
#pragma unroll
      for (int g = 0; g < G; g++) {
        const int c = c0 + g;
        const uint32_t id = __shfl_sync(FULL, my, c & 31);
        part[g] = 0.f;
        row[g] = c < cnt ? reinterpret_cast<const float4 *>(base + (size_t)id * d) : nullptr;
      }
      // chunk-major: the G rows' loads of one step are independent
      for (uint32_t k = lane; k < d4; k += 32) {
        const float4 qk = q4[k];
#pragma unroll
        for (int g = 0; g < G; g++)
          if (row[g]) part[g] += group4(__ldg(row[g] + k), qk);
      }
#pragma unroll
      for (int g = 0; g < G; g++) {
        float v = part[g];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(FULL, v, o);
        if (lane == c0 + g) out = v;
      }
    }
  } else if (lane < cnt) {
    const float4 *row = reinterpret_cast<const float4 *>(base + (size_t)my * d);
    const float4 *q4 = reinterpret_cast<const float4 *>(qv);
#pragma unroll 8
    for (uint32_t g = 0; g < d4; g++) out = __fadd_rn(out, group4(__ldg(row + g), q4[g]));
  }
  return out;
}

__device__ __forceinline__ float cand_dist(const SearchArgs &a, bool ints, uint32_t my, int cnt, const float *qv,
                                           int lane) {
  if (a.storage != 0) return lowp_rows_dist(LowpRows{a.qbase, a.qscale, a.storage, a.d}, my, cnt, qv, lane);
  return ints ? batch_dist<true>(a.base, a.d, my, cnt, qv, lane) : batch_dist<false>(a.base, a.d, my, cnt, qv, lane);
}

// BUILD = false: SearchEntry* + ROUTER_GREEDY (seeds not marked visited,
//   DistCount / HopCount kept, top-K written).
// BUILD = true: CandidateNSG::CandidateInner for base points: seeds are
//   marked visited, and every visited (id, dist) -- the seeds in drawn order,
//   then each newly visited id in visit order -- is appended to the query's
//   visit list (vis, vcap apart, vlimit entries kept, count in vcnt).
template <bool BUILD>
__global__ void __launch_bounds__(WARPS * 32) k_search(SearchArgs a) {
  extern __shared__ __align__(16) uint8_t smem[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const size_t wbytes = warp_smem_bytes(a.d, a.Lmax, a.cap);
  WarpSmem s = carve(smem + warp * wbytes, a.d, a.Lmax, a.cap);
  const uint32_t slot = blockIdx.x * WARPS + warp;
  Visited vis;
  vis.hash = s.hash;
  vis.mask = hash_cap(a.Lmax) - 1;
  vis.limit = hash_cap(a.Lmax) / 2;
  vis.bits = a.visited + (size_t)slot * a.words;
  vis.touched = a.touched + (size_t)slot * a.words;
  vis.ntouch = 0;
  vis.inserted = 0;
  vis.spill = false;
  unsigned long long dcount = 0, hcount = 0;
  const unsigned lt = (1u << lane) - 1u;

  while (true) {
    uint32_t q = 0;
    if (lane == 0) q = atomicAdd(a.next_query, 1u);
    q = __shfl_sync(FULL, q, 0);
    if (q >= a.nq) break;
    const int L = (int)(a.Lq ? a.Lq[q] : a.L);
    const int K = (int)(a.Kq ? a.Kq[q] : a.K);
    const float *qsrc = a.queries + (size_t)q * a.d;
    bool qint = true;
    for (uint32_t i = lane; i < a.d; i += 32) {
      const float v = qsrc[i];
      s.qv[i] = v;
      qint &= v >= 0.f && v <= 255.f && v == rintf(v);
    }
    // integer base and query: any summation order gives the reference's value
    const bool ints = a.int_exact && a.d <= 256 && __all_sync(FULL, qint);
    // ---- seeds (SearchEntryInner): distances in drawn order ----
    const uint32_t *seeds = a.seeds + (size_t)q * a.seed_stride;
    uint32_t nvis = 0;
    DI *vis_out = BUILD ? a.vis + (size_t)q * a.vcap : nullptr;
    __syncwarp();
    for (int b = 0; b < L; b += 32) {
      const int cnt = min(32, L - b);
      uint32_t id = lane < cnt ? seeds[b + lane] : 0u;
      if (lane < cnt && id >= a.n) {
        set_err(a.status, DEV_BAD_ID);
        id = 0;
      }
      const float dist = cand_dist(a, ints, id, cnt, s.qv, lane);
      if (lane < cnt) {
        s.pa_d[b + lane] = dist;
        s.pa_i[b + lane] = id;
        if (BUILD && nvis + lane < a.vlimit) vis_out[nvis + lane] = DI{dist, id};
      }
      nvis += cnt;
    }
    dcount += L;
    __syncwarp();
    sort_seeds(s, L, lane);
    vis.clear(lane);  // the seed sort used the hash as scratch
    if (BUILD) {
      // CandidateNSG flags its seeds (component_candidate.cpp:21-29)
      for (int b = 0; b < L; b += 32) {
        const int i = b + lane;
        const uint32_t id = i < L ? (s.pb_i[i] & ID_MASK) : EMPTY;
        // duplicate seeds among lanes: only the first tests
        const unsigned same = __match_any_sync(FULL, id);
        vis.test_and_set(i < L && (__ffs(same) - 1) == lane, id, lane);
      }
    }
    float *pd = s.pb_d, *od = s.pa_d;
    uint32_t *pi = s.pb_i, *oi = s.pa_i;

    // ---- route (RouteInner) ----
    int k = first_flag(pi, 0, L, lane);
    while (k < L) {
      const uint32_t node = pi[k] & ID_MASK;
      __syncwarp();
      if (lane == 0) pi[k] = node;  // flag = false
      __syncwarp();
      hcount++;
      const uint32_t *row = a.gids + (size_t)node * a.gw;
      // the degree and the first 32 slots of the row are loaded together
      // (slots past the degree are read but ignored; rows are gw wide)
      uint32_t deg = __ldg(a.gdeg + node);
      const uint32_t head = lane < a.gw ? __ldg(row + lane) : INVALID;
      if (deg > a.gw) {
        set_err(a.status, DEV_BAD_ID);
        deg = a.gw;
      }
      const float thr = pd[L - 1];
      // 1) the fresh neighbours, in adjacency order
      uint32_t nfresh = 0;
      for (uint32_t m0 = 0; m0 < deg; m0 += 32) {
        const uint32_t m = m0 + lane;
        uint32_t id = m < deg ? (m0 == 0 ? head : __ldg(row + m)) : INVALID;
        if (id != INVALID && id >= a.n) {
          set_err(a.status, DEV_BAD_ID);
          id = INVALID;
        }
        // a repeated id inside this chunk: only its first position visits it
        const unsigned same = __match_any_sync(FULL, id);
        const bool leader = (__ffs(same) - 1) == lane;
        const bool fresh = vis.test_and_set(id != INVALID && leader, id, lane);
        const unsigned fm = __ballot_sync(FULL, fresh);
        if (fresh) s.fi[nfresh + __popc(fm & lt)] = id;
        nfresh += __popc(fm);
      }
      __syncwarp();
      // 2) their distances, 3) the accepted ones in adjacency order
      int ncand = 0;
      for (uint32_t b = 0; b < nfresh; b += 32) {
        const int cnt = (int)min(32u, nfresh - b);
        const uint32_t my = lane < cnt ? s.fi[b + lane] : 0u;
        const float dist = cand_dist(a, ints, my, cnt, s.qv, lane);
        if (BUILD) {
          if (lane < cnt && nvis + lane < a.vlimit) vis_out[nvis + lane] = DI{dist, my};
          nvis += cnt;
        }
        bool acc = false;
        if (lane < cnt && dist < thr) {
          // reject an id already in the pool (an unvisited seed): same id
          // implies same distance, so look inside the run of equal distances
          int lo = lower_bound_f(pd, L, dist), hi = upper_bound_f(pd, L, dist);
          acc = true;
          for (int t = lo; t < hi; t++)
            if ((pi[t] & ID_MASK) == my) acc = false;
        }
        const unsigned am = __ballot_sync(FULL, acc);
        if (acc) {
          const int r = ncand + __popc(am & lt);
          s.cd[r] = dist;
          s.ci[r] = my;
        }
        ncand += __popc(am);
      }
      dcount += nfresh;
      __syncwarp();
      int nk = L;
      if (ncand > 0) {
        // stable rank of each candidate by distance (adjacency order on ties)
        float myd[8];
        uint32_t myi[8];
        int myr[8];
        int nmine = 0;
        for (int c = lane; c < ncand; c += 32) {
          const float dc = s.cd[c];
          int r = 0;
          for (int c2 = 0; c2 < ncand; c2++) {
            const float d2 = s.cd[c2];
            r += (d2 < dc) || (d2 == dc && c2 < c);
          }
          myd[nmine] = dc;
          myi[nmine] = s.ci[c];
          myr[nmine] = r;
          nmine++;
        }
        __syncwarp();
        for (int t = 0; t < nmine; t++) s.cd[myr[t]] = myd[t];  // sorted distances
        __syncwarp();
        // pool entries move down by the number of strictly closer candidates
        for (int j = lane; j < L; j += 32) {
          const int pos = j + lower_bound_f(s.cd, ncand, pd[j]);
          if (pos < L) {
            od[pos] = pd[j];
            oi[pos] = pi[j];
          }
        }
        // candidates go after every pool entry of equal or smaller distance
        int mink = L;
        for (int t = 0; t < nmine; t++) {
          const int pos = myr[t] + upper_bound_f(pd, L, myd[t]);
          if (pos < L) {
            od[pos] = myd[t];
            oi[pos] = myi[t] | FLAG;
            mink = min(mink, pos);
          }
        }
        for (int o = 16; o > 0; o >>= 1) mink = min(mink, __shfl_xor_sync(FULL, mink, o));
        nk = mink;
        __syncwarp();
        float *t1 = pd;
        pd = od;
        od = t1;
        uint32_t *t2 = pi;
        pi = oi;
        oi = t2;
      }
      const int next = (nk <= k) ? nk : k + 1;
      k = first_flag(pi, next, L, lane);
    }
    // ---- exact FP32 rerank of the final pool (low-precision storage) ----
    if (!BUILD && a.storage != 0 && a.rerank > 0) {
      const int R = min((int)a.rerank, L);
      for (int b = 0; b < R; b += 32) {
        const int cnt = min(32, R - b);
        const uint32_t id = lane < cnt ? (pi[b + lane] & ID_MASK) : 0u;
        const float ex = ints ? batch_dist<true>(a.base, a.d, id, cnt, s.qv, lane)
                              : batch_dist<false>(a.base, a.d, id, cnt, s.qv, lane);
        if (lane < cnt) {
          od[b + lane] = ex;
          oi[b + lane] = id;
        }
      }
      dcount += R;
      __syncwarp();
      // stable order by the exact distance (pool position breaks ties)
      for (int c = lane; c < R; c += 32) {
        const float dc = od[c];
        int r = 0;
        for (int c2 = 0; c2 < R; c2++) {
          const float d2 = od[c2];
          r += (d2 < dc) || (d2 == dc && c2 < c);
        }
        pd[r] = dc;  // pd / pi receive the re-sorted head of the pool
        pi[r] = oi[c];
      }
      __syncwarp();
    }
    // ---- results ----
    if (BUILD && lane == 0) {
      a.vcnt[q] = nvis;
      if (nvis > a.vlimit) set_err(a.status, DEV_OVERFLOW);
    }
    if (a.out_ids)
      for (int i = lane; i < K; i += 32) {
        a.out_ids[(size_t)q * a.out_stride + i] = pi[i] & ID_MASK;
        if (a.out_dist) a.out_dist[(size_t)q * a.out_stride + i] = pd[i];
      }
    vis.clear(lane);
  }
  if (!BUILD && lane == 0 && a.counters) {
    atomicAdd(a.counters + 0, dcount);
    atomicAdd(a.counters + 1, hcount);
  }
}

template <bool B>
void set_attr(size_t smem) {
  cudaFuncSetAttribute(k_search<B>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
}

}  // namespace

size_t search_block_smem(uint32_t d, uint32_t Lmax, uint32_t cap) { return WARPS * warp_smem_bytes(d, Lmax, cap); }

int search_warps_per_block() { return WARPS; }

int search_grid(uint32_t d, uint32_t Lmax, uint32_t cap, int device) {
  const size_t smem = search_block_smem(d, Lmax, cap);
  if (smem > 227 * 1024) return 0;
  set_attr<false>(smem);
  set_attr<true>(smem);
  if (cudaGetLastError() != cudaSuccess) return 0;
  int per_sm = 0, sms = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_search<true>, WARPS * 32, smem) != cudaSuccess)
    return 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) return 0;
  return per_sm * sms;
}

cudaError_t launch_search_exact(const SearchArgs &a, int blocks, cudaStream_t stream) {
  const size_t smem = search_block_smem(a.d, a.Lmax, a.cap);
  if (a.vis) k_search<true><<<blocks, WARPS * 32, smem, stream>>>(a);
  else k_search<false><<<blocks, WARPS * 32, smem, stream>>>(a);
  return cudaGetLastError();
}

}  // namespace wv
