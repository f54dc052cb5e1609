// K6: batched greedy beam search (ROUTER_GREEDY) on GB300.
//
// Replaces the per-query loop of IndexBuilder::search (src/builder.cpp:445-454)
// over ComponentSearchEntry*::SearchEntryInner + ComponentSearchRouteGreedy::
// RouteInner (src/component_route.cpp:9-53).  One warp owns one query at a time
// (persistent warps pull query indices from a global counter), so queries of
// different beam widths L and result sizes K share one launch.
//
// Exactness (the plain FP32 form): the result ids, the pool order and the
// DistCount/HopCount counters equal the reference's, because
//  * every distance is folded in the reference's order (wv_common.cuh);
//  * the seed pool is ordered as std::sort orders it: a bitonic sort on
//    (dist, seed position) gives the stable order, which is std::sort's order
//    whenever L <= 16 or no two seed distances tie; otherwise one lane replays
//    libstdc++'s introsort (stl_order.cuh) on the seeds in their drawn order;
//  * one expansion's sequential InsertIntoPool calls (index.h:152-180) equal a
//    stable merge of the pool with the accepted candidates sorted by
//    (distance, adjacency position), pool entries before equal candidates,
//    truncated to L; candidates whose id is already pooled (unvisited seeds)
//    are rejected; and the restart index nk is the smallest final position of
//    an accepted candidate (positions before it never move);
//  * the visited set is an exact per-warp bitset (flags, route.cpp:14), seeds
//    are not marked, as in the reference.
#include <cstdio>

#include "warp_sort.cuh"
#include "wv_common.cuh"
#include "wv_search.h"

namespace wv {

namespace {

constexpr int WARPS = 4;  // warps per block

struct WarpSmem {
  float *stage;   // STAGE_FLOATS
  float *qv;      // dpad
  float *pa_d;    // pool A (Lmax + 1)
  uint32_t *pa_i;
  float *pb_d;    // pool B (Lmax + 1)
  uint32_t *pb_i;
  float *cd;      // accepted candidates (cap)
  uint32_t *ci;
};

__host__ __device__ inline size_t align16(size_t x) { return (x + 15) & ~size_t(15); }

__host__ __device__ inline size_t warp_smem_bytes(uint32_t d, uint32_t Lmax, uint32_t cap) {
  size_t b = 0;
  b += align16(STAGE_FLOATS * 4);
  b += align16(((d + 3) & ~3u) * 4);
  b += 4 * align16((Lmax + 1) * 4);
  b += 2 * align16(cap * 4);
  return b;
}

__device__ inline WarpSmem carve(uint8_t *p, uint32_t d, uint32_t Lmax, uint32_t cap) {
  WarpSmem s;
  s.stage = (float *)p;
  p += align16(STAGE_FLOATS * 4);
  s.qv = (float *)p;
  p += align16(((d + 3) & ~3u) * 4);
  s.pa_d = (float *)p;
  p += align16((Lmax + 1) * 4);
  s.pa_i = (uint32_t *)p;
  p += align16((Lmax + 1) * 4);
  s.pb_d = (float *)p;
  p += align16((Lmax + 1) * 4);
  s.pb_i = (uint32_t *)p;
  p += align16((Lmax + 1) * 4);
  s.cd = (float *)p;
  p += align16(cap * 4);
  s.ci = (uint32_t *)p;
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

// Orders the L seeds (pa_*, in drawn order) into pb_* exactly as std::sort
// would, flags set.  A bitonic sort on (dist, seed position) gives the stable
// order, which is std::sort's whenever L <= 16 or no two seed distances tie;
// otherwise the warp replays libstdc++'s introsort (warp_sort.cuh).  Uses
// stage as scratch.
__device__ void sort_seeds(WarpSmem &s, int L, int lane) {
  int P = 1;
  while (P < L) P <<= 1;
  // keys in stage: dist (P floats) then position (P u32)
  float *kd = s.stage;
  uint32_t *kx = (uint32_t *)(s.stage + P);
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
    for (int i = lane; i < L; i += 32) {
      uint32_t x = kx[i];
      s.pb_d[i] = s.pa_d[x];
      s.pb_i[i] = s.pa_i[x] | FLAG;
    }
  } else {
    // ties and L > 16: replay libstdc++ introsort on the drawn order.  The
    // pairs sort in the B pool region (2 x (Lmax+1) words), the partition
    // scratch sits in stage; the result goes through stage into B.
    __syncwarp();
    DI *tmp = reinterpret_cast<DI *>(s.pb_d);
    for (int i = lane; i < L; i += 32) tmp[i] = DI{s.pa_d[i], s.pa_i[i]};
    int *scr = reinterpret_cast<int *>(s.stage);
    __syncwarp();
    warp_std_sort(tmp, L, DILess(), WarpSortScratch{scr, scr + L, scr + 2 * L, scr + 2 * L + 192}, lane);
    DI *out = reinterpret_cast<DI *>(s.stage);
    for (int i = lane; i < L; i += 32) out[i] = tmp[i];
    __syncwarp();
    for (int i = lane; i < L; i += 32) {
      s.pb_d[i] = out[i].d;
      s.pb_i[i] = out[i].i | FLAG;
    }
  }
  __syncwarp();
}

// BUILD = false: SearchEntry* + ROUTER_GREEDY (seeds not marked visited,
//   DistCount / HopCount kept, top-K written).
// BUILD = true: CandidateNSG::CandidateInner (component_candidate.cpp:10-85)
//   for base points: seeds are marked visited, and every visited (id, dist)
//   -- the seeds in drawn order, then each newly visited id in visit order --
//   is appended to the query's visit list (vis, vcap entries, count in vcnt).
template <bool BUILD>
__global__ void __launch_bounds__(WARPS * 32) k_search(SearchArgs a) {
  extern __shared__ __align__(16) uint8_t smem[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const size_t wbytes = warp_smem_bytes(a.d, a.Lmax, a.cap);
  WarpSmem s = carve(smem + warp * wbytes, a.d, a.Lmax, a.cap);
  const uint32_t slot = blockIdx.x * WARPS + warp;
  uint32_t *vis = a.visited + (size_t)slot * a.words;
  uint32_t *touched = a.touched + (size_t)slot * a.words;
  unsigned long long dcount = 0, hcount = 0;

  while (true) {
    uint32_t q = 0;
    if (lane == 0) q = atomicAdd(a.next_query, 1u);
    q = __shfl_sync(FULL, q, 0);
    if (q >= a.nq) break;
    const int L = (int)(a.Lq ? a.Lq[q] : a.L);
    const int K = (int)(a.Kq ? a.Kq[q] : a.K);
    const float *qsrc = a.queries + (size_t)q * a.d;
    for (uint32_t i = lane; i < a.d; i += 32) s.qv[i] = qsrc[i];
    // ---- seeds (SearchEntryInner): distances in drawn order ----
    const uint32_t *seeds = a.seeds + (size_t)q * a.seed_stride;
    uint32_t ntouch = 0;
    uint32_t nvis = 0;
    DI *vis_out = BUILD ? a.vis + (size_t)q * a.vcap : nullptr;
    __syncwarp();
    for (int b = 0; b < L; b += 32) {
      int cnt = min(32, L - b);
      uint32_t id = lane < cnt ? seeds[b + lane] : 0u;
      if (lane < cnt && id >= a.n) {
        set_err(a.status, DEV_BAD_ID);
        id = 0;
      }
      if (BUILD) {
        // CandidateNSG flags its seeds (component_candidate.cpp:21-29)
        bool newword = false;
        if (lane < cnt) {
          const uint32_t bit = 1u << (id & 31);
          newword = atomicOr(vis + (id >> 5), bit) == 0;
        }
        const unsigned nwm = __ballot_sync(FULL, newword);
        if (newword) touched[ntouch + __popc(nwm & ((1u << lane) - 1u))] = id >> 5;
        ntouch += __popc(nwm);
      }
      float dist = warp_l2_rows(a.base, a.d, id, cnt, s.qv, s.stage, lane);
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
      uint32_t deg = a.gdeg[node];
      if (deg > a.gw) {
        set_err(a.status, DEV_BAD_ID);
        deg = a.gw;
      }
      const uint32_t *row = a.gids + (size_t)node * a.gw;
      const float thr = pd[L - 1];
      int ncand = 0;
      for (uint32_t m0 = 0; m0 < deg; m0 += 32) {
        const uint32_t m = m0 + lane;
        uint32_t id = m < deg ? row[m] : INVALID;
        if (id != INVALID && id >= a.n) {
          set_err(a.status, DEV_BAD_ID);
          id = INVALID;
        }
        // a repeated id inside this chunk: only its first position visits it
        const unsigned same = __match_any_sync(FULL, id);
        const bool leader = (__ffs(same) - 1) == lane;
        bool fresh = false, newword = false;
        if (id != INVALID && leader) {
          const uint32_t bit = 1u << (id & 31);
          const uint32_t old = atomicOr(vis + (id >> 5), bit);
          fresh = (old & bit) == 0;
          newword = old == 0;
        }
        // words that became non-zero are recorded so the query can clear them
        const unsigned lt = (1u << lane) - 1u;
        const unsigned nwm = __ballot_sync(FULL, newword);
        if (newword) touched[ntouch + __popc(nwm & lt)] = id >> 5;
        ntouch += __popc(nwm);
        const unsigned fm = __ballot_sync(FULL, fresh);
        const int cnt = __popc(fm);
        if (cnt == 0) continue;
        // compact the fresh ids to lanes 0..cnt-1, adjacency order kept
        uint32_t *xch = s.ci + a.cap - 32;
        if (fresh) xch[__popc(fm & lt)] = id;
        __syncwarp();
        const uint32_t my = lane < cnt ? xch[lane] : 0u;
        __syncwarp();
        float dist = warp_l2_rows(a.base, a.d, my, cnt, s.qv, s.stage, lane);
        dcount += cnt;
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
        unsigned am = __ballot_sync(FULL, acc);
        if (acc) {
          int r = ncand + __popc(am & ((1u << lane) - 1));
          s.cd[r] = dist;
          s.ci[r] = my;
        }
        ncand += __popc(am);
        __syncwarp();
      }
      int nk = L;
      if (ncand > 0) {
        // stable rank of each candidate by distance (adjacency order on ties)
        float myd[8];
        uint32_t myi[8];
        int myr[8];
        int nmine = 0;
        for (int c = lane; c < ncand; c += 32) {
          float dc = s.cd[c];
          int r = 0;
          for (int c2 = 0; c2 < ncand; c2++) {
            float d2 = s.cd[c2];
            r += (d2 < dc) || (d2 == dc && c2 < c);
          }
          myd[nmine] = dc;
          myi[nmine] = s.ci[c];
          myr[nmine] = r;
          nmine++;
        }
        __syncwarp();
        // sorted candidate distances into cd (for the pool-side bound search)
        for (int t = 0; t < nmine; t++) s.cd[myr[t]] = myd[t];
        __syncwarp();
        // pool entries move down by the number of strictly closer candidates
        for (int j = lane; j < L; j += 32) {
          int pos = j + lower_bound_f(s.cd, ncand, pd[j]);
          if (pos < L) {
            od[pos] = pd[j];
            oi[pos] = pi[j];
          }
        }
        // candidates go after every pool entry of equal or smaller distance
        int mink = L;
        for (int t = 0; t < nmine; t++) {
          int pos = myr[t] + upper_bound_f(pd, L, myd[t]);
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
      int next = (nk <= k) ? nk : k + 1;
      k = first_flag(pi, next, L, lane);
    }
    // ---- results ----
    if (BUILD) {
      if (lane == 0) {
        a.vcnt[q] = nvis;
        if (nvis > a.vlimit) set_err(a.status, DEV_OVERFLOW);
      }
      if (a.out_ids)
        for (int i = lane; i < K; i += 32) {
          a.out_ids[(size_t)q * a.out_stride + i] = pi[i] & ID_MASK;
          if (a.out_dist) a.out_dist[(size_t)q * a.out_stride + i] = pd[i];
        }
    } else {
      for (int i = lane; i < K; i += 32) {
        a.out_ids[(size_t)q * a.out_stride + i] = pi[i] & ID_MASK;
        if (a.out_dist) a.out_dist[(size_t)q * a.out_stride + i] = pd[i];
      }
    }
    // clear this query's visited words for the warp's next query
    __syncwarp();
    for (uint32_t i = lane; i < ntouch; i += 32) vis[touched[i]] = 0u;
    __syncwarp();
  }
  if (!BUILD && lane == 0 && a.counters) {
    atomicAdd(a.counters + 0, dcount);
    atomicAdd(a.counters + 1, hcount);
  }
}

}  // namespace

}  // namespace wv

namespace wv {

size_t search_block_smem(uint32_t d, uint32_t Lmax, uint32_t cap) { return WARPS * warp_smem_bytes(d, Lmax, cap); }

int search_warps_per_block() { return WARPS; }

int search_grid(uint32_t d, uint32_t Lmax, uint32_t cap, int device) {
  size_t smem = search_block_smem(d, Lmax, cap);
  if (cudaFuncSetAttribute(k_search<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess ||
      cudaFuncSetAttribute(k_search<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
    return 0;
  int per_sm = 0, sms = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_search<true>, WARPS * 32, smem) != cudaSuccess)
    return 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) return 0;
  return per_sm * sms;
}

cudaError_t launch_search_exact(const SearchArgs &a, int blocks, cudaStream_t stream) {
  size_t smem = search_block_smem(a.d, a.Lmax, a.cap);
  if (a.vis) k_search<true><<<blocks, WARPS * 32, smem, stream>>>(a);
  else k_search<false><<<blocks, WARPS * 32, smem, stream>>>(a);
  return cudaGetLastError();
}

}  // namespace wv
