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

#include <algorithm>
#include <cstdio>

#include "warp_sort.cuh"
#include "wv_common.cuh"
#include "wv_lowp.cuh"
#include "wv_search.h"
#include "wv_search_common.cuh"

namespace wv {

namespace {


struct WarpSmem {
  uint32_t *hash;  // hcap words: visited set; scratch of the seed sort and the rerank
  float *qv;       // dpad
  float *pd;       // pool distances (pcap), directly followed by
  uint32_t *pi;    // pool ids | FLAG (unexpanded) (pcap)
  float *cd;       // accepted candidates of one expansion, adjacency order (cap)
  uint32_t *ci;    //   (then the candidates' insertion bounds)
  float *sd;       // accepted candidates sorted (cap)
  uint32_t *si;    //   (before that: the expansion's fresh ids)
};

__host__ __device__ inline size_t warp_smem_bytes(uint32_t d, uint32_t Lmax, uint32_t cap, uint32_t hcap) {
  size_t b = 0;
  b += align16((size_t)hash_slots(Lmax, hcap) * 4);
  b += align16(((d + 3) & ~3u) * 4);
  b += 2 * align16((size_t)pool_cap(Lmax) * 4);
  b += 4 * align16(cap * 4);
  return b;
}

__device__ inline WarpSmem carve(uint8_t *p, uint32_t d, uint32_t Lmax, uint32_t cap, uint32_t hcap) {
  WarpSmem s;
  const uint32_t pc = pool_cap(Lmax);
  s.hash = (uint32_t *)p;
  p += align16((size_t)hash_slots(Lmax, hcap) * 4);
  s.qv = (float *)p;
  p += align16(((d + 3) & ~3u) * 4);
  s.pd = (float *)p;
  p += align16((size_t)pc * 4);
  s.pi = (uint32_t *)p;
  p += align16((size_t)pc * 4);
  s.cd = (float *)p;
  p += align16(cap * 4);
  s.ci = (uint32_t *)p;
  p += align16(cap * 4);
  s.sd = (float *)p;
  p += align16(cap * 4);
  s.si = (uint32_t *)p;
  return s;
}

// Orders the L seeds -- (dist, id) pairs in drawn order, stored as DI over the
// pool region -- into the pool exactly as std::sort would, flags set.  A
// bitonic sort on (dist, seed position) gives the stable order, which is
// std::sort's whenever L <= 16 or no two seed distances tie; otherwise the
// warp replays libstdc++'s introsort (warp_sort.cuh) on the drawn order.  The
// hash area is the scratch (the caller clears it afterwards).
__device__ void sort_seeds(WarpSmem &s, int L, uint32_t hwords, uint32_t *gscratch, int lane) {
  const int P = (int)pow2_at_least((uint32_t)L);
  const DI *dv = reinterpret_cast<const DI *>(s.pd);
  float *kd = reinterpret_cast<float *>(s.hash);
  uint32_t *kx = s.hash + P;
  for (int i = lane; i < P; i += 32) {
    kd[i] = i < L ? dv[i].d : __int_as_float(0x7f800000);
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
    for (int i = lane; i < L; i += 32) kx[i] = dv[kx[i]].i;
    __syncwarp();
    for (int i = lane; i < L; i += 32) {
      s.pd[i] = kd[i];
      s.pi[i] = kx[i] | FLAG;
    }
  } else {
    // ties and L > 16: libstdc++ introsort on the drawn order, in place over
    // the pool region (pd and pi are contiguous, 2 * pcap >= 2L words), the
    // partition scratch (2L + 256 words) in the hash area when it fits, else
    // in the warp's global scratch; unpacked through the same place
    __syncwarp();
    DI *tmp = reinterpret_cast<DI *>(s.pd);
    uint32_t *area = hwords >= (uint32_t)(2 * L + 256) ? s.hash : gscratch;
    int *scr = reinterpret_cast<int *>(area);
    warp_std_sort(tmp, L, DILess(), WarpSortScratch{scr, scr + L, scr + 2 * L, scr + 2 * L + 192}, lane);
    __syncwarp();
    DI *cp = reinterpret_cast<DI *>(area);
    for (int i = lane; i < L; i += 32) cp[i] = tmp[i];
    __syncwarp();
    for (int i = lane; i < L; i += 32) {
      s.pd[i] = cp[i].d;
      s.pi[i] = cp[i].i | FLAG;
    }
  }
  __syncwarp();
}


__device__ __forceinline__ float cand_dist(const SearchArgs &a, bool ints, uint32_t my, int cnt, const float *qv,
                                           int lane, float qn) {
  if (a.storage != 0)
    // the norm form unless integer data at d > 128 (where only the
    // difference form stays exact)
    return lowp_rows_dist(LowpRows{a.qbase, a.qscale, (ints && a.d > 128) ? nullptr : a.qnorm, a.storage, a.d}, my,
                          cnt, qv, qn, lane);
  return ints ? batch_dist<true>(a.base, a.d, my, cnt, qv, lane, qn, a.d <= 128 ? a.xnorm : nullptr)
              : batch_dist<false>(a.base, a.d, my, cnt, qv, lane);
}

// SearchEntrySubCentroid's seed distance (component_search_entry.cpp:84-89):
// the row pointer is advanced by one float and d floats are compared from
// there, in the reference's order (one lane per seed; the last row reads the
// zero float that follows the base)
__device__ __forceinline__ float shifted_seed_dist(const float *__restrict__ base, uint32_t d, uint32_t id,
                                                   const float *qv) {
  const float *x = base + (size_t)id * d + 1;
  const float4 *q4 = reinterpret_cast<const float4 *>(qv);
  float acc = 0.f;
  for (uint32_t g = 0; g < (d >> 2); g++) {
    const float4 xv = make_float4(__ldg(x + 4 * g), __ldg(x + 4 * g + 1), __ldg(x + 4 * g + 2), __ldg(x + 4 * g + 3));
    acc = __fadd_rn(acc, group4(xv, q4[g]));
  }
  return acc;
}

// BUILD = false: SearchEntry* + ROUTER_GREEDY (seeds not marked visited,
//   DistCount / HopCount kept, top-K written).
// BUILD = true: CandidateNSG::CandidateInner for base points: seeds are
//   marked visited, and every visited (id, dist) -- the seeds in drawn order,
//   then each newly visited id in visit order -- is appended to the query's
//   visit list (vis, vcap apart, vlimit entries kept, count in vcnt).
template <bool BUILD, int W>
__global__ void __maxnreg__(128) k_search(SearchArgs a) {
  extern __shared__ __align__(16) uint8_t smem[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const size_t wbytes = warp_smem_bytes(a.d, a.Lmax, a.cap, a.hcap);
  WarpSmem s = carve(smem + warp * wbytes, a.d, a.Lmax, a.cap, a.hcap);
  const uint32_t slot = blockIdx.x * W + warp;
  const uint32_t hs = hash_slots(a.Lmax, a.hcap);
  const uint32_t nq = a.nq_dev ? *a.nq_dev : a.nq;
  Visited vis;
  vis.init(s.hash, hs, a.n, a.wide_hash != 0);
  vis.bits = a.visited + (size_t)slot * a.words;
  vis.touched = a.touched + (size_t)slot * a.words;
  unsigned long long dcount = 0, hcount = 0;
  const unsigned lt = (1u << lane) - 1u;
  float *pd = s.pd;
  uint32_t *pi = s.pi;

  while (true) {
    uint32_t q = 0;
    if (lane == 0) {
      q = atomicAdd(a.next_query, 1u);
      if (q < nq && a.order) q = q < a.nq ? a.order[q] : nq;  // (order holds a.nq entries)
    }
    q = __shfl_sync(FULL, q, 0);
    if (q >= nq) break;
    const int L = (int)(a.Lq ? a.Lq[q] : a.L);
    const int K = (int)(a.Kq ? a.Kq[q] : a.K);
    // per-query sizes may come from device memory the host never checked
    if (L < 1 || L > (int)a.Lmax || K < 1 || K > L || (uint32_t)L >= a.n || (a.out_ids && (uint32_t)K > a.out_stride)) {
      if (lane == 0) set_err(a.status, DEV_OVERFLOW);
      continue;
    }
    const float *qsrc = a.queries + (size_t)q * a.d;
    bool qint = true;
    float qn = 0.f;  // |q|^2 (exact on integer data)
    for (uint32_t i = lane; i < a.d; i += 32) {
      const float v = qsrc[i];
      s.qv[i] = v;
      qn = fmaf(v, v, qn);
      qint &= v >= 0.f && v <= 255.f && v == rintf(v);
    }
    for (int o = 16; o > 0; o >>= 1) qn += __shfl_xor_sync(FULL, qn, o);
    // integer base and query: any summation order gives the reference's value
    const bool ints = a.int_exact && a.d <= 256 && __all_sync(FULL, qint);
    // ---- seeds (SearchEntryInner): distances in drawn order, as (dist, id)
    // pairs over the pool region ----
    const uint32_t *seeds = a.seeds + (size_t)q * a.seed_stride;
    uint32_t nvis = 0;
    DI *vis_out = BUILD ? a.vis + (size_t)q * a.vcap : nullptr;
    DI *drawn = reinterpret_cast<DI *>(s.pd);
    __syncwarp();
    for (int b = 0; b < L; b += 32) {
      const int cnt = min(32, L - b);
      uint32_t id = lane < cnt ? seeds[b + lane] : 0u;
      if (lane < cnt && id >= a.n) {
        set_err(a.status, DEV_BAD_ID);
        id = 0;
      }
      const float dist = (!BUILD && a.seed_shift) ? (lane < cnt ? shifted_seed_dist(a.base, a.d, id, s.qv) : 0.f)
                                                 : cand_dist(a, ints, id, cnt, s.qv, lane, qn);
      if (lane < cnt) {
        drawn[b + lane] = DI{dist, id};
        if (BUILD && nvis + lane < a.vlimit) vis_out[nvis + lane] = DI{dist, id};
      }
      nvis += cnt;
    }
    dcount += L;
    __syncwarp();
    sort_seeds(s, L, hs, vis.touched, lane);  // (the touched list is empty between queries)
    vis.clear(lane);  // the seed sort used the hash as scratch
    // CandidateNSG flags its seeds (component_candidate.cpp:21-29); the route
    // leaves them unvisited and records them as seeds
    for (int b = 0; b < L; b += 32) {
      const int i = b + lane;
      const uint32_t id = i < L ? (pi[i] & ID_MASK) : EMPTY;
      // duplicate seeds among lanes: only the first records
      const unsigned same = __match_any_sync(FULL, id);
      const bool first = i < L && (__ffs(same) - 1) == lane;
      if (BUILD) {
        bool sd;
        vis.test_and_set(first, id, lane, sd);
      } else {
        vis.add_seed(first, id);
      }
    }

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
      // the row most likely expanded next (the next unexpanded pool entry,
      // unless this expansion inserts a closer one) is fetched toward L2
      // while this one is processed
      {
        const int g = first_flag(pi, k + 1, L, lane);
        if (g < L && lane == 0) {
          const uint32_t nx = pi[g] & ID_MASK;
          asm volatile("prefetch.global.L2 [%0];" ::"l"(a.gids + (size_t)nx * a.gw));
          asm volatile("prefetch.global.L2 [%0];" ::"l"(a.gdeg + nx));
        }
      }
      // 1) the fresh neighbours, in adjacency order (a seed marked SEEDBIT)
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
        bool was_seed;
        const bool fresh = vis.test_and_set(id != INVALID && leader, id, lane, was_seed);
        const unsigned fm = __ballot_sync(FULL, fresh);
        if (fresh) s.si[nfresh + __popc(fm & lt)] = id | (was_seed ? SEEDBIT : 0u);
        nfresh += __popc(fm);
      }
      __syncwarp();
      // 2) their distances, 3) the accepted ones in adjacency order: closer
      // than the pool's last entry, and not a seed (a seed still closer than
      // the last entry is still in the pool: InsertIntoPool rejects it)
      int ncand = 0;
      // sub-centroid seeds sit in the pool under their shifted distances, so
      // a returning seed is not simply a duplicate: such expansions replay
      // InsertIntoPool one candidate at a time (below)
      const bool shift = !BUILD && a.seed_shift;
      bool replay = false;
      for (uint32_t b = 0; b < nfresh; b += 32) {
        const int cnt = (int)min(32u, nfresh - b);
        const uint32_t raw = lane < cnt ? s.si[b + lane] : 0u;
        const uint32_t my = raw & ID_MASK;
        const float dist = cand_dist(a, ints, my, cnt, s.qv, lane, qn);
        if (BUILD) {
          if (lane < cnt && nvis + lane < a.vlimit) vis_out[nvis + lane] = DI{dist, my};
          nvis += cnt;
        }
        bool acc = lane < cnt && dist < thr && (shift || !(raw & SEEDBIT));
        if (shift) replay |= __any_sync(FULL, acc && ((raw & SEEDBIT) || vis.seed_over));
        if (acc && vis.seed_over && !shift) {
          // a seed the hash could not record: look for the id in the pool
          // (same id, same distance: inside the run of equal distances)
          const int lo = lower_bound_of(pd, L, dist), hi = upper_bound_of(pd, L, dist);
          for (int t = lo; t < hi && acc; t++)
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
      if (ncand > 0 && replay) {
        // InsertIntoPool (include/weavess/index.h), candidate by candidate in
        // adjacency order: skipped unless closer than the current last entry;
        // put in front of a farther first entry unchecked; otherwise placed
        // after its equal-distance run unless its id is in that run, just
        // below it, or just above it
        for (int c = 0; c < ncand; c++) {
          const float dist = s.cd[c];
          const uint32_t id = s.ci[c];
          if (!(dist < pd[L - 1])) continue;
          int pos = 0;
          if (!(pd[0] > dist)) {
            const int ub = upper_bound_of(pd, L, dist), lb = lower_bound_of(pd, L, dist);
            bool hit = false;
            for (int t = max(lb - 1, 0) + lane; t <= ub && t < L; t += 32) hit |= (pi[t] & ID_MASK) == id;
            if (__any_sync(FULL, hit)) continue;
            pos = ub;
          }
          // entries pos..L-2 move up one slot (chunks from the end: each chunk
          // reads its sources before writing, and no chunk writes a slot a
          // later chunk still reads)
          for (int jt = L - 1; jt > pos; jt -= 32) {
            const int j = jt - lane;
            const bool act = j > pos;
            float v = 0.f;
            uint32_t x = 0;
            if (act) {
              v = pd[j - 1];
              x = pi[j - 1];
            }
            __syncwarp();
            if (act) {
              pd[j] = v;
              pi[j] = x;
            }
            __syncwarp();
          }
          if (lane == 0) {
            pd[pos] = dist;
            pi[pos] = id | FLAG;
          }
          __syncwarp();
          nk = min(nk, pos);
        }
      } else if (ncand > 0) {
        // stable order of the candidates by distance (adjacency order on ties)
        for (int c = lane; c < ncand; c += 32) {
          const float dc = s.cd[c];
          int r = 0;
          for (int c2 = 0; c2 < ncand; c2++) {
            const float d2 = s.cd[c2];
            r += (d2 < dc) || (d2 == dc && c2 < c);
          }
          s.sd[r] = dc;
          s.si[r] = s.ci[c];
        }
        __syncwarp();
        // candidate c goes after every pool entry of equal or smaller
        // distance: final position ub[c] + c (ub non-decreasing in c)
        uint32_t *ub = s.ci;
        int mink = L;
        for (int c = lane; c < ncand; c += 32) {
          const int u = upper_bound_of(pd, L, s.sd[c]);
          ub[c] = (uint32_t)u;
          if (u + c < L) mink = min(mink, u + c);
        }
        for (int o = 16; o > 0; o >>= 1) mink = min(mink, __shfl_xor_sync(FULL, mink, o));
        __syncwarp();
        // pool entry j moves down by the number of candidates placed before
        // it (those with ub <= j); in place, from the end, 32 at a time: a
        // chunk is read before it is written and only moves to higher slots
        const int lo = (int)ub[0];
        for (int jt = L; jt > lo; jt -= 32) {
          const int j = jt - 32 + lane;
          const bool act = j >= lo;
          float v = 0.f;
          uint32_t id = 0;
          int pos = L;
          if (act) {
            v = pd[j];
            id = pi[j];
            pos = j + upper_bound_of(ub, ncand, (uint32_t)j);
          }
          __syncwarp();
          if (act && pos < L) {
            pd[pos] = v;
            pi[pos] = id;
          }
          __syncwarp();
        }
        for (int c = lane; c < ncand; c += 32) {
          const int pos = (int)ub[c] + c;
          if (pos < L) {
            pd[pos] = s.sd[c];
            pi[pos] = s.si[c] | FLAG;
          }
        }
        nk = mink;
        __syncwarp();
      }
      const int next = (nk <= k) ? nk : k + 1;
      k = first_flag(pi, next, L, lane);
    }
    // ---- exact FP32 rerank of the final pool (low-precision storage) ----
    if (!BUILD && a.storage != 0 && a.rerank > 0) {
      const int R = min((int)a.rerank, L);
      float *xd = reinterpret_cast<float *>(s.hash);  // the visited set is done with
      uint32_t *xi = s.hash + R;
      for (int b = 0; b < R; b += 32) {
        const int cnt = min(32, R - b);
        const uint32_t id = lane < cnt ? (pi[b + lane] & ID_MASK) : 0u;
        const float ex = ints ? batch_dist<true>(a.base, a.d, id, cnt, s.qv, lane, qn, a.d <= 128 ? a.xnorm : nullptr)
                              : batch_dist<false>(a.base, a.d, id, cnt, s.qv, lane);
        if (lane < cnt) {
          xd[b + lane] = ex;
          xi[b + lane] = id;
        }
      }
      dcount += R;
      __syncwarp();
      // stable order by the exact distance (pool position breaks ties)
      for (int c = lane; c < R; c += 32) {
        const float dc = xd[c];
        int r = 0;
        for (int c2 = 0; c2 < R; c2++) {
          const float d2 = xd[c2];
          r += (d2 < dc) || (d2 == dc && c2 < c);
        }
        pd[r] = dc;  // the head of the pool, re-sorted
        pi[r] = xi[c];
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
    __syncwarp();
    vis.clear(lane);
  }
  if (!BUILD && lane == 0 && a.counters) {
    atomicAdd(a.counters + 0, dcount);
    atomicAdd(a.counters + 1, hcount);
  }
}

template <bool B, int W>
cudaError_t launch_w(const SearchArgs &a, int blocks, size_t smem, cudaStream_t stream) {
  k_search<B, W><<<blocks, W * 32, smem, stream>>>(a);
  return cudaGetLastError();
}

template <bool B, int W>
int max_blocks_w(size_t smem) {
  if (cudaFuncSetAttribute(k_search<B, W>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
    return -1;
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_search<B, W>, W * 32, smem) != cudaSuccess) return -1;
  return per_sm;
}

bool shape_ok(const SearchShape &sh) { return sh.wpb == 1 || sh.wpb == 2 || sh.wpb == 4 || sh.wpb == 8; }

}  // namespace

size_t search_block_smem(uint32_t d, uint32_t Lmax, uint32_t cap, SearchShape sh) {
  return (size_t)sh.wpb * warp_smem_bytes(d, Lmax, cap, sh.hcap);
}
size_t search_block_smem(uint32_t d, uint32_t Lmax, uint32_t cap) {
  return search_block_smem(d, Lmax, cap, SearchShape{});
}

int search_warps_per_block() { return WARPS; }

uint32_t search_hash_slots(uint32_t Lmax, uint32_t want) { return hash_slots(Lmax, want); }
uint32_t search_hash_min(uint32_t Lmax, uint32_t n) {
  const size_t words = ((size_t)n + 31) / 32;
  return words >= 2 * (size_t)Lmax + 256 ? hash_min(Lmax) : hash_cap(Lmax);
}

int search_grid(uint32_t d, uint32_t Lmax, uint32_t cap, int device, SearchShape sh) {
  if (!shape_ok(sh)) return 0;
  const size_t smem = search_block_smem(d, Lmax, cap, sh);
  if (smem > 227 * 1024) return 0;
  int per_sm = -1;
  // (the build variant exists in the default shape only)
  switch (sh.wpb) {
    case 1: per_sm = max_blocks_w<false, 1>(smem); break;
    case 2: per_sm = max_blocks_w<false, 2>(smem); break;
    case 4: per_sm = std::min(max_blocks_w<false, 4>(smem), max_blocks_w<true, 4>(smem)); break;
    default: per_sm = max_blocks_w<false, 8>(smem); break;
  }
  if (per_sm <= 0) {
    cudaGetLastError();
    return 0;
  }
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) return 0;
  return per_sm * sms;
}
int search_grid(uint32_t d, uint32_t Lmax, uint32_t cap, int device) {
  return search_grid(d, Lmax, cap, device, SearchShape{});
}

// the dispatch order of a launch with per-query beams: a counting sort of
// the query indices by beam width, widest first (one block; beams above Lmax
// count as Lmax, the search kernel rejects them).  Within one width the order
// is that of the shared-memory atomics, which no result depends on.
constexpr int ORDER_BUCKETS = 4096, ORDER_THREADS = 1024;
static __global__ void __launch_bounds__(ORDER_THREADS)
    k_order_by_beam(const uint32_t *Lq, uint32_t nq, const uint32_t *nq_dev, uint32_t Lmax, uint32_t *order) {
  __shared__ uint32_t cnt[ORDER_BUCKETS];
  __shared__ uint32_t wsum[ORDER_THREADS / 32];
  const uint32_t t = threadIdx.x, lane = t & 31, w = t >> 5;
  const uint32_t n = nq_dev ? min(*nq_dev, nq) : nq;
  uint32_t shift = 0;
  while ((Lmax >> shift) >= (uint32_t)ORDER_BUCKETS) shift++;
  for (uint32_t i = t; i < ORDER_BUCKETS; i += ORDER_THREADS) cnt[i] = 0;
  __syncthreads();
  // bucket ORDER_BUCKETS - 1 - width: ascending buckets are descending widths
  for (uint32_t q = t; q < n; q += ORDER_THREADS) atomicAdd(&cnt[ORDER_BUCKETS - 1 - (min(Lq[q], Lmax) >> shift)], 1u);
  __syncthreads();
  constexpr int PER = ORDER_BUCKETS / ORDER_THREADS;
  uint32_t v[PER], run = 0;
  for (int i = 0; i < PER; i++) {
    v[i] = cnt[t * PER + i];
    run += v[i];
  }
  uint32_t incl = run;
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(FULL, incl, o);
    if ((int)lane >= o) incl += y;
  }
  if (lane == 31) wsum[w] = incl;
  __syncthreads();
  if (w == 0) {
    uint32_t x = wsum[lane], xi = x;
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(FULL, xi, o);
      if ((int)lane >= o) xi += y;
    }
    wsum[lane] = xi - x;  // exclusive prefix of the warps' totals
  }
  __syncthreads();
  uint32_t off = wsum[w] + incl - run;
  for (int i = 0; i < PER; i++) {
    cnt[t * PER + i] = off;
    off += v[i];
  }
  __syncthreads();
  for (uint32_t q = t; q < n; q += ORDER_THREADS)
    order[atomicAdd(&cnt[ORDER_BUCKETS - 1 - (min(Lq[q], Lmax) >> shift)], 1u)] = q;
}

cudaError_t launch_search(const SearchArgs &a, SearchShape sh, int blocks, cudaStream_t stream) {
  if (!shape_ok(sh)) return cudaErrorInvalidValue;
  if (a.order && a.Lq && !a.vis) {
    k_order_by_beam<<<1, ORDER_THREADS, 0, stream>>>(a.Lq, a.nq, a.nq_dev, a.Lmax, a.order);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  SearchArgs b = a;
  if (!b.Lq || b.vis) b.order = nullptr;
  if (b.parents > 0 && !b.vis && !b.seed_shift) return launch_beam(b, sh, blocks, stream);
  b.hcap = sh.hcap;
  b.wide_hash = sh.wide ? 1 : 0;
  const size_t smem = search_block_smem(a.d, a.Lmax, a.cap, sh);
  if (a.vis) return sh.wpb == WARPS ? launch_w<true, WARPS>(b, blocks, smem, stream) : cudaErrorInvalidValue;
  switch (sh.wpb) {
    case 1: return launch_w<false, 1>(b, blocks, smem, stream);
    case 2: return launch_w<false, 2>(b, blocks, smem, stream);
    case 4: return launch_w<false, 4>(b, blocks, smem, stream);
    default: return launch_w<false, 8>(b, blocks, smem, stream);
  }
}
cudaError_t launch_search_exact(const SearchArgs &a, int blocks, cudaStream_t stream) {
  return launch_search(a, SearchShape{}, blocks, stream);
}

}  // namespace wv
