// Throughput form of the batched greedy beam search.
//
// The exact form (wv_search.cu) follows ComponentSearchRouteGreedy::RouteInner
// (src/component_route.cpp:9-53) expansion by expansion, so its ids and
// DistCount/HopCount equal the reference's.  This kernel answers the same
// question -- the K nearest entries of a beam of width L grown best-first
// over the graph from the query's seeds -- in an order chosen for the GPU,
// for callers that do not need the reference's traversal (the learned entry,
// low-precision candidates, or a caller that sets an expansion width):
//
//  * each step expands the E best unexpanded pool entries at once (E =
//    SearchArgs::parents, 1..4): their rows are read together, the fresh
//    neighbours of all E tested against the visited set, their distances
//    taken in one pass and merged into the pool in one merge, so the
//    per-step latency (row reads, merge) is paid once per E expansions;
//  * candidate distances of bf16 rows (d = 96 or 128), and of FP32 rows of
//    integer data in [0, 255] at d = 128 (converted to bf16 exactly), run on
//    the tensor cores: a warp-wide mma.sync m16n8k16 takes 16 rows x 16
//    dimensions per instruction, rows as the A operand read straight from
//    HBM into registers (each lane 16 contiguous bytes of a row per load, up
//    to 32 rows' loads in flight per warp), the query as the B operand in
//    all eight columns (a hi + lo bf16 split of the FP32 query, so the
//    products keep 16 bits of the query's mantissa; on integer queries the
//    lo part is zero and skipped), FP32 accumulation.  The dot product's
//    dimension order is permuted so that each lane's 16-byte load feeds its
//    fragment registers directly (the order of a dot product's terms does
//    not change it beyond rounding; on integer data every partial sum is an
//    integer below 2^24, so the result is exact).  Distance = |q|^2 + |x|^2 -
//    2 q.x with the stored rows' squared norms;
//  * the seeds are marked visited when they enter the pool (a seed met again
//    as a neighbour is not re-scored), duplicate seeds keep one entry;
//  * the rows of the next step's parents are read before the merge that
//    settles them (the next parents are the E closest of the pool's next
//    unexpanded entries and the sorted candidates), so the row reads of a
//    step overlap the previous merge;
//  * with query_warps = 2 or 4 (a launch-shape dimension; one query per
//    block) member warps take shares of the leader warp's distance passes
//    through a named barrier -- the separately compiled COOP variant; the
//    single-warp variant keeps its distances in registers.
//
// Other row layouts (fp8, other d) use warp-cooperative row distances (a
// warp per row, coalesced; FP32 rows of real-valued data in an order that is
// not the reference's).  The final pool of low-precision candidates is re-ranked in
// FP32 as in the exact form, except bf16 candidates of integer data at
// d <= 128, which are exact already.  DistCount counts every distance taken (seeds
// included), HopCount every expanded node.
#include <cuda_bf16.h>

#include <algorithm>

#include "wv_common.cuh"
#include "wv_lowp.cuh"
#include "wv_search.h"
#include "wv_search_common.cuh"

namespace wv {

namespace {

constexpr uint32_t BEAM_NONE = ID_MASK;  // id of an empty pool slot (never expanded, never output first)

// the distance path a launch compiles in
enum BeamDist : int {
  BD_GENERIC = 0,   // the exact form's warp-cooperative rows (any storage, any d)
  BD_BF16_128 = 1,  // bf16 rows, d = 128, mma
  BD_BF16_96 = 2,   // bf16 rows, d = 96, mma
  BD_F32INT_128 = 3 // FP32 rows of integer data, d = 128, mma (exact)
};

// query fragments in shared memory: for each 32-dimension step t and lane
// column j (lane & 3), the four bf16x2 words (dimensions 32t + 8j + 0..7)
// of the B operand; hi then lo
__host__ __device__ inline uint32_t qfrag_words(uint32_t d) { return (d % 32 == 0 && d <= 256) ? 2 * (d / 32) * 16 : 0; }

struct BeamSmem {
  uint32_t *task;  // a distance pass shared by the query's warps: kind, count, |q|^2 bits, flags
  uint32_t *hash;  // visited set; scratch of the seed sort and the rerank
  float *qv;       // the query (FP32)
  uint32_t *qf;    // query fragments
  float *pd;       // pool distances
  uint32_t *pi;    // pool ids | FLAG (unexpanded)
  float *cd;       // accepted candidates of one step, in visit order
  uint32_t *ci;    //   (then their insertion bounds)
  float *sd;       // accepted candidates sorted
  uint32_t *si;    //   (before that: the step's fresh ids)
};

// shared memory of one query (one group of query_warps warps)
__host__ __device__ inline size_t beam_warp_bytes(uint32_t d, uint32_t Lmax, uint32_t cap, uint32_t hcap) {
  size_t b = 16 + align16((size_t)hash_slots(Lmax, hcap) * 4);
  b += align16(((d + 3) & ~3u) * 4);
  b += align16((size_t)qfrag_words(d) * 4);
  b += 2 * align16((size_t)pool_cap(Lmax) * 4);
  b += 4 * align16((size_t)cap * 4);
  return b;
}

__device__ inline BeamSmem beam_carve(uint8_t *p, uint32_t d, uint32_t Lmax, uint32_t cap, uint32_t hcap) {
  BeamSmem s;
  s.task = (uint32_t *)p;
  p += 16;
  s.hash = (uint32_t *)p;
  p += align16((size_t)hash_slots(Lmax, hcap) * 4);
  s.qv = (float *)p;
  p += align16(((d + 3) & ~3u) * 4);
  s.qf = (uint32_t *)p;
  p += align16((size_t)qfrag_words(d) * 4);
  const uint32_t pc = pool_cap(Lmax);
  s.pd = (float *)p;
  p += align16((size_t)pc * 4);
  s.pi = (uint32_t *)p;
  p += align16((size_t)pc * 4);
  s.cd = (float *)p;
  p += align16((size_t)cap * 4);
  s.ci = (uint32_t *)p;
  p += align16((size_t)cap * 4);
  s.sd = (float *)p;
  p += align16((size_t)cap * 4);
  s.si = (uint32_t *)p;
  return s;
}

__device__ __forceinline__ uint32_t pack_bf16x2(float lo, float hi) {
  const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<const uint32_t *>(&v);
}

// D += A B: m16n8k16, bf16 operands, FP32 accumulators
__device__ __forceinline__ void mma16816(float (&c)[4], uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3,
                                         uint32_t b0, uint32_t b1) {
  asm("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

// the query's B fragments (hi, lo) for T steps of 32 dimensions; returns
// whether the lo part is non-zero somewhere
template <int T>
__device__ bool build_qfrag(const float *qv, uint32_t *qf, int lane) {
  bool lo = false;
  for (int w = lane; w < T * 16; w += 32) {  // word w: step t = w / 16, column j = (w / 4) % 4, pair u = w % 4
    const int t = w >> 4, j = (w >> 2) & 3, u = w & 3;
    const float x0 = qv[32 * t + 8 * j + 2 * u], x1 = qv[32 * t + 8 * j + 2 * u + 1];
    const float h0 = __bfloat162float(__float2bfloat16_rn(x0)), h1 = __bfloat162float(__float2bfloat16_rn(x1));
    const float l0 = x0 - h0, l1 = x1 - h1;
    qf[w] = pack_bf16x2(h0, h1);
    qf[T * 16 + w] = pack_bf16x2(l0, l1);
    lo |= l0 != 0.f || l1 != 0.f;
  }
  return __any_sync(FULL, lo);
}

// Distances of cnt (<= 32) rows -- ids in lanes 0..cnt-1 of `my` -- by mma:
// lane (g = lane / 4, j = lane % 4) reads dimensions 32t + 8j .. +7 of rows
// g and g + 8 of each 16-row group; lane i returns row i's distance
// (|q|^2 + |x|^2 - 2 q.x, never below 0).  F32: the rows are FP32 (integer
// values, converted to bf16 exactly), one 16-row group per pass; else bf16
// rows, two groups (32 rows) per pass.
template <int T, bool F32>
__device__ __forceinline__ float mma_rows(const void *__restrict__ rows, const float *__restrict__ norms,
                                          const uint32_t *qf, bool lo, uint32_t my, int cnt, float qn, int lane) {
  constexpr int NG = F32 ? 1 : 2;
  constexpr uint32_t D = 32 * T;
  const int g = lane >> 2, j = lane & 3;
  const float xn = lane < cnt ? __ldg(norms + my) : 0.f;
  float v = 0.f;
  for (int c0 = 0; c0 < cnt; c0 += 16 * NG) {
    uint4 A[NG][2][T];
#pragma unroll
    for (int gi = 0; gi < NG; gi++) {
#pragma unroll
      for (int h = 0; h < 2; h++) {
        const int r = c0 + gi * 16 + h * 8 + g;
        const uint32_t id = __shfl_sync(FULL, my, r & 31);
        const uint32_t row = r < cnt ? id : 0u;  // rows past cnt read row 0 (in bounds), ignored
        if (F32) {
          const float4 *p = reinterpret_cast<const float4 *>(reinterpret_cast<const float *>(rows) + (size_t)row * D) +
                            2 * j;
#pragma unroll
          for (int t = 0; t < T; t++) {
            const float4 x0 = __ldg(p + 8 * t), x1 = __ldg(p + 8 * t + 1);
            A[gi][h][t] = make_uint4(pack_bf16x2(x0.x, x0.y), pack_bf16x2(x0.z, x0.w), pack_bf16x2(x1.x, x1.y),
                                     pack_bf16x2(x1.z, x1.w));
          }
        } else {
          const uint4 *p = reinterpret_cast<const uint4 *>(reinterpret_cast<const __nv_bfloat16 *>(rows) +
                                                           (size_t)row * D) + j;
#pragma unroll
          for (int t = 0; t < T; t++) A[gi][h][t] = __ldg(p + 4 * t);
        }
      }
    }
    float acc[NG][4];
#pragma unroll
    for (int gi = 0; gi < NG; gi++) acc[gi][0] = acc[gi][1] = acc[gi][2] = acc[gi][3] = 0.f;
#pragma unroll
    for (int t = 0; t < T; t++) {
      const uint4 bh = *reinterpret_cast<const uint4 *>(qf + 16 * t + 4 * j);
#pragma unroll
      for (int gi = 0; gi < NG; gi++) {
        mma16816(acc[gi], A[gi][0][t].x, A[gi][1][t].x, A[gi][0][t].y, A[gi][1][t].y, bh.x, bh.y);
        mma16816(acc[gi], A[gi][0][t].z, A[gi][1][t].z, A[gi][0][t].w, A[gi][1][t].w, bh.z, bh.w);
      }
      if (lo) {
        const uint4 bl = *reinterpret_cast<const uint4 *>(qf + 16 * T + 16 * t + 4 * j);
#pragma unroll
        for (int gi = 0; gi < NG; gi++) {
          mma16816(acc[gi], A[gi][0][t].x, A[gi][1][t].x, A[gi][0][t].y, A[gi][1][t].y, bl.x, bl.y);
          mma16816(acc[gi], A[gi][0][t].z, A[gi][1][t].z, A[gi][0][t].w, A[gi][1][t].w, bl.z, bl.w);
        }
      }
    }
    // lane 4g holds row 16 gi + g in acc[gi][0] and row 16 gi + g + 8 in acc[gi][2]
    const int rr = lane - c0;
    const int src = 4 * (rr & 7);
#pragma unroll
    for (int gi = 0; gi < NG; gi++) {
      const float a0 = __shfl_sync(FULL, acc[gi][0], src), a2 = __shfl_sync(FULL, acc[gi][2], src);
      if (rr >= 16 * gi && rr < 16 * gi + 16) v = ((rr - 16 * gi) & 8) ? a2 : a0;
    }
  }
  return lane < cnt ? fmaxf(qn + xn - 2.f * v, 0.f) : 0.f;
}

template <int DK>
__device__ __forceinline__ float beam_dist(const SearchArgs &a, bool ints, bool lo, const uint32_t *qf, uint32_t my,
                                           int cnt, const float *qv, float qn, int lane) {
  if (DK == BD_BF16_128) return mma_rows<4, false>(a.qbase, a.qnorm, qf, lo, my, cnt, qn, lane);
  if (DK == BD_BF16_96) return mma_rows<3, false>(a.qbase, a.qnorm, qf, lo, my, cnt, qn, lane);
  if (DK == BD_F32INT_128 && ints) return mma_rows<4, true>(a.base, a.xnorm, qf, false, my, cnt, qn, lane);
  if (a.storage != 0)
    return lowp_rows_dist(LowpRows{a.qbase, a.qscale, (ints && a.d > 128) ? nullptr : a.qnorm, a.storage, a.d}, my,
                          cnt, qv, qn, lane);
  // FP32 rows: a warp per row with coalesced loads (the norm form on integer
  // data up to d = 128, else the difference form; the summation order is not
  // the reference's, which the throughput form does not promise)
  return batch_dist<true>(a.base, a.d, my, cnt, qv, lane, qn, (ints && a.d <= 128) ? a.xnorm : nullptr);
}

// stable bitonic sort of the L seeds -- distances pd[i] of ids pi[i] in
// drawn order -- into (pd, pi | FLAG); the hash area is the scratch
__device__ void beam_sort_seeds(const BeamSmem &s, int L, int lane) {
  const int P = (int)pow2_at_least((uint32_t)L);
  float *kd = reinterpret_cast<float *>(s.hash);
  uint32_t *kx = s.hash + P;
  for (int i = lane; i < P; i += 32) {
    kd[i] = i < L ? s.pd[i] : __int_as_float(0x7f800000);
    kx[i] = i;
  }
  __syncwarp();
  for (int k = 2; k <= P; k <<= 1) {
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int i = lane; i < P; i += 32) {
        const int l = i ^ j;
        if (l > i) {
          const bool up = (i & k) == 0;
          const float di = kd[i], dl = kd[l];
          const uint32_t xi = kx[i], xl = kx[l];
          const bool gt = di > dl || (di == dl && xi > xl);
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
  for (int i = lane; i < L; i += 32) kx[i] = s.pi[kx[i]];
  __syncwarp();
  for (int i = lane; i < L; i += 32) {
    s.pd[i] = kd[i];
    s.pi[i] = kx[i] | FLAG;
  }
  __syncwarp();
}

// ---- the warps of one query (query_warps > 1, one query group per block):
// a leader warp runs the search; at each distance pass it posts the task in
// shared memory and named barrier 1 releases the member warps, which take
// 32-row chunks m, m + QW, ... of the pass; a second barrier joins them.
// Kind 0 ends the members' loop (the leader has no more queries).  (A
// constant barrier id keeps the kernel at two barriers per block; an id per
// group made ptxas reserve all sixteen, which cut the resident blocks.)
enum BeamTask : uint32_t { BT_EXIT = 0, BT_FRESH = 1, BT_SEEDS = 2, BT_RERANK = 3 };

__device__ __forceinline__ void group_bar(int grp, int qw) {
  (void)grp;  // (one query group per block when qw > 1)
  asm volatile("bar.sync 1, %0;" ::"r"(qw * 32) : "memory");
}

// this warp's chunks of a distance pass
template <int DK>
__device__ void beam_share(const SearchArgs &a, const BeamSmem &s, uint32_t kind, int n, bool ints, bool lo,
                           float qn, int mem, int qw, int lane) {
  for (int c = mem * 32; c < n; c += qw * 32) {
    const int cnt = min(32, n - c);
    if (kind == BT_RERANK) {
      const int R = n;
      float *xd = reinterpret_cast<float *>(s.hash);
      uint32_t *xi = s.hash + R;
      const uint32_t id = lane < cnt ? (s.pi[c + lane] & ID_MASK) : 0u;
      const float ex = ints ? batch_dist<true>(a.base, a.d, id, cnt, s.qv, lane, qn, a.d <= 128 ? a.xnorm : nullptr)
                            : batch_dist<false>(a.base, a.d, id, cnt, s.qv, lane);
      if (lane < cnt) {
        xd[c + lane] = ex;
        xi[c + lane] = id;
      }
    } else {
      const uint32_t *ids = kind == BT_FRESH ? s.si : s.pi;
      float *out = kind == BT_FRESH ? s.sd : s.pd;
      const uint32_t my = lane < cnt ? ids[c + lane] : 0u;
      const float dist = beam_dist<DK>(a, ints, lo, s.qf, my, cnt, s.qv, qn, lane);
      if (lane < cnt) out[c + lane] = dist;
    }
  }
}

// the leader's side of a distance pass over n items
template <int DK>
__device__ void beam_pass(const SearchArgs &a, const BeamSmem &s, uint32_t kind, int n, bool ints, bool lo, float qn,
                          int grp, int qw, int lane) {
  __syncwarp();
  if (qw > 1) {
    if (lane == 0) {
      s.task[0] = kind;
      s.task[1] = (uint32_t)n;
      s.task[2] = __float_as_uint(qn);
      s.task[3] = (ints ? 1u : 0u) | (lo ? 2u : 0u);
    }
    group_bar(grp, qw);
  }
  beam_share<DK>(a, s, kind, n, ints, lo, qn, 0, qw, lane);
  if (qw > 1) group_bar(grp, qw);
  __syncwarp();
}

// a member warp's loop (until the leader posts BT_EXIT)
template <int DK>
__device__ void beam_member(const SearchArgs &a, const BeamSmem &s, int grp, int mem, int qw, int lane) {
  while (true) {
    group_bar(grp, qw);
    const uint32_t kind = s.task[0];
    if (kind == BT_EXIT) return;
    const int n = (int)s.task[1];
    const float qn = __uint_as_float(s.task[2]);
    const uint32_t fl = s.task[3];
    beam_share<DK>(a, s, kind, n, (fl & 1u) != 0, (fl & 2u) != 0, qn, mem, qw, lane);
    group_bar(grp, qw);
  }
}

// the ncand accepted candidates (cd, ci; visit order) sorted stably by
// distance into (sd, si)
__device__ void beam_sort_cands(const BeamSmem &s, int ncand, int lane) {
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
}

// merges the ncand sorted candidates (sd, si) into the sorted pool of L
// entries, stably (pool entries before equal candidates); returns the
// smallest final position of a candidate (L if none stays)
__device__ int beam_merge(const BeamSmem &s, int L, int ncand, int lane) {
  uint32_t *ub = s.ci;
  int mink = L;
  for (int c = lane; c < ncand; c += 32) {
    const int u = upper_bound_of(s.pd, L, s.sd[c]);
    ub[c] = (uint32_t)u;
    if (u + c < L) mink = min(mink, u + c);
  }
  for (int o = 16; o > 0; o >>= 1) mink = min(mink, __shfl_xor_sync(FULL, mink, o));
  __syncwarp();
  const int lo = (int)ub[0];
  for (int jt = L; jt > lo; jt -= 32) {
    const int j = jt - 32 + lane;
    const bool act = j >= lo;
    float v = 0.f;
    uint32_t id = 0;
    int pos = L;
    if (act) {
      v = s.pd[j];
      id = s.pi[j];
      pos = j + upper_bound_of(ub, ncand, (uint32_t)j);
    }
    __syncwarp();
    if (act && pos < L) {
      s.pd[pos] = v;
      s.pi[pos] = id;
    }
    __syncwarp();
  }
  for (int c = lane; c < ncand; c += 32) {
    const int pos = (int)ub[c] + c;
    if (pos < L) {
      s.pd[pos] = s.sd[c];
      s.pi[pos] = s.si[c] | FLAG;
    }
  }
  __syncwarp();
  return mink;
}

// COOP: the variant with several warps per query (launches with
// query_warps > 1); the single-warp variant keeps its distances in registers
// and uses no named barrier
template <int DK, bool COOP>
__global__ void __maxnreg__(128) k_beam(SearchArgs a) {
  extern __shared__ __align__(16) uint8_t smem[];
  const int W = blockDim.x >> 5;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // query groups of QW warps (the launch keeps W a multiple of QW)
  const int QW = COOP && a.query_warps > 1 ? a.query_warps : 1;
  const int grp = warp / QW, mem = warp % QW;
  const size_t wbytes = beam_warp_bytes(a.d, a.Lmax, a.cap, a.hcap);
  const BeamSmem s = beam_carve(smem + grp * wbytes, a.d, a.Lmax, a.cap, a.hcap);
  if (COOP && mem != 0) {
    beam_member<DK>(a, s, grp, mem, QW, lane);
    return;
  }
  const uint32_t slot = blockIdx.x * (W / QW) + grp;
  const uint32_t hs = hash_slots(a.Lmax, a.hcap);
  const uint32_t nq = a.nq_dev ? *a.nq_dev : a.nq;
  const int E = (int)min(max(a.parents, 1u), BEAM_MAX_PARENTS);
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
      if (q < nq && a.order) q = q < a.nq ? a.order[q] : nq;
    }
    q = __shfl_sync(FULL, q, 0);
    if (q >= nq) break;
    const int L = (int)(a.Lq ? a.Lq[q] : a.L);
    const int K = (int)(a.Kq ? a.Kq[q] : a.K);
    if (L < 1 || L > (int)a.Lmax || K < 1 || K > L || (uint32_t)L >= a.n || (a.out_ids && (uint32_t)K > a.out_stride)) {
      if (lane == 0) set_err(a.status, DEV_OVERFLOW);
      continue;
    }
    const float *qsrc = a.queries + (size_t)q * a.d;
    bool qint = true;
    float qn = 0.f;
    for (uint32_t i = lane; i < a.d; i += 32) {
      const float v = qsrc[i];
      s.qv[i] = v;
      qn = fmaf(v, v, qn);
      qint &= v >= 0.f && v <= 255.f && v == rintf(v);
    }
    for (int o = 16; o > 0; o >>= 1) qn += __shfl_xor_sync(FULL, qn, o);
    __syncwarp();
    const bool ints = a.int_exact && a.d <= 256 && __all_sync(FULL, qint);
    bool lo = false;
    if (DK == BD_BF16_128 || DK == BD_F32INT_128) lo = build_qfrag<4>(s.qv, s.qf, lane);
    if (DK == BD_BF16_96) lo = build_qfrag<3>(s.qv, s.qf, lane);
    __syncwarp();
    // ---- seeds: distances in drawn order, sorted, then entered into the
    // visited set in pool order (a repeated seed keeps its first entry)
    const uint32_t *seeds = a.seeds + (size_t)q * a.seed_stride;
    for (int i = lane; i < L; i += 32) {
      uint32_t id = seeds[i];
      if (id >= a.n) {
        set_err(a.status, DEV_BAD_ID);
        id = 0;
      }
      pi[i] = id;
    }
    beam_pass<DK>(a, s, BT_SEEDS, L, ints, lo, qn, grp, QW, lane);  // pd[i]: distance of pi[i]
    dcount += L;
    beam_sort_seeds(s, L, lane);
    vis.clear(lane);
    int m = 0;  // pool entries kept
    for (int b = 0; b < L; b += 32) {
      const int i = b + lane;
      const float dv = i < L ? pd[i] : 0.f;
      const uint32_t id = i < L ? (pi[i] & ID_MASK) : EMPTY;
      const unsigned same = __match_any_sync(FULL, id);
      const bool first = i < L && (__ffs(same) - 1) == lane;
      bool sd;
      const bool keep = vis.test_and_set(first, id, lane, sd);
      const unsigned km = __ballot_sync(FULL, keep);
      __syncwarp();
      if (keep) {
        const int r = m + __popc(km & lt);
        pd[r] = dv;
        pi[r] = id | FLAG;
      }
      m += __popc(km);
      __syncwarp();
    }
    for (int i = m + lane; i < L; i += 32) {
      pd[i] = __int_as_float(0x7f800000);
      pi[i] = BEAM_NONE;
    }
    __syncwarp();

    // ---- steps of E expansions.  The rows of the next step's parents are
    // read before the merge that settles them: the next parents are the
    // first E unexpanded entries of the merged pool, i.e. the E closest of
    // the pool's next unexpanded entries and the sorted candidates, so their
    // row reads overlap the merge; a step takes the rows read for its
    // parents and reads only those of parents that were not foreseen.
    uint32_t pnode = INVALID, pdeg = 0;  // lane t < npred: foreseen parent t, its degree
    uint32_t phead[BEAM_MAX_PARENTS];    // the first 32 slots of their rows
    int npred = 0;
#pragma unroll
    for (int c = 0; c < BEAM_MAX_PARENTS; c++) phead[c] = INVALID;
    int k = first_flag(pi, 0, L, lane);
    while (k < L) {
      // the first E unexpanded entries from k (lane p < got holds the p-th
      // position), and the next E after them (lane p < pf)
      int got = 0, pf = 0, mypos = -1, pfpos = -1;
      for (int b = k; b < L && pf < E; b += 32) {
        unsigned fm = __ballot_sync(FULL, b + lane < L && (pi[b + lane] & FLAG));
        while (fm && pf < E) {
          const int p = b + __ffs(fm) - 1;
          fm &= fm - 1;
          if (got < E) {
            if (lane == got) mypos = p;
            got++;
          } else {
            if (lane == pf) pfpos = p;
            pf++;
          }
        }
      }
      const int last = __shfl_sync(FULL, mypos, got - 1);
      uint32_t node = 0;
      if (lane < got) node = pi[mypos] & ID_MASK;
      __syncwarp();
      if (lane < got) pi[mypos] = node;  // expanded
      __syncwarp();
      hcount += got;
      const float thr = pd[L - 1];
      // each parent's degree and the first 32 slots of its row (slots past
      // the degree are read and ignored: rows are gw wide), from the rows
      // read ahead when the parent was foreseen
      uint32_t head[BEAM_MAX_PARENTS], dgs[BEAM_MAX_PARENTS];
#pragma unroll
      for (int c = 0; c < BEAM_MAX_PARENTS; c++) {
        head[c] = INVALID;
        dgs[c] = 0;
        if (c < got) {
          const uint32_t nd = __shfl_sync(FULL, node, c);
          const unsigned hit = __ballot_sync(FULL, lane < npred && pnode == nd);
          if (hit) {
            const int m = __ffs(hit) - 1;
            dgs[c] = __shfl_sync(FULL, pdeg, m);
#pragma unroll
            for (int t = 0; t < BEAM_MAX_PARENTS; t++)
              if (t == m) head[c] = phead[t];
          } else {
            dgs[c] = __ldg(a.gdeg + nd);
            head[c] = (uint32_t)lane < a.gw ? __ldg(a.gids + (size_t)nd * a.gw + lane) : INVALID;
          }
        }
      }
      // fresh neighbours, parent by parent in adjacency order
      uint32_t nfresh = 0;
#pragma unroll
      for (int c = 0; c < BEAM_MAX_PARENTS; c++) {
        if (c >= got) break;
        const uint32_t nd = __shfl_sync(FULL, node, c);
        uint32_t dg = dgs[c];
        if (dg > a.gw) {
          if (lane == 0) set_err(a.status, DEV_BAD_ID);
          dg = a.gw;
        }
        for (uint32_t m0 = 0; m0 < dg; m0 += 32) {
          const uint32_t mm = m0 + lane;
          uint32_t id = mm < dg ? (m0 == 0 ? head[c] : __ldg(a.gids + (size_t)nd * a.gw + mm)) : INVALID;
          if (id != INVALID && id >= a.n) {
            set_err(a.status, DEV_BAD_ID);
            id = INVALID;
          }
          const unsigned same = __match_any_sync(FULL, id);
          const bool leader = (__ffs(same) - 1) == lane;
          bool ws;
          const bool fresh = vis.test_and_set(id != INVALID && leader, id, lane, ws);
          const unsigned fm = __ballot_sync(FULL, fresh);
          if (fresh) s.si[nfresh + __popc(fm & lt)] = id;
          nfresh += __popc(fm);
        }
      }
      __syncwarp();
      // distances (in registers, or with several warps per query through sd);
      // the ones closer than the pool's last entry are accepted
      if (COOP && nfresh > 0) beam_pass<DK>(a, s, BT_FRESH, (int)nfresh, ints, lo, qn, grp, QW, lane);
      int ncand = 0;
      for (uint32_t b = 0; b < nfresh; b += 32) {
        const int cnt = (int)min(32u, nfresh - b);
        const uint32_t my = lane < cnt ? s.si[b + lane] : 0u;
        const float dist = COOP ? (lane < cnt ? s.sd[b + lane] : 0.f)
                                : beam_dist<DK>(a, ints, lo, s.qf, my, cnt, s.qv, qn, lane);
        const bool acc = lane < cnt && dist < thr;
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
      if (ncand > 0) beam_sort_cands(s, ncand, lane);
      // foresee the next parents and read their rows
      {
        int i = 0, j = 0;
        npred = 0;
        pnode = INVALID;
#pragma unroll
        for (int t = 0; t < BEAM_MAX_PARENTS; t++) {
          phead[t] = INVALID;
          if (t < E) {
            const int pp = __shfl_sync(FULL, pfpos, i & 31);
            const float dp = i < pf ? pd[pp] : __int_as_float(0x7f800000);
            const float dc = j < ncand ? s.sd[j] : __int_as_float(0x7f800000);
            uint32_t nd = INVALID;
            if (i < pf && (j >= ncand || dp <= dc)) {
              nd = pi[pp] & ID_MASK;
              i++;
            } else if (j < ncand) {
              nd = s.si[j];
              j++;
            }
            if (nd != INVALID) {
              if (lane == t) {
                pnode = nd;
                pdeg = __ldg(a.gdeg + nd);
              }
              phead[t] = (uint32_t)lane < a.gw ? __ldg(a.gids + (size_t)nd * a.gw + lane) : INVALID;
              npred = t + 1;
            }
          }
        }
      }
      __syncwarp();
      int nk = L;
      if (ncand > 0) nk = beam_merge(s, L, ncand, lane);
      k = first_flag(pi, min(nk, last + 1), L, lane);
    }
    // ---- exact FP32 rerank of the final pool (low-precision storage); bf16
    // candidates of integer data at d <= 128 are already exact (integer
    // values, products and partial sums below 2^24), so they keep their order
    if (a.storage != 0 && a.rerank > 0 && !(a.storage == 1 && ints && a.d <= 128)) {
      // (empty slots, +inf, sit at the tail when seeds repeated)
      const int R = min((int)a.rerank, lower_bound_of(pd, L, __int_as_float(0x7f800000)));
      float *xd = reinterpret_cast<float *>(s.hash);
      uint32_t *xi = s.hash + R;
      beam_pass<DK>(a, s, BT_RERANK, R, ints, lo, qn, grp, QW, lane);  // xd, xi
      dcount += R;
      for (int c = lane; c < R; c += 32) {
        const float dc = xd[c];
        int r = 0;
        for (int c2 = 0; c2 < R; c2++) {
          const float d2 = xd[c2];
          r += (d2 < dc) || (d2 == dc && c2 < c);
        }
        pd[r] = dc;
        pi[r] = xi[c];
      }
      __syncwarp();
    }
    if (a.out_ids)
      for (int i = lane; i < K; i += 32) {
        a.out_ids[(size_t)q * a.out_stride + i] = pi[i] & ID_MASK;
        if (a.out_dist) a.out_dist[(size_t)q * a.out_stride + i] = pd[i];
      }
    __syncwarp();
    vis.clear(lane);
  }
  // the member warps leave with the leader
  if (COOP && QW > 1) {
    __syncwarp();
    if (lane == 0) s.task[0] = BT_EXIT;
    group_bar(grp, QW);
  }
  if (lane == 0 && a.counters) {
    atomicAdd(a.counters + 0, dcount);
    atomicAdd(a.counters + 1, hcount);
  }
}

int beam_kind(const SearchArgs &a) {
  if (a.storage == 1 && a.d == 128) return BD_BF16_128;
  if (a.storage == 1 && a.d == 96) return BD_BF16_96;
  if (a.storage == 0 && a.d == 128 && a.int_exact) return BD_F32INT_128;
  return BD_GENERIC;
}

template <int DK, bool COOP>
int beam_blocks_per_sm(int threads, size_t smem) {
  if (cudaFuncSetAttribute(k_beam<DK, COOP>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
    return -1;
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_beam<DK, COOP>, threads, smem) != cudaSuccess)
    return -1;
  return per_sm;
}

template <bool COOP>
int beam_blocks_all(int threads, size_t smem) {
  int per_sm = 1 << 30;
  // every distance path a launch may pick must fit
  for (int v : {beam_blocks_per_sm<BD_GENERIC, COOP>(threads, smem), beam_blocks_per_sm<BD_BF16_128, COOP>(threads, smem),
                beam_blocks_per_sm<BD_BF16_96, COOP>(threads, smem),
                beam_blocks_per_sm<BD_F32INT_128, COOP>(threads, smem)})
    per_sm = std::min(per_sm, v);
  return per_sm;
}

template <bool COOP>
void beam_launch(int dk, int blocks, int threads, size_t smem, cudaStream_t stream, const SearchArgs &b) {
  switch (dk) {
    case BD_BF16_128: k_beam<BD_BF16_128, COOP><<<blocks, threads, smem, stream>>>(b); break;
    case BD_BF16_96: k_beam<BD_BF16_96, COOP><<<blocks, threads, smem, stream>>>(b); break;
    case BD_F32INT_128: k_beam<BD_F32INT_128, COOP><<<blocks, threads, smem, stream>>>(b); break;
    default: k_beam<BD_GENERIC, COOP><<<blocks, threads, smem, stream>>>(b); break;
  }
}

}  // namespace

uint32_t beam_cap(uint32_t gw, uint32_t parents) {
  const uint32_t e = std::min(std::max(parents, 1u), BEAM_MAX_PARENTS);
  return e * gw + 32;
}

bool beam_shape_ok(const SearchShape &sh) {
  // several warps per query: one query group per block
  return (sh.wpb == 1 || sh.wpb == 2 || sh.wpb == 4 || sh.wpb == 8) &&
         (sh.qw == 1 || ((sh.qw == 2 || sh.qw == 4) && sh.wpb == sh.qw));
}

int beam_grid(uint32_t d, uint32_t Lmax, uint32_t gw, uint32_t parents, int device, SearchShape sh) {
  if (!beam_shape_ok(sh)) return 0;
  const size_t smem = (size_t)(sh.wpb / sh.qw) * beam_warp_bytes(d, Lmax, beam_cap(gw, parents), sh.hcap);
  if (smem > 227 * 1024) return 0;
  const int per_sm = sh.qw > 1 ? beam_blocks_all<true>(sh.wpb * 32, smem) : beam_blocks_all<false>(sh.wpb * 32, smem);
  if (per_sm <= 0) {
    cudaGetLastError();
    return 0;
  }
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) return 0;
  return per_sm * sms;
}

cudaError_t launch_beam(const SearchArgs &a, SearchShape sh, int blocks, cudaStream_t stream) {
  if (!beam_shape_ok(sh)) return cudaErrorInvalidValue;
  SearchArgs b = a;
  b.cap = beam_cap(a.gw, a.parents);
  b.hcap = sh.hcap;
  b.wide_hash = sh.wide ? 1 : 0;
  b.query_warps = sh.qw;
  const size_t smem = (size_t)(sh.wpb / sh.qw) * beam_warp_bytes(b.d, b.Lmax, b.cap, b.hcap);
  if (sh.qw > 1) beam_launch<true>(beam_kind(b), blocks, sh.wpb * 32, smem, stream, b);
  else beam_launch<false>(beam_kind(b), blocks, sh.wpb * 32, smem, stream, b);
  return cudaGetLastError();
}

}  // namespace wv
