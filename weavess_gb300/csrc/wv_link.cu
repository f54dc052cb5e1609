// K3/K4/K5: the Vamana, NSG and SSG link (REFINE_VAMANA / REFINE_NSG /
// REFINE_SSG) on GB300.
//
// Replaces ComponentRefineVAMANA::RefineInner / Link / InterInsert
// (src/component_refine.cpp:794-950), ComponentRefineNSG::RefineInner / Link /
// InterInsert (component_refine.cpp:393-541), ComponentRefineSSG::
// RefineInner / Link / InterInsert (component_refine.cpp:550-720),
// ComponentCandidateNSG and ComponentCandidatePropagation2
// (component_candidate.cpp:10-109), ComponentPruneVAMANA / ComponentPruneNSG /
// ComponentPruneSSG (component_prune.cpp:20-122, 245-300) and
// ComponentRefineEntryCentroid (component_entry.cpp:9-92).
// ComponentConnNSGDFS walks on the host (the depth-first walk fixes which
// nodes get linked), with its greedy searches batched on the GPU and taken
// in repair order; ComponentConnSSGDFS (component_conn.cpp:
// 169-225) walks on the GPU (frontier kernels) with the repairs on the device.
//
// Plain form, bit-exact with the single-threaded reference:
//  * candidates: the beam kernel in build mode (seeds flagged, every visit
//    recorded in order), seeds drawn on the host in node order;
//  * prune: one warp per node sorts the visit pool with the warp replica of
//    std::sort, then picks in pool order 32 candidates at a time: each lane
//    tests its candidate against the rows picked before the batch, and a
//    bitmask records which earlier batch members would occlude it, so the
//    sequential pick/skip walk over the batch needs no further distances.
//    VAMANA refills from the skipped items through libstdc++'s heap steps;
//  * InterInsert: sequentially, node n walks its current row and inserts
//    itself into each neighbour's row (dedup, append, or re-prune).  Node n's
//    row at that moment is its pruned row plus the insertions from nodes < n
//    that still listed n -- and those can only be nodes m < n with n in m's
//    PRUNED row.  So nodes are processed by level (level(n) = 1 + max level
//    of such m): all nodes of a level run in parallel, each applying the
//    insertions from lower ids in id order, which gives its row at its turn
//    (kept as a snapshot).  Then every row applies, in id order, the
//    insertions from higher ids, read from their snapshots.  Each warp keeps
//    the vectors' pairwise distances of its row in shared memory, so an
//    insertion costs one new distance column.
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <string>
#include <vector>

#include "warp_sort.cuh"
#include "wv_bfs.cuh"
#include "wv_common.cuh"
#include "wv_link.h"
#include "wv_scan.h"
#include "wv_search.h"
#include "wv_segsort.h"

namespace wv {
namespace {

constexpr int PR_WARPS = 4;
constexpr uint32_t LINK_MAX_R = 63;  // row slots (R + 1) index a 64-bit mask

// exact-order squared L2 of two base rows, read from global memory by one lane
__device__ __forceinline__ float l2g(const float *__restrict__ base, uint32_t d, uint32_t a, uint32_t b) {
  const float4 *x = reinterpret_cast<const float4 *>(base + (size_t)a * d);
  const float4 *y = reinterpret_cast<const float4 *>(base + (size_t)b * d);
  float acc = 0.f;
  const uint32_t d4 = d >> 2;
#pragma unroll 4
  for (uint32_t g = 0; g < d4; g++) acc = __fadd_rn(acc, group4(__ldg(x + g), __ldg(y + g)));
  return acc;
}

struct HeapItem {  // Index::MinHeap<float, SimpleNeighbor>::Item
  float key;
  DI data;
};
struct HeapItemLess {  // Item::operator< is key > other.key
  __device__ bool operator()(const HeapItem &a, const HeapItem &b) const { return a.key > b.key; }
};

// ---------------------------------------------------------------- prune
struct PruneArgs {
  const float *base;
  uint32_t d, n;
  DI *vis;              // chunk x vcap pools (sorted in place)
  const uint32_t *vcnt;
  uint32_t vcap;
  uint32_t n0, cnt;     // nodes [n0, n0 + cnt)
  uint32_t R;
  float alpha;
  uint32_t maxc;        // NSG: C_refine
  float threshold;      // SSG: cos of the angle bound
  const uint32_t *g_ids;  // NSG: the candidate graph (final_graph_)
  const uint32_t *g_deg;
  uint32_t gw;
  int clean;            // Vamana: a short pool is sorted too (clean mode)
  const float *xnorm;   // integer data, d % 32 == 0, d <= 128, R <= 32: the Gram-tile variant's row norms
  int *gscr;            // per warp: 2 * vcap + 256 ints
  HeapItem *hscr;       // per warp: vcap items (VAMANA refill)
  uint32_t *out_ids;    // rows of width R, indexed by node
  float *out_dist;
  uint32_t *out_deg;
  int *status;
};

// the angle test of ComponentPruneSSG / RefineSSG::InterInsert
// (component_prune.cpp:96-104, component_refine.cpp:685-693) with the
// reference's operand types: float sums, a float quotient by 2, and the
// quotient by ::sqrt(double) of the float product taken in double, then
// stored to float
__device__ __forceinline__ bool ssg_occludes(float pd, float rd, float djk, float threshold) {
  const float num = __fmul_rn(__fsub_rn(__fadd_rn(pd, rd), djk), 0.5f);  // x / 2 is exact as x * 0.5
  const double den = __dsqrt_rn((double)__fmul_rn(pd, rd));
  const float cos_ij = __double2float_rn(__ddiv_rn((double)num, den));
  return cos_ij > threshold;
}

// ---- pair distances of a prune batch as Gram tiles (integer data)
// On integer data in [0, 255] with d a multiple of 32 up to 128, the exact
// distance of rows x, y equals |x|^2 + |y|^2 - 2 x.y computed in FP32 (every
// value an integer below 2^24), and x.y comes from BF16 tensor-core tiles
// (integers up to 255 are exact in BF16).  Per warp, shared memory holds the
// rows picked so far and the batch's 32 candidate rows as BF16 (row stride
// an odd multiple of 64 bytes: the fragment loads are free of bank
// conflicts), and the two tiles candidate x picked and candidate x candidate.
constexpr uint32_t PT_ROWS = 32;  // rows picked (R <= 32) and candidates per batch

__host__ __device__ inline uint32_t pt_stride(uint32_t d) { return (d * 2) % 128 == 64 ? d * 2 : d * 2 + 64; }
__host__ __device__ inline size_t pt_warp_bytes(uint32_t d) {
  return 2 * (size_t)PT_ROWS * pt_stride(d) + 2 * (size_t)PT_ROWS * PT_ROWS * 4 + PT_ROWS * 4;
}

__device__ __forceinline__ uint32_t pt_pack(float lo, float hi) {
  const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<const uint32_t *>(&v);
}

// row `id` of the FP32 base into slot `r` of a BF16 row area (16 lanes per row)
__device__ __forceinline__ void pt_stage_row(uint8_t *area, uint32_t stride, uint32_t r, const float *base,
                                             uint32_t d, uint32_t id, int sub) {
  for (uint32_t k = (uint32_t)sub * 8; k < d; k += 16 * 8) {
    const float4 *src = reinterpret_cast<const float4 *>(base + (size_t)id * d + k);
    const float4 x0 = __ldg(src), x1 = __ldg(src + 1);
    *reinterpret_cast<uint4 *>(area + (size_t)r * stride + k * 2) =
        make_uint4(pt_pack(x0.x, x0.y), pt_pack(x0.z, x0.w), pt_pack(x1.x, x1.y), pt_pack(x1.z, x1.w));
  }
}

__device__ __forceinline__ void pt_mma(float (&c)[4], uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3, uint32_t b0,
                                       uint32_t b1) {
  asm("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

// G[x][y] = X_x . Y_y for the 32 rows of X and the first ncol (a multiple of
// 8, <= 32) rows of Y; lane (g, j) loads dimensions 32t + 8j .. +7 of its
// rows (the dot product's terms permuted alike in A and B)
__device__ void pt_gram(const uint8_t *X, const uint8_t *Y, uint32_t stride, uint32_t d, uint32_t ncol, float *G,
                        int lane) {
  const int g = lane >> 2, j = lane & 3;
  const uint32_t T = d / 32;
  for (int gi = 0; gi < 2; gi++) {
    for (uint32_t nt = 0; nt * 8 < ncol; nt++) {
      float acc[4] = {0.f, 0.f, 0.f, 0.f};
      for (uint32_t t = 0; t < T; t++) {
        const uint32_t off = (32 * t + 8 * j) * 2;
        const uint4 a0 = *reinterpret_cast<const uint4 *>(X + (size_t)(16 * gi + g) * stride + off);
        const uint4 a1 = *reinterpret_cast<const uint4 *>(X + (size_t)(16 * gi + g + 8) * stride + off);
        const uint4 b = *reinterpret_cast<const uint4 *>(Y + (size_t)(8 * nt + g) * stride + off);
        pt_mma(acc, a0.x, a1.x, a0.y, a1.y, b.x, b.y);
        pt_mma(acc, a0.z, a1.z, a0.w, a1.w, b.z, b.w);
      }
      // lane (g, j): rows 16 gi + g (c0, c1) and + 8 (c2, c3), columns 8 nt + 2j, + 1
      float *r0 = G + (size_t)(16 * gi + g) * PT_ROWS + 8 * nt + 2 * j;
      float *r1 = G + (size_t)(16 * gi + g + 8) * PT_ROWS + 8 * nt + 2 * j;
      r0[0] = acc[0];
      r0[1] = acc[1];
      r1[0] = acc[2];
      r1[1] = acc[3];
    }
  }
}

// MODE: 0 Vamana, 1 NSG, 2 SSG.  TC: the pair distances from Gram tiles
// (integer data, d a multiple of 32 up to 128, R <= 32; same values)
template <int MODE, bool TC>
__global__ void __launch_bounds__(PR_WARPS * 32) k_prune(PruneArgs a) {
  constexpr bool NSG = MODE != 0;  // the NSG-style walk (SSG shares it with the angle test)
  __shared__ uint32_t pk_id[PR_WARPS][LINK_MAX_R];
  __shared__ float pk_d[PR_WARPS][LINK_MAX_R];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t gwarp = blockIdx.x * PR_WARPS + warp, nwarps = gridDim.x * PR_WARPS;
  int *scr = a.gscr + (size_t)gwarp * (2 * a.vcap + 256);
  HeapItem *heap = a.hscr + (size_t)gwarp * a.vcap;
  uint32_t *pid = pk_id[warp];
  float *pd = pk_d[warp];
  // TC: per warp, the picked rows, the batch's rows, the two tiles, the
  // picked rows' norms
  extern __shared__ __align__(16) uint8_t pt_smem[];
  const uint32_t pst = pt_stride(a.d);
  uint8_t *prow = pt_smem + (TC ? (size_t)warp * pt_warp_bytes(a.d) : 0);
  uint8_t *crow = prow + (size_t)PT_ROWS * pst;
  float *G1 = reinterpret_cast<float *>(crow + (size_t)PT_ROWS * pst);
  float *G2 = G1 + PT_ROWS * PT_ROWS;
  float *pxn = G2 + PT_ROWS * PT_ROWS;
  for (uint32_t qi = gwarp; qi < a.cnt; qi += nwarps) {
    const uint32_t node = a.n0 + qi;
    DI *pool = a.vis + (size_t)qi * a.vcap;
    uint32_t m = min(a.vcnt[qi], a.vcap);
    uint32_t *oid = a.out_ids + (size_t)node * a.R;
    float *od = a.out_dist + (size_t)node * a.R;
    // clean Vamana (this library's clean build mode): the pool is the visited
    // set plus the node's own row, as DiskANN's RobustPrune prunes V u
    // N_out(p); the node itself and repeated ids are dropped, not skipped
    const bool cv = !NSG && a.clean;
    if (NSG || cv) {
      // the node's own row joins the pool, distances recomputed
      // (component_prune.cpp:26-34); vcap leaves room for it
      const uint32_t deg = min(a.g_deg[node], a.gw);
      for (uint32_t j = lane; j < deg; j += 32) {
        uint32_t id = a.g_ids[(size_t)node * a.gw + j];
        if (id >= a.n) {
          set_err(a.status, DEV_BAD_ID);
          id = 0;
        }
        if (m + j < a.vcap) pool[m + j] = DI{l2g(a.base, a.d, node, id), id};
      }
      if (m + deg > a.vcap) set_err(a.status, DEV_OVERFLOW);
      m = min(m + deg, a.vcap);
      __syncwarp();
    }
    if (!NSG && m <= a.R && !a.clean) {  // PruneVAMANA keeps a short pool unsorted
      for (uint32_t j = lane; j < m; j += 32) {
        oid[j] = pool[j].i;
        od[j] = pool[j].d;
      }
      if (lane == 0) a.out_deg[node] = m;
      continue;
    }
    if (m == 0) {
      if (lane == 0) a.out_deg[node] = 0;
      continue;
    }
    warp_std_sort(pool, (int)m, DILess(), WarpSortScratch{scr, scr + a.vcap, scr + 2 * a.vcap,
                                                          scr + 2 * a.vcap + 192}, lane);
    uint32_t np = 0;   // picked
    uint32_t ex = 0;   // next pool index to examine
    uint32_t end = m;  // examination bound
    uint32_t nskip = 0;
    if (NSG) {
      // start skips the node itself at position 0; pool[start] is taken as is
      uint32_t start = pool[0].i == node ? 1u : 0u;
      if (start >= m) {
        if (lane == 0) a.out_deg[node] = 0;
        continue;
      }
      if (lane == 0) {
        pid[0] = pool[start].i;
        pd[0] = pool[start].d;
      }
      np = 1;
      ex = start + 1;
      end = MODE == 2 ? m : min(m, a.maxc);  // SSG examines the whole pool
      __syncwarp();
      if (TC) {
        const uint32_t id0 = pid[0];
        if (lane < 16) pt_stage_row(prow, pst, 0, a.base, a.d, id0, lane);
        if (lane == 0) pxn[0] = __ldg(a.xnorm + id0);
        __syncwarp();
      }
    }
    bool done = np >= a.R;
    while (!done && ex < end) {
      const uint32_t cnt = min(32u, end - ex);
      DI cand = lane < (int)cnt ? pool[ex + lane] : DI{0.f, 0u};
      float cxn = 0.f;
      if (TC) {
        // the batch's rows (rows past cnt: row 0 of the base, never read) and
        // the tiles candidate x picked-before-the-batch, candidate x candidate
        for (uint32_t r = lane >> 4; r < PT_ROWS; r += 2) {
          const uint32_t id = __shfl_sync(0xffffffffu, cand.i, r);
          pt_stage_row(crow, pst, r, a.base, a.d, r < cnt ? id : 0u, lane & 15);
        }
        cxn = lane < (int)cnt ? __ldg(a.xnorm + cand.i) : 0.f;
        __syncwarp();
        if (np > 0) pt_gram(crow, prow, pst, a.d, (np + 7) & ~7u, G1, lane);
        pt_gram(crow, crow, pst, a.d, (cnt + 7) & ~7u, G2, lane);
        __syncwarp();
      }
      // against the rows picked before this batch
      bool s1 = false, dup1 = false;  // dup1 (clean Vamana): the node itself or an id picked before
      if (lane < (int)cnt) {
        if (cv) {
          dup1 = cand.i == node;
          for (uint32_t j = 0; j < np && !dup1; j++) dup1 = pid[j] == cand.i;
          s1 = dup1;
        }
        for (uint32_t j = 0; j < np && !s1; j++) {
          if (NSG && pid[j] == cand.i) s1 = true;
          else {
            float dd = TC ? (pxn[j] + cxn) - 2.f * G1[lane * PT_ROWS + j] : l2g(a.base, a.d, pid[j], cand.i);
            s1 = MODE == 2 ? ssg_occludes(cand.d, pd[j], dd, a.threshold)
                           : (NSG ? (dd < cand.d) : (__fmul_rn(a.alpha, dd) < cand.d));
          }
        }
      }
      // which earlier batch members would occlude this one
      uint32_t occl = 0;
      uint32_t dupo = 0;  // clean Vamana: earlier batch members with the same id
      for (int b = 0; b < (int)cnt; b++) {
        const uint32_t bid = __shfl_sync(FULL, cand.i, b);
        const float bd = __shfl_sync(FULL, cand.d, b);
        const float bxn = TC ? __shfl_sync(FULL, cxn, b) : 0.f;
        if (b < lane && lane < (int)cnt) {
          bool hit;
          if ((NSG || cv) && bid == cand.i) {
            hit = true;
            if (cv) dupo |= 1u << b;
          } else {
            float dd = TC ? (bxn + cxn) - 2.f * G2[lane * PT_ROWS + b] : l2g(a.base, a.d, bid, cand.i);
            hit = MODE == 2 ? ssg_occludes(cand.d, bd, dd, a.threshold)
                            : (NSG ? (dd < cand.d) : (__fmul_rn(a.alpha, dd) < cand.d));
          }
          if (hit) occl |= 1u << b;
        }
      }
      // the sequential walk of the reference over this batch
      const uint32_t np0 = np;
      uint32_t pm = 0;
      uint32_t stop = cnt;
      for (int b = 0; b < (int)cnt; b++) {
        const bool sb = __shfl_sync(FULL, s1, b);
        const uint32_t ob = __shfl_sync(FULL, occl, b);
        const bool db = __shfl_sync(FULL, dup1, b) || (__shfl_sync(FULL, dupo, b) & pm);
        const DI cb = DI{__shfl_sync(FULL, cand.d, b), __shfl_sync(FULL, cand.i, b)};
        const bool skip = sb || (ob & pm);
        if (!skip) {
          pm |= 1u << b;
          if (lane == 0) {
            pid[np] = cb.i;
            pd[np] = cb.d;
          }
          np++;
          if (np == a.R) {
            stop = b + 1;
            done = true;
            break;
          }
        } else if (!NSG && !db) {
          if (lane == 0) heap[nskip] = HeapItem{cb.d, cb};
          nskip++;
        }
      }
      __syncwarp();
      if (TC) {
        // the rows picked in this batch join the picked rows (and norms)
        uint32_t k = np0;
        for (uint32_t mm = pm; mm; mm &= mm - 1, k++) {
          const int b = __ffs(mm) - 1;
          const float bxn = __shfl_sync(FULL, cxn, b);
          for (uint32_t o = (uint32_t)lane * 16; o < a.d * 2; o += 32 * 16)
            *reinterpret_cast<uint4 *>(prow + (size_t)k * pst + o) =
                *reinterpret_cast<const uint4 *>(crow + (size_t)b * pst + o);
          if (lane == 0) pxn[k] = bxn;
        }
        __syncwarp();
      }
      ex += stop;
    }
    if (!NSG && np < a.R && nskip > 0) {
      // refill from the skipped min-heap (component_prune.cpp:276-279)
      if (lane == 0) {
        for (uint32_t k = 1; k <= nskip; k++) stl::push_heap(heap, (int)k, HeapItemLess());
        uint32_t hs = nskip;
        while (np < a.R && hs > 0) {
          bool again = false;  // clean Vamana: an id skipped twice is taken once
          for (uint32_t j = 0; cv && j < np && !again; j++) again = pid[j] == heap[0].data.i;
          if (!again) {
            pid[np] = heap[0].data.i;
            pd[np] = heap[0].data.d;
            np++;
          }
          stl::pop_heap(heap, (int)hs, HeapItemLess());
          hs--;
        }
      }
      np = __shfl_sync(FULL, np, 0);
      __syncwarp();
    }
    for (uint32_t j = lane; j < np; j += 32) {
      oid[j] = pid[j];
      od[j] = pd[j];
    }
    if (lane == 0) a.out_deg[node] = np;
    __syncwarp();
  }
}

// ---------------------------------------------------------------- InterInsert
struct IIArgs {
  const float *base;
  uint32_t d, n, R;
  float alpha;
  int vamana;
  int clean;               // Vamana re-prune closest first, each candidate against its own distance
  int ssg;                 // SSG re-prune: angle test, sentinel after a short result
  int ints;                // integer rows in [0, 255], d <= 256: any summation order is exact
  float threshold;
  const uint32_t *p_ids;   // pruned rows (width R)
  const float *p_dist;
  const uint32_t *p_deg;
  uint32_t *s_ids;         // rows at each node's turn (width R)
  float *s_dist;
  uint32_t *s_deg;
  uint32_t *f_ids;         // final rows (width R)
  float *f_dist;
  uint32_t *f_deg;
  const uint32_t *nodes;   // nodes of this launch
  uint32_t nn;
  const unsigned long long *req;  // per target: (sender << 32 | index) sorted
  const uint32_t *req_off, *req_cnt;
  int *status;
};

constexpr int II_WARPS = 4;
constexpr int II_SLOTS = LINK_MAX_R + 1;

struct Ent3 {
  float d;
  uint32_t i;
  uint32_t slot;
};
struct Ent3Less {
  __device__ bool operator()(const Ent3 &a, const Ent3 &b) const { return a.d < b.d; }
};
struct HeapIdx {  // MinHeap item of the re-prune: key and temp index
  float key;
  uint32_t k;
};
struct HeapIdxLess {
  __device__ bool operator()(const HeapIdx &a, const HeapIdx &b) const { return a.key > b.key; }
};

// per-warp state: the row (with the slot holding each entry's vector), the
// re-prune scratch, and -- in the dynamic tail -- the pairwise distances of
// the slot vectors (S x S, S = R + 1) and the vectors themselves (S rows)
struct IIWarp {
  Ent3 row[II_SLOTS];
  Ent3 tmp[II_SLOTS];
  uint32_t sid[II_SLOTS];  // id held by each slot
  uint32_t res[II_SLOTS];
  HeapIdx heap[II_SLOTS];
  float *D;                // S x S
  float *V;                // S x vs floats, or null: distances from global memory
};

__host__ __device__ inline size_t ii_warp_bytes(uint32_t R, uint32_t vs) {
  const size_t S = R + 1;
  return ((sizeof(IIWarp) + 15) & ~size_t(15)) + ((S * S * 4 + 15) & ~size_t(15)) + S * vs * 4;
}

__device__ inline IIWarp &ii_carve(uint8_t *smem, int warp, uint32_t R, uint32_t vs) {
  uint8_t *p = smem + (size_t)warp * ii_warp_bytes(R, vs);
  IIWarp &w = *reinterpret_cast<IIWarp *>(p);
  p += (sizeof(IIWarp) + 15) & ~size_t(15);
  w.D = reinterpret_cast<float *>(p);
  p += ((size_t)(R + 1) * (R + 1) * 4 + 15) & ~size_t(15);
  w.V = vs ? reinterpret_cast<float *>(p) : nullptr;
  return w;
}

// copies base row `id` into vector slot f (one warp, 16-byte pieces)
__device__ __forceinline__ void ii_stage(const IIArgs &a, IIWarp &w, uint32_t vs, uint32_t f, uint32_t id, int lane) {
  if (!w.V) return;
  const float4 *src = reinterpret_cast<const float4 *>(a.base + (size_t)id * a.d);
  float4 *dst = reinterpret_cast<float4 *>(w.V + (size_t)f * vs);
  for (uint32_t k = lane; k < (a.d >> 2); k += 32) dst[k] = __ldg(src + k);
}

// exact-order distance between the vectors of slots x and y
__device__ __forceinline__ float ii_dist(const IIArgs &a, const IIWarp &w, uint32_t vs, uint32_t x, uint32_t y) {
  if (!w.V) return l2g(a.base, a.d, w.sid[x], w.sid[y]);
  const float4 *p = reinterpret_cast<const float4 *>(w.V + (size_t)x * vs);
  const float4 *q = reinterpret_cast<const float4 *>(w.V + (size_t)y * vs);
  const uint32_t d4 = a.d >> 2;
  if (a.ints) {
    // every partial sum is an integer below 2^24, so four chains give the
    // exact-order value
    float s0 = 0.f, s1 = 0.f, s2 = 0.f, s3 = 0.f;
    uint32_t g = 0;
    for (; g + 4 <= d4; g += 4) {
      s0 = __fadd_rn(s0, group4(p[g], q[g]));
      s1 = __fadd_rn(s1, group4(p[g + 1], q[g + 1]));
      s2 = __fadd_rn(s2, group4(p[g + 2], q[g + 2]));
      s3 = __fadd_rn(s3, group4(p[g + 3], q[g + 3]));
    }
    for (; g < d4; g++) s0 = __fadd_rn(s0, group4(p[g], q[g]));
    return __fadd_rn(__fadd_rn(s0, s1), __fadd_rn(s2, s3));
  }
  float acc = 0.f;
#pragma unroll 4
  for (uint32_t g = 0; g < d4; g++) acc = __fadd_rn(acc, group4(p[g], q[g]));
  return acc;
}

// gives row entry j (slot INVALID) a free slot, its vector and its distance
// column to the other slotted entries (dvalid rows only)
__device__ void ii_slot_entry(const IIArgs &a, IIWarp &w, uint32_t vs, uint32_t rs, uint32_t j, int lane) {
  const uint32_t S = a.R + 1;
  unsigned long long used = 0;
  for (uint32_t t = 0; t < rs; t++)
    if (t != j) used |= 1ull << w.row[t].slot;
  const uint32_t f = __ffsll(~used) - 1;
  if (lane == 0) {
    w.row[j].slot = f;
    w.sid[f] = w.row[j].i;
  }
  __syncwarp();
  ii_stage(a, w, vs, f, w.row[j].i, lane);
  __syncwarp();
  for (uint32_t t = lane; t < rs; t += 32) {
    if (t == j) continue;
    const uint32_t o = w.row[t].slot;
    const float dd = ii_dist(a, w, vs, o, f);
    w.D[f * S + o] = dd;
    w.D[o * S + f] = dd;
  }
  __syncwarp();
}

// applies "insert `s` (distance dist, sender index i) into this row" exactly
// as InterInsert does to des_pool (component_refine.cpp:484-540 / 884-949).
// `kept` (NSG): the last re-prune took R entries with distinct keys, so the
// row is sorted and no entry is occluded by a nearer one.  Re-pruning such a
// row with s gives the same row when s ties no key and is either farther
// than every entry (the walk is full before it reaches s) or occluded by a
// nearer entry (s is skipped and every entry is taken again), so those
// insertions stop early.
__device__ void ii_apply(const IIArgs &a, IIWarp &w, uint32_t vs, uint32_t &rs, bool &dvalid, bool &kept, uint32_t s,
                         float dist, uint32_t i, int lane) {
  bool dup = false;
  for (uint32_t j = lane; j < rs; j += 32) dup |= w.row[j].i == s;
  if (__any_sync(FULL, dup)) return;
  const uint32_t R = a.R, S = R + 1;
  if (rs + 1 <= R) {  // room: append at the sentinel
    if (lane == 0) w.row[rs] = Ent3{dist, s, INVALID};
    __syncwarp();
    if (dvalid) ii_slot_entry(a, w, vs, rs + 1, rs, lane);
    rs++;
    kept = false;
    return;
  }
  const bool nsg = !a.vamana && !a.ssg;
  bool tie_s = false;
  if (nsg && kept) {
    bool far = true;
    for (uint32_t j = lane; j < rs; j += 32) {
      const float rd = w.row[j].d;
      tie_s |= rd == dist;
      far &= rd < dist;
    }
    tie_s = __any_sync(FULL, tie_s);
    if (!tie_s && __all_sync(FULL, far)) return;
  }
  // a re-prune needs the pairwise distances of row + s
  if (!dvalid) {
    for (uint32_t j = lane; j < rs; j += 32) {
      w.row[j].slot = j;
      w.sid[j] = w.row[j].i;
    }
    __syncwarp();
    for (uint32_t j = 0; j < rs; j++) ii_stage(a, w, vs, j, w.row[j].i, lane);
    __syncwarp();
    for (uint32_t p = lane; p < rs * rs; p += 32) {
      const uint32_t x = p / rs, y = p % rs;
      if (x < y) {
        const float dd = ii_dist(a, w, vs, x, y);
        w.D[x * S + y] = dd;
        w.D[y * S + x] = dd;
      }
    }
    dvalid = true;
    __syncwarp();
  }
  // s takes the free slot (the row holds at most R of the R + 1 slots)
  if (lane == 0) w.row[rs] = Ent3{dist, s, INVALID};
  __syncwarp();
  ii_slot_entry(a, w, vs, rs + 1, rs, lane);
  if (nsg && kept && !tie_s) {
    const uint32_t fs = w.row[rs].slot;
    bool occ = false;
    for (uint32_t j = lane; j < rs; j += 32) {
      const Ent3 r = w.row[j];
      occ |= r.d < dist && w.D[r.slot * S + fs] < dist;
    }
    if (__any_sync(FULL, occ)) return;
  }
  const uint32_t T = rs + 1;
  bool any_tie = false;
  // std::sort(temp_pool) (component_refine.cpp:503 / 901): with distinct keys
  // the sorted array is unique, so each lane places its entries by rank;
  // tied keys take the one-lane replica of std::sort
  {
    const Ent3 e0 = lane < T ? w.row[lane] : Ent3{0.f, 0u, 0u};
    const Ent3 e1 = lane + 32 < T ? w.row[lane + 32] : Ent3{0.f, 0u, 0u};
    uint32_t r0 = 0, r1 = 0;
    bool tie = false;
    for (uint32_t t = 0; t < T; t++) {
      const float kt = w.row[t].d;
      r0 += kt < e0.d;
      r1 += kt < e1.d;
      tie |= (lane < T && t != lane && kt == e0.d) || (lane + 32 < T && t != lane + 32 && kt == e1.d);
    }
    any_tie = __any_sync(FULL, tie);
    if (any_tie) {
      for (uint32_t j = lane; j < T; j += 32) w.tmp[j] = w.row[j];
      __syncwarp();
      if (lane == 0) stl::sort(w.tmp, (int)T, Ent3Less());
    } else {
      if (lane < T) w.tmp[r0] = e0;
      if (lane + 32 < T) w.tmp[r1] = e1;
    }
    __syncwarp();
  }
  uint32_t nres = 0;
  if (a.vamana) {
    // compat: farthest first, every candidate against temp_pool[i].d (the
    // outer index, refine.cpp:907); clean: closest first, each candidate
    // against its own distance (the rule of PruneVAMANA)
    uint32_t nskip = 0;
    for (int kk = 0; kk < (int)T; kk++) {
      const int k = a.clean ? kk : (int)T - 1 - kk;
      const float cur = a.clean ? w.tmp[k].d : w.tmp[i].d;
      const uint32_t ks = w.tmp[k].slot;
      bool hit = false;
      for (uint32_t j = lane; j < nres; j += 32) hit |= __fmul_rn(a.alpha, w.D[w.tmp[w.res[j]].slot * S + ks]) < cur;
      const bool skip = __any_sync(FULL, hit);
      if (!skip) {
        if (lane == 0) w.res[nres] = (uint32_t)k;
        nres++;
      } else {
        if (lane == 0) {
          w.heap[nskip] = HeapIdx{cur, (uint32_t)k};
          stl::push_heap(w.heap, (int)(nskip + 1), HeapIdxLess());
        }
        nskip++;
      }
      __syncwarp();
      if (nres == R) break;
    }
    if (nres < R && nskip > 0) {
      if (lane == 0) {
        uint32_t hs = nskip;
        while (nres < R && hs > 0) {
          w.res[nres++] = w.heap[0].k;
          stl::pop_heap(w.heap, (int)hs, HeapIdxLess());
          hs--;
        }
      }
      nres = __shfl_sync(FULL, nres, 0);
      __syncwarp();
    }
  } else if (!a.ssg) {
    // NSG (component_refine.cpp:505-526): bit r of o0 / o1 is set when sorted
    // entry r < p occludes this lane's entry p = lane / lane + 32 (the same
    // id, or nearer to p than p is to the node); the walk then takes entry 0
    // and each later entry that no taken entry occludes, up to R
    const Ent3 p0 = lane < T ? w.tmp[lane] : Ent3{0.f, 0u, 0u};
    const Ent3 p1 = lane + 32 < T ? w.tmp[lane + 32] : Ent3{0.f, 0u, 0u};
    unsigned long long o0 = 0, o1 = 0;
    for (uint32_t r = 0; r + 1 < T; r++) {
      const Ent3 q = w.tmp[r];
      if (r < lane && lane < T && (q.i == p0.i || w.D[q.slot * S + p0.slot] < p0.d)) o0 |= 1ull << r;
      if (r < lane + 32 && lane + 32 < T && (q.i == p1.i || w.D[q.slot * S + p1.slot] < p1.d)) o1 |= 1ull << r;
    }
    unsigned long long taken = 1ull;
    nres = 1;
    for (uint32_t st = 1; nres < R && st < T; st++) {
      const unsigned long long o = st < 32 ? __shfl_sync(FULL, o0, st) : __shfl_sync(FULL, o1, st - 32);
      if (!(o & taken)) {
        taken |= 1ull << st;
        nres++;
      }
    }
    if (lane < T && ((taken >> lane) & 1ull)) w.res[__popcll(taken & ((1ull << lane) - 1ull))] = lane;
    if (lane + 32 < T && ((taken >> (lane + 32)) & 1ull))
      w.res[__popcll(taken & ((1ull << (lane + 32)) - 1ull))] = lane + 32;
    __syncwarp();
  } else {
    if (lane == 0) w.res[0] = 0;
    nres = 1;
    __syncwarp();
    for (uint32_t st = 1; nres < R && st < T; st++) {
      const Ent3 p = w.tmp[st];
      bool occ = false;
      for (uint32_t j = lane; j < nres; j += 32) {
        const Ent3 r = w.tmp[w.res[j]];
        const float djk = w.D[r.slot * S + p.slot];
        occ |= (r.i == p.i) || (a.ssg ? ssg_occludes(p.d, r.d, djk, a.threshold) : (djk < p.d));
      }
      if (!__any_sync(FULL, occ)) {
        if (lane == 0) w.res[nres] = st;
        nres++;
      }
      __syncwarp();
    }
  }
  // des_pool[t] = result[t] for t < result.size() (refine.cpp:527-530,
  // 943-946, 706-712).  Vamana results always hold R entries; an NSG result
  // may be shorter and then, with no sentinel written, the old entries at
  // positions result.size()..R-1 stay in the row; SSG writes the sentinel.
  for (uint32_t j = lane; j < nres; j += 32) w.row[j] = w.tmp[w.res[j]];
  __syncwarp();
  kept = nsg && nres == R && !any_tie;
  if (a.vamana || a.ssg) rs = nres;  // SSG writes a sentinel after a short result
  __syncwarp();
}

__device__ void ii_load_row(IIWarp &w, const uint32_t *ids, const float *dist, uint32_t deg, int lane) {
  for (uint32_t j = lane; j < deg; j += 32) w.row[j] = Ent3{dist[j], ids[j], INVALID};
  __syncwarp();
}

// forward: each node of this level applies the insertions from lower ids
// (senders m < n whose row at their turn lists n), then snapshots its row
__global__ void __launch_bounds__(II_WARPS * 32) k_ii_forward(IIArgs a, uint32_t vs) {
  extern __shared__ __align__(16) uint8_t smem[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  IIWarp &w = ii_carve(smem, warp, a.R, vs);
  for (uint32_t t = blockIdx.x * II_WARPS + warp; t < a.nn; t += gridDim.x * II_WARPS) {
    const uint32_t n = a.nodes[t];
    uint32_t rs = a.p_deg[n];
    ii_load_row(w, a.p_ids + (size_t)n * a.R, a.p_dist + (size_t)n * a.R, rs, lane);
    bool dvalid = false, kept = false;
    const uint32_t off = a.req_off[n], cnt = a.req_cnt[n];
    for (uint32_t r = 0; r < cnt; r++) {
      const uint32_t m = (uint32_t)(a.req[off + r] >> 32);
      // each position of n in m's row at m's turn sends one insertion
      // (an NSG row can list an id twice), in position order
      const uint32_t mdeg = a.s_deg[m];
      for (uint32_t b = 0; b < mdeg; b += 32) {
        const uint32_t j = b + lane;
        unsigned hits = __ballot_sync(FULL, j < mdeg && a.s_ids[(size_t)m * a.R + j] == n);
        while (hits) {
          const uint32_t pos = b + __ffs(hits) - 1;
          hits &= hits - 1;
          ii_apply(a, w, vs, rs, dvalid, kept, m, a.s_dist[(size_t)m * a.R + pos], pos, lane);
        }
      }
    }
    for (uint32_t j = lane; j < rs; j += 32) {
      a.s_ids[(size_t)n * a.R + j] = w.row[j].i;
      a.s_dist[(size_t)n * a.R + j] = w.row[j].d;
    }
    if (lane == 0) a.s_deg[n] = rs;
    __syncwarp();
  }
}

// backward: every row applies the insertions from higher ids in id order
__global__ void __launch_bounds__(II_WARPS * 32) k_ii_backward(IIArgs a, uint32_t vs) {
  extern __shared__ __align__(16) uint8_t smem[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  IIWarp &w = ii_carve(smem, warp, a.R, vs);
  for (uint32_t r = blockIdx.x * II_WARPS + warp; r < a.n; r += gridDim.x * II_WARPS) {
    uint32_t rs = a.s_deg[r];
    ii_load_row(w, a.s_ids + (size_t)r * a.R, a.s_dist + (size_t)r * a.R, rs, lane);
    bool dvalid = false, kept = false;
    const uint32_t off = a.req_off[r], cnt = a.req_cnt[r];
    for (uint32_t q = 0; q < cnt; q++) {
      const unsigned long long key = a.req[off + q];
      const uint32_t m = (uint32_t)(key >> 32), pos = (uint32_t)key;
      ii_apply(a, w, vs, rs, dvalid, kept, m, a.s_dist[(size_t)m * a.R + pos], pos, lane);
    }
    for (uint32_t j = lane; j < rs; j += 32) {
      a.f_ids[(size_t)r * a.R + j] = w.row[j].i;
      a.f_dist[(size_t)r * a.R + j] = w.row[j].d;
    }
    if (lane == 0) a.f_deg[r] = rs;
    __syncwarp();
  }
}

// requests index: count edges m -> t of rows (ids, deg) with m < t (fwd) or m > t
__global__ void k_req_count(uint32_t n, uint32_t R, const uint32_t *ids, const uint32_t *deg, int fwd, uint32_t *cnt) {
  const uint32_t m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= n) return;
  for (uint32_t j = 0; j < deg[m]; j++) {
    const uint32_t t = ids[(size_t)m * R + j];
    if (t < n && (fwd ? m < t : m > t)) atomicAdd(&cnt[t], 1u);
  }
}
__global__ void k_req_fill(uint32_t n, uint32_t R, const uint32_t *ids, const uint32_t *deg, int fwd,
                           const uint32_t *off, uint32_t *cur, unsigned long long *req) {
  const uint32_t m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= n) return;
  for (uint32_t j = 0; j < deg[m]; j++) {
    const uint32_t t = ids[(size_t)m * R + j];
    if (t < n && (fwd ? m < t : m > t))
      req[off[t] + atomicAdd(&cur[t], 1u)] = ((unsigned long long)m << 32) | j;
  }
}

// level(t) = max(level(t), level(m) + 1) over forward edges of the pruned rows
__global__ void k_level_relax(uint32_t n, uint32_t R, const uint32_t *ids, const uint32_t *deg, uint32_t *level,
                              uint32_t *changed) {
  const uint32_t m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= n) return;
  const uint32_t lm = level[m];
  for (uint32_t j = 0; j < deg[m]; j++) {
    const uint32_t t = ids[(size_t)m * R + j];
    if (t < n && m < t && level[t] < lm + 1) {
      atomicMax(&level[t], lm + 1);
      *changed = 1;
    }
  }
}
__global__ void k_level_count(uint32_t n, const uint32_t *level, uint32_t *lcnt) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) atomicAdd(&lcnt[level[i]], 1u);
}
__global__ void k_level_fill(uint32_t n, const uint32_t *level, const uint32_t *loff, uint32_t *lcur,
                             uint32_t *order) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) order[loff[level[i]] + atomicAdd(&lcur[level[i]], 1u)] = i;
}

// ---------------------------------------------------------------- centroid
// EntryCentroid's FP32 column sums in the reference's order (i ascending)
__global__ void k_centroid(const float *base, uint32_t n, uint32_t d, float *center) {
  const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= d) return;
  float acc = 0.f;
  for (uint32_t i = 0; i < n; i++) acc = __fadd_rn(acc, base[(size_t)i * d + j]);
  center[j] = __fdiv_rn(acc, (float)n);
}

// ---------------------------------------------------------------- Propagation2
// ComponentCandidatePropagation2::CandidateInner (component_candidate.cpp:90-109):
// the pool takes the unseen neighbours of the node's neighbours, walking the
// node's row and each neighbour's row in order, and stops at L entries.  One
// warp per node handles a neighbour row 32 entries at a time: a lane's entry
// is new when the seen-set lacks it and no lower lane holds the same id; the
// first (L - size) new entries, in lane order, are appended and marked.  The
// seen-set is an open-addressing hash in shared memory (at most L + 1 of its
// 2^k >= 2(L + 1) words are ever used, so a probe always ends).
constexpr int P2_WARPS_MAX = 8;
constexpr uint32_t P2_EMPTY = 0xffffffffu;

struct Prop2Args {
  const float *base;
  uint32_t d, n;
  const uint32_t *g_ids, *g_deg;
  uint32_t gw;
  uint32_t n0, cnt;   // nodes [n0, n0 + cnt)
  uint32_t L;
  uint32_t hwords;    // seen-set words per warp (power of two)
  DI *vis;            // cnt x vcap pools
  uint32_t vcap;
  uint32_t *vcnt;
  int *status;
};

__device__ __forceinline__ uint32_t p2_slot(uint32_t v, uint32_t mask) { return (v * 0x9E3779B1u) & mask; }

__device__ __forceinline__ bool p2_find(const uint32_t *H, uint32_t mask, uint32_t v) {
  uint32_t h = p2_slot(v, mask);
  for (uint32_t t = 0; t <= mask; t++, h = (h + 1) & mask) {
    const uint32_t x = H[h];
    if (x == v) return true;
    if (x == P2_EMPTY) return false;
  }
  return false;
}

__device__ __forceinline__ void p2_insert(uint32_t *H, uint32_t mask, uint32_t v) {
  uint32_t h = p2_slot(v, mask);
  for (uint32_t t = 0; t <= mask; t++, h = (h + 1) & mask) {
    const uint32_t old = atomicCAS(H + h, P2_EMPTY, v);
    if (old == P2_EMPTY || old == v) return;
  }
}

__global__ void k_prop2(Prop2Args a) {
  extern __shared__ uint32_t p2_smem[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int wpb = blockDim.x >> 5;
  uint32_t *H = p2_smem + (size_t)warp * a.hwords;
  const uint32_t mask = a.hwords - 1;
  const unsigned lt = (1u << lane) - 1u;
  for (uint32_t qi = blockIdx.x * wpb + warp; qi < a.cnt; qi += gridDim.x * wpb) {
    const uint32_t q = a.n0 + qi;
    DI *pool = a.vis + (size_t)qi * a.vcap;
    for (uint32_t k = lane; k < a.hwords; k += 32) H[k] = P2_EMPTY;
    __syncwarp();
    if (lane == 0) p2_insert(H, mask, q);
    __syncwarp();
    uint32_t size = 0;
    const uint32_t qdeg = min(a.g_deg[q], a.gw);
    for (uint32_t i = 0; i < qdeg && size < a.L; i++) {
      const uint32_t nid = a.g_ids[(size_t)q * a.gw + i];
      if (nid >= a.n) {
        if (lane == 0) set_err(a.status, DEV_BAD_ID);
        continue;
      }
      const uint32_t ndeg = min(a.g_deg[nid], a.gw);
      for (uint32_t b = 0; b < ndeg && size < a.L; b += 32) {
        const uint32_t j = b + lane;
        uint32_t v = j < ndeg ? a.g_ids[(size_t)nid * a.gw + j] : P2_EMPTY;
        if (j < ndeg && v >= a.n) {
          set_err(a.status, DEV_BAD_ID);
          v = P2_EMPTY;
        }
        bool fresh = v != P2_EMPTY && !p2_find(H, mask, v);
        const unsigned same = __match_any_sync(FULL, v);
        fresh = fresh && (same & lt) == 0;  // the lowest lane holding v speaks for it
        const unsigned newm = __ballot_sync(FULL, fresh);
        const uint32_t take = min((uint32_t)__popc(newm), a.L - size);
        const uint32_t rank = __popc(newm & lt);
        __syncwarp();  // every lookup of this batch precedes its insertions
        if (fresh && rank < take) {
          pool[size + rank] = DI{0.f, v};
          p2_insert(H, mask, v);
        }
        size += take;
        __syncwarp();
      }
    }
    // distances in the reference's order, one lane per entry
    for (uint32_t j = lane; j < size; j += 32) pool[j].d = l2g(a.base, a.d, q, pool[j].i);
    if (lane == 0) a.vcnt[qi] = size;
    __syncwarp();
  }
}

// ---------------------------------------------------------------- SSG conn
// smallest reached node whose row has a free slot (deg < R); *out starts at ~0
__global__ void k_first_open(const uint32_t *bits, const uint32_t *deg, uint32_t n, uint32_t R, uint32_t *out) {
  for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
    if (((bits[j >> 5] >> (j & 31)) & 1u) && deg[j] < R) {
      atomicMin(out, j);
      return;  // later j of this thread are larger
    }
  }
}

// one repair of ConnSSGDFS (component_conn.cpp:205-221): node u = the smallest
// unreached id; the first reached node j with a free slot gets the edge
// j -> u (distance in the reference's order); u is marked and becomes the
// frontier.  u >= n ends the root's pass (frontier size 0).
__global__ void k_ssg_repair(const float *base, uint32_t d, uint32_t n, uint32_t w, uint32_t R, uint32_t *ids,
                             float *dist, uint32_t *deg, const uint32_t *u_in, uint32_t *j_in, uint32_t *bits,
                             uint32_t *front, uint32_t *nfront, uint32_t *added) {
  if (threadIdx.x != 0) return;
  const uint32_t u = *u_in, j = *j_in;
  *j_in = 0xffffffffu;
  if (u >= n) {
    *nfront = 0;
    return;
  }
  if (j < n && deg[j] < R) {
    const uint32_t pos = deg[j];
    ids[(size_t)j * w + pos] = u;
    dist[(size_t)j * w + pos] = l2g(base, d, j, u);
    deg[j] = pos + 1;
    *added += 1;
  }
  bits[u >> 5] |= 1u << (u & 31);
  front[0] = u;
  *nfront = 1;
}

__global__ void k_mark_root(uint32_t *bits, uint32_t r, uint32_t *front) {
  bits[r >> 5] |= 1u << (r & 31);
  front[0] = r;
}

}  // namespace

// ================================================================ host side
namespace {

int run_build_search(wv_ctx *c, const float *d_queries, uint32_t nq, const uint32_t *d_seeds, uint32_t seed_stride,
                     uint32_t L, const uint32_t *gids, const uint32_t *gdeg, uint32_t gw, DI *vis, uint32_t *vcnt,
                     uint32_t vcap, uint32_t *out_ids, uint32_t K, uint32_t vlimit = 0) {
  if (vlimit == 0) vlimit = vcap;
  const uint32_t cap = gw + 32;
  int blocks = search_grid(c->d, L, cap, c->device);
  WV_CHECK(c, blocks > 0, WV_ERR_LIMIT, "candidate search cannot run with d=%u L=%u width=%u", c->d, L, gw);
  size_t slots = (size_t)blocks * search_warps_per_block();
  size_t words = (c->n + 31) / 32;
  if (slots > c->vis_slots || words != c->vis_words) {
    c->visited.release();
    c->touched.release();
    WV_CUDA(c, c->visited.ensure(slots * words * 4));
    WV_CUDA(c, c->touched.ensure(slots * words * 4));
    WV_CUDA(c, cudaMemsetAsync(c->visited.p, 0, slots * words * 4, c->stream));
    c->vis_slots = slots;
    c->vis_words = words;
  }
  WV_CUDA(c, cudaMemsetAsync(c->misc.p, 0, 32, c->stream));
  SearchArgs a{};
  a.base = c->base.as<float>();
  a.n = c->n;
  a.d = c->d;
  a.gids = gids;
  a.gdeg = gdeg;
  a.gw = gw;
  a.queries = d_queries;
  a.nq = nq;
  a.seeds = d_seeds;
  a.seed_stride = seed_stride;
  a.L = L;
  a.K = K;
  a.Lmax = L;
  a.out_ids = out_ids;
  a.out_stride = K;
  a.visited = c->visited.as<uint32_t>();
  a.touched = c->touched.as<uint32_t>();
  a.words = (uint32_t)words;
  a.cap = cap;
  a.next_query = c->d_next();
  a.status = c->d_status();
  a.vis = vis;
  a.vcnt = vcnt;
  a.vcap = vcap;
  a.vlimit = vlimit;
  a.int_exact = c->base_int;
  a.xnorm = c->xnorm.as<float>();
  int nb = (int)std::min<size_t>((size_t)blocks, ((size_t)nq + search_warps_per_block() - 1) / search_warps_per_block());
  WV_CUDA(c, launch_search_exact(a, std::max(nb, 1), c->stream));
  return WV_OK;
}

// seen-set words per warp for pool size L, and the warps per block that fit
uint32_t prop2_hwords(uint32_t L) {
  uint32_t h = 64;
  while (h < 2 * (L + 1)) h <<= 1;
  return h;
}

int run_prop2(wv_ctx *c, uint32_t n0, uint32_t cnt, uint32_t L, DI *vis, uint32_t *vcnt, uint32_t vcap) {
  Prop2Args a{};
  a.base = c->base.as<float>();
  a.d = c->d;
  a.n = c->n;
  a.g_ids = c->fg_ids.as<uint32_t>();
  a.g_deg = c->fg_deg.as<uint32_t>();
  a.gw = c->fg_w;
  a.n0 = n0;
  a.cnt = cnt;
  a.L = L;
  a.hwords = prop2_hwords(L);
  a.vis = vis;
  a.vcap = vcap;
  a.vcnt = vcnt;
  a.status = c->d_status();
  const size_t per_warp = (size_t)a.hwords * 4;
  const int wpb = (int)std::max<size_t>(1, std::min<size_t>(P2_WARPS_MAX, (96u << 10) / per_warp));
  const size_t smem = per_warp * wpb;
  WV_CUDA(c, cudaFuncSetAttribute(k_prop2, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const int blocks = (int)std::min<size_t>(((size_t)cnt + wpb - 1) / wpb, (size_t)c->sms * 16);
  k_prop2<<<std::max(blocks, 1), wpb * 32, smem, c->stream>>>(a);
  WV_CUDA(c, cudaGetLastError());
  return WV_OK;
}

// float threshold = std::cos(A / 180 * kPi) (component_prune.cpp:92-93,
// component_refine.cpp:640-641): float quotient, double product and cosine
float ssg_threshold(float A) {
  const double kPi = std::acos(-1.0);
  return (float)std::cos((double)(A / 180) * kPi);
}

}  // namespace

int link_gpu(wv_ctx *c, const LinkParams &p, LinkStats *st) {
  const bool ssg = p.mode == LinkMode::SSG, vamana = p.mode == LinkMode::VAMANA;
  WV_CHECK(c, c->n > 0 && c->fg_n == c->n, WV_ERR_STATE, "the link needs the base and a candidate graph");
  WV_CHECK(c, p.R >= 1 && p.R <= LINK_MAX_R, WV_ERR_LIMIT, "R_refine=%u: this build supports 1..%u", p.R, LINK_MAX_R);
  if (ssg)
    WV_CHECK(c, p.L >= 1 && p.L <= (1u << 13), WV_ERR_ARG, "L_refine=%u out of range", p.L);
  else
    WV_CHECK(c, p.L >= 1 && p.L < c->n && p.L <= SEARCH_MAX_L, WV_ERR_ARG, "L_refine=%u out of range", p.L);
  WV_CHECK(c, c->fg_w <= SEARCH_MAX_WIDTH, WV_ERR_LIMIT, "candidate graph width %u above %u", c->fg_w,
           SEARCH_MAX_WIDTH);
  WV_CHECK(c, c->d % 4 == 0, WV_ERR_LIMIT, "dimension %u is not a multiple of 4", c->d);
  LinkStats local;
  LinkStats &S = st ? *st : local;
  S = LinkStats();
  cudaError_t e = cudaSuccess;
  const uint32_t n = c->n, R = p.R, gw = c->fg_w;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventRecord(e0, c->stream);
  // host copies of what the host-side draws need
  std::vector<uint32_t> hdeg(n);
  WV_CUDA(c, cudaMemcpyAsync(hdeg.data(), c->fg_deg.p, (size_t)n * 4, cudaMemcpyDeviceToHost, c->stream));
  WV_CUDA(c, cudaStreamSynchronize(c->stream));
  auto host_row = [&](uint32_t v, std::vector<uint32_t> &out) -> int {
    out.resize(hdeg[v]);
    if (hdeg[v])
      WV_CUDA(c, cudaMemcpy(out.data(), c->fg_ids.as<uint32_t>() + (size_t)v * gw, hdeg[v] * 4, cudaMemcpyDeviceToHost));
    return WV_OK;
  };
  float *center = c->buf<float>("center", c->d, &e);
  uint32_t *seed1 = c->buf<uint32_t>("seed1", p.L, &e);
  uint32_t *one = c->buf<uint32_t>("one", 4, &e);
  WV_CUDA(c, e);
  // ---- entry point (ComponentRefineEntryCentroid::EntryInner); SSG has none
  // (its RefineInner leaves the entry step out) and draws no rand() here
  uint32_t ep = 0;
  if (!ssg) {
  k_centroid<<<(c->d + 127) / 128, 128, 0, c->stream>>>(c->base.as<float>(), n, c->d, center);
  WV_CUDA(c, cudaGetLastError());
  ep = (uint32_t)c->rnd.next() % n;
  if (p.entry_L == 0) {
    ep = 0;  // get_neighbors with L = 0 leaves retset[0] value-initialised
  } else {
    std::vector<uint32_t> row, sd(p.entry_L);
    int rc = host_row(ep, row);
    if (rc) return rc;
    draw_seeds_row(c->rnd, p.entry_L, n, row.data(), (uint32_t)row.size(), sd.data());
    WV_CUDA(c, cudaMemcpyAsync(seed1, sd.data(), p.entry_L * 4, cudaMemcpyHostToDevice, c->stream));
    DI *v1 = c->buf<DI>("vis1", (size_t)n + p.entry_L + 64, &e);
    WV_CUDA(c, e);
    rc = run_build_search(c, center, 1, seed1, p.entry_L, p.entry_L, c->fg_ids.as<uint32_t>(),
                          c->fg_deg.as<uint32_t>(), gw, v1, one + 1, n + p.entry_L + 64, one, 1);
    if (rc) return rc;
    WV_CUDA(c, cudaMemcpyAsync(&ep, one, 4, cudaMemcpyDeviceToHost, c->stream));
    WV_CUDA(c, cudaStreamSynchronize(c->stream));
  }
  }
  S.ep = ep;
  // ---- candidates + prune, in chunks of nodes
  uint32_t *p_ids = c->buf<uint32_t>("lk_pids", (size_t)n * R, &e);
  float *p_dist = c->buf<float>("lk_pdist", (size_t)n * R, &e);
  uint32_t *p_deg = c->buf<uint32_t>("lk_pdeg", n, &e);
  WV_CUDA(c, e);
  std::vector<uint32_t> ep_row;
  if (!ssg) {
    int rc = host_row(ep, ep_row);
    if (rc) return rc;
  }
  const bool shared_seeds = ssg || p.L <= ep_row.size();  // no rand() fill needed
  // SSG pools hold at most L candidates plus the node's row
  uint32_t vcap = ssg ? p.L + gw : std::max<uint32_t>(2048, 8 * p.L) + gw;
  const uint32_t CH = std::min<uint32_t>(n, 1u << 17);
  std::vector<uint32_t> hseeds;
  uint32_t *dseeds = c->buf<uint32_t>("lk_seeds", (size_t)(shared_seeds ? 1 : CH) * p.L, &e);
  WV_CUDA(c, e);
  if (shared_seeds && !ssg)
    WV_CUDA(c, cudaMemcpyAsync(dseeds, ep_row.data(), p.L * 4, cudaMemcpyHostToDevice, c->stream));
  const int prune_blocks = c->sms * 8;
  const size_t nwarps = (size_t)prune_blocks * PR_WARPS;
  const float threshold = ssg ? ssg_threshold(p.A) : 0.f;
  for (uint32_t n0 = 0; n0 < n; n0 += CH) {
    const uint32_t cnt = std::min(CH, n - n0);
    if (!shared_seeds) {
      hseeds.resize((size_t)cnt * p.L);
      for (uint32_t q = 0; q < cnt; q++) {
        // the fill draws rand() % N until L ids are taken (candidate.cpp:25-31)
        draw_seeds_row(c->rnd, p.L, n, ep_row.data(), (uint32_t)ep_row.size(), hseeds.data() + (size_t)q * p.L);
      }
      WV_CUDA(c, cudaMemcpyAsync(dseeds, hseeds.data(), (size_t)cnt * p.L * 4, cudaMemcpyHostToDevice, c->stream));
    }
    while (true) {
      DI *vis = c->buf<DI>("lk_vis", (size_t)cnt * vcap, &e);
      uint32_t *vcnt = c->buf<uint32_t>("lk_vcnt", cnt, &e);
      int *gscr = c->buf<int>("lk_gscr", nwarps * (2 * (size_t)vcap + 256), &e);
      HeapItem *hscr = c->buf<HeapItem>("lk_hscr", nwarps * (size_t)vcap, &e);
      WV_CUDA(c, e);
      int rc = ssg ? run_prop2(c, n0, cnt, p.L, vis, vcnt, vcap)
                   : run_build_search(c, c->base.as<float>() + (size_t)n0 * c->d, cnt, dseeds,
                                      shared_seeds ? 0 : p.L, p.L, c->fg_ids.as<uint32_t>(),
                                      c->fg_deg.as<uint32_t>(), gw, vis, vcnt, vcap, nullptr, 1,
                                      vcap - ((vamana && !p.clean) ? 0 : gw));
      if (rc) return rc;
      int st0 = 0;
      WV_CUDA(c, cudaMemcpyAsync(&st0, c->d_status(), 4, cudaMemcpyDeviceToHost, c->stream));
      WV_CUDA(c, cudaStreamSynchronize(c->stream));
      if (st0 == DEV_OVERFLOW && !ssg) {  // a visit list outgrew vcap: redo the chunk with room
        WV_CUDA(c, cudaMemsetAsync(c->d_status(), 0, 4, c->stream));
        vcap = vcap * 2;
        continue;
      }
      rc = check_device_status(c, "candidate search");
      if (rc) return rc;
      PruneArgs pa{};
      pa.base = c->base.as<float>();
      pa.d = c->d;
      pa.n = n;
      pa.vis = vis;
      pa.vcnt = vcnt;
      pa.vcap = vcap;
      pa.n0 = n0;
      pa.cnt = cnt;
      pa.R = R;
      pa.alpha = p.alpha;
      pa.clean = p.clean ? 1 : 0;
      pa.maxc = p.C;
      pa.threshold = threshold;
      pa.g_ids = c->fg_ids.as<uint32_t>();
      pa.g_deg = c->fg_deg.as<uint32_t>();
      pa.gw = gw;
      pa.gscr = gscr;
      pa.hscr = hscr;
      pa.out_ids = p_ids;
      pa.out_dist = p_dist;
      pa.out_deg = p_deg;
      pa.status = c->d_status();
      // integer data (d % 32 == 0, d <= 128) and R <= 32: the pair distances
      // from Gram tiles, the same values (WV_LINK_PRUNE=fp32 keeps the
      // exact-order FP32 sums)
      const char *pr_env = getenv("WV_LINK_PRUNE");
      const bool tc = c->base_int && c->d % 32 == 0 && c->d <= 128 && R <= PT_ROWS &&
                      !(pr_env && std::string(pr_env) == "fp32");
      pa.xnorm = tc ? c->xnorm.as<float>() : nullptr;
      const size_t tsm = tc ? (size_t)PR_WARPS * pt_warp_bytes(c->d) : 0;
      if (tc) {
        if (ssg) WV_CUDA(c, cudaFuncSetAttribute(k_prune<2, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tsm));
        else if (!vamana) WV_CUDA(c, cudaFuncSetAttribute(k_prune<1, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tsm));
        else WV_CUDA(c, cudaFuncSetAttribute(k_prune<0, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tsm));
      }
      if (ssg) {
        if (tc) k_prune<2, true><<<prune_blocks, PR_WARPS * 32, tsm, c->stream>>>(pa);
        else k_prune<2, false><<<prune_blocks, PR_WARPS * 32, 0, c->stream>>>(pa);
      } else if (!vamana) {
        if (tc) k_prune<1, true><<<prune_blocks, PR_WARPS * 32, tsm, c->stream>>>(pa);
        else k_prune<1, false><<<prune_blocks, PR_WARPS * 32, 0, c->stream>>>(pa);
      } else {
        if (tc) k_prune<0, true><<<prune_blocks, PR_WARPS * 32, tsm, c->stream>>>(pa);
        else k_prune<0, false><<<prune_blocks, PR_WARPS * 32, 0, c->stream>>>(pa);
      }
      WV_CUDA(c, cudaGetLastError());
      rc = check_device_status(c, "prune");
      if (rc) return rc;
      break;
    }
  }
  // ---- InterInsert
  uint32_t *level = c->buf<uint32_t>("lk_level", n, &e);
  uint32_t *flag = c->buf<uint32_t>("lk_flag", 4, &e);
  uint32_t *rcnt = c->buf<uint32_t>("lk_rcnt", n, &e);
  uint32_t *roff = c->buf<uint32_t>("lk_roff", n + 1, &e);
  uint32_t *rcur = c->buf<uint32_t>("lk_rcur", n, &e);
  uint32_t *scan_tmp = c->buf<uint32_t>("lk_scan", scan_scratch_words((size_t)n + 1), &e);
  unsigned long long *req = c->buf<unsigned long long>("lk_req", (size_t)n * R + 1, &e);
  uint32_t *s_ids = c->buf<uint32_t>("lk_sids", (size_t)n * R, &e);
  float *s_dist = c->buf<float>("lk_sdist", (size_t)n * R, &e);
  uint32_t *s_deg = c->buf<uint32_t>("lk_sdeg", n, &e);
  uint32_t *order = c->buf<uint32_t>("lk_order", n, &e);
  WV_CUDA(c, e);
  const int nb = (int)((n + 255) / 256);
  WV_CUDA(c, cudaMemsetAsync(level, 0, (size_t)n * 4, c->stream));
  uint32_t iters = 0;
  while (true) {
    WV_CUDA(c, cudaMemsetAsync(flag, 0, 4, c->stream));
    k_level_relax<<<nb, 256, 0, c->stream>>>(n, R, p_ids, p_deg, level, flag);
    uint32_t ch = 0;
    WV_CUDA(c, cudaMemcpyAsync(&ch, flag, 4, cudaMemcpyDeviceToHost, c->stream));
    WV_CUDA(c, cudaStreamSynchronize(c->stream));
    iters++;
    if (!ch) break;
    WV_CHECK(c, iters <= n + 1, WV_ERR_DEVICE, "level relaxation did not converge");
  }
  std::vector<uint32_t> hlevel(n);
  WV_CUDA(c, cudaMemcpyAsync(hlevel.data(), level, (size_t)n * 4, cudaMemcpyDeviceToHost, c->stream));
  WV_CUDA(c, cudaStreamSynchronize(c->stream));
  const uint32_t nlev = *std::max_element(hlevel.begin(), hlevel.end()) + 1;
  S.levels = nlev;
  uint32_t *lcnt = c->buf<uint32_t>("lk_lcnt", nlev + 1, &e);
  uint32_t *loff = c->buf<uint32_t>("lk_loff", nlev + 1, &e);
  uint32_t *lcur = c->buf<uint32_t>("lk_lcur", nlev + 1, &e);
  uint32_t *scan_l = c->buf<uint32_t>("lk_scanl", scan_scratch_words(nlev + 1), &e);
  WV_CUDA(c, e);
  WV_CUDA(c, cudaMemsetAsync(lcnt, 0, (size_t)(nlev + 1) * 4, c->stream));
  WV_CUDA(c, cudaMemsetAsync(lcur, 0, (size_t)(nlev + 1) * 4, c->stream));
  k_level_count<<<nb, 256, 0, c->stream>>>(n, level, lcnt);
  WV_CUDA(c, exclusive_scan_u32(lcnt, loff, nlev + 1, scan_l, c->stream));
  k_level_fill<<<nb, 256, 0, c->stream>>>(n, level, loff, lcur, order);
  std::vector<uint32_t> hloff(nlev + 1);
  WV_CUDA(c, cudaMemcpyAsync(hloff.data(), loff, (size_t)(nlev + 1) * 4, cudaMemcpyDeviceToHost, c->stream));
  // forward request lists from the pruned rows, sorted by sender
  WV_CUDA(c, cudaMemsetAsync(rcnt, 0, (size_t)n * 4, c->stream));
  WV_CUDA(c, cudaMemsetAsync(rcur, 0, (size_t)n * 4, c->stream));
  k_req_count<<<nb, 256, 0, c->stream>>>(n, R, p_ids, p_deg, 1, rcnt);
  WV_CUDA(c, exclusive_scan_u32(rcnt, roff, n, scan_tmp, c->stream));
  k_req_fill<<<nb, 256, 0, c->stream>>>(n, R, p_ids, p_deg, 1, roff, rcur, req);
  int rc = segsort_u64(c, req, roff, rcnt, n);
  if (rc) return rc;
  IIArgs ia{};
  ia.base = c->base.as<float>();
  ia.d = c->d;
  ia.n = n;
  ia.R = R;
  ia.alpha = p.alpha;
  ia.vamana = vamana;
  ia.clean = p.clean ? 1 : 0;
  ia.ssg = ssg;
  ia.ints = c->base_int && c->d <= 256;
  ia.threshold = threshold;
  ia.p_ids = p_ids;
  ia.p_dist = p_dist;
  ia.p_deg = p_deg;
  ia.s_ids = s_ids;
  ia.s_dist = s_dist;
  ia.s_deg = s_deg;
  ia.req = req;
  ia.req_off = roff;
  ia.req_cnt = rcnt;
  ia.status = c->d_status();
  // row vectors in shared memory when they fit, else read from global memory
  uint32_t vs = ((c->d + 3) & ~3u) + 4;
  if (II_WARPS * ii_warp_bytes(R, vs) > 200 * 1024) vs = 0;
  const size_t ii_smem = II_WARPS * ii_warp_bytes(R, vs);
  WV_CUDA(c, cudaFuncSetAttribute(k_ii_forward, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ii_smem));
  WV_CUDA(c, cudaFuncSetAttribute(k_ii_backward, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ii_smem));
  WV_CUDA(c, cudaStreamSynchronize(c->stream));
  for (uint32_t t = 0; t < nlev; t++) {
    const uint32_t cnt = hloff[t + 1] - hloff[t];
    if (!cnt) continue;
    ia.nodes = order + hloff[t];
    ia.nn = cnt;
    const int blocks = (int)std::min<uint32_t>((cnt + II_WARPS - 1) / II_WARPS, (uint32_t)c->sms * 16);
    k_ii_forward<<<blocks, II_WARPS * 32, ii_smem, c->stream>>>(ia, vs);
  }
  WV_CUDA(c, cudaGetLastError());
  // backward request lists from the snapshots, sorted by sender
  WV_CUDA(c, cudaMemsetAsync(rcnt, 0, (size_t)n * 4, c->stream));
  WV_CUDA(c, cudaMemsetAsync(rcur, 0, (size_t)n * 4, c->stream));
  k_req_count<<<nb, 256, 0, c->stream>>>(n, R, s_ids, s_deg, 0, rcnt);
  WV_CUDA(c, exclusive_scan_u32(rcnt, roff, n, scan_tmp, c->stream));
  k_req_fill<<<nb, 256, 0, c->stream>>>(n, R, s_ids, s_deg, 0, roff, rcur, req);
  rc = segsort_u64(c, req, roff, rcnt, n);
  if (rc) return rc;
  // final rows (width R) replace the build graph
  WV_CUDA(c, c->fg_ids.ensure((size_t)n * R * 4));
  WV_CUDA(c, c->fg_dist.ensure((size_t)n * R * 4));
  WV_CUDA(c, c->fg_deg.ensure((size_t)n * 4));
  ia.f_ids = c->fg_ids.as<uint32_t>();
  ia.f_dist = c->fg_dist.as<float>();
  ia.f_deg = c->fg_deg.as<uint32_t>();
  k_ii_backward<<<c->sms * 16, II_WARPS * 32, ii_smem, c->stream>>>(ia, vs);
  WV_CUDA(c, cudaGetLastError());
  rc = check_device_status(c, "inter-insert");
  if (rc) return rc;
  c->fg_w = R;
  c->fg_ep = ep;
  c->fg_has_ep = !ssg;
  c->fg_eps.clear();
  cudaEventRecord(e1, c->stream);
  cudaEventSynchronize(e1);
  cudaEventElapsedTime(&S.ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return WV_OK;
}

// The conn edges root -> id at row position pos, applied on the device: the
// id, the distance compare(base[root], base[id]) (ComponentConnNSGDFS::
// findroot, component_conn.cpp:94-97) and the row's degree.
struct ConnEdge {
  uint32_t root, id, pos;
};

__global__ void k_conn_edges(const float *base, uint32_t d, const ConnEdge *e, uint32_t ne, uint32_t *gids,
                             float *gdist, uint32_t *gdeg, uint32_t w) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < ne; i += gridDim.x * blockDim.x) {
    const ConnEdge x = e[i];
    gids[(size_t)x.root * w + x.pos] = x.id;
    gdist[(size_t)x.root * w + x.pos] = l2g(base, d, x.root, x.id);
    atomicMax(gdeg + x.root, x.pos + 1);
  }
}

// rows ids[0..B) of the base, packed (the queries of a batch of searches)
__global__ void k_conn_rows(const float *base, uint32_t d, const uint32_t *ids, uint32_t B, float *out) {
  const size_t total = (size_t)B * d;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total; t += (size_t)gridDim.x * blockDim.x)
    out[t] = base[(size_t)ids[t / d] * d + t % d];
}

// the rows (width w0) re-laid out with width w1, entries past a row's
// degree zero
__global__ void k_conn_relayout(const uint32_t *ids, const float *dist, const uint32_t *deg, uint32_t n, uint32_t w0,
                                uint32_t w1, uint32_t *ids1, float *dist1) {
  const size_t total = (size_t)n * w1;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total; t += (size_t)gridDim.x * blockDim.x) {
    const uint32_t v = (uint32_t)(t / w1), j = (uint32_t)(t % w1);
    const bool in = j < w0 && j < deg[v];
    ids1[t] = in ? ids[(size_t)v * w0 + j] : 0u;
    dist1[t] = in ? dist[(size_t)v * w0 + j] : 0.f;
  }
}

int conn_dfs_gpu(wv_ctx *c, uint32_t L_refine, uint32_t *added) {
  // ComponentConnNSGDFS::tree_grow (component_conn.cpp:14-98).
  //
  // Which nodes get linked, and in which order, follows from the rows alone:
  // everything reachable from a flagged node is flagged, so the DFS after a
  // repair leaves the new root only through the new edge, the flagged set
  // after repair k is the closure of ep and the first k linked nodes over
  // the rows as they were, and the next linked node is the smallest
  // unflagged id.  The host walks that first: ft[x] is the repair after
  // which x is flagged (0: the walk from ep), tgt the linked nodes in order.
  //
  // The roots come from greedy searches (get_neighbors from ep's row) that
  // read the rows with the edges added so far and draw rand() for their
  // seeds.  They run as one batch over the linked nodes still to do, all on
  // the rows and the rand() stream as they stand at the batch's start (the
  // seeds from a copy of the stream).  The host then takes the results in
  // repair order and accepts search k while (a) the real stream, at k's
  // turn, gives the same seeds (the fallback's extra draws and an edge
  // appended to a short ep row change them) and (b) none of the rows it
  // read -- its seeds' and its visits' -- got an edge earlier in the batch.
  // The first search that fails starts the next batch, so every accepted
  // search is the one the serial walk runs and the first of a batch is
  // always accepted.  With a caller's rand() function (the stream cannot be
  // copied) each batch is one search.
  //
  // The rows stay on the device (edges appended there, widths changed by a
  // copy kernel); the host keeps the rows as they were, for the walk, and
  // ep's row with its new edges, for the seeds.
  const uint32_t n = c->n, ep = c->fg_ep, w0 = c->fg_w;
  uint32_t w = w0;
  std::vector<uint32_t> deg(n), ids((size_t)n * w0);
  WV_CUDA(c, cudaMemcpyAsync(deg.data(), c->fg_deg.p, (size_t)n * 4, cudaMemcpyDeviceToHost, c->stream));
  WV_CUDA(c, cudaMemcpyAsync(ids.data(), c->fg_ids.p, (size_t)n * w0 * 4, cudaMemcpyDeviceToHost, c->stream));
  WV_CUDA(c, cudaStreamSynchronize(c->stream));
  *added = 0;
  // the walk: flag times and the linked nodes
  constexpr uint32_t NONE = 0xffffffffu;
  std::vector<uint32_t> ft(n, NONE), tgt, st;
  for (uint32_t v = 0; v < n; v++) {
    WV_CHECK(c, deg[v] <= w0, WV_ERR_STATE, "row %u: degree %u > width %u", v, deg[v], w0);
    for (uint32_t j = 0; j < deg[v]; j++)
      WV_CHECK(c, ids[(size_t)v * w0 + j] < n, WV_ERR_STATE, "row %u holds id %u >= n", v, ids[(size_t)v * w0 + j]);
  }
  auto walk = [&](uint32_t start, uint32_t t) {  // DFS (component_conn.cpp:31-57)
    st.assign(1, start);
    ft[start] = t;
    uint32_t tmp = start;
    while (!st.empty()) {
      uint32_t next = NONE;
      for (uint32_t j = 0; j < deg[tmp]; j++)
        if (ft[ids[(size_t)tmp * w0 + j]] == NONE) {
          next = ids[(size_t)tmp * w0 + j];
          break;
        }
      if (next == NONE) {
        st.pop_back();
        if (st.empty()) break;
        tmp = st.back();
        continue;
      }
      tmp = next;
      ft[tmp] = t;
      st.push_back(tmp);
    }
  };
  walk(ep, 0);
  for (uint32_t cur = 0;;) {  // findroot's first unflagged id only grows
    while (cur < n && ft[cur] != NONE) cur++;
    if (cur == n) break;
    tgt.push_back(cur);
    walk(cur, (uint32_t)tgt.size());
  }
  const uint32_t m = (uint32_t)tgt.size();
  if (m == 0) return WV_OK;
  std::vector<uint32_t> ep_row(ids.begin() + (size_t)ep * w0, ids.begin() + (size_t)ep * w0 + deg[ep]);
  // re-lays the device rows out with width nw
  auto relayout = [&](uint32_t nw) -> int {
    DevBuf &ti = c->work["conn_ri"], &td = c->work["conn_rd"];
    WV_CUDA(c, ti.ensure((size_t)n * nw * 4));
    WV_CUDA(c, td.ensure((size_t)n * nw * 4));
    const size_t total = (size_t)n * nw;
    const int nb = (int)std::min<size_t>((total + 255) / 256, (size_t)c->sms * 16);
    k_conn_relayout<<<nb, 256, 0, c->stream>>>(c->fg_ids.as<uint32_t>(), c->fg_dist.as<float>(),
                                                c->fg_deg.as<uint32_t>(), n, w, nw, ti.as<uint32_t>(),
                                                td.as<float>());
    WV_CUDA(c, cudaGetLastError());
    std::swap(c->fg_ids, ti);
    std::swap(c->fg_dist, td);
    w = nw;
    c->fg_w = w;
    return WV_OK;
  };
  // accepted edges not yet in the device rows
  std::vector<ConnEdge> edges;
  auto flush = [&]() -> int {
    if (edges.empty()) return WV_OK;
    const uint32_t ne = (uint32_t)edges.size();
    cudaError_t e2 = cudaSuccess;
    ConnEdge *de = c->buf<ConnEdge>("conn_e", ne, &e2);
    WV_CUDA(c, e2);
    WV_CUDA(c, cudaMemcpyAsync(de, edges.data(), (size_t)ne * sizeof(ConnEdge), cudaMemcpyHostToDevice, c->stream));
    k_conn_edges<<<(ne + 127) / 128, 128, 0, c->stream>>>(c->base.as<float>(), c->d, de, ne, c->fg_ids.as<uint32_t>(),
                                                          c->fg_dist.as<float>(), c->fg_deg.as<uint32_t>(), w);
    WV_CUDA(c, cudaGetLastError());
    edges.clear();
    return WV_OK;
  };
  int rc = relayout(w + 16);  // spare width for the edges this pass adds
  if (rc) return rc;
  const bool own = c->rnd.fn == nullptr;
  // searches per batch at most (WV_CONN_BATCH=1 runs them one at a time)
  uint32_t batch_max = 4096;
  if (const char *be = getenv("WV_CONN_BATCH")) batch_max = (uint32_t)std::min(4096L, std::max(1L, atol(be)));
  uint32_t vcap = L_refine + std::max<uint32_t>(1024, 16 * L_refine);
  std::vector<uint32_t> sd, real(L_refine), vcnt_h;
  std::vector<DI> vis_h, hv;
  std::vector<char> changed(n, 0);
  std::vector<uint32_t> changed_list;
  uint32_t k0 = 0;
  while (k0 < m) {
    rc = flush();  // the rows as they stand
    if (rc) return rc;
    for (uint32_t v : changed_list) changed[v] = 0;
    changed_list.clear();
    const uint32_t B = own ? std::min(m - k0, batch_max) : 1;
    sd.resize((size_t)B * L_refine);
    if (own) {
      RandSource spec = c->rnd;
      for (uint32_t b = 0; b < B; b++)
        draw_seeds_row(spec, L_refine, n, ep_row.data(), (uint32_t)ep_row.size(), sd.data() + (size_t)b * L_refine);
    } else {
      draw_seeds_row(c->rnd, L_refine, n, ep_row.data(), (uint32_t)ep_row.size(), sd.data());
    }
    cudaError_t e = cudaSuccess;
    uint32_t *dseed = c->buf<uint32_t>("conn_seed", (size_t)B * L_refine, &e);
    uint32_t *dtg = c->buf<uint32_t>("conn_tg", B, &e);
    float *dq = c->buf<float>("conn_q", (size_t)B * c->d, &e);
    uint32_t *dvc = c->buf<uint32_t>("conn_vc", B, &e);
    uint32_t *dout = c->buf<uint32_t>("conn_out", B, &e);
    WV_CUDA(c, e);
    WV_CUDA(c, cudaMemcpyAsync(dseed, sd.data(), (size_t)B * L_refine * 4, cudaMemcpyHostToDevice, c->stream));
    WV_CUDA(c, cudaMemcpyAsync(dtg, tgt.data() + k0, (size_t)B * 4, cudaMemcpyHostToDevice, c->stream));
    {
      const size_t total = (size_t)B * c->d;
      const int nb = (int)std::min<size_t>((total + 255) / 256, (size_t)c->sms * 8);
      k_conn_rows<<<nb, 256, 0, c->stream>>>(c->base.as<float>(), c->d, dtg, B, dq);
      WV_CUDA(c, cudaGetLastError());
    }
    DI *vis = nullptr;
    while (true) {  // get_neighbors(base[id]) from ep's row (component_conn.cpp:100-160)
      vis = c->buf<DI>("conn_vis", (size_t)B * vcap, &e);
      WV_CUDA(c, e);
      rc = run_build_search(c, dq, B, dseed, L_refine, L_refine, c->fg_ids.as<uint32_t>(), c->fg_deg.as<uint32_t>(),
                            w, vis, dvc, vcap, dout, 1);
      if (rc) return rc;
      int st0 = 0;
      WV_CUDA(c, cudaMemcpyAsync(&st0, c->d_status(), 4, cudaMemcpyDeviceToHost, c->stream));
      WV_CUDA(c, cudaStreamSynchronize(c->stream));
      if (st0 == DEV_OVERFLOW) {  // a visit list outgrew vcap: redo the batch with room
        WV_CUDA(c, cudaMemsetAsync(c->d_status(), 0, 4, c->stream));
        vcap *= 2;
        continue;
      }
      rc = check_device_status(c, "conn search");
      if (rc) return rc;
      break;
    }
    vcnt_h.resize(B);
    vis_h.resize((size_t)B * vcap);
    WV_CUDA(c, cudaMemcpyAsync(vcnt_h.data(), dvc, (size_t)B * 4, cudaMemcpyDeviceToHost, c->stream));
    WV_CUDA(c, cudaStreamSynchronize(c->stream));
    // the visit lists come back in growing chunks, each list only as far as
    // the chunk's longest: a batch is usually cut after a few searches
    uint32_t have = 0, chunk = 16;
    uint32_t acc = 0;
    for (uint32_t b = 0; b < B; b++) {
      if (b == have) {
        const uint32_t hi = std::min(B, have + chunk);
        uint32_t wmax = 1;
        for (uint32_t q = have; q < hi; q++) wmax = std::max(wmax, std::min(vcnt_h[q], vcap));
        WV_CUDA(c, cudaMemcpy2DAsync(vis_h.data() + (size_t)have * vcap, (size_t)vcap * sizeof(DI),
                                     vis + (size_t)have * vcap, (size_t)vcap * sizeof(DI), (size_t)wmax * sizeof(DI),
                                     hi - have, cudaMemcpyDeviceToHost, c->stream));
        WV_CUDA(c, cudaStreamSynchronize(c->stream));
        have = hi;
        chunk *= 2;
      }
      const uint32_t k = k0 + b, u = tgt[k];
      const uint32_t nv = std::min(vcnt_h[b], vcap);
      const DI *v = vis_h.data() + (size_t)b * vcap;
      bool stale = false;
      for (uint32_t j = 0; j < nv && !stale; j++) stale = v[j].i < n && changed[v[j].i];
      if (stale) break;
      if (own) {
        const RandSource keep = c->rnd;
        draw_seeds_row(c->rnd, L_refine, n, ep_row.data(), (uint32_t)ep_row.size(), real.data());
        if (!std::equal(real.begin(), real.end(), sd.data() + (size_t)b * L_refine)) {
          c->rnd = keep;
          break;
        }
      }
      // the pool: the expansion visits (the seeds are not part of it), sorted
      hv.assign(v + std::min(nv, L_refine), v + nv);
      stl::sort(hv.data(), (int)hv.size(), DILess());
      uint32_t root = NONE;
      for (auto &x : hv)
        if (x.i < n && ft[x.i] <= k) {
          root = x.i;
          break;
        }
      if (root == NONE) {
        while (true) {
          const uint32_t rid = (uint32_t)c->rnd.next() % n;
          if (ft[rid] <= k) {
            root = rid;
            break;
          }
        }
      }
      if (deg[root] == w) {
        rc = flush();
        if (rc) return rc;
        rc = relayout(w + 16);
        if (rc) return rc;
      }
      const uint32_t pos = deg[root]++;
      edges.push_back(ConnEdge{root, u, pos});
      if (root == ep) ep_row.push_back(u);
      if (!changed[root]) {
        changed[root] = 1;
        changed_list.push_back(root);
      }
      (*added)++;
      acc++;
    }
    WV_CHECK(c, acc > 0, WV_ERR_STATE, "conn: the first search of a batch was not accepted");
    k0 += acc;
  }
  rc = flush();
  if (rc) return rc;
  uint32_t nw = 1;  // trim to the widest row
  for (uint32_t v = 0; v < n; v++) nw = std::max(nw, deg[v]);
  if (nw != w) rc = relayout(nw);
  if (rc) return rc;
  WV_CUDA(c, cudaStreamSynchronize(c->stream));
  return WV_OK;
}

int conn_ssg_gpu(wv_ctx *c, uint32_t n_try, uint32_t R, std::vector<uint32_t> &eps, uint32_t *added) {
  // ComponentConnSSGDFS::ConnInner (component_conn.cpp:169-225).  The roots
  // are the first n_try ids of std::random_shuffle(0..n-1) on rand()
  // (libstdc++: for i = 1..n-1 swap ids[i] with ids[rand() % (i + 1)]).
  // From each root a breadth-first walk; while nodes stay unreached, the
  // smallest unreached id u is linked from the first reached node with a free
  // slot (if any), marked, and walked from.  Reach does not depend on the
  // walk's order, so the walk runs level-synchronously on the GPU.
  const uint32_t n = c->n, w = c->fg_w;
  WV_CHECK(c, n_try >= 1 && n_try <= n, WV_ERR_ARG, "n_try=%u out of range (n=%u)", n_try, n);
  WV_CHECK(c, R <= w, WV_ERR_ARG, "range %u above the row width %u", R, w);
  std::vector<uint32_t> perm(n);
  for (uint32_t i = 0; i < n; i++) perm[i] = i;
  for (uint32_t i = 1; i < n; i++) {
    const uint32_t j = (uint32_t)c->rnd.next() % (i + 1);
    if (i != j) std::swap(perm[i], perm[j]);
  }
  eps.assign(perm.begin(), perm.begin() + n_try);
  cudaError_t e = cudaSuccess;
  const uint32_t words = (n + 31) / 32;
  uint32_t *bits = c->buf<uint32_t>("sc_bits", words, &e);
  uint32_t *fa = c->buf<uint32_t>("sc_fa", n, &e);
  uint32_t *fb = c->buf<uint32_t>("sc_fb", n, &e);
  uint32_t *cnt = c->buf<uint32_t>("sc_cnt", 8, &e);  // [0] frontier size, [1] u, [2] j, [3] added
  WV_CUDA(c, e);
  WV_CUDA(c, cudaMemsetAsync(cnt, 0, 32, c->stream));
  WV_CUDA(c, cudaMemsetAsync(cnt + 2, 0xff, 4, c->stream));
  uint32_t *ids = c->fg_ids.as<uint32_t>(), *deg = c->fg_deg.as<uint32_t>();
  float *dist = c->fg_dist.as<float>();
  const int scan_blocks = c->sms * 4;
  for (uint32_t t = 0; t < n_try; t++) {
    WV_CUDA(c, cudaMemsetAsync(bits, 0, (size_t)words * 4, c->stream));
    k_mark_root<<<1, 1, 0, c->stream>>>(bits, eps[t], fa);
    uint32_t nf = 1;
    for (;;) {
      while (nf) {
        WV_CUDA(c, cudaMemsetAsync(cnt, 0, 4, c->stream));
        const uint32_t blocks = std::min<uint32_t>((nf + 7) / 8, (uint32_t)c->sms * 32);
        k_bfs_level<<<blocks, 256, 0, c->stream>>>(ids, deg, w, n, fa, nf, bits, fb, cnt, c->d_status());
        WV_CUDA(c, cudaGetLastError());
        WV_CUDA(c, cudaMemcpyAsync(&nf, cnt, 4, cudaMemcpyDeviceToHost, c->stream));
        WV_CUDA(c, cudaStreamSynchronize(c->stream));
        std::swap(fa, fb);
      }
      k_first_unreached<<<1, 1024, 0, c->stream>>>(bits, n, cnt + 1);
      k_first_open<<<scan_blocks, 256, 0, c->stream>>>(bits, deg, n, R, cnt + 2);
      k_ssg_repair<<<1, 32, 0, c->stream>>>(c->base.as<float>(), c->d, n, w, R, ids, dist, deg, cnt + 1,
                                            cnt + 2, bits, fa, cnt, cnt + 3);
      WV_CUDA(c, cudaGetLastError());
      WV_CUDA(c, cudaMemcpyAsync(&nf, cnt, 4, cudaMemcpyDeviceToHost, c->stream));
      WV_CUDA(c, cudaStreamSynchronize(c->stream));
      if (!nf) break;
    }
  }
  WV_CUDA(c, cudaMemcpyAsync(added, cnt + 3, 4, cudaMemcpyDeviceToHost, c->stream));
  WV_CUDA(c, cudaStreamSynchronize(c->stream));
  return check_device_status(c, "ssg conn");
}

}  // namespace wv
