// Warp-parallel replica of libstdc++ std::sort (introsort) on shared memory.
//
// std::sort's result on tied keys depends on its exact sequence of
// median-of-three pivots, Hoare partitions, heapsort fallbacks and the final
// insertion sort (stl_order.cuh restates them for one thread).  Here one
// warp produces the same array, faster:
//  * a Hoare partition [f+1, l) around P = a[f] swaps, in order, the k-th
//    element (from the left) that is not < P with the k-th element (from the
//    right) that P is not < -- for as long as the k-th left position is below
//    the k-th right position.  Those positions are found with ballots, the
//    swaps done in parallel, and the returned cut is the (K+1)-th left stop,
//    capped by the K-th right stop (where the left scan meets a swapped-in
//    element), K being the number of swaps;
//  * disjoint sub-ranges never interact, so the recursion runs from an
//    explicit stack in any order;
//  * the final insertion sort only moves elements inside the <=16-element
//    ranges the recursion stopped at (every element of a range is >= every
//    element before it), so those ranges are insertion-sorted one per lane.
// tests/test_sort_gpu.py checks it against the host std::sort on tie-heavy data.
#pragma once
#include "stl_order.cuh"

namespace wv {

struct WarpSortScratch {
  int *apos;   // >= n ints
  int *bpos;   // >= n ints
  int *stack;  // 3 * 64 ints
  int *leaf;   // 64 ints: up to 32 pending (first, last) insertion ranges
};

template <class T, class Less>
__device__ __forceinline__ void flush_leaves(T *a, Less less, const int *leaf, int nleaf, int lane) {
  if (lane < nleaf) stl::insertion_sort(a + leaf[2 * lane], a + leaf[2 * lane + 1], less);
  __syncwarp();
}

template <class T, class Less>
__device__ __forceinline__ void warp_std_sort(T *a, int n, Less less, WarpSortScratch s, int lane) {
  if (n <= 1) return;
  const unsigned FULLM = 0xffffffffu;
  const unsigned lt = (1u << lane) - 1u;
  int sp = 0, nleaf = 0;
  if (lane == 0) {
    s.stack[0] = 0;
    s.stack[1] = n;
    s.stack[2] = 2 * stl::lg2(n);
  }
  sp = 1;
  __syncwarp();
  while (sp > 0) {
    sp--;
    int f = s.stack[3 * sp], l = s.stack[3 * sp + 1], depth = s.stack[3 * sp + 2];
    __syncwarp();
    while (l - f > 16) {
      if (depth == 0) {
        // std::__partial_sort(f, l, l): heapsort; sorted, so no insertion range
        if (lane == 0) {
          stl::make_heap(a + f, l - f, less);
          stl::sort_heap(a + f, l - f, less);
        }
        __syncwarp();
        f = l;
        break;
      }
      --depth;
      const int m = l - f;
      if (lane == 0) stl::move_median_to_first(a + f, a + f + 1, a + f + m / 2, a + l - 1, less);
      __syncwarp();
      const T P = a[f];
      const int M = m - 1;
      const T *r = a + f + 1;
      // left stops (not < P) ascending, right stops (P not <) descending
      int na = 0, nb = 0;
      for (int b = 0; b < M; b += 32) {
        const int p = b + lane;
        const bool isl = p < M && !less(r[p], P);
        const unsigned bl = __ballot_sync(FULLM, isl);
        if (isl) s.apos[na + __popc(bl & lt)] = p;
        na += __popc(bl);
        const int q = M - 1 - p;
        const bool isr = p < M && !less(P, r[q]);
        const unsigned br = __ballot_sync(FULLM, isr);
        if (isr) s.bpos[nb + __popc(br & lt)] = q;
        nb += __popc(br);
      }
      __syncwarp();
      const int lim = min(na, nb);
      int K = lim;
      for (int b = 0; b < lim; b += 32) {
        const int k = b + lane;
        const bool stop = k < lim && !(s.apos[k] < s.bpos[k]);
        const unsigned bs = __ballot_sync(FULLM, stop);
        if (bs) {
          K = b + __ffs(bs) - 1;
          break;
        }
      }
      int cut;
      if (K == 0) {
        cut = s.apos[0];
      } else {
        cut = s.bpos[K - 1];
        if (K < na) cut = min(cut, s.apos[K]);
      }
      for (int k = lane; k < K; k += 32) {
        T t = a[f + 1 + s.apos[k]];
        a[f + 1 + s.apos[k]] = a[f + 1 + s.bpos[k]];
        a[f + 1 + s.bpos[k]] = t;
      }
      __syncwarp();
      const int c = f + 1 + cut;
      // right part later (same depth), left part now
      if (lane == 0) {
        s.stack[3 * sp] = c;
        s.stack[3 * sp + 1] = l;
        s.stack[3 * sp + 2] = depth;
      }
      sp++;
      l = c;
      __syncwarp();
    }
    if (l - f > 1) {
      if (lane == 0) {
        s.leaf[2 * nleaf] = f;
        s.leaf[2 * nleaf + 1] = l;
      }
      nleaf++;
      __syncwarp();
      if (nleaf == 32) {
        flush_leaves(a, less, s.leaf, nleaf, lane);
        nleaf = 0;
      }
    }
    __syncwarp();
  }
  // the final insertion sort, range by range (ranges are disjoint)
  flush_leaves(a, less, s.leaf, nleaf, lane);
}

}  // namespace wv
