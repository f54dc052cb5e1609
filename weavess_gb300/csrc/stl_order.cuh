// Order-exact restatements of the GNU libstdc++ sorting and heap algorithms
// that WEAVESS calls on its hot path (std::sort, std::make_heap,
// std::push_heap, std::pop_heap).  When distances tie, the reference's output
// order is whatever these algorithms leave, so the GPU path runs the same
// steps (one thread per array) wherever a tie could change the result.
//
// The algorithms are the published libstdc++ ones (introsort with a
// median-of-three pivot, threshold 16, heapsort fallback at depth
// 2*floor(log2 n), final insertion sort; Floyd heap construction with the
// hole/sift-down-then-up adjust).  tests/test_stl_order.py checks every routine
// against the host's std:: on tie-heavy inputs.
//
// Usable from host and device code.  `Less` is a functor bool(const T&, const T&).
#pragma once

#ifdef __CUDACC__
#define WV_HD __host__ __device__ __forceinline__
#else
#define WV_HD inline
#endif

namespace wv {
namespace stl {

template <class T>
WV_HD void swap_(T &a, T &b) {
  T t = a;
  a = b;
  b = t;
}

WV_HD int lg2(int n) {  // floor(log2(n)), n > 0
  int r = 0;
  while (n >>= 1) r++;
  return r;
}

// ---- heap ----
// The heap routines take any handle `first` with first[i] yielding an
// assignable element (a plain pointer, or an array split across memories).
template <class P, class T, class Less>
WV_HD void push_heap_hole(P first, int hole, int top, T value, Less less) {
  int parent = (hole - 1) / 2;
  while (hole > top && less(first[parent], value)) {
    first[hole] = first[parent];
    hole = parent;
    parent = (hole - 1) / 2;
  }
  first[hole] = value;
}

template <class P, class T, class Less>
WV_HD void adjust_heap(P first, int hole, int len, T value, Less less) {
  const int top = hole;
  int child = hole;
  while (child < (len - 1) / 2) {
    child = 2 * (child + 1);
    if (less(first[child], first[child - 1])) child--;
    first[hole] = first[child];
    hole = child;
  }
  if ((len & 1) == 0 && child == (len - 2) / 2) {
    child = 2 * (child + 1);
    first[hole] = first[child - 1];
    hole = child - 1;
  }
  push_heap_hole(first, hole, top, value, less);
}

template <class P, class Less>
WV_HD void make_heap(P first, int len, Less less) {
  if (len < 2) return;
  int parent = (len - 2) / 2;
  while (true) {
    auto value = first[parent];
    adjust_heap(first, parent, len, value, less);
    if (parent == 0) return;
    parent--;
  }
}

// std::push_heap(first, first + len): the new element is first[len - 1]
template <class P, class Less>
WV_HD void push_heap(P first, int len, Less less) {
  auto value = first[len - 1];
  push_heap_hole(first, len - 1, 0, value, less);
}

// moves *first into *result and re-heaps [first, first + len)
template <class T, class Less>
WV_HD void pop_heap_into(T *first, int len, T *result, Less less) {
  T value = *result;
  *result = *first;
  adjust_heap(first, 0, len, value, less);
}

// std::pop_heap(first, first + len)
template <class P, class Less>
WV_HD void pop_heap(P first, int len, Less less) {
  if (len > 1) {
    auto value = first[len - 1];
    first[len - 1] = first[0];
    adjust_heap(first, 0, len - 1, value, less);
  }
}

template <class T, class Less>
WV_HD void sort_heap(T *first, int len, Less less) {
  while (len > 1) {
    --len;
    pop_heap_into(first, len, first + len, less);
  }
}

// ---- introsort ----
template <class T, class Less>
WV_HD void move_median_to_first(T *result, T *a, T *b, T *c, Less less) {
  if (less(*a, *b)) {
    if (less(*b, *c)) swap_(*result, *b);
    else if (less(*a, *c)) swap_(*result, *c);
    else swap_(*result, *a);
  } else if (less(*a, *c)) swap_(*result, *a);
  else if (less(*b, *c)) swap_(*result, *c);
  else swap_(*result, *b);
}

template <class T, class Less>
WV_HD T *unguarded_partition(T *first, T *last, T *pivot, Less less) {
  while (true) {
    while (less(*first, *pivot)) ++first;
    --last;
    while (less(*pivot, *last)) --last;
    if (!(first < last)) return first;
    swap_(*first, *last);
    ++first;
  }
}

template <class T, class Less>
WV_HD void unguarded_linear_insert(T *last, Less less) {
  T val = *last;
  T *next = last - 1;
  while (less(val, *next)) {
    *last = *next;
    last = next;
    --next;
  }
  *last = val;
}

template <class T, class Less>
WV_HD void insertion_sort(T *first, T *last, Less less) {
  if (first == last) return;
  for (T *i = first + 1; i != last; ++i) {
    if (less(*i, *first)) {
      T val = *i;
      for (T *p = i; p != first; --p) *p = *(p - 1);
      *first = val;
    } else {
      unguarded_linear_insert(i, less);
    }
  }
}

// std::sort(first, first + n).  The recursion on the right part is replaced by
// an explicit stack; the parts are disjoint, so the order in which they are
// finished does not change the result.
template <class T, class Less>
WV_HD void sort(T *first, int n, Less less) {
  if (n <= 1) return;
  const int threshold = 16;
  struct Part {
    T *f, *l;
    int depth;
  } stack[64];
  int sp = 0;
  stack[sp++] = Part{first, first + n, 2 * lg2(n)};
  while (sp > 0) {
    Part p = stack[--sp];
    T *f = p.f, *l = p.l;
    int depth = p.depth;
    while (l - f > threshold) {
      if (depth == 0) {  // std::__partial_sort(f, l, l): heapsort
        make_heap(f, (int)(l - f), less);
        sort_heap(f, (int)(l - f), less);
        break;
      }
      --depth;
      T *mid = f + (l - f) / 2;
      move_median_to_first(f, f + 1, mid, l - 1, less);
      T *cut = unguarded_partition(f + 1, l, f, less);
      stack[sp++] = Part{cut, l, depth};
      l = cut;
    }
  }
  if (n > threshold) {
    insertion_sort(first, first + threshold, less);
    for (T *i = first + threshold; i != first + n; ++i) unguarded_linear_insert(i, less);
  } else {
    insertion_sort(first, first + n, less);
  }
}

}  // namespace stl
}  // namespace wv
