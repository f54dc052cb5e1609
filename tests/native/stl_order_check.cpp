// Checks weavess_gb300/csrc/stl_order.cuh against the host libstdc++ on
// tie-heavy arrays: same final order of (key, payload) pairs after every
// operation.  Prints "OK <cases>" or the first mismatch.
#include <algorithm>
#include <cstdio>
#include <random>
#include <vector>
#include "../../weavess_gb300/csrc/stl_order.cuh"

struct E {
  float d;
  unsigned id;
  bool operator<(const E &o) const { return d < o.d; }
};
struct Lt {
  bool operator()(const E &a, const E &b) const { return a.d < b.d; }
};
struct Gt {  // Index::MinHeap item order (key > other.key)
  bool operator()(const E &a, const E &b) const { return a.d > b.d; }
};
static bool same(const std::vector<E> &a, const std::vector<E> &b) {
  for (size_t i = 0; i < a.size(); i++)
    if (a[i].d != b[i].d || a[i].id != b[i].id) return false;
  return true;
}
int main() {
  std::mt19937 rng(123);
  int cases = 0;
  for (int trial = 0; trial < 4000; trial++) {
    int n = trial % 7 == 0 ? (int)(rng() % 2000) : (int)(rng() % 300);
    int levels = 1 + (int)(rng() % (trial % 3 == 0 ? 3 : 50));
    std::vector<E> a(n);
    for (int i = 0; i < n; i++) a[i] = E{(float)(rng() % levels), (unsigned)i};
    // sort
    std::vector<E> x = a, y = a;
    std::sort(x.begin(), x.end());
    wv::stl::sort(y.data(), n, Lt());
    if (!same(x, y)) { printf("sort mismatch n=%d levels=%d\n", n, levels); return 1; }
    // sorted input with descending values (depth-limit heapsort path)
    std::vector<E> s = a;
    for (int i = 0; i < n; i++) s[i].d = (float)((i * 7919) % (levels + 1));
    x = s; y = s;
    std::sort(x.begin(), x.end());
    wv::stl::sort(y.data(), n, Lt());
    if (!same(x, y)) { printf("sort2 mismatch n=%d\n", n); return 1; }
    // make_heap
    x = a; y = a;
    std::make_heap(x.begin(), x.end());
    wv::stl::make_heap(y.data(), n, Lt());
    if (!same(x, y)) { printf("make_heap mismatch n=%d\n", n); return 1; }
    // push / pop sequences, both orders
    std::vector<E> hx, hy;
    for (int i = 0; i < n; i++) {
      if (rng() % 3 == 0 && !hx.empty()) {
        std::pop_heap(hx.begin(), hx.end());
        hx.pop_back();
        wv::stl::pop_heap(hy.data(), (int)hy.size(), Lt());
        hy.pop_back();
      } else {
        hx.push_back(a[i]);
        std::push_heap(hx.begin(), hx.end());
        hy.push_back(a[i]);
        wv::stl::push_heap(hy.data(), (int)hy.size(), Lt());
      }
      if (!same(hx, hy)) { printf("push/pop mismatch n=%d i=%d\n", n, i); return 1; }
    }
    std::vector<E> gx, gy;
    for (int i = 0; i < n; i++) {
      gx.push_back(a[i]);
      std::push_heap(gx.begin(), gx.end(), Gt());
      gy.push_back(a[i]);
      wv::stl::push_heap(gy.data(), (int)gy.size(), Gt());
    }
    while (!gx.empty()) {
      std::pop_heap(gx.begin(), gx.end(), Gt());
      gx.pop_back();
      wv::stl::pop_heap(gy.data(), (int)gy.size(), Gt());
      gy.pop_back();
      if (!same(gx, gy)) { printf("min-heap mismatch n=%d\n", n); return 1; }
    }
    cases++;
  }
  printf("OK %d\n", cases);
  return 0;
}
