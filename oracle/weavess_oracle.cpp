// ORACLE -- test infrastructure only.
//
// A plain C++ restatement of the WEAVESS hot path, used by tests/ (and by the
// CPU-baseline leg of bench.py) as the checker for the GPU implementation.
// Nothing in the product links, loads or calls this file.  Its parity with the
// reference itself is pinned by tests/test_oracle_golden.py against fixtures
// produced by the unmodified reference sources (oracle/ref_driver.cpp,
// tests/golden/make_golden.py).
//
// Every routine cites the reference function it restates.  Single-threaded
// calls reproduce the reference's single-threaded results bit for bit,
// including the glibc rand() stream, std::sort/std::make_heap tie behaviour
// and the reference's known defects.  With threads > 1 the OpenMP structure of
// the reference is kept (the results are then as nondeterministic as the
// reference's; this mode is only used for timing).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <random>
#include <stack>
#include <queue>
#include <set>
#include <vector>
#include <omp.h>

namespace {

// ---------------------------------------------------------------- rand()
// glibc's default rand() (TYPE_3 additive feedback generator, degree 31,
// separation 3): r[i] = r[i-31] + r[i-3] mod 2^32, output r[i] >> 1, with a
// Lehmer (16807) seeding of the first 31 words and 310 discarded outputs.
// This is the generator the reference's rand() calls draw from (srand is never
// called on the hot path, so the seed is glibc's default 1).
struct GlibcRand {
  uint32_t r[34];
  int i = 0;  // ring position
  std::mutex mu;
  explicit GlibcRand(uint32_t seed) { reseed(seed); }
  void reseed(uint32_t seed) {
    if (seed == 0) seed = 1;
    int32_t w[34];
    w[0] = (int32_t)seed;
    for (int k = 1; k < 31; k++) {
      // 16807 * w mod (2^31 - 1) via Schrage's method, as glibc does
      int32_t hi = w[k - 1] / 127773, lo = w[k - 1] % 127773;
      int32_t word = 16807 * lo - 2836 * hi;
      if (word < 0) word += 2147483647;
      w[k] = word;
    }
    for (int k = 31; k < 34; k++) w[k] = w[k - 31];
    for (int k = 0; k < 34; k++) r[k] = (uint32_t)w[k];
    i = 0;
    // ring holds the last 34 words; position i is the oldest
    for (int k = 0; k < 310; k++) step();
  }
  // advance: new word = r[n-31] + r[n-3]; return it
  uint32_t step() {
    // ring of 34 words where r[(i + 34 - m) % 34] is r[n - m] for the next n
    uint32_t v = r[(i + 34 - 31) % 34] + r[(i + 34 - 3) % 34];
    r[i] = v;
    i = (i + 1) % 34;
    return v;
  }
  int next() { return (int)(step() >> 1); }
  int next_locked() {
    std::lock_guard<std::mutex> g(mu);
    return next();
  }
};

// ---------------------------------------------------------------- distance
// Distance::compare (include/weavess/distance.h:12-36): groups of four,
// result += d0*d0 + d1*d1 + d2*d2 + d3*d3 in that order, then the tail.
// Built with -ffp-contract=off so no FMA changes the rounding.
inline float l2(const float *a, const float *b, unsigned d) {
  float result = 0;
  unsigned k = 0;
  for (; k + 3 < d; k += 4) {
    float d0 = a[k] - b[k], d1 = a[k + 1] - b[k + 1], d2 = a[k + 2] - b[k + 2], d3 = a[k + 3] - b[k + 3];
    result += d0 * d0 + d1 * d1 + d2 * d2 + d3 * d3;
  }
  for (; k < d; k++) {
    float t = a[k] - b[k];
    result += t * t;
  }
  return result;
}

struct Neighbor {  // NNDescent::Neighbor (index.h:66-82)
  unsigned id;
  float distance;
  bool flag;
  Neighbor() = default;
  Neighbor(unsigned i, float dd, bool f) : id(i), distance(dd), flag(f) {}
  bool operator<(const Neighbor &o) const { return distance < o.distance; }
};
struct SimpleNeighbor {  // Index::SimpleNeighbor (index.h:1530-1541)
  unsigned id;
  float distance;
  SimpleNeighbor() = default;
  SimpleNeighbor(unsigned i, float dd) : id(i), distance(dd) {}
  bool operator<(const SimpleNeighbor &o) const { return distance < o.distance; }
};

// Index::MinHeap (index.h:339-382): std heap with an inverted comparator
struct MinHeapItem {
  float key;
  SimpleNeighbor data;
  bool operator<(const MinHeapItem &o) const { return key > o.key; }
};
struct MinHeap {
  std::vector<MinHeapItem> v;
  void push(float k, const SimpleNeighbor &d) {
    v.push_back(MinHeapItem{k, d});
    std::push_heap(v.begin(), v.end());
  }
  const MinHeapItem &top() const { return v[0]; }
  void pop() {
    std::pop_heap(v.begin(), v.end());
    v.pop_back();
  }
  size_t size() const { return v.size(); }
};

// NNDescent::InsertIntoPool (index.h:152-180)
int insert_into_pool(Neighbor *addr, unsigned K, Neighbor nn) {
  int left = 0, right = (int)K - 1;
  if (addr[left].distance > nn.distance) {
    memmove((char *)&addr[left + 1], &addr[left], K * sizeof(Neighbor));
    addr[left] = nn;
    return left;
  }
  if (addr[right].distance < nn.distance) {
    addr[K] = nn;
    return (int)K;
  }
  while (left < right - 1) {
    int mid = (left + right) / 2;
    if (addr[mid].distance > nn.distance) right = mid;
    else left = mid;
  }
  while (left > 0) {
    if (addr[left].distance < nn.distance) break;
    if (addr[left].id == nn.id) return (int)K + 1;
    left--;
  }
  if (addr[left].id == nn.id || addr[right].id == nn.id) return (int)K + 1;
  memmove((char *)&addr[right + 1], &addr[right], (K - right) * sizeof(Neighbor));
  addr[right] = nn;
  return right;
}

// GenRandom (util.h:13-27; same body as ComponentInitRandom::GenRandom,
// component_init.cpp:51-68)
void gen_random(std::mt19937 &rng, unsigned *addr, unsigned size, unsigned N) {
  for (unsigned i = 0; i < size; ++i) addr[i] = rng() % (N - size);
  std::sort(addr, addr + size);
  for (unsigned i = 1; i < size; ++i)
    if (addr[i] <= addr[i - 1]) addr[i] = addr[i - 1] + 1;
  unsigned off = rng() % N;
  for (unsigned i = 0; i < size; ++i) addr[i] = (addr[i] + off) % N;
}

struct Data {
  const float *base;
  unsigned n, d;
  const float *row(size_t i) const { return base + i * (size_t)d; }
};

typedef std::vector<std::vector<SimpleNeighbor>> FinalGraph;

FinalGraph graph_from_arrays(const unsigned *ids, const float *dist, const unsigned *deg, unsigned n, unsigned w) {
  FinalGraph g(n);
  for (unsigned i = 0; i < n; i++) {
    g[i].reserve(deg[i]);
    for (unsigned j = 0; j < deg[i]; j++) g[i].emplace_back(ids[(size_t)i * w + j], dist ? dist[(size_t)i * w + j] : 0.f);
  }
  return g;
}

int graph_to_arrays(const FinalGraph &g, unsigned *ids, float *dist, unsigned *deg, unsigned w) {
  for (size_t i = 0; i < g.size(); i++) {
    if (g[i].size() > w) return -1;
    deg[i] = (unsigned)g[i].size();
    for (size_t j = 0; j < g[i].size(); j++) {
      ids[i * w + j] = g[i][j].id;
      if (dist) dist[i * w + j] = g[i][j].distance;
    }
  }
  return 0;
}

// ---------------------------------------------------------------- NN-Descent
struct NHood {  // NNDescent::nhood (index.h:86-150)
  std::mutex lock;
  std::vector<Neighbor> pool;
  unsigned M = 0;
  std::vector<unsigned> nn_old, nn_new, rnn_old, rnn_new;
};

struct NNDescent {
  const Data &D;
  unsigned S, K, L, ITER, R;
  GlibcRand &rnd;
  int threads;
  std::vector<NHood> graph;
  uint64_t overflow_events = 0, dist_evals = 0;

  NNDescent(const Data &d, unsigned s, unsigned k, unsigned l, unsigned it, unsigned r, GlibcRand &rr, int th)
      : D(d), S(s), K(k), L(l), ITER(it), R(r), rnd(rr), threads(th), graph(d.n) {}

  // nhood::insert (index.h:120-135); pool capacity is L (reserved once)
  void insert(unsigned t, unsigned id, float dist) {
    NHood &h = graph[t];
    std::lock_guard<std::mutex> guard(h.lock);
    if (dist > h.pool.front().distance) return;
    for (unsigned i = 0; i < h.pool.size(); i++)
      if (id == h.pool[i].id) return;
    if (h.pool.size() < L) {
      h.pool.push_back(Neighbor(id, dist, true));
      std::push_heap(h.pool.begin(), h.pool.end());
    } else {
      std::pop_heap(h.pool.begin(), h.pool.end());
      h.pool[h.pool.size() - 1] = Neighbor(id, dist, true);
      std::push_heap(h.pool.begin(), h.pool.end());
    }
  }

  // ComponentRefineNNDescent::init (component_refine.cpp:87-104); nhood(L,S)
  // leaves nn_new as 2S zeros (index.h:98-103), so the first join does nothing
  void init(const FinalGraph &fg) {
    for (unsigned i = 0; i < D.n; i++) {
      graph[i].M = S;
      graph[i].nn_new.assign(2 * S, 0u);
      graph[i].pool.reserve(L);
      for (auto &nb : fg[i]) graph[i].pool.emplace_back(nb.id, nb.distance, true);
      std::make_heap(graph[i].pool.begin(), graph[i].pool.end());
    }
  }

  // ComponentRefineEFANNA::init (component_refine.cpp:1036-1058): one rand()
  // seeds an mt19937 from which nhood(L, S, rng, N) (index.h:105-111) draws
  // 2S random ids into each node's nn_new in node order (GenRandom); the
  // pool takes the node's row sorted by distance (std::sort), skipping the
  // node itself and an id equal to its predecessor in that order.  The
  // first join therefore has work to do.
  void init_efanna(FinalGraph fg) {
    std::mt19937 rng(rnd.next());
    for (unsigned i = 0; i < D.n; i++) {
      graph[i].M = S;
      graph[i].nn_new.assign(2 * S, 0u);
      gen_random(rng, graph[i].nn_new.data(), 2 * S, D.n);
      graph[i].pool.reserve(L);
    }
    for (unsigned i = 0; i < D.n; i++) {
      auto &ids = fg[i];
      std::sort(ids.begin(), ids.end());
      for (unsigned j = 0; j < ids.size(); j++) {
        const unsigned id = ids[j].id;
        if (id == i || (j > 0 && id == ids[j - 1].id)) continue;
        graph[i].pool.emplace_back(id, ids[j].distance, true);
      }
      std::make_heap(graph[i].pool.begin(), graph[i].pool.end());
    }
  }

  // ComponentRefineNNDescent::join (component_refine.cpp:127-143) with
  // nhood::join (index.h:137-149)
  void join() {
#pragma omp parallel for schedule(dynamic, 100) num_threads(threads)
    for (unsigned n = 0; n < D.n; n++) {
      auto cb = [&](unsigned i, unsigned j) {
        if (i != j) {
          float dist = l2(D.row(i), D.row(j), D.d);
          insert(i, j, dist);
          insert(j, i, dist);
        }
      };
      const NHood &h = graph[n];
      for (unsigned const i : h.nn_new) {
        for (unsigned const j : h.nn_new)
          if (i < j) cb(i, j);
        for (unsigned j : h.nn_old) cb(i, j);
      }
    }
  }

  // ComponentRefineNNDescent::update (component_refine.cpp:145-239)
  void update() {
#pragma omp parallel for num_threads(threads)
    for (unsigned i = 0; i < D.n; i++) {
      std::vector<unsigned>().swap(graph[i].nn_new);
      std::vector<unsigned>().swap(graph[i].nn_old);
    }
#pragma omp parallel for num_threads(threads)
    for (unsigned n = 0; n < D.n; ++n) {
      auto &nn = graph[n];
      std::sort(nn.pool.begin(), nn.pool.end());
      if (nn.pool.size() > L) nn.pool.resize(L);
      unsigned maxl = std::min(nn.M + S, (unsigned)nn.pool.size());
      unsigned c = 0, l = 0;
      while ((l < maxl) && (c < S)) {
        if (nn.pool[l].flag) ++c;
        ++l;
      }
      nn.M = l;
    }
#pragma omp parallel for num_threads(threads)
    for (unsigned n = 0; n < D.n; ++n) {
      auto &nnhd = graph[n];
      for (unsigned l = 0; l < nnhd.M; ++l) {
        auto &nn = nnhd.pool[l];
        auto &nhood_o = graph[nn.id];
        // pool.back() of the other node: the max if it is still sorted, the
        // last slot of its heap if it was already make_heap'd this pass
        if (nn.flag) {
          nnhd.nn_new.push_back(nn.id);
          if (nn.distance > nhood_o.pool.back().distance) {
            std::lock_guard<std::mutex> guard(nhood_o.lock);
            if (nhood_o.rnn_new.size() < R) nhood_o.rnn_new.push_back(n);
            else {
              unsigned pos = (unsigned)rnd.next_locked() % R;
              nhood_o.rnn_new[pos] = n;
              overflow_events++;
            }
          }
          nn.flag = false;
        } else {
          nnhd.nn_old.push_back(nn.id);
          if (nn.distance > nhood_o.pool.back().distance) {
            std::lock_guard<std::mutex> guard(nhood_o.lock);
            if (nhood_o.rnn_old.size() < R) nhood_o.rnn_old.push_back(n);
            else {
              unsigned pos = (unsigned)rnd.next_locked() % R;
              nhood_o.rnn_old[pos] = n;
              overflow_events++;
            }
          }
        }
      }
      std::make_heap(nnhd.pool.begin(), nnhd.pool.end());
    }
#pragma omp parallel for num_threads(threads)
    for (unsigned i = 0; i < D.n; ++i) {
      auto &g = graph[i];
      // the random_shuffle branches of the reference are unreachable: the
      // reverse lists are capped at R when they are filled
      g.nn_new.insert(g.nn_new.end(), g.rnn_new.begin(), g.rnn_new.end());
      g.nn_old.insert(g.nn_old.end(), g.rnn_old.begin(), g.rnn_old.end());
      if (g.nn_old.size() > R * 2) g.nn_old.resize(R * 2);
      std::vector<unsigned>().swap(g.rnn_new);
      std::vector<unsigned>().swap(g.rnn_old);
    }
  }

  // RefineInner tail (component_refine.cpp:21-74): sort pools, naive prune to K
  FinalGraph finish() {
    FinalGraph fg(D.n);
    for (unsigned i = 0; i < D.n; i++) {
      std::sort(graph[i].pool.begin(), graph[i].pool.end());
      unsigned len = std::min<unsigned>((unsigned)graph[i].pool.size(), K);  // PruneNaive
      for (unsigned j = 0; j < len; j++) fg[i].emplace_back(graph[i].pool[j].id, graph[i].pool[j].distance);
    }
    return fg;
  }
};

// ComponentInitRandom::InitInner (component_init.cpp:11-45)
FinalGraph init_random(const Data &D, unsigned S, GlibcRand &rnd) {
  FinalGraph g(D.n);
  std::mt19937 rng(rnd.next());
  std::vector<unsigned> tmp(S);
  for (unsigned i = 0; i < D.n; i++) {
    g[i].reserve(S);
    gen_random(rng, tmp.data(), S, D.n);
    for (unsigned j = 0; j < S; j++) {
      unsigned id = tmp[j];
      if (id == i) continue;
      g[i].emplace_back(id, l2(D.row(i), D.row(id), D.d));
    }
    std::sort(g[i].begin(), g[i].end());
  }
  return g;
}

// ComponentInitRand::InitInner (component_init.cpp:979-1025), the Vamana
// init: one rand() seeds an mt19937 from which every node, in node order,
// draws L ids (GenRandom); the node itself is skipped; the pool (Neighbor,
// flag true) is make_heap'd, then std::sort'ed -- the heap arrangement is
// the order the sort starts from, which decides equal distances
FinalGraph init_rand(const Data &D, unsigned L, GlibcRand &rnd) {
  FinalGraph g(D.n);
  std::mt19937 rng(rnd.next());
  std::vector<unsigned> tmp(L);
  std::vector<Neighbor> pool;
  for (unsigned i = 0; i < D.n; i++) {
    gen_random(rng, tmp.data(), L, D.n);
    pool.clear();
    for (unsigned j = 0; j < L; j++) {
      const unsigned id = tmp[j];
      if (id == i) continue;
      pool.emplace_back(id, l2(D.row(i), D.row(id), D.d), true);
    }
    std::make_heap(pool.begin(), pool.end());
    std::sort(pool.begin(), pool.end());
    g[i].reserve(pool.size());
    for (auto &x : pool) g[i].emplace_back(x.id, x.distance);
  }
  return g;
}

// ---------------------------------------------------------------- greedy searches
// Seeds for a build-time greedy search: the first L ids of `enter`'s row, then
// rand() % N draws that skip flagged ids (component_candidate.cpp:17-31,
// component_entry.cpp:39-52, component_conn.cpp:93-106).
void build_seeds(const FinalGraph &g, unsigned enter, unsigned L, unsigned N, GlibcRand &rnd,
                 std::vector<unsigned> &init_ids, std::vector<char> &flags) {
  init_ids.assign(L, 0);
  unsigned l = 0;
  for (unsigned i = 0; i < init_ids.size() && i < g[enter].size(); i++) {
    init_ids[i] = g[enter][i].id;
    flags[init_ids[i]] = 1;
    l++;
  }
  while (l < init_ids.size()) {
    unsigned id = (unsigned)rnd.next_locked() % N;
    if (flags[id]) continue;
    init_ids[l] = id;
    l++;
    flags[id] = 1;
  }
}

// The greedy loop shared by CandidateNSG::CandidateInner
// (component_candidate.cpp:46-81), EntryCentroid::get_neighbors
// (component_entry.cpp:66-91) and ConnNSGDFS::get_neighbors
// (component_conn.cpp:121-159).  `visit` is called with every newly flagged
// (id, dist) in visit order.
template <class F>
void greedy_expand(const Data &D, const FinalGraph &g, const float *q, std::vector<Neighbor> &retset, unsigned L,
                   std::vector<char> &flags, F visit) {
  int k = 0;
  while (k < (int)L) {
    int nk = (int)L;
    if (retset[k].flag) {
      retset[k].flag = false;
      unsigned n = retset[k].id;
      for (unsigned m = 0; m < g[n].size(); ++m) {
        unsigned id = g[n][m].id;
        if (flags[id]) continue;
        flags[id] = 1;
        float dist = l2(q, D.row(id), D.d);
        Neighbor nn(id, dist, true);
        visit(nn);
        if (dist >= retset[L - 1].distance) continue;
        int r = insert_into_pool(retset.data(), L, nn);
        if (L + 1 < retset.size()) ++L;
        if (r < nk) nk = r;
      }
    }
    if (nk <= k) k = nk;
    else ++k;
  }
}

// ComponentCandidateNSG::CandidateInner (component_candidate.cpp:10-85)
void candidate_nsg(const Data &D, const FinalGraph &g, unsigned query, unsigned enter, unsigned Lr, GlibcRand &rnd,
                   std::vector<SimpleNeighbor> &result, std::vector<char> &flags) {
  std::vector<unsigned> init_ids;
  build_seeds(g, enter, Lr, D.n, rnd, init_ids, flags);
  std::vector<Neighbor> retset(Lr + 1);
  unsigned L = 0;
  for (unsigned i = 0; i < init_ids.size(); i++) {
    unsigned id = init_ids[i];
    float dist = l2(D.row(id), D.row(query), D.d);
    retset[i] = Neighbor(id, dist, true);
    result.emplace_back(id, dist);
    L++;
  }
  std::sort(retset.begin(), retset.begin() + L);
  greedy_expand(D, g, D.row(query), retset, L, flags,
                [&](const Neighbor &nn) { result.push_back(SimpleNeighbor(nn.id, nn.distance)); });
}

// greedy search for an arbitrary vector (EntryCentroid / ConnNSGDFS
// get_neighbors); returns retset, fills fullset with the expansion visits
void get_neighbors(const Data &D, const FinalGraph &g, unsigned ep, const float *q, unsigned Lr, GlibcRand &rnd,
                   std::vector<Neighbor> &retset, std::vector<Neighbor> *fullset) {
  std::vector<char> flags(D.n, 0);
  std::vector<unsigned> init_ids;
  build_seeds(g, ep, Lr, D.n, rnd, init_ids, flags);
  retset.assign(Lr + 1, Neighbor(0, 0.f, false));
  unsigned L = 0;
  for (unsigned i = 0; i < init_ids.size(); i++) {
    unsigned id = init_ids[i];
    retset[i] = Neighbor(id, l2(D.row(id), q, D.d), true);
    L++;
  }
  std::sort(retset.begin(), retset.begin() + L);
  greedy_expand(D, g, q, retset, L, flags, [&](const Neighbor &nn) {
    if (fullset) fullset->push_back(nn);
  });
}

// ComponentRefineEntryCentroid::EntryInner (component_entry.cpp:9-28).
// `entry_L` is the index's L_refine member: the NSG refine sets it, the
// Vamana refine never does, so there it is 0 and ep_ ends as node 0.
unsigned entry_centroid(const Data &D, const FinalGraph &g, unsigned entry_L, GlibcRand &rnd) {
  std::vector<float> center(D.d, 0.f);
  for (unsigned i = 0; i < D.n; i++)
    for (unsigned j = 0; j < D.d; j++) center[j] += D.row(i)[j];
  for (unsigned j = 0; j < D.d; j++) center[j] /= D.n;
  unsigned ep = (unsigned)rnd.next() % D.n;
  std::vector<Neighbor> tmp;
  if (entry_L == 0) return 0;  // retset of one value-initialised Neighbor
  get_neighbors(D, g, ep, center.data(), entry_L, rnd, tmp, nullptr);
  return tmp[0].id;
}

// ComponentPruneNSG::PruneInner (component_prune.cpp:20-69)
void prune_nsg(const Data &D, const FinalGraph &g, unsigned query, unsigned range, unsigned maxc,
               std::vector<SimpleNeighbor> &pool, SimpleNeighbor *cut_graph) {
  unsigned start = 0;
  for (unsigned nn = 0; nn < g[query].size(); nn++) {
    unsigned id = g[query][nn].id;
    pool.push_back(SimpleNeighbor(id, l2(D.row(query), D.row(id), D.d)));
  }
  std::sort(pool.begin(), pool.end());
  std::vector<SimpleNeighbor> result;
  if (pool[start].id == query) start++;
  result.push_back(pool[start]);
  while (result.size() < range && (++start) < pool.size() && start < maxc) {
    auto &p = pool[start];
    bool occlude = false;
    for (unsigned t = 0; t < result.size(); t++) {
      if (p.id == result[t].id) {
        occlude = true;
        break;
      }
      float djk = l2(D.row(result[t].id), D.row(p.id), D.d);
      if (djk < p.distance) {
        occlude = true;
        break;
      }
    }
    if (!occlude) result.push_back(p);
  }
  SimpleNeighbor *des = cut_graph + (size_t)query * range;
  for (size_t t = 0; t < result.size(); t++) des[t] = result[t];
  if (result.size() < range) des[result.size()].distance = -1;
}

// ComponentPruneVAMANA::PruneInner (component_prune.cpp:245-300)
void prune_vamana(const Data &D, const FinalGraph &g, unsigned query, unsigned range, float alpha,
                  std::vector<SimpleNeighbor> &pool, SimpleNeighbor *cut_graph, bool clean = false) {
  std::vector<SimpleNeighbor> picked;
  if (clean) {
    // clean mode (this library's WV_BUILD_CLEAN, not the reference): the
    // pool is the visited set plus the node's own row (DiskANN's RobustPrune
    // prunes V u N_out(p)), sorted whatever its size; the node itself and
    // ids already picked are dropped, not skipped; the refill takes an id
    // once
    for (unsigned nn = 0; nn < g[query].size(); nn++) {
      unsigned id = g[query][nn].id;
      pool.push_back(SimpleNeighbor(id, l2(D.row(query), D.row(id), D.d)));
    }
    std::sort(pool.begin(), pool.end());
    MinHeap skipped;
    auto taken = [&](unsigned id) {
      for (auto &x : picked)
        if (x.id == id) return true;
      return false;
    };
    for (size_t i = 0; i < pool.size(); i++) {
      if (pool[i].id == query || taken(pool[i].id)) continue;
      bool skip = false;
      float cur_dist = pool[i].distance;
      for (size_t j = 0; j < picked.size(); j++) {
        float dist = l2(D.row(picked[j].id), D.row(pool[i].id), D.d);
        if (alpha * dist < cur_dist) {
          skip = true;
          break;
        }
      }
      if (!skip) picked.push_back(pool[i]);
      else skipped.push(cur_dist, pool[i]);
      if (picked.size() == range) break;
    }
    while (picked.size() < range && skipped.size()) {
      if (!taken(skipped.top().data.id)) picked.push_back(skipped.top().data);
      skipped.pop();
    }
  } else if (pool.size() > range) {
    std::sort(pool.begin(), pool.end());
    MinHeap skipped;
    for (size_t i = 0; i < pool.size(); i++) {
      bool skip = false;
      float cur_dist = pool[i].distance;
      for (size_t j = 0; j < picked.size(); j++) {
        float dist = l2(D.row(picked[j].id), D.row(pool[i].id), D.d);
        if (alpha * dist < cur_dist) {
          skip = true;
          break;
        }
      }
      if (!skip) picked.push_back(pool[i]);
      else skipped.push(cur_dist, pool[i]);
      if (picked.size() == range) break;
    }
    while (picked.size() < range && skipped.size()) {
      picked.push_back(skipped.top().data);
      skipped.pop();
    }
  } else {
    for (size_t i = 0; i < pool.size(); i++) picked.push_back(pool[i]);
  }
  SimpleNeighbor *des = cut_graph + (size_t)query * range;
  for (size_t t = 0; t < picked.size(); t++) des[t] = picked[t];
  if (picked.size() < range) des[picked.size()].distance = -1;
}

// ComponentRefineNSG::InterInsert (component_refine.cpp:474-541) and
// ComponentRefineVAMANA::InterInsert (component_refine.cpp:874-950).  The
// Vamana re-prune reads temp_pool[i] (the outer index) as the distance to
// beat, as the reference does at component_refine.cpp:907.
void inter_insert(const Data &D, unsigned n, unsigned range, bool vamana, float alpha, std::vector<std::mutex> &locks,
                  SimpleNeighbor *cut_graph, bool clean = false) {
  SimpleNeighbor *src_pool = cut_graph + (size_t)n * range;
  for (size_t i = 0; i < range; i++) {
    if (src_pool[i].distance == -1) break;
    SimpleNeighbor sn(n, src_pool[i].distance);
    size_t des = src_pool[i].id;
    SimpleNeighbor *des_pool = cut_graph + des * range;
    std::vector<SimpleNeighbor> temp_pool;
    int dup = 0;
    {
      std::lock_guard<std::mutex> guard(locks[des]);
      for (size_t j = 0; j < range; j++) {
        if (des_pool[j].distance == -1) break;
        if (n == des_pool[j].id) {
          dup = 1;
          break;
        }
        temp_pool.push_back(des_pool[j]);
      }
    }
    if (dup) continue;
    temp_pool.push_back(sn);
    if (temp_pool.size() > range) {
      std::vector<SimpleNeighbor> result;
      std::sort(temp_pool.begin(), temp_pool.end());
      if (!vamana) {
        unsigned start = 0;
        result.push_back(temp_pool[start]);
        while (result.size() < range && (++start) < temp_pool.size()) {
          auto &p = temp_pool[start];
          bool occlude = false;
          for (unsigned t = 0; t < result.size(); t++) {
            if (p.id == result[t].id) {
              occlude = true;
              break;
            }
            float djk = l2(D.row(result[t].id), D.row(p.id), D.d);
            if (djk < p.distance) {
              occlude = true;
              break;
            }
          }
          if (!occlude) result.push_back(p);
        }
      } else {
        MinHeap skipped;
        // clean mode (WV_BUILD_CLEAN): closest first, each candidate against
        // its own distance -- the rule of PruneVAMANA
        for (int kk = 0; kk < (int)temp_pool.size(); ++kk) {
          const int k = clean ? kk : (int)temp_pool.size() - 1 - kk;
          bool skip = false;
          float cur_dist = clean ? temp_pool[k].distance : temp_pool[i].distance;
          for (size_t j = 0; j < result.size(); j++) {
            float dist = l2(D.row(result[j].id), D.row(temp_pool[k].id), D.d);
            if (alpha * dist < cur_dist) {
              skip = true;
              break;
            }
          }
          if (!skip) result.push_back(temp_pool[k]);
          else skipped.push(cur_dist, temp_pool[k]);
          if (result.size() == range) break;
        }
        while (result.size() < range && skipped.size()) {
          result.push_back(skipped.top().data);
          skipped.pop();
        }
      }
      std::lock_guard<std::mutex> guard(locks[des]);
      for (unsigned t = 0; t < result.size(); t++) des_pool[t] = result[t];
    } else {
      std::lock_guard<std::mutex> guard(locks[des]);
      for (unsigned t = 0; t < range; t++) {
        if (des_pool[t].distance == -1) {
          des_pool[t] = sn;
          if (t + 1 < range) des_pool[t + 1].distance = -1;
          break;
        }
      }
    }
  }
}

// cut_graph_ -> final_graph_ (component_refine.cpp:406-421, 807-824),
// including the reference's row length rule (an empty row keeps one entry)
FinalGraph cut_to_final(const std::vector<SimpleNeighbor> &cut, unsigned n, unsigned range) {
  FinalGraph fg(n);
  for (size_t i = 0; i < n; i++) {
    const SimpleNeighbor *pool = cut.data() + i * range;
    unsigned pool_size = 0;
    for (unsigned j = 0; j < range; j++) {
      if (pool[j].distance == -1) break;
      pool_size = j;
    }
    pool_size++;
    fg[i].assign(pool, pool + pool_size);
  }
  return fg;
}

// Link for both refines (component_refine.cpp:438-472, 835-872)
FinalGraph link(const Data &D, const FinalGraph &g, unsigned ep, unsigned Lr, unsigned Rr, unsigned Cr, bool vamana,
                float alpha, GlibcRand &rnd, int threads, bool clean = false) {
  std::vector<SimpleNeighbor> cut((size_t)D.n * Rr);
  std::vector<std::mutex> locks(D.n);
#pragma omp parallel num_threads(threads)
  {
    std::vector<SimpleNeighbor> pool;
    std::vector<char> flags(D.n);
#pragma omp for schedule(dynamic, 100)
    for (unsigned n = 0; n < D.n; ++n) {
      pool.clear();
      std::fill(flags.begin(), flags.end(), 0);
      candidate_nsg(D, g, n, ep, Lr, rnd, pool, flags);
      if (vamana) prune_vamana(D, g, n, Rr, alpha, pool, cut.data(), clean);
      else prune_nsg(D, g, n, Rr, Cr, pool, cut.data());
    }
#pragma omp for schedule(dynamic, 100)
    for (unsigned n = 0; n < D.n; ++n) inter_insert(D, n, Rr, vamana, alpha, locks, cut.data(), clean);
  }
  return cut_to_final(cut, D.n, Rr);
}

// ComponentConnNSGDFS (component_conn.cpp:10-166)
void conn_dfs(const Data &D, FinalGraph &g, unsigned ep, unsigned Lr, GlibcRand &rnd, unsigned *added) {
  std::vector<char> flag(D.n, 0);
  unsigned root = ep, cnt = 0;
  *added = 0;
  while (cnt < D.n) {
    // DFS (component_conn.cpp:30-58)
    unsigned tmp = root;
    std::stack<unsigned> s;
    s.push(root);
    if (!flag[root]) cnt++;
    flag[root] = 1;
    while (!s.empty()) {
      unsigned next = D.n + 1;
      for (unsigned i = 0; i < g[tmp].size(); i++)
        if (!flag[g[tmp][i].id]) {
          next = g[tmp][i].id;
          break;
        }
      if (next == D.n + 1) {
        s.pop();
        if (s.empty()) break;
        tmp = s.top();
        continue;
      }
      tmp = next;
      flag[tmp] = 1;
      s.push(tmp);
      cnt++;
    }
    if (cnt >= D.n) break;
    // findroot (component_conn.cpp:60-91)
    unsigned id = D.n;
    for (unsigned i = 0; i < D.n; i++)
      if (!flag[i]) {
        id = i;
        break;
      }
    if (id == D.n) break;
    std::vector<Neighbor> tmpv, pool;
    get_neighbors(D, g, ep, D.row(id), Lr, rnd, tmpv, &pool);
    std::sort(pool.begin(), pool.end());
    bool found = false;
    for (unsigned i = 0; i < pool.size(); i++)
      if (flag[pool[i].id]) {
        root = pool[i].id;
        found = true;
        break;
      }
    if (!found) {
      while (true) {
        unsigned rid = (unsigned)rnd.next() % D.n;
        if (flag[rid]) {
          root = rid;
          break;
        }
      }
    }
    g[root].push_back(SimpleNeighbor(id, l2(D.row(root), D.row(id), D.d)));
    (*added)++;
  }
}

}  // namespace

namespace {

// ---------------------------------------------------------------- SSG
// The angle test of ComponentPruneSSG::PruneInner (component_prune.cpp:96-104)
// and ComponentRefineSSG::InterInsert (component_refine.cpp:685-693):
// cos_ij = (p + r - djk) / 2 / sqrt(p * r) with the reference's operand
// types -- float sums, a float quotient by 2, and the unqualified sqrt of the
// float product resolving to ::sqrt(double) there -- so the quotient is
// taken in double and stored to float.
inline bool ssg_occludes(float pd, float rd, float djk, float threshold) {
  const float num = (pd + rd - djk) / 2;
  const float cos_ij = (float)((double)num / std::sqrt((double)(pd * rd)));
  return cos_ij > threshold;
}

// float threshold = std::cos((float)A / 180 * kPi) (component_prune.cpp:92-93,
// component_refine.cpp:640-641): float quotient, double product and cosine
float ssg_threshold(float A) {
  const double kPi = std::acos(-1.0);
  return (float)std::cos(A / 180 * kPi);
}

// ComponentCandidatePropagation2::CandidateInner (component_candidate.cpp:90-109).
// The reference takes `flags` by value, so every call starts from a clear copy.
void candidate_prop2(const Data &D, const FinalGraph &g, unsigned query, unsigned Lr, std::vector<char> &flags,
                     std::vector<SimpleNeighbor> &pool) {
  std::fill(flags.begin(), flags.end(), 0);
  flags[query] = 1;
  for (unsigned i = 0; i < g[query].size(); i++) {
    unsigned nid = g[query][i].id;
    for (unsigned nn = 0; nn < g[nid].size(); nn++) {
      unsigned nnid = g[nid][nn].id;
      if (flags[nnid]) continue;
      flags[nnid] = 1;
      pool.emplace_back(nnid, l2(D.row(query), D.row(nnid), D.d));
      if (pool.size() >= Lr) break;
    }
    if (pool.size() >= Lr) break;
  }
}

// ComponentPruneSSG::PruneInner (component_prune.cpp:71-122); the flags it
// receives are the caller's clear bitset (a by-value copy), so the node's
// whole row joins the pool
void prune_ssg(const Data &D, const FinalGraph &g, unsigned query, unsigned range, float threshold,
               std::vector<SimpleNeighbor> &pool, SimpleNeighbor *cut_graph) {
  unsigned start = 0;
  for (unsigned nn = 0; nn < g[query].size(); nn++) {
    unsigned id = g[query][nn].id;
    pool.push_back(SimpleNeighbor(id, l2(D.row(query), D.row(id), D.d)));
  }
  std::sort(pool.begin(), pool.end());
  std::vector<SimpleNeighbor> result;
  if (pool[start].id == query) start++;
  result.push_back(pool[start]);
  while (result.size() < range && (++start) < pool.size()) {
    auto &p = pool[start];
    bool occlude = false;
    for (unsigned t = 0; t < result.size(); t++) {
      if (p.id == result[t].id) {
        occlude = true;
        break;
      }
      float djk = l2(D.row(result[t].id), D.row(p.id), D.d);
      if (ssg_occludes(p.distance, result[t].distance, djk, threshold)) {
        occlude = true;
        break;
      }
    }
    if (!occlude) result.push_back(p);
  }
  SimpleNeighbor *des_pool = cut_graph + (size_t)query * range;
  for (size_t t = 0; t < result.size(); t++) des_pool[t] = result[t];
  if (result.size() < range) des_pool[result.size()].distance = -1;
}

// ComponentRefineSSG::InterInsert (component_refine.cpp:647-720): NSG's
// structure with the angle test, and a sentinel after a short re-prune
void inter_insert_ssg(const Data &D, unsigned n, unsigned range, float threshold, SimpleNeighbor *cut_graph) {
  SimpleNeighbor *src_pool = cut_graph + (size_t)n * range;
  for (size_t i = 0; i < range; i++) {
    if (src_pool[i].distance == -1) break;
    SimpleNeighbor sn(n, src_pool[i].distance);
    size_t des = src_pool[i].id;
    SimpleNeighbor *des_pool = cut_graph + des * range;
    std::vector<SimpleNeighbor> temp_pool;
    int dup = 0;
    for (size_t j = 0; j < range; j++) {
      if (des_pool[j].distance == -1) break;
      if (n == des_pool[j].id) {
        dup = 1;
        break;
      }
      temp_pool.push_back(des_pool[j]);
    }
    if (dup) continue;
    temp_pool.push_back(sn);
    if (temp_pool.size() > range) {
      std::vector<SimpleNeighbor> result;
      unsigned start = 0;
      std::sort(temp_pool.begin(), temp_pool.end());
      result.push_back(temp_pool[start]);
      while (result.size() < range && (++start) < temp_pool.size()) {
        auto &p = temp_pool[start];
        bool occlude = false;
        for (unsigned t = 0; t < result.size(); t++) {
          if (p.id == result[t].id) {
            occlude = true;
            break;
          }
          float djk = l2(D.row(result[t].id), D.row(p.id), D.d);
          if (ssg_occludes(p.distance, result[t].distance, djk, threshold)) {
            occlude = true;
            break;
          }
        }
        if (!occlude) result.push_back(p);
      }
      for (unsigned t = 0; t < result.size(); t++) des_pool[t] = result[t];
      if (result.size() < range) des_pool[result.size()].distance = -1;
    } else {
      for (unsigned t = 0; t < range; t++) {
        if (des_pool[t].distance == -1) {
          des_pool[t] = sn;
          if (t + 1 < range) des_pool[t + 1].distance = -1;
          break;
        }
      }
    }
  }
}

// ComponentConnSSGDFS::ConnInner (component_conn.cpp:169-225): n_try roots
// from a std::random_shuffle of 0..n-1 (libstdc++: for i = 1..n-1 swap ids[i]
// with ids[rand() % (i + 1)]); from each root a breadth-first walk, and while
// nodes stay unreached the first reached node with a free slot gets an edge
// to the smallest unreached id, which the walk continues from
void conn_ssg(const Data &D, FinalGraph &g, unsigned n_try, unsigned range, GlibcRand &rnd,
              std::vector<unsigned> &eps, unsigned *added) {
  std::vector<unsigned> ids(D.n);
  for (unsigned i = 0; i < D.n; i++) ids[i] = i;
  for (unsigned i = 1; i < D.n; i++) {
    unsigned j = (unsigned)((long)rnd.next() % (long)(i + 1));
    if (i != j) std::swap(ids[i], ids[j]);
  }
  *added = 0;
  for (unsigned i = 0; i < n_try; i++) eps.push_back(ids[i]);
  for (unsigned i = 0; i < n_try; i++) {
    unsigned rootid = eps[i];
    std::vector<char> flags(D.n, 0);
    std::vector<unsigned> queue;
    size_t head = 0;
    queue.push_back(rootid);
    flags[rootid] = 1;
    std::vector<unsigned> uncheck_set(1);
    while (uncheck_set.size() > 0) {
      while (head < queue.size()) {
        unsigned q_front = queue[head++];
        for (unsigned j = 0; j < g[q_front].size(); j++) {
          unsigned child = g[q_front][j].id;
          if (flags[child]) continue;
          flags[child] = 1;
          queue.push_back(child);
        }
      }
      uncheck_set.clear();
      for (unsigned j = 0; j < D.n; j++)
        if (!flags[j]) uncheck_set.push_back(j);
      if (uncheck_set.size() > 0) {
        for (unsigned j = 0; j < D.n; j++) {
          if (flags[j] && g[j].size() < range) {
            g[j].push_back(SimpleNeighbor(uncheck_set[0], l2(D.row(j), D.row(uncheck_set[0]), D.d)));
            (*added)++;
            break;
          }
        }
        queue.push_back(uncheck_set[0]);
        flags[uncheck_set[0]] = 1;
      }
    }
  }
}

// ComponentRefineSSG::RefineInner / Link (component_refine.cpp:550-645)
FinalGraph link_ssg(const Data &D, const FinalGraph &g, unsigned Lr, unsigned Rr, float A) {
  std::vector<SimpleNeighbor> cut((size_t)D.n * Rr);
  std::vector<SimpleNeighbor> pool;
  std::vector<char> flags(D.n);
  const float threshold = ssg_threshold(A);
  for (unsigned n = 0; n < D.n; ++n) {
    pool.clear();
    candidate_prop2(D, g, n, Lr, flags, pool);
    prune_ssg(D, g, n, Rr, threshold, pool, cut.data());
  }
  for (unsigned n = 0; n < D.n; ++n) inter_insert_ssg(D, n, Rr, threshold, cut.data());
  return cut_to_final(cut, D.n, Rr);
}

// ---------------------------------------------------------------- HNSW / NSW routing
// The graph as IndexBuilder::load_graph(INDEX_HNSW) reads it (builder.cpp:
// 1096-1124): enterpoint id, max level, then per node its id, its layer count
// and, per layer, the friend count and ids.
struct HnswGraph {
  unsigned ep = 0, max_level = 0;
  std::vector<std::vector<std::vector<unsigned>>> fr;  // node -> layer -> friends
};

bool parse_hnsw(const unsigned *w, size_t count, unsigned n, HnswGraph &g) {
  size_t p = 0;
  auto next = [&](unsigned &x) {
    if (p >= count) return false;
    x = w[p++];
    return true;
  };
  if (!next(g.ep) || !next(g.max_level)) return false;
  g.fr.assign(n, std::vector<std::vector<unsigned>>(1));
  for (unsigned i = 0; i < n; i++) {
    unsigned id, layers;
    if (!next(id) || !next(layers) || id >= n) return false;
    g.fr[id].assign(std::max(layers, 1u), {});
    for (unsigned l = 0; l < layers; l++) {
      unsigned gk;
      if (!next(gk)) return false;
      g.fr[id][l].resize(gk);
      for (unsigned k = 0; k < gk; k++)
        if (!next(g.fr[id][l][k]) || g.fr[id][l][k] >= n) return false;
    }
  }
  return g.ep < n;
}

struct FurtherFirst {  // Index::FurtherFirst (index.h:435-447)
  float d;
  unsigned id;
  bool operator<(const FurtherFirst &o) const { return d < o.d; }
};
struct CloserFirst {  // Index::CloserFirst (index.h:449-459)
  float d;
  unsigned id;
  bool operator<(const CloserFirst &o) const { return d > o.d; }
};

struct RouteCtx {
  const Data &D;
  const HnswGraph &g;
  const float *q;
  unsigned L;
  std::vector<unsigned> visited;  // VisitedList (index.h:461-491): a mark per reset
  unsigned mark = 0;
  unsigned long long dc = 0, hc = 0;
  void reset() { ++mark; }
};

// SearchAtLayer (component_route.cpp:85-131 and 214-260, the same body)
void search_at_layer(RouteCtx &c, unsigned entry, unsigned level, std::priority_queue<FurtherFirst> &result) {
  std::priority_queue<CloserFirst> candidates;
  float d = l2(c.q, c.D.row(entry), c.D.d);
  c.dc++;
  result.push(FurtherFirst{d, entry});
  candidates.push(CloserFirst{d, entry});
  c.reset();
  c.visited[entry] = c.mark;
  while (!candidates.empty()) {
    const CloserFirst cand = candidates.top();
    const float lower_bound = result.top().d;
    if (cand.d > lower_bound) break;
    const std::vector<unsigned> &nb = c.g.fr[cand.id][level];
    candidates.pop();
    c.hc++;
    for (unsigned id : nb) {
      if (c.visited[id] == c.mark) continue;
      c.visited[id] = c.mark;
      d = l2(c.q, c.D.row(id), c.D.d);
      c.dc++;
      if (result.size() < c.L || result.top().d > d) {
        result.push(FurtherFirst{d, id});
        candidates.push(CloserFirst{d, id});
        if (result.size() > c.L) result.pop();
      }
    }
  }
}

// the K nearest of `result`, through the CloserFirst queue the reference
// moves them into (unfilled slots stay 0, as res.resize(K) leaves them)
void take_k(std::priority_queue<FurtherFirst> &result, unsigned K, unsigned *res) {
  std::priority_queue<CloserFirst> tmp;
  while (!result.empty()) {
    tmp.push(CloserFirst{result.top().d, result.top().id});
    result.pop();
  }
  for (unsigned pos = 0; pos < K; pos++) {
    res[pos] = 0;
    if (!tmp.empty()) {
      res[pos] = tmp.top().id;
      tmp.pop();
    }
  }
}

// ComponentSearchRouteHNSW::RouteInner (component_route.cpp:134-212): greedy
// descent from the enterpoint through every layer down to 0 (a fresh visited
// mark per layer; every improvement appended to the path), then the layer-0
// search from the path element before the last one.  When the path holds
// only the enterpoint the reference reads before its vector's start; here
// the search then starts from the enterpoint.
void route_hnsw(RouteCtx &c, unsigned K, unsigned *res) {
  unsigned cur = c.g.ep;
  float cur_dist = l2(c.q, c.D.row(cur), c.D.d);
  c.dc++;
  std::vector<std::pair<unsigned, float>> path{{cur, cur_dist}};
  for (int i = (int)c.g.max_level; i >= 0; --i) {
    c.reset();
    c.visited[cur] = c.mark;
    bool changed = true;
    while (changed) {
      changed = false;
      const std::vector<unsigned> &nb = c.g.fr[cur][i];
      c.hc++;
      for (unsigned id : nb) {
        if (c.visited[id] == c.mark) continue;
        c.visited[id] = c.mark;
        const float d = l2(c.q, c.D.row(id), c.D.d);
        c.dc++;
        if (d < cur_dist) {
          cur_dist = d;
          cur = id;
          changed = true;
          path.emplace_back(cur, cur_dist);
        }
      }
    }
  }
  std::priority_queue<FurtherFirst> result;
  while (result.size() < K && !path.empty()) {
    path.pop_back();
    const unsigned entry = path.empty() ? c.g.ep : path.back().first;
    search_at_layer(c, entry, 0, result);
  }
  take_k(result, K, res);
}

// ComponentSearchRouteNSW::RouteInner (component_route.cpp:56-83): the
// layer-0 search from node 0
void route_nsw(RouteCtx &c, unsigned K, unsigned *res) {
  std::priority_queue<FurtherFirst> result;
  search_at_layer(c, 0, 0, result);
  take_k(result, K, res);
}


// ---------------------------------------------------------------- INIT_KDT
// ComponentInitKDT (component_init.cpp:500-912): nTrees randomised KD-trees
// over rand()-shuffled id lists, leaf-to-leaf merges below depth mLevel into
// per-point bounded candidate sets, then the final graph.  One thread, as the
// reference's results with IndexBuilder(1): every split's std::mt19937 is
// seeded 1998 ^ omp_get_thread_num() = 1998.
struct KdtNode {
  int div_dim = -1;
  float div_val = 0.f;
  unsigned start = 0, end = 0;
  int left = -1, right = -1;  // -1: leaf
};
struct KdtForest {
  unsigned n = 0, T = 0;
  std::vector<std::vector<unsigned>> leaf;  // LeafLists
  std::vector<std::vector<KdtNode>> nodes;  // node 0 = root of the tree
};
constexpr unsigned KDT_TNS = 10, KDT_SAMPLE = 100, KDT_RAND_DIM = 5, KDT_ACTIVE_MAX = 1100;

// selectDivision (component_init.cpp:732-756): one of the RAND_DIM largest
// variances, by the first rng() output % their count
unsigned kdt_select_division(std::mt19937 &rng, const float *v, unsigned d) {
  int num = 0;
  size_t top[KDT_RAND_DIM];
  for (size_t i = 0; i < d; ++i) {
    if (num < (int)KDT_RAND_DIM || v[i] > v[top[num - 1]]) {
      if (num < (int)KDT_RAND_DIM) top[num++] = i;
      else top[num - 1] = i;
      int j = num - 1;
      while (j > 0 && v[top[j]] > v[top[j - 1]]) {
        std::swap(top[j], top[j - 1]);
        --j;
      }
    }
  }
  return (unsigned)top[rng() % (unsigned)num];
}

// planeSplit (component_init.cpp:698-730): Hoare partitions by < cutval, then
// by <= cutval from lim1 (the element reads are guarded where the reference
// reads one past the range without using the value)
void kdt_plane_split(const Data &D, unsigned *ids, unsigned count, unsigned cutdim, float cutval, unsigned &lim1,
                     unsigned &lim2) {
  auto val = [&](int i) { return D.base[(size_t)ids[i] * D.d + cutdim]; };
  int left = 0, right = (int)count - 1;
  for (;;) {
    while (left <= right && val(left) < cutval) ++left;
    while (left <= right && val(right) >= cutval) --right;
    if (left > right) break;
    std::swap(ids[left], ids[right]);
    ++left;
    --right;
  }
  lim1 = (unsigned)left;
  right = (int)count - 1;
  for (;;) {
    while (left <= right && val(left) <= cutval) ++left;
    while (left <= right && val(right) > cutval) --right;
    if (left > right) break;
    std::swap(ids[left], ids[right]);
    ++left;
    --right;
  }
  lim2 = (unsigned)left;
}

// meanSplit (component_init.cpp:648-696): mean and variance of the first
// SAMPLE_NUM + 1 ids, the cut at the mean of a high-variance dimension
void kdt_mean_split(const Data &D, std::mt19937 &rng, unsigned *ids, unsigned count, unsigned &index1,
                    unsigned &cutdim, float &cutval) {
  std::vector<float> mean(D.d, 0.f), var(D.d, 0.f);
  const unsigned cnt = std::min(KDT_SAMPLE + 1, count);
  for (unsigned j = 0; j < cnt; ++j) {
    const float *v = D.base + (size_t)ids[j] * D.d;
    for (unsigned k = 0; k < D.d; ++k) mean[k] += v[k];
  }
  const float div_factor = float(1) / cnt;
  for (unsigned k = 0; k < D.d; ++k) mean[k] *= div_factor;
  for (unsigned j = 0; j < cnt; ++j) {
    const float *v = D.base + (size_t)ids[j] * D.d;
    for (unsigned k = 0; k < D.d; ++k) {
      const float dd = v[k] - mean[k];
      var[k] += dd * dd;
    }
  }
  cutdim = kdt_select_division(rng, var.data(), D.d);
  cutval = mean[cutdim];
  unsigned lim1, lim2;
  kdt_plane_split(D, ids, count, cutdim, cutval, lim1, lim2);
  if (lim1 > count / 2) index1 = lim1;
  else if (lim2 < count / 2) index1 = lim2;
  else index1 = count / 2;
  if (lim1 == count || lim2 == 0) index1 = count / 2;
}

int kdt_new_node(std::vector<KdtNode> &nodes, unsigned start, unsigned end) {
  KdtNode x;
  x.start = start;
  x.end = end;
  nodes.push_back(x);
  return (int)nodes.size() - 1;
}

// DFSbuild (component_init.cpp:758-787); nodes of TNS ids or fewer are leaves
void kdt_dfs_build(const Data &D, std::vector<KdtNode> &nodes, std::vector<unsigned> &leaf, int nd,
                   std::mt19937 &rng) {
  const unsigned start = nodes[nd].start, count = nodes[nd].end - nodes[nd].start;
  if (count <= KDT_TNS) return;
  unsigned idx, cutdim;
  float cutval;
  kdt_mean_split(D, rng, leaf.data() + start, count, idx, cutdim, cutval);
  nodes[nd].div_dim = (int)cutdim;
  nodes[nd].div_val = cutval;
  const int l = kdt_new_node(nodes, start, start + idx);
  const int r = kdt_new_node(nodes, start + idx, start + count);
  nodes[nd].left = l;
  nodes[nd].right = r;
  kdt_dfs_build(D, nodes, leaf, l, rng);
  kdt_dfs_build(D, nodes, leaf, r, rng);
}

// the trees of InitInner (component_init.cpp:500-580): shuffled id lists
// (std::random_shuffle on rand(), tree by tree), level-by-level splits while
// fewer than 1,100 nodes are active (children of more than K ids stay
// active; each split with a fresh rng), then DFSbuild below each active node
// (one fresh rng per active node, shared down its subtree)
KdtForest kdt_build(const Data &D, unsigned T, unsigned K, GlibcRand &rnd) {
  KdtForest F;
  F.n = D.n;
  F.T = T;
  F.leaf.assign(T, std::vector<unsigned>(D.n));
  F.nodes.assign(T, std::vector<KdtNode>());
  std::vector<std::pair<unsigned, int>> active, next;
  for (unsigned t = 0; t < T; t++) {
    kdt_new_node(F.nodes[t], 0, D.n);
    active.emplace_back(t, 0);
  }
  for (unsigned t = 0; t < T; t++) {
    std::vector<unsigned> &ids = F.leaf[t];
    for (unsigned i = 0; i < D.n; i++) ids[i] = i;
    for (unsigned i = 1; i < D.n; i++) {
      const unsigned j = (unsigned)((long)rnd.next() % (long)(i + 1));
      if (i != j) std::swap(ids[i], ids[j]);
    }
  }
  while (!active.empty() && active.size() < KDT_ACTIVE_MAX) {
    next.clear();
    for (auto &a : active) {
      std::vector<KdtNode> &nodes = F.nodes[a.first];
      const unsigned start = nodes[a.second].start, count = nodes[a.second].end - start;
      std::mt19937 rng(1998);
      unsigned mid, cutdim;
      float cutval;
      kdt_mean_split(D, rng, F.leaf[a.first].data() + start, count, mid, cutdim, cutval);
      nodes[a.second].div_dim = (int)cutdim;
      nodes[a.second].div_val = cutval;
      const int l = kdt_new_node(nodes, start, start + mid);
      const int r = kdt_new_node(nodes, start + mid, start + count);
      nodes[a.second].left = l;
      nodes[a.second].right = r;
      if (mid > K) next.emplace_back(a.first, l);
      if (count - mid > K) next.emplace_back(a.first, r);
    }
    active.swap(next);
  }
  for (auto &a : active) {
    std::mt19937 rng(1998);
    kdt_dfs_build(D, F.nodes[a.first], F.leaf[a.first], a.second, rng);
  }
  return F;
}

// SearchToLeaf (component_init.cpp:828-838)
int kdt_search_to_leaf(const Data &D, const std::vector<KdtNode> &nodes, int nd, size_t id) {
  while (nodes[nd].left >= 0 && nodes[nd].right >= 0)
    nd = D.base[id * D.d + nodes[nd].div_dim] < nodes[nd].div_val ? nodes[nd].left : nodes[nd].right;
  return nd;
}

struct KdtCand {  // Index::Candidate (index.h:234-253)
  size_t row_id;
  float distance;
  bool operator>(const KdtCand &o) const {
    return distance == o.distance ? row_id > o.row_id : distance > o.distance;
  }
};
typedef std::set<KdtCand, std::greater<KdtCand>> KdtHeap;

void kdt_offer(KdtHeap &h, unsigned K, size_t id, float dist) {
  if (h.size() < K || dist < h.begin()->distance) {
    h.insert(KdtCand{id, dist});
    if (h.size() > K) h.erase(h.begin());
  }
}

// mergeSubGraphs (component_init.cpp:840-912)
void kdt_merge(const Data &D, const KdtForest &F, unsigned t, int nd, unsigned K, std::vector<KdtHeap> &knn) {
  const std::vector<KdtNode> &nodes = F.nodes[t];
  const KdtNode &x = nodes[nd];
  if (x.left < 0 || x.right < 0) return;
  kdt_merge(D, F, t, x.left, K, knn);
  kdt_merge(D, F, t, x.right, K, knn);
  const size_t numL = nodes[x.left].end - nodes[x.left].start, numR = nodes[x.right].end - nodes[x.right].start;
  int root;
  size_t start, end;
  if (numL < numR) {
    root = x.right;
    start = nodes[x.left].start;
    end = nodes[x.left].end;
  } else {
    root = x.left;
    start = nodes[x.right].start;
    end = nodes[x.right].end;
  }
  for (; start < end; start++) {
    const size_t feature_id = F.leaf[t][start];
    const int lf = kdt_search_to_leaf(D, nodes, root, feature_id);
    for (size_t i = nodes[lf].start; i < nodes[lf].end; i++) {
      const size_t tmpfea = F.leaf[t][i];
      const float dist = l2(D.base + tmpfea * D.d, D.base + feature_id * D.d, D.d);
      kdt_offer(knn[tmpfea], K, feature_id, dist);
      kdt_offer(knn[feature_id], K, tmpfea, dist);
    }
  }
}

// getMergeLevelNodeList (component_init.cpp:814-826)
void kdt_merge_level(const KdtForest &F, unsigned t, int nd, unsigned depth, unsigned ml,
                     std::vector<std::pair<int, unsigned>> &out) {
  const KdtNode &x = F.nodes[t][nd];
  if (x.left >= 0 && x.right >= 0 && depth < ml) {
    kdt_merge_level(F, t, x.left, depth + 1, ml, out);
    kdt_merge_level(F, t, x.right, depth + 1, ml, out);
  } else if (depth == ml) {
    out.emplace_back(nd, t);
  }
}

// InitInner's merge and final graph (component_init.cpp:582-640): rows in
// ascending (distance, id); a row of fewer than K gets rng() % n fills into a
// set ordered by distance alone (equal distances kept once).  Returns false
// when a row cannot reach K distinct distances (the reference loops forever).
bool kdt_graph(const Data &D, const KdtForest &F, unsigned K, unsigned ml, FinalGraph &g) {
  std::vector<std::pair<int, unsigned>> mlist;
  for (unsigned t = 0; t < F.T; t++) kdt_merge_level(F, t, 0, 0, ml, mlist);
  std::vector<KdtHeap> knn(D.n);
  for (auto &m : mlist) kdt_merge(D, F, m.second, m.first, K, knn);
  g.assign(D.n, {});
  std::mt19937 rng(1998);
  for (unsigned i = 0; i < D.n; i++) {
    std::vector<SimpleNeighbor> tmp;
    for (auto it = knn[i].rbegin(); it != knn[i].rend(); it++)
      tmp.push_back(SimpleNeighbor((unsigned)it->row_id,
                                   l2(D.base + (size_t)i * D.d, D.base + it->row_id * D.d, D.d)));
    if (tmp.size() < K) {
      auto by_dist = [](const SimpleNeighbor &a, const SimpleNeighbor &b) { return a.distance < b.distance; };
      std::set<SimpleNeighbor, decltype(by_dist)> result(by_dist);
      for (auto &x : tmp) result.insert(x);
      size_t tries = 0;
      while (result.size() < K) {
        if (++tries > 64ull * D.n + 1000000ull) return false;
        const unsigned id = (unsigned)(rng() % D.n);
        result.insert(SimpleNeighbor(id, l2(D.base + (size_t)i * D.d, D.base + (size_t)id * D.d, D.d)));
      }
      tmp.assign(result.begin(), result.end());
    }
    g[i] = tmp;
  }
  return true;
}

// ComponentSearchEntryKDT::getSearchNodeList (component_search_entry.cpp:156-170)
void kdt_leaf_list(const std::vector<KdtNode> &nodes, int nd, const float *q, unsigned lsize, std::vector<int> &vn) {
  if (vn.size() >= lsize) return;
  const KdtNode &x = nodes[nd];
  if (x.left >= 0 && x.right >= 0) {
    const bool lt = q[x.div_dim] < x.div_val;
    kdt_leaf_list(nodes, lt ? x.left : x.right, q, lsize, vn);
    kdt_leaf_list(nodes, lt ? x.right : x.left, q, lsize, vn);
  } else {
    vn.push_back(nd);
  }
}

// ComponentSearchEntryKDT::SearchEntryInner's seeds (component_search_entry.cpp:102-141):
// the ids of lsize = L / (nTrees * TNS) + 1 leaves per tree, taken leaf-major
// across the trees (the base id equal to the query's index is skipped, as the
// reference flags it), then rand() % n fills without repeats.  A tree with
// fewer leaves than lsize contributes the leaves it has (the reference reads
// past its list there).
void kdt_seeds(const KdtForest &F, const float *q, unsigned qidx, unsigned L, GlibcRand &rnd, unsigned *s) {
  const unsigned lsize = L / (F.T * KDT_TNS) + 1;
  std::vector<std::vector<int>> vnl(F.T);
  for (unsigned t = 0; t < F.T; t++) kdt_leaf_list(F.nodes[t], 0, q, lsize, vnl[t]);
  std::vector<char> flags(F.n, 0);
  if (qidx < F.n) flags[qidx] = 1;
  unsigned p = 0;
  for (unsigned ni = 0; ni < lsize && p < L; ni++) {
    for (unsigned t = 0; t < F.T && p < L; t++) {
      if (ni >= vnl[t].size()) continue;
      const KdtNode &lf = F.nodes[t][vnl[t][ni]];
      for (unsigned j = lf.start; j < lf.end && p < L; j++) {
        const unsigned nn = F.leaf[t][j];
        if (flags[nn]) continue;
        flags[nn] = 1;
        s[p++] = nn;
      }
    }
  }
  while (p < L) {
    const unsigned nn = (unsigned)rnd.next() % F.n;
    if (flags[nn]) continue;
    flags[nn] = 1;
    s[p++] = nn;
  }
}

// the pool and route of IndexBuilder::search on given seeds (builder.cpp:445-454,
// component_route.cpp:9-53)
void route_seeded(const Data &D, const unsigned *g_ids, const unsigned *g_deg, unsigned g_w, const float *qv,
                  const unsigned *seeds, unsigned L, unsigned K, unsigned *res, unsigned long long &dc,
                  unsigned long long &hc) {
  std::vector<char> flags(D.n, 0);
  std::vector<Neighbor> pool(L + 1);
  for (unsigned i = 0; i < L; i++) {
    pool[i] = Neighbor(seeds[i], l2(qv, D.base + (size_t)seeds[i] * D.d, D.d), true);
    dc++;
  }
  std::sort(pool.begin(), pool.begin() + L);
  int k = 0;
  while (k < (int)L) {
    int nk = (int)L;
    if (pool[k].flag) {
      pool[k].flag = false;
      const unsigned nd = pool[k].id;
      hc++;
      for (unsigned m = 0; m < g_deg[nd]; ++m) {
        const unsigned id = g_ids[(size_t)nd * g_w + m];
        if (flags[id]) continue;
        flags[id] = 1;
        const float dist = l2(qv, D.base + (size_t)id * D.d, D.d);
        dc++;
        if (dist >= pool[L - 1].distance) continue;
        const int rr = insert_into_pool(pool.data(), L, Neighbor(id, dist, true));
        if (rr < nk) nk = rr;
      }
    }
    if (nk <= k) k = nk;
    else ++k;
  }
  for (unsigned i = 0; i < K; i++) res[i] = pool[i].id;
}

// flat forest arrays: per tree nodes[t * ncap + j] = (div_dim, div_val bits,
// start, end, left, right), node counts cnt[t]; leaf lists T x n
void kdt_export(const KdtForest &F, unsigned ncap, int *nodes, unsigned *cnt, unsigned *leaf) {
  for (unsigned t = 0; t < F.T; t++) {
    cnt[t] = (unsigned)F.nodes[t].size();
    for (size_t j = 0; j < F.nodes[t].size() && j < ncap; j++) {
      const KdtNode &x = F.nodes[t][j];
      int *o = nodes + ((size_t)t * ncap + j) * 6;
      o[0] = x.div_dim;
      std::memcpy(&o[1], &x.div_val, 4);
      o[2] = (int)x.start;
      o[3] = (int)x.end;
      o[4] = x.left;
      o[5] = x.right;
    }
    std::memcpy(leaf + (size_t)t * F.n, F.leaf[t].data(), (size_t)F.n * 4);
  }
}
KdtForest kdt_import(unsigned n, unsigned T, unsigned ncap, const int *nodes, const unsigned *cnt,
                     const unsigned *leaf) {
  KdtForest F;
  F.n = n;
  F.T = T;
  F.leaf.assign(T, std::vector<unsigned>(n));
  F.nodes.assign(T, std::vector<KdtNode>());
  for (unsigned t = 0; t < T; t++) {
    for (unsigned j = 0; j < cnt[t]; j++) {
      const int *o = nodes + ((size_t)t * ncap + j) * 6;
      KdtNode x;
      x.div_dim = o[0];
      std::memcpy(&x.div_val, &o[1], 4);
      x.start = (unsigned)o[2];
      x.end = (unsigned)o[3];
      x.left = o[4];
      x.right = o[5];
      F.nodes[t].push_back(x);
    }
    std::memcpy(F.leaf[t].data(), leaf + (size_t)t * n, (size_t)n * 4);
  }
  return F;
}

}  // namespace

extern "C" {

// ROUTER_HNSW (router 0) / ROUTER_NSW (router 1) over a graph in the
// INDEX_HNSW file layout (words), every query: res nq x K, counters
// [dist_count, hop_count]
int orc_search_hnsw(const float *base, unsigned n, unsigned d, const float *query, unsigned nq, const unsigned *words,
                    size_t nwords, int router, unsigned L, unsigned K, unsigned *res, unsigned long long *counters) {
  HnswGraph g;
  if (!parse_hnsw(words, nwords, n, g)) return -1;
  if (g.max_level >= g.fr[g.ep].size() && router == 0) return -2;
  Data D{base, n, d};
  RouteCtx c{D, g, nullptr, L, std::vector<unsigned>(n, 0u)};
  for (unsigned q = 0; q < nq; q++) {
    c.q = query + (size_t)q * d;
    if (router == 0) route_hnsw(c, K, res + (size_t)q * K);
    else route_nsw(c, K, res + (size_t)q * K);
  }
  counters[0] = c.dc;
  counters[1] = c.hc;
  return 0;
}

void *orc_rand_create(unsigned seed) { return new GlibcRand(seed); }
void orc_rand_destroy(void *r) { delete (GlibcRand *)r; }
int orc_rand_next(void *r) { return ((GlibcRand *)r)->next(); }
void orc_rand_fill(void *r, int *out, unsigned n) {
  for (unsigned i = 0; i < n; i++) out[i] = ((GlibcRand *)r)->next();
}

// L2 in the reference's summation order, row by row (for tests)
void orc_l2_rows(const float *a, const float *b, unsigned n, unsigned d, float *out) {
  for (unsigned i = 0; i < n; i++) out[i] = l2(a + (size_t)i * d, b + (size_t)i * d, d);
}

// INIT_RAND: out rows of width L (self hits dropped, so deg may be L-1)
int orc_init_rand(const float *base, unsigned n, unsigned d, unsigned L, void *rnd, unsigned *ids, float *dist,
                  unsigned *deg) {
  Data D{base, n, d};
  FinalGraph g = init_rand(D, L, *(GlibcRand *)rnd);
  return graph_to_arrays(g, ids, dist, deg, L);
}

// INIT_RANDOM: out rows of width S (self hits dropped, so deg may be S-1)
int orc_init_random(const float *base, unsigned n, unsigned d, unsigned S, void *rnd, unsigned *ids, float *dist,
                    unsigned *deg) {
  Data D{base, n, d};
  FinalGraph g = init_random(D, S, *(GlibcRand *)rnd);
  return graph_to_arrays(g, ids, dist, deg, S);
}

// REFINE_NN_DESCENT from a given init graph; out rows of width K.
// stats[0] = reverse-list overflow events (rand() draws), stats[1] unused
int orc_nndescent(const float *base, unsigned n, unsigned d, const unsigned *in_ids, const float *in_dist,
                  const unsigned *in_deg, unsigned in_w, unsigned S, unsigned K, unsigned L, unsigned ITER, unsigned R,
                  void *rnd, int threads, unsigned *ids, float *dist, unsigned *deg, unsigned long long *stats) {
  Data D{base, n, d};
  FinalGraph init = graph_from_arrays(in_ids, in_dist, in_deg, n, in_w);
  NNDescent nd(D, S, K, L, ITER, R, *(GlibcRand *)rnd, threads < 1 ? 1 : threads);
  nd.init(init);
  for (unsigned it = 0; it < ITER; it++) {
    nd.join();
    nd.update();
  }
  FinalGraph fg = nd.finish();
  if (stats) stats[0] = nd.overflow_events;
  return graph_to_arrays(fg, ids, dist, deg, K);
}

// REFINE_EFANNA (component_refine.cpp:959-1178) from a given init graph: the
// NN-Descent of REFINE_NN_DESCENT with EFANNA's init; out rows of width K.
// Init rows longer than L are refused (the reference's pool would outgrow
// its reserved capacity).
int orc_efanna(const float *base, unsigned n, unsigned d, const unsigned *in_ids, const float *in_dist,
               const unsigned *in_deg, unsigned in_w, unsigned S, unsigned K, unsigned L, unsigned ITER, unsigned R,
               void *rnd, unsigned *ids, float *dist, unsigned *deg, unsigned long long *stats) {
  Data D{base, n, d};
  for (unsigned i = 0; i < n; i++)
    if (in_deg[i] > L) return -1;
  FinalGraph init = graph_from_arrays(in_ids, in_dist, in_deg, n, in_w);
  NNDescent nd(D, S, K, L, ITER, R, *(GlibcRand *)rnd, 1);
  nd.init_efanna(init);
  for (unsigned it = 0; it < ITER; it++) {
    nd.join();
    nd.update();
  }
  FinalGraph fg = nd.finish();
  if (stats) stats[0] = nd.overflow_events;
  return graph_to_arrays(fg, ids, dist, deg, K);
}

// NN-Descent pool state after `iters` iterations (debug / fine-grained parity):
// pools sorted, with flags; width L
int orc_nndescent_pools(const float *base, unsigned n, unsigned d, const unsigned *in_ids, const float *in_dist,
                        const unsigned *in_deg, unsigned in_w, unsigned S, unsigned L, unsigned iters, unsigned R,
                        void *rnd, unsigned *ids, float *dist, unsigned char *flag, unsigned *deg, unsigned *M) {
  Data D{base, n, d};
  FinalGraph init = graph_from_arrays(in_ids, in_dist, in_deg, n, in_w);
  NNDescent nd(D, S, L, L, iters, R, *(GlibcRand *)rnd, 1);
  nd.init(init);
  for (unsigned it = 0; it < iters; it++) {
    nd.join();
    nd.update();
  }
  for (unsigned i = 0; i < n; i++) {
    // the pool as the update left it (a heap); report it as stored
    deg[i] = (unsigned)nd.graph[i].pool.size();
    M[i] = nd.graph[i].M;
    for (unsigned j = 0; j < deg[i]; j++) {
      ids[(size_t)i * L + j] = nd.graph[i].pool[j].id;
      dist[(size_t)i * L + j] = nd.graph[i].pool[j].distance;
      flag[(size_t)i * L + j] = nd.graph[i].pool[j].flag;
    }
  }
  return 0;
}

// REFINE_VAMANA (component_refine.cpp:794-872) on graph `in`; entry_L is the
// index's L_refine member (0 unless an NSG refine ran before).  Out width R.
int orc_vamana(const float *base, unsigned n, unsigned d, const unsigned *in_ids, const float *in_dist,
               const unsigned *in_deg, unsigned in_w, unsigned L_refine, unsigned R_refine, float alpha,
               unsigned entry_L, void *rnd, int threads, unsigned *ids, float *dist, unsigned *deg, unsigned *ep,
               int clean) {
  Data D{base, n, d};
  GlibcRand &r = *(GlibcRand *)rnd;
  FinalGraph g = graph_from_arrays(in_ids, in_dist, in_deg, n, in_w);
  // clean mode: the entry search the link intends (L_refine when unset)
  unsigned e = entry_centroid(D, g, (clean && entry_L == 0) ? L_refine : entry_L, r);
  FinalGraph out = link(D, g, e, L_refine, R_refine, 0, true, alpha, r, threads < 1 ? 1 : threads, clean != 0);
  *ep = e;
  return graph_to_arrays(out, ids, dist, deg, R_refine);
}

// REFINE_NSG (component_refine.cpp:393-428) incl. ConnNSGDFS; out width out_w
// (>= R_refine: the connectivity pass may lengthen rows)
int orc_nsg(const float *base, unsigned n, unsigned d, const unsigned *in_ids, const float *in_dist,
            const unsigned *in_deg, unsigned in_w, unsigned L_refine, unsigned R_refine, unsigned C_refine,
            void *rnd, int threads, unsigned *ids, float *dist, unsigned *deg, unsigned out_w, unsigned *ep,
            unsigned *conn_added) {
  Data D{base, n, d};
  GlibcRand &r = *(GlibcRand *)rnd;
  FinalGraph g = graph_from_arrays(in_ids, in_dist, in_deg, n, in_w);
  unsigned e = entry_centroid(D, g, L_refine, r);
  FinalGraph out = link(D, g, e, L_refine, R_refine, C_refine, false, 1.0f, r, threads < 1 ? 1 : threads);
  conn_dfs(D, out, e, L_refine, r, conn_added);
  *ep = e;
  return graph_to_arrays(out, ids, dist, deg, out_w);
}

// REFINE_SSG (component_refine.cpp:550-582): link + DFS-expand conn; eps
// receives the n_try roots
int orc_ssg(const float *base, unsigned n, unsigned d, const unsigned *in_ids, const float *in_dist,
            const unsigned *in_deg, unsigned in_w, unsigned L_refine, unsigned R_refine, float A, unsigned n_try,
            void *rnd, unsigned *ids, float *dist, unsigned *deg, unsigned out_w, unsigned *eps,
            unsigned *conn_added) {
  Data D{base, n, d};
  GlibcRand &r = *(GlibcRand *)rnd;
  FinalGraph g = graph_from_arrays(in_ids, in_dist, in_deg, n, in_w);
  FinalGraph out = link_ssg(D, g, L_refine, R_refine, A);
  std::vector<unsigned> e;
  conn_ssg(D, out, n_try, R_refine, r, e, conn_added);
  for (unsigned i = 0; i < n_try; i++) eps[i] = e[i];
  return graph_to_arrays(out, ids, dist, deg, out_w);
}

// Seed draws of the three entries (the host side of the GPU search makes the
// same draws):
// entry 0 = SearchEntryRand (component_search_entry.cpp:9-30): one rand()
//   seeds an mt19937, GenRandom draws L distinct ids;
// entry 1 = SearchEntryCentroid (component_search_entry.cpp:33-67): the entry
//   point's row, then rand() % n fills (no repeats);
// entry 2 = SearchEntrySubCentroid (component_search_entry.cpp:70-99): the
//   Rand draw with its first n_eps ids replaced by the SSG roots (the pool
//   may then hold an id twice).
static void draw_entry(unsigned n, const unsigned *g_ids, const unsigned *g_deg, unsigned g_w, unsigned ep, int entry,
                unsigned L, const unsigned *eps, unsigned n_eps, GlibcRand &r, unsigned *s) {
  if (entry == 0 || entry == 2) {
    std::mt19937 rng(r.next());
    gen_random(rng, s, L, n);
    if (entry == 2)
      for (unsigned i = 0; i < n_eps && i < L; i++) s[i] = eps[i];
  } else {
    std::vector<char> flags(n, 0);
    unsigned t = 0;
    for (; t < L && t < g_deg[ep]; t++) {
      s[t] = g_ids[(size_t)ep * g_w + t];
      flags[s[t]] = 1;
    }
    while (t < L) {
      unsigned id = (unsigned)r.next() % n;
      if (flags[id]) continue;
      flags[id] = 1;
      s[t++] = id;
    }
  }
}

// SearchEntrySubCentroid's seed distance (component_search_entry.cpp:84-89):
// the row pointer is advanced by one float (its first value taken as a
// norm) and d floats compared from there -- for the last row that is one
// float past the base, read as 0 here
static float sub_centroid_dist(const float *base, unsigned n, unsigned d, unsigned id, const float *qv) {
  std::vector<float> x(d);
  const float *row = base + (size_t)id * d + 1;
  for (unsigned j = 0; j + 1 < d; j++) x[j] = row[j];
  x[d - 1] = id + 1 < n ? row[d - 1] : 0.0f;
  return l2(x.data(), qv, d);
}

// IndexBuilder::search with L_SEARCH_ASSIGN (builder.cpp:430-454): seeds by
// draw_entry, route = ComponentSearchRouteGreedy (component_route.cpp:9-53).
// res: nq x K ids; counters: [dist_count, hop_count].  With threads > 1 the
// seed draws are made first in query order (so results stay deterministic)
// and the queries then run in an OpenMP loop like builder.cpp:285-295.
int orc_search(const float *base, unsigned n, unsigned d, const float *query, unsigned nq, const unsigned *g_ids,
               const unsigned *g_deg, unsigned g_w, unsigned ep, int entry, unsigned L, unsigned K, void *rnd,
               int threads, unsigned *res, unsigned long long *counters, const unsigned *eps, unsigned n_eps) {
  if (L < K) return -1;
  if (entry == 2 && n_eps > L) return -1;  // the reference asserts eps_.size() <= L
  GlibcRand &r = *(GlibcRand *)rnd;
  std::vector<std::vector<unsigned>> seeds(nq, std::vector<unsigned>(L));
  for (unsigned q = 0; q < nq; q++) draw_entry(n, g_ids, g_deg, g_w, ep, entry, L, eps, n_eps, r, seeds[q].data());
  unsigned long long dc = 0, hc = 0;
#pragma omp parallel num_threads(threads < 1 ? 1 : threads) reduction(+ : dc, hc)
  {
    std::vector<char> flags(n);
    std::vector<Neighbor> pool(L + 1);
#pragma omp for schedule(dynamic, 16)
    for (unsigned q = 0; q < nq; q++) {
      const float *qv = query + (size_t)q * d;
      for (unsigned i = 0; i < L; i++) {
        unsigned id = seeds[q][i];
        const float dist = entry == 2 ? sub_centroid_dist(base, n, d, id, qv) : l2(qv, base + (size_t)id * d, d);
        pool[i] = Neighbor(id, dist, true);
        dc++;
      }
      std::sort(pool.begin(), pool.begin() + L);
      std::fill(flags.begin(), flags.end(), 0);
      int k = 0;
      while (k < (int)L) {
        int nk = (int)L;
        if (pool[k].flag) {
          pool[k].flag = false;
          unsigned nd = pool[k].id;
          hc++;
          for (unsigned m = 0; m < g_deg[nd]; ++m) {
            unsigned id = g_ids[(size_t)nd * g_w + m];
            if (flags[id]) continue;
            flags[id] = 1;
            float dist = l2(qv, base + (size_t)id * d, d);
            dc++;
            if (dist >= pool[L - 1].distance) continue;
            int rr = insert_into_pool(pool.data(), L, Neighbor(id, dist, true));
            if (rr < nk) nk = rr;
          }
        }
        if (nk <= k) k = nk;
        else ++k;
      }
      for (unsigned i = 0; i < K; i++) res[(size_t)q * K + i] = pool[i].id;
    }
  }
  counters[0] = dc;
  counters[1] = hc;
  return 0;
}

// Seeds only (the host side of the GPU search does the same draws)
int orc_search_seeds(unsigned n, unsigned nq, const unsigned *g_ids, const unsigned *g_deg, unsigned g_w, unsigned ep,
                     int entry, unsigned L, void *rnd, unsigned *seeds, const unsigned *eps, unsigned n_eps) {
  GlibcRand &r = *(GlibcRand *)rnd;
  for (unsigned q = 0; q < nq; q++)
    draw_entry(n, g_ids, g_deg, g_w, ep, entry, L, eps, n_eps, r, seeds + (size_t)q * L);
  return 0;
}


// INIT_KDT (component_init.cpp:500-640): the final graph (rows of width K,
// ascending) and the forest (nodes: T x ncap x 6 words, node counts, leaf
// lists T x n).  -1: ncap too small; -2: a row cannot reach K distinct
// distances.
int orc_init_kdt(const float *base, unsigned n, unsigned d, unsigned T, unsigned K, unsigned mlevel, void *rnd,
                 unsigned *ids, float *dist, unsigned *deg, unsigned ncap, int *nodes, unsigned *cnt, unsigned *leaf) {
  Data D{base, n, d};
  KdtForest F = kdt_build(D, T, K, *(GlibcRand *)rnd);
  for (unsigned t = 0; t < T; t++)
    if (F.nodes[t].size() > ncap) return -1;
  FinalGraph g;
  if (!kdt_graph(D, F, K, mlevel, g)) return -2;
  kdt_export(F, ncap, nodes, cnt, leaf);
  return graph_to_arrays(g, ids, dist, deg, K);
}

// SEARCH_ENTRY_KDT + ROUTER_GREEDY (component_search_entry.cpp:102-154,
// component_route.cpp:9-53) over a forest in the orc_init_kdt layout; queries
// in order (their seed draws share the rand() stream)
int orc_search_kdt(const float *base, unsigned n, unsigned d, const float *query, unsigned nq, const unsigned *g_ids,
                   const unsigned *g_deg, unsigned g_w, unsigned T, unsigned ncap, const int *nodes,
                   const unsigned *cnt, const unsigned *leaf, unsigned L, unsigned K, void *rnd, unsigned *res,
                   unsigned long long *counters, unsigned *seeds_out) {
  if (L < K || L >= n) return -1;
  Data D{base, n, d};
  KdtForest F = kdt_import(n, T, ncap, nodes, cnt, leaf);
  GlibcRand &r = *(GlibcRand *)rnd;
  std::vector<unsigned> s(L);
  unsigned long long dc = 0, hc = 0;
  for (unsigned q = 0; q < nq; q++) {
    const float *qv = query + (size_t)q * d;
    kdt_seeds(F, qv, q, L, r, s.data());
    if (seeds_out) std::memcpy(seeds_out + (size_t)q * L, s.data(), (size_t)L * 4);
    route_seeded(D, g_ids, g_deg, g_w, qv, s.data(), L, K, res + (size_t)q * K, dc, hc);
  }
  counters[0] = dc;
  counters[1] = hc;
  return 0;
}

}  // extern "C"
