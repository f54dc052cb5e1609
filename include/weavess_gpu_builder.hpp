// weavess_gpu_builder.hpp -- the reference's component-pipeline API over the
// GPU library, header-only C++ on top of the C ABI (weavess_gpu.h).
//
// Mirrors weavess::IndexBuilder (include/weavess/builder.h:11-58 of the
// reference) for the path this library implements: the same method names and
// chaining (load / init / refine / save_graph / load_graph / search /
// print_index_info), the same TYPE names, a string-keyed Parameters with
// set<T> / get<T>, the reference's console lines, and its error convention (a
// message, then exit(-1), on an unsupported type or an unreadable file;
// Parameters::get throws on a missing name).  A program written against the
// reference's builder for these components changes its namespace and links
// libweavess_gpu.so:
//
//   weavess_gpu::IndexBuilder b(n_threads);
//   b.load(base, query, gt, params)->init(weavess_gpu::INIT_RANDOM)
//    ->refine(weavess_gpu::REFINE_NN_DESCENT, false)->refine(weavess_gpu::REFINE_NSG, false)
//    ->save_graph(weavess_gpu::INDEX_NSG, file);
//
// Supported: INIT_RANDOM, INIT_RAND, INIT_KDT; REFINE_NN_DESCENT, REFINE_NSG,
// REFINE_VAMANA, REFINE_SSG, REFINE_EFANNA; search entries RAND, CENTROID,
// SUB_CENTROID, KDT (ROUTER_GREEDY) and NONE (ROUTER_HNSW, ROUTER_NSW); the three
// L policies; graph files KGRAPH / EFANNA (no header), NSG / VAMANA (entry
// point), SSG (roots), HNSW and NSW (load only).  The rand() values the components
// draw come from the process's own rand(), as in the reference.
#pragma once

#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <set>
#include <sstream>
#include <stdexcept>
#include <string>
#include <typeinfo>
#include <unordered_map>
#include <vector>

#include "weavess_gpu.h"

namespace weavess_gpu {

// the reference's TYPE names (include/weavess/policy.h:9-31)
enum TYPE {
  INDEX_KGRAPH, INDEX_FANNG, INDEX_NSG, INDEX_SSG, INDEX_DPG, INDEX_VAMANA, INDEX_EFANNA, INDEX_IEH,
  INDEX_NSW, INDEX_HNSW, INDEX_ONNG, INDEX_PANNG, INDEX_HCNNG, INDEX_SPTAG_KDT, INDEX_SPTAG_BKT, INDEX_EXACT_KNNG,
  INDEX_KDRG,
  INIT_RANDOM, INIT_KNNG, INIT_KDT,
  REFINE_NN_DESCENT, REFINE_KDRG,
  INIT_NN_DESCENT, INIT_RAND, INIT_IEH, INIT_NSW, INIT_HNSW, INIT_ANNG, INIT_SPTAG_KDT, INIT_SPTAG_BKT, INIT_FANNG,
  INIT_HCNNG,
  REFINE_NSG, REFINE_SSG, REFINE_DPG, REFINE_VAMANA, REFINE_EFANNA, REFINE_PANNG, REFINE_SPTAG_KDT,
  REFINE_SPTAG_BKT, REFINE_FANNG, REFINE_ONNG,
  SEARCH_ENTRY_RAND, SEARCH_ENTRY_CENTROID, SEARCH_ENTRY_SUB_CENTROID, SEARCH_ENTRY_KDT, SEARCH_ENTRY_KDT_SINGLE,
  SEARCH_ENTRY_NONE, SEARCH_ENTRY_HASH, SEARCH_ENTRY_SPTAG_KDT, SEARCH_ENTRY_SPTAG_BKT, SEARCH_ENTRY_VPT,
  L_SEARCH_ASCEND, L_SEARCH_SET_RECALL, L_SEARCH_ASSIGN,
  ROUTER_GREEDY, ROUTER_IEH, ROUTER_NSW, ROUTER_HNSW, ROUTER_NGT, ROUTER_BACKTRACK, ROUTER_SPTAG_KDT,
  ROUTER_SPTAG_BKT, ROUTER_GUIDE
};

// string-keyed parameters (the reference's Parameters, parameters.h:11-56):
// values are kept as text and converted on get; a missing name throws
// std::invalid_argument, an unconvertible value std::runtime_error
class Parameters {
 public:
  template <typename T>
  void set(const std::string &name, const T &val) {
    std::ostringstream os;
    os << val;
    kv_[name] = os.str();
  }
  template <typename T>
  T get(const std::string &name) const {
    const auto it = kv_.find(name);
    if (it == kv_.end()) throw std::invalid_argument("Invalid paramter name : " + name + ".");
    std::istringstream is(it->second);
    T v;
    if (!(is >> v) || !is.eof())
      throw std::runtime_error("Fail to convert value" + it->second + " to type: " + typeid(v).name());
    return v;
  }
  bool has(const std::string &name) const { return kv_.count(name) != 0; }
  std::string toString() const {
    std::string out;
    for (const auto &p : kv_) out += p.first + ":" + p.second + " ";
    return out;
  }

 private:
  std::unordered_map<std::string, std::string> kv_;
};

namespace detail {

[[noreturn]] inline void die(const std::string &msg) {
  std::cerr << msg << std::endl;
  exit(-1);
}

// the reference's fvecs / ivecs reader (component_load.cpp:9-28): the first
// word is the dimension, num = file size / (dim + 1) / 4, every record's
// 4-byte header skipped
template <class T>
inline void load_vecs(const char *file, std::vector<T> &data, unsigned &num, unsigned &dim) {
  std::ifstream in(file, std::ios::binary);
  if (!in.is_open()) die("open file error");
  in.read(reinterpret_cast<char *>(&dim), 4);
  in.seekg(0, std::ios::end);
  const size_t bytes = static_cast<size_t>(in.tellg());
  num = static_cast<unsigned>(bytes / (dim + 1) / 4);
  data.resize(static_cast<size_t>(num) * dim);
  in.seekg(0, std::ios::beg);
  for (size_t i = 0; i < num; i++) {
    in.seekg(4, std::ios::cur);
    in.read(reinterpret_cast<char *>(data.data() + i * dim), dim * sizeof(T));
  }
}

// 1 - misses / (GroundLen * K) in FP32 (builder.cpp:306-320)
inline float accuracy(const std::vector<unsigned> &res, unsigned nq, unsigned K, const std::vector<unsigned> &gt,
                      unsigned gt_len, unsigned gt_dim) {
  int cnt = 0;
  for (unsigned i = 0; i < gt_len && i < nq; i++)
    for (unsigned j = 0; j < K; j++) {
      unsigned k = 0;
      for (; k < K; k++)
        if (res[static_cast<size_t>(i) * K + j] == gt[static_cast<size_t>(i) * gt_dim + k]) break;
      if (k == K) cnt++;
    }
  return 1 - static_cast<float>(cnt) / (gt_len * K);
}

}  // namespace detail

// the component pipeline (the reference's IndexBuilder, builder.cpp:22-487,
// 501-780, 918-1311) on one GPU
class IndexBuilder {
 public:
  // `num_threads` sizes the host-side work (the oracle-free library has
  // none that needs it); the GPU is device `device`
  explicit IndexBuilder(unsigned num_threads, int device = 0) {
    (void)num_threads;
    if (wv_ctx_create(&ctx_, device) != WV_OK) detail::die("no CUDA device for the GPU index builder");
    wv_set_rand_source(ctx_, &rand);  // the process's rand() stream, as the reference draws it
  }
  virtual ~IndexBuilder() {
    if (ctx_) wv_ctx_destroy(ctx_);
  }
  IndexBuilder(const IndexBuilder &) = delete;
  IndexBuilder &operator=(const IndexBuilder &) = delete;

  // the GPU context (for the batched and learned entry points of weavess_gpu.h)
  wv_ctx *context() { return ctx_; }
  // VAMANA::alpha (index.h:213-216): 1 at first; a Vamana link leaves it at 2
  float alpha = 1.0f;

  IndexBuilder *load(char *data_file, char *query_file, char *ground_file, Parameters &parameters) {
    detail::load_vecs(data_file, base_, n_, d_);
    detail::load_vecs(query_file, query_, nq_, qd_);
    detail::load_vecs(ground_file, gt_, gt_len_, gt_dim_);
    if (n_ == 0 || d_ == 0 || nq_ == 0 || qd_ != d_ || gt_len_ == 0) detail::die("load: bad base / query / ground file");
    params_ = parameters;
    check(wv_upload_base(ctx_, base_.data(), n_, d_), "upload base");
    std::cout << "base data len : " << n_ << std::endl;
    std::cout << "base data dim : " << d_ << std::endl;
    std::cout << "query data len : " << nq_ << std::endl;
    std::cout << "query data dim : " << qd_ << std::endl;
    std::cout << "ground truth data len : " << gt_len_ << std::endl;
    std::cout << "ground truth data dim : " << gt_dim_ << std::endl;
    std::cout << "=====================" << std::endl;
    std::cout << params_.toString() << std::endl;
    std::cout << "=====================" << std::endl;
    return this;
  }

  IndexBuilder *init(TYPE type, bool debug = false) {
    (void)debug;
    s_ = std::chrono::high_resolution_clock::now();
    if (type == INIT_RANDOM) {
      std::cout << "__INIT : RANDOM__" << std::endl;
      check(wv_init_random(ctx_, params_.get<unsigned>("S"), nullptr), "INIT_RANDOM");
    } else if (type == INIT_RAND) {
      std::cout << "__INIT : RAND__" << std::endl;
      check(wv_init_rand(ctx_, params_.get<unsigned>("L"), nullptr), "INIT_RAND");
    } else if (type == INIT_KDT) {
      std::cout << "__INIT : KDT__" << std::endl;
      check(wv_init_kdt(ctx_, params_.get<unsigned>("nTrees"), params_.get<unsigned>("K"),
                        params_.get<unsigned>("mLevel"), nullptr),
            "INIT_KDT");
    } else {
      detail::die("__INIT : WRONG TYPE__");
    }
    e_ = std::chrono::high_resolution_clock::now();
    std::cout << "__INIT FINISH__" << std::endl;
    return this;
  }

  IndexBuilder *refine(TYPE type, bool debug) {
    (void)debug;
    const Parameters &P = params_;
    if (type == REFINE_NN_DESCENT) {
      std::cout << "__REFINE : KGRAPH__" << std::endl;
      check(wv_nnd_refine(ctx_, P.get<unsigned>("S"), P.get<unsigned>("K"), P.get<unsigned>("L"),
                          P.get<unsigned>("ITER"), P.get<unsigned>("R"), nullptr), "REFINE_NN_DESCENT");
    } else if (type == REFINE_NSG) {
      std::cout << "__REFINE : NSG__" << std::endl;
      L_refine_ = P.get<unsigned>("L_refine");
      check(wv_nsg_refine(ctx_, L_refine_, P.get<unsigned>("R_refine"), P.get<unsigned>("C_refine"), nullptr),
            "REFINE_NSG");
    } else if (type == REFINE_VAMANA) {
      std::cout << "__REFINE : VAMANA__" << std::endl;
      // the entry search reads the index's L_refine member, which only the
      // NSG and SSG refines set (component_entry.cpp:32)
      check(wv_vamana_refine(ctx_, P.get<unsigned>("L_refine"), P.get<unsigned>("R_refine"), alpha, L_refine_,
                             nullptr), "REFINE_VAMANA");
      alpha = 2.0f;  // component_refine.cpp:871
    } else if (type == REFINE_SSG) {
      std::cout << "__REFINE : NSSG__" << std::endl;
      L_refine_ = P.get<unsigned>("L_refine");
      const unsigned n_try = P.get<unsigned>("n_try");
      eps_.assign(n_try, 0u);
      check(wv_ssg_refine(ctx_, L_refine_, P.get<unsigned>("R_refine"), P.get<float>("A"), n_try, eps_.data(),
                          nullptr), "REFINE_SSG");
    } else if (type == REFINE_EFANNA) {
      std::cout << "__REFINE : EFANNA__" << std::endl;
      check(wv_efanna_refine(ctx_, P.get<unsigned>("S"), P.get<unsigned>("K"), P.get<unsigned>("L"),
                             P.get<unsigned>("ITER"), P.get<unsigned>("R"), nullptr), "REFINE_EFANNA");
    } else {
      detail::die("__REFINE : WRONG TYPE__");
    }
    std::cout << "===================" << std::endl;
    std::cout << "__REFINE : FINISH__" << std::endl;
    std::cout << "===================" << std::endl;
    e_ = std::chrono::high_resolution_clock::now();
    return this;
  }

  std::chrono::duration<double> GetBuildTime() { return e_ - s_; }

  // the parameters the components read (the index's copy, as the reference keeps one)
  Parameters &getParam() { return params_; }

  IndexBuilder *save_graph(TYPE type, char *graph_file) {
    int hdr = WV_GRAPH_PLAIN;
    if (type == INDEX_NSG || type == INDEX_VAMANA) hdr = WV_GRAPH_EP;
    else if (type == INDEX_SSG) hdr = WV_GRAPH_EPS;
    else if (type != INDEX_KGRAPH && type != INDEX_EFANNA) detail::die("save_graph: type not supported here");
    check(wv_save_graph(ctx_, graph_file, hdr), "save_graph");
    return this;
  }

  IndexBuilder *load_graph(TYPE type, char *graph_file) {
    int hdr = WV_GRAPH_PLAIN;
    if (type == INDEX_NSG || type == INDEX_VAMANA) hdr = WV_GRAPH_EP;
    else if (type == INDEX_SSG) hdr = WV_GRAPH_EPS;
    else if (type == INDEX_HNSW) hdr = WV_GRAPH_HNSW;
    else if (type == INDEX_NSW) hdr = WV_GRAPH_NSW;
    else if (type == INDEX_EXACT_KNNG) return load_exact(graph_file);
    else if (type != INDEX_KGRAPH && type != INDEX_EFANNA) detail::die("load_graph: type not supported here");
    {
      std::ifstream probe(graph_file, std::ios::binary);
      if (!probe.is_open()) detail::die("load graph error");
    }
    check(wv_load_graph(ctx_, graph_file, hdr), "load_graph");
    loaded_ = type;
    return this;
  }

  IndexBuilder *search(TYPE entry_type, TYPE route_type, TYPE L_type) {
    std::cout << "__SEARCH__" << std::endl;
    const unsigned K = 10;
    params_.set<unsigned>("K_search", K);
    int entry = -1;
    if (route_type == ROUTER_GREEDY) {
      if (entry_type == SEARCH_ENTRY_RAND) entry = WV_ENTRY_RAND;
      else if (entry_type == SEARCH_ENTRY_CENTROID) entry = WV_ENTRY_CENTROID;
      else if (entry_type == SEARCH_ENTRY_SUB_CENTROID) entry = WV_ENTRY_SUB_CENTROID;
      // ComponentSearchEntryKDTSingle (component_search_entry.cpp:173-240) is
      // the same entry, line for line
      else if (entry_type == SEARCH_ENTRY_KDT || entry_type == SEARCH_ENTRY_KDT_SINGLE) entry = WV_ENTRY_KDT;
      else detail::die("__SEARCH ENTRY : WRONG TYPE__");
    } else if (route_type == ROUTER_HNSW || route_type == ROUTER_NSW) {
      if (entry_type != SEARCH_ENTRY_NONE) detail::die("__SEARCH ENTRY : WRONG TYPE__");
    } else {
      detail::die("__ROUTER : WRONG TYPE__");
    }
    res_.assign(static_cast<size_t>(nq_) * K, 0u);
    auto run = [&](unsigned L) -> float {
      std::cout << "SEARCH_L : " << L << std::endl;
      if (L < K) detail::die("search_L cannot be smaller than search_K! ");
      params_.set<unsigned>("L_search", L);
      wv_counters cnt{0, 0};
      const auto t0 = std::chrono::high_resolution_clock::now();
      if (route_type == ROUTER_GREEDY)
        check(wv_search(ctx_, query_.data(), nq_, entry, L, K, nullptr, res_.data(), nullptr, &cnt), "search");
      else
        check(wv_search_hnsw(ctx_, query_.data(), nq_, route_type == ROUTER_HNSW ? 0 : 1, L, K, res_.data(),
                             nullptr, &cnt), "search");
      const std::chrono::duration<double> dt = std::chrono::high_resolution_clock::now() - t0;
      std::cout << "search time: " << dt.count() << "\n";
      std::cout << "DistCount: " << cnt.dist_count << std::endl;
      std::cout << "HopCount: " << cnt.hop_count << std::endl;
      const float acc = detail::accuracy(res_, nq_, K, gt_, gt_len_, gt_dim_);
      std::cout << K << " NN accuracy: " << acc << std::endl;
      return acc;
    };
    if (L_type == L_SEARCH_SET_RECALL) {
      // the reference's walk toward the smallest L with accuracy >= 0.99 (builder.cpp:262-351)
      std::set<unsigned> visited;
      const unsigned sg = 1000;
      const float acc_set = 0.99f;
      bool flag = false;
      int L_sl = 1;
      unsigned L = K;
      visited.insert(L);
      unsigned L_min = 0x7fffffff;
      while (true) {
        const float acc = run(L);
        if (acc_set - acc <= 0) {
          if (L_min > L) L_min = L;
          if (L == K || L_sl == 1) break;
          if (!flag) {
            L_sl < 0 ? L_sl-- : L_sl++;
            flag = true;
          }
          L_sl /= 2;
          if (L_sl == 0) break;
          if (L_sl > 0) L_sl = -L_sl;
        } else {
          if (L_min < L) break;
          L_sl = static_cast<int>(sg * (acc_set - acc));
          if (L_sl == 0) L_sl++;
          flag = false;
        }
        L += L_sl;
        if (visited.count(L)) break;
        visited.insert(L);
      }
      std::cout << "L_min: " << L_min << std::endl;
    } else if (L_type == L_SEARCH_ASCEND) {
      unsigned L_st = 5, L_st2 = 8;
      for (unsigned i = 0; i < 10; i++) {
        const unsigned L = L_st + L_st2;
        L_st = L_st2;
        L_st2 = L;
        run(L);
      }
    } else if (L_type == L_SEARCH_ASSIGN) {
      run(params_.get<unsigned>("L_search"));
    } else {
      detail::die("__L TYPE : WRONG TYPE__");
    }
    return this;
  }

  // the last search's result ids, nq x 10 (what the reference keeps in `res`)
  const std::vector<unsigned> &results() const { return res_; }

  // degree statistics, conn and (with the parameter exact_knng_path) graph
  // quality of the loaded search graph, printed as the reference prints them
  IndexBuilder *print_index_info(TYPE type) {
    int hdr = WV_GRAPH_PLAIN;
    if (type == INDEX_NSG || type == INDEX_VAMANA) hdr = WV_GRAPH_EP;
    else if (type == INDEX_SSG) hdr = WV_GRAPH_EPS;
    else if (type == INDEX_HNSW || type == INDEX_NSW) hdr = WV_GRAPH_HNSW;
    std::vector<uint32_t> ex_ids, ex_deg;
    uint32_t ex_w = 0;
    if (params_.has("exact_knng_path")) {
      load_exact(const_cast<char *>(params_.get<std::string>("exact_knng_path").c_str()));
      for (const auto &r : exact_) ex_w = std::max<uint32_t>(ex_w, static_cast<uint32_t>(r.size()));
      ex_w = std::max<uint32_t>(ex_w, 1u);
      ex_ids.assign(static_cast<size_t>(n_) * ex_w, 0u);
      ex_deg.assign(n_, 0u);
      for (size_t i = 0; i < exact_.size() && i < n_; i++) {
        ex_deg[i] = static_cast<uint32_t>(exact_[i].size());
        std::copy(exact_[i].begin(), exact_[i].end(), ex_ids.begin() + i * ex_w);
      }
    }
    wv_index_stats st{};
    check(wv_index_info(ctx_, hdr, ex_w ? ex_ids.data() : nullptr, ex_w ? ex_deg.data() : nullptr, ex_w, &st),
          "print_index_info");
    printf("Degree Statistics: Max out degree = %d, Min out degree= %d, Avg out degree = %lf\n",
           static_cast<int>(st.max_out), static_cast<int>(st.min_out), st.avg_out);
    printf("Conn Statistics: conn = %d\n", static_cast<int>(st.conn));
    if (ex_w) std::cout << "Graph Quality : " << static_cast<float>(st.quality) << std::endl;
    return this;
  }

  // the SSG roots of the last SSG refine
  const std::vector<uint32_t> &eps() const { return eps_; }

 private:
  void check(int rc, const char *what) {
    if (rc != WV_OK) detail::die(std::string(what) + ": " + wv_last_error(ctx_));
  }

  // INDEX_EXACT_KNNG (builder.cpp:1289-1298): per node its count and ids, to
  // the end of the file
  IndexBuilder *load_exact(char *file) {
    std::ifstream in(file, std::ios::binary);
    if (!in.is_open()) detail::die("load graph error");
    exact_.clear();
    while (true) {
      unsigned gk;
      in.read(reinterpret_cast<char *>(&gk), 4);
      if (in.eof()) break;
      std::vector<unsigned> row(gk);
      in.read(reinterpret_cast<char *>(row.data()), static_cast<std::streamsize>(gk) * 4);
      exact_.push_back(std::move(row));
    }
    return this;
  }

  wv_ctx *ctx_ = nullptr;
  Parameters params_;
  std::vector<float> base_, query_;
  std::vector<unsigned> gt_, res_, eps_;
  std::vector<std::vector<unsigned>> exact_;
  unsigned n_ = 0, d_ = 0, nq_ = 0, qd_ = 0, gt_len_ = 0, gt_dim_ = 0;
  unsigned L_refine_ = 0;  // the index's L_refine member (set by the NSG and SSG refines)
  TYPE loaded_ = INDEX_KGRAPH;
  std::chrono::high_resolution_clock::time_point s_, e_;
};

}  // namespace weavess_gpu
