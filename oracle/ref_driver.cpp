// Reference driver: runs the UNMODIFIED WEAVESS component sources (compiled from
// where they lie by oracle/Makefile) on seeded inputs and dumps every
// intermediate result the GPU path is checked against.  Test infrastructure
// only -- never linked into the product.
//
// It follows the reference pipelines:
//   KGraph build   test/main.cpp:15-21   (init INIT_RANDOM, refine REFINE_NN_DESCENT)
//   Vamana link    src/component_refine.cpp:794-872 (alpha set on the index, as
//                  the reference has no parameter for it, index.h:213-216)
//   NSG link       src/component_refine.cpp:393-472
//   SSG link       src/component_refine.cpp:550-720, component_conn.cpp:169-225
//   search loop    src/builder.cpp:445-454 (L_SEARCH_ASSIGN, serial), with the
//                  result ids kept instead of only the recall print.
// One thread (IndexBuilder(1)), so the glibc rand() stream and every sort are
// deterministic.
//
// usage: ref_driver base.fvecs query.fvecs gt.ivecs outprefix key=val ... -- step ...
//   steps: init_random | init_rand | init_kdt | nndescent | efanna | vamana | nsg | ssg | load:<kgraph|vamana|nsg|ssg|efanna>
//          | hnsw | search_rand:<L> | search_centroid:<L> | search_sub:<L> | search_kdt:<L> | search_hnsw:<L>
//          | search_nsw:<L> | nsw | search_nswidx:<L> | policy:<rand|centroid>_<set_recall|ascend>
//          | rand_probe
//   (search_sub: SEARCH_ENTRY_SUB_CENTROID, the entry the reference's SSG
//   test searches with, test/main.cpp:117)
#include <bits/stdc++.h>
#include <omp.h>
#include <boost/dynamic_bitset.hpp>
#include <boost/shared_ptr.hpp>
#include <boost/heap/d_ary_heap.hpp>
#define private public
#define protected public
#include <weavess/builder.h>
#include <weavess/component.h>
#undef private
#undef protected

using namespace weavess;

static void write_final_graph(const std::string &path, Index *idx, bool with_ep) {
  FILE *f = fopen(path.c_str(), "wb");
  unsigned n = idx->getBaseLen();
  unsigned ep = with_ep ? idx->ep_ : 0xffffffffu;
  fwrite(&n, 4, 1, f);
  fwrite(&ep, 4, 1, f);
  auto &g = idx->getFinalGraph();
  for (unsigned i = 0; i < n; i++) {
    unsigned deg = (unsigned)g[i].size();
    fwrite(&deg, 4, 1, f);
    for (unsigned j = 0; j < deg; j++) {
      fwrite(&g[i][j].id, 4, 1, f);
      fwrite(&g[i][j].distance, 4, 1, f);
    }
  }
  fclose(f);
}

int main(int argc, char **argv) {
  if (argc < 6) {
    fprintf(stderr, "usage: %s base query gt outprefix k=v ... -- steps\n", argv[0]);
    return 2;
  }
  std::string prefix = argv[4];
  Parameters params;
  float alpha = 1.0f;
  int a = 5;
  for (; a < argc && std::string(argv[a]) != "--"; a++) {
    std::string kv = argv[a];
    auto p = kv.find('=');
    std::string k = kv.substr(0, p), v = kv.substr(p + 1);
    if (k == "alpha") alpha = std::stof(v);
    else params.set<std::string>(k, v);
  }
  a++;
  auto *builder = new IndexBuilder(1);
  builder->load(argv[1], argv[2], argv[3], params);
  Index *idx = builder->final_index_;
  // Members the reference reads without ever setting on these paths
  // (e.g. L_refine for the Vamana entry, component_entry.cpp:32) start at 0,
  // as they do in a fresh process where `new Index()` gets zeroed pages.
  idx->L_refine = 0;
  idx->R_refine = 0;
  idx->C_refine = 0;
  idx->alpha = alpha;
  // ComponentSearchEntrySubCentroid reads the base row shifted by one float
  // (component_search_entry.cpp:84-86), so for the last row it reads one
  // float past the array.  The driver gives that float a defined value, 0 --
  // what a fresh allocation above the mmap threshold holds there.
  {
    const size_t nd = (size_t)idx->getBaseLen() * idx->getBaseDim();
    float *padded = new float[nd + 4]();
    std::memcpy(padded, idx->getBaseData(), nd * sizeof(float));
    idx->setBaseData(padded);
  }
  for (; a < argc; a++) {
    std::string step = argv[a];
    std::string arg;
    auto c = step.find(':');
    if (c != std::string::npos) {
      arg = step.substr(c + 1);
      step = step.substr(0, c);
    }
    auto t0 = std::chrono::high_resolution_clock::now();
    if (step == "init_random") {
      builder->init(INIT_RANDOM, false);
      write_final_graph(prefix + ".init.bin", idx, false);
    } else if (step == "init_kdt") {
      // INIT_KDT (component_init.cpp:500-640): the graph and the trees' id lists
      builder->init(INIT_KDT, false);
      write_final_graph(prefix + ".initkdt.bin", idx, false);
      FILE *f = fopen((prefix + ".kdtleaf.bin").c_str(), "wb");
      unsigned T = (unsigned)idx->LeafLists.size(), n = idx->getBaseLen();
      fwrite(&T, 4, 1, f);
      fwrite(&n, 4, 1, f);
      for (unsigned t = 0; t < T; t++) fwrite(idx->LeafLists[t].data(), 4, n, f);
      fclose(f);
    } else if (step == "init_rand") {
      builder->init(INIT_RAND, false);
      write_final_graph(prefix + ".initrand.bin", idx, false);
    } else if (step == "nndescent") {
      builder->refine(REFINE_NN_DESCENT, false);
      write_final_graph(prefix + ".nnd.bin", idx, false);
    } else if (step == "hnsw") {
      // INIT_HNSW (component_init.cpp:1340-1540; its level rng is seeded per
      // thread, so one thread makes it deterministic); the graph file the
      // reference writes for it (save_graph, builder.cpp:925-944) is dumped
      // byte for byte
      builder->init(INIT_HNSW, false);
      std::string gf = prefix + ".hnswgraph.bin";
      builder->save_graph(INDEX_HNSW, &gf[0]);
    } else if (step == "nsw") {
      // INIT_NSW (component_init.cpp:1242-1340), one thread; the INDEX_NSW file
      // the reference writes for it (builder.cpp:987-999) dumped byte for byte
      builder->init(INIT_NSW, false);
      std::string gf = prefix + ".nswgraph.bin";
      builder->save_graph(INDEX_NSW, &gf[0]);
    } else if (step == "search_nswidx") {
      // ROUTER_NSW over the graph load_graph(INDEX_NSW) reads back (builder.cpp:1171-1189)
      std::string gf = prefix + ".nswgraph.bin";
      builder->load_graph(INDEX_NSW, &gf[0]);
      unsigned L = (unsigned)std::stoul(arg);
      idx->getParam().set<unsigned>("K_search", 10);
      idx->getParam().set<unsigned>("L_search", L);
      auto *r = new ComponentSearchRouteNSW(idx);
      idx->resetDistCount();
      idx->resetHopCount();
      unsigned nq = idx->getQueryLen();
      std::vector<std::vector<unsigned>> res(nq);
      for (unsigned i = 0; i < nq; i++) {
        std::vector<Index::Neighbor> pool;
        r->RouteInner(i, pool, res[i]);
      }
      std::string out = prefix + "." + step + "_" + arg + ".bin";
      FILE *f = fopen(out.c_str(), "wb");
      fwrite(&nq, 4, 1, f);
      unsigned k = 10;
      fwrite(&k, 4, 1, f);
      for (unsigned i = 0; i < nq; i++) fwrite(res[i].data(), 4, 10, f);
      unsigned dc = idx->getDistCount(), hc = idx->getHopCount();
      fwrite(&dc, 4, 1, f);
      fwrite(&hc, 4, 1, f);
      fclose(f);
    } else if (step == "search_hnsw" || step == "search_nsw") {
      // ROUTER_HNSW / ROUTER_NSW (component_route.cpp:56-260) over the graph
      // as load_graph(INDEX_HNSW) reads it back
      std::string gf = prefix + ".hnswgraph.bin";
      builder->load_graph(INDEX_HNSW, &gf[0]);
      unsigned L = (unsigned)std::stoul(arg);
      idx->getParam().set<unsigned>("K_search", 10);
      idx->getParam().set<unsigned>("L_search", L);
      ComponentSearchRoute *r = step == "search_hnsw" ? (ComponentSearchRoute *)new ComponentSearchRouteHNSW(idx)
                                                      : (ComponentSearchRoute *)new ComponentSearchRouteNSW(idx);
      idx->resetDistCount();
      idx->resetHopCount();
      unsigned nq = idx->getQueryLen();
      std::vector<std::vector<unsigned>> res(nq);
      for (unsigned i = 0; i < nq; i++) {
        std::vector<Index::Neighbor> pool;
        r->RouteInner(i, pool, res[i]);
      }
      std::string out = prefix + "." + step + "_" + arg + ".bin";
      FILE *f = fopen(out.c_str(), "wb");
      fwrite(&nq, 4, 1, f);
      unsigned k = 10;
      fwrite(&k, 4, 1, f);
      for (unsigned i = 0; i < nq; i++) fwrite(res[i].data(), 4, 10, f);
      unsigned dc = idx->getDistCount(), hc = idx->getHopCount();
      fwrite(&dc, 4, 1, f);
      fwrite(&hc, 4, 1, f);
      fclose(f);
    } else if (step == "efanna") {
      // REFINE_EFANNA (component_refine.cpp:959-1178) on the current graph
      builder->refine(REFINE_EFANNA, false);
      write_final_graph(prefix + ".efanna.bin", idx, false);
    } else if (step == "vamana") {
      // alpha is set once, at load; the reference itself sets it to 2 at the
      // end of every Vamana link (component_refine.cpp:871)
      builder->refine(REFINE_VAMANA, false);
      write_final_graph(prefix + ".vamana.bin", idx, true);
    } else if (step == "nsg") {
      builder->refine(REFINE_NSG, false);
      write_final_graph(prefix + ".nsg.bin", idx, true);
    } else if (step == "ssg") {
      // REFINE_SSG (component_refine.cpp:550-582): Propagation2 candidates,
      // SSG prune, InterInsert, DFS-expand conn from n_try shuffled roots
      builder->refine(REFINE_SSG, false);
      write_final_graph(prefix + ".ssg.bin", idx, false);
      FILE *f = fopen((prefix + ".ssgeps.bin").c_str(), "wb");
      unsigned ne = (unsigned)idx->eps_.size();
      fwrite(&ne, 4, 1, f);
      fwrite(idx->eps_.data(), 4, ne, f);
      fclose(f);
    } else if (step == "load") {
      TYPE t = arg == "kgraph" ? INDEX_KGRAPH
               : arg == "vamana" ? INDEX_VAMANA
               : arg == "ssg"    ? INDEX_SSG
               : arg == "efanna" ? INDEX_KGRAPH
                                 : INDEX_NSG;
      std::string gf = prefix + "." + arg + ".graph";
      builder->save_graph(t, &gf[0]);
      idx->getLoadGraph().clear();
      builder->load_graph(t, &gf[0]);
    } else if (step == "search_rand" || step == "search_centroid" || step == "search_sub" || step == "search_kdt") {
      unsigned L = (unsigned)std::stoul(arg);
      idx->getParam().set<unsigned>("K_search", 10);
      idx->getParam().set<unsigned>("L_search", L);
      ComponentSearchEntry *e =
          step == "search_rand"       ? (ComponentSearchEntry *)new ComponentSearchEntryRand(idx)
          : step == "search_centroid" ? (ComponentSearchEntry *)new ComponentSearchEntryCentroid(idx)
          : step == "search_kdt"      ? (ComponentSearchEntry *)new ComponentSearchEntryKDT(idx)
                                      : (ComponentSearchEntry *)new ComponentSearchEntrySubCentroid(idx);
      auto *r = new ComponentSearchRouteGreedy(idx);
      idx->resetDistCount();
      idx->resetHopCount();
      unsigned nq = idx->getQueryLen();
      std::vector<std::vector<unsigned>> res(nq);
      for (unsigned i = 0; i < nq; i++) {
        std::vector<Index::Neighbor> pool;
        e->SearchEntryInner(i, pool);
        r->RouteInner(i, pool, res[i]);
      }
      std::string out = prefix + "." + step + "_" + arg + ".bin";
      FILE *f = fopen(out.c_str(), "wb");
      fwrite(&nq, 4, 1, f);
      unsigned k = 10;
      fwrite(&k, 4, 1, f);
      for (unsigned i = 0; i < nq; i++) fwrite(res[i].data(), 4, 10, f);
      unsigned dc = idx->getDistCount(), hc = idx->getHopCount();
      fwrite(&dc, 4, 1, f);
      fwrite(&hc, 4, 1, f);
      fclose(f);
      // components own (and would delete) the index; leak them as the reference does
    } else if (step == "policy") {
      // IndexBuilder::search (builder.cpp:187-487) with its L policy, entry
      // rand or centroid, ROUTER_GREEDY: arg = "<rand|centroid>_<set_recall|ascend>".
      // The loop prints each L, DistCount, HopCount and accuracy; they are
      // captured from std::cout and dumped as (L, dist_count, hop_count, acc).
      auto us = arg.find('_');
      std::string ent = arg.substr(0, us), pol = arg.substr(us + 1);
      idx->resetDistCount();  // the counters start from zero, as in a fresh search
      idx->resetHopCount();
      std::stringstream ss;
      std::streambuf *old = std::cout.rdbuf(ss.rdbuf());
      builder->search(ent == "rand" ? SEARCH_ENTRY_RAND : SEARCH_ENTRY_CENTROID, ROUTER_GREEDY,
                      pol == "ascend" ? L_SEARCH_ASCEND : L_SEARCH_SET_RECALL);
      std::cout.rdbuf(old);
      std::vector<unsigned> Ls, dcs, hcs;
      std::vector<float> accs;
      std::string line;
      while (std::getline(ss, line)) {
        unsigned v;
        float a;
        if (sscanf(line.c_str(), "SEARCH_L : %u", &v) == 1) Ls.push_back(v);
        else if (sscanf(line.c_str(), "DistCount: %u", &v) == 1) dcs.push_back(v);
        else if (sscanf(line.c_str(), "HopCount: %u", &v) == 1) hcs.push_back(v);
        else if (sscanf(line.c_str(), "10 NN accuracy: %f", &a) == 1) accs.push_back(a);
      }
      std::string out = prefix + ".policy_" + arg + ".bin";
      FILE *f = fopen(out.c_str(), "wb");
      unsigned cnt = (unsigned)Ls.size();
      fwrite(&cnt, 4, 1, f);
      for (unsigned i = 0; i < cnt; i++) {
        unsigned rec[3] = {Ls[i], i < dcs.size() ? dcs[i] : 0u, i < hcs.size() ? hcs[i] : 0u};
        float a = i < accs.size() ? accs[i] : -1.f;
        fwrite(rec, 4, 3, f);
        fwrite(&a, 4, 1, f);
      }
      fclose(f);
    } else if (step == "rand_probe") {
      // consumes one value of the process rand() stream and reports it
      printf("rand_probe %d\n", rand());
    } else {
      fprintf(stderr, "unknown step %s\n", step.c_str());
      return 2;
    }
    auto t1 = std::chrono::high_resolution_clock::now();
    printf("step %s%s%s %.6f s\n", step.c_str(), arg.empty() ? "" : ":", arg.c_str(),
           std::chrono::duration<double>(t1 - t0).count());
    fflush(stdout);
  }
  return 0;
}
