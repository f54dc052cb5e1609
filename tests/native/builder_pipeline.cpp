// A test program written the way the reference's test/main.cpp drives its
// builder, against weavess_gpu::IndexBuilder (include/weavess_gpu_builder.hpp).
//
// usage: builder_pipeline base.fvecs query.fvecs gt.ivecs outprefix key=value ... -- step ...
//   steps: init_random | init_rand | init_kdt | nndescent | nsg | vamana | ssg | efanna
//          | save:<kgraph|nsg|vamana|ssg> | load:<kgraph|nsg|vamana|ssg|hnsw>
//          | search:<rand|centroid|sub|kdt|hnsw|nsw>:<L>   (L_SEARCH_ASSIGN; ids to outprefix.sN.bin)
//          | policy:<rand|centroid>:<set_recall|ascend> | info:<nsg|...>
// The parameter alpha (if given) sets the builder's Vamana alpha before the
// first step, as a harness sets the reference's index member.
#include <cstdio>
#include <cstring>
#include <string>

#include "weavess_gpu_builder.hpp"

using namespace weavess_gpu;

static TYPE index_type(const std::string &s) {
  if (s == "nsg") return INDEX_NSG;
  if (s == "vamana") return INDEX_VAMANA;
  if (s == "ssg") return INDEX_SSG;
  if (s == "efanna") return INDEX_EFANNA;
  if (s == "hnsw") return INDEX_HNSW;
  return INDEX_KGRAPH;
}

int main(int argc, char **argv) {
  if (argc < 6) {
    fprintf(stderr, "usage: %s base query gt outprefix k=v ... -- steps\n", argv[0]);
    return 2;
  }
  const std::string prefix = argv[4];
  Parameters params;
  float alpha = -1.f;
  int a = 5;
  for (; a < argc && std::string(argv[a]) != "--"; a++) {
    const std::string kv = argv[a];
    const auto eq = kv.find('=');
    const std::string k = kv.substr(0, eq), v = kv.substr(eq + 1);
    if (k == "alpha") alpha = std::stof(v);
    else params.set<std::string>(k, v);
  }
  a++;
  IndexBuilder builder(1);
  builder.load(argv[1], argv[2], argv[3], params);
  if (alpha > 0) builder.alpha = alpha;
  int nsearch = 0;
  for (; a < argc; a++) {
    std::string step = argv[a], arg, arg2;
    auto c = step.find(':');
    if (c != std::string::npos) {
      arg = step.substr(c + 1);
      step = step.substr(0, c);
      auto c2 = arg.find(':');
      if (c2 != std::string::npos) {
        arg2 = arg.substr(c2 + 1);
        arg = arg.substr(0, c2);
      }
    }
    std::string file = prefix + "." + arg + ".graph";
    if (step == "init_random") builder.init(INIT_RANDOM);
    else if (step == "init_rand") builder.init(INIT_RAND);
    else if (step == "init_kdt") builder.init(INIT_KDT);
    else if (step == "nndescent") builder.refine(REFINE_NN_DESCENT, false);
    else if (step == "nsg") builder.refine(REFINE_NSG, false);
    else if (step == "vamana") builder.refine(REFINE_VAMANA, false);
    else if (step == "ssg") builder.refine(REFINE_SSG, false);
    else if (step == "efanna") builder.refine(REFINE_EFANNA, false);
    else if (step == "save") builder.save_graph(index_type(arg), &file[0]);
    else if (step == "load") builder.load_graph(index_type(arg), &file[0]);
    else if (step == "info") builder.print_index_info(index_type(arg));
    else if (step == "search" || step == "policy") {
      TYPE entry = SEARCH_ENTRY_RAND, route = ROUTER_GREEDY;
      if (arg == "centroid") entry = SEARCH_ENTRY_CENTROID;
      else if (arg == "sub") entry = SEARCH_ENTRY_SUB_CENTROID;
      else if (arg == "kdt") entry = SEARCH_ENTRY_KDT;
      else if (arg == "hnsw" || arg == "nsw") {
        entry = SEARCH_ENTRY_NONE;
        route = arg == "hnsw" ? ROUTER_HNSW : ROUTER_NSW;
      }
      if (step == "search") {
        builder.getParam().set<unsigned>("L_search", (unsigned)std::stoul(arg2));
        builder.search(entry, route, L_SEARCH_ASSIGN);
        const std::string out = prefix + ".s" + std::to_string(nsearch++) + ".bin";
        FILE *f = fopen(out.c_str(), "wb");
        fwrite(builder.results().data(), 4, builder.results().size(), f);
        fclose(f);
      } else {
        builder.search(entry, route, arg2 == "ascend" ? L_SEARCH_ASCEND : L_SEARCH_SET_RECALL);
      }
    } else {
      fprintf(stderr, "unknown step %s\n", step.c_str());
      return 2;
    }
  }
  printf("pipeline done\n");
  return 0;
}
