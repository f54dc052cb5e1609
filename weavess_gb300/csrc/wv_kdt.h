// INIT_KDT and the SEARCH_ENTRY_KDT seeds (wv_kdt.cu).
#pragma once
#include <cstdint>
#include <vector>

struct wv_ctx;

namespace wv {

// one node of a randomised KD-tree (Index::EFANNA::Node, index.h:219-231):
// ids [start, end) of the tree's id list; left / right -1 for a leaf
struct KNode {
  int dim;
  float val;
  uint32_t start, end;
  int left, right, parent;
  int depth, tree;
};

// the forest of the last wv_init_kdt on the current base (n, T, node count;
// all 0 while none): its nodes and T x n id lists stay in the context's work
// buffers "kd_nodes" / "kd_leaf" (node t is the root of tree t) for the
// search entry.  Set only when an init completed: an init that fails part
// way (the buffers then hold a partial forest) leaves it cleared.
struct KdtForest {
  uint32_t n = 0, T = 0, nodes = 0;
};

// INIT_KDT on the uploaded base: the current graph becomes the KD-tree graph
// (rows of K, ascending) and the forest is kept for SEARCH_ENTRY_KDT
int init_kdt_gpu(wv_ctx *c, uint32_t T, uint32_t K, uint32_t mlevel);

// SEARCH_ENTRY_KDT seeds of nq host queries (numbered 0..nq-1, the numbers
// the reference flags), rand() fills drawn from the context's stream
int draw_seeds_kdt(wv_ctx *c, const float *queries, uint32_t nq, uint32_t L, uint32_t *seeds, uint32_t stride);

}  // namespace wv
