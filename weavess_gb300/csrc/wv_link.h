// Vamana / NSG / SSG link on the GPU (REFINE_VAMANA, REFINE_NSG, REFINE_SSG).
#pragma once
#include <cstdint>
#include <vector>

#include "wv_ctx.h"

namespace wv {

enum class LinkMode { VAMANA, NSG, SSG };

struct LinkParams {
  uint32_t L;        // L_refine: beam of the candidate searches (SSG: candidate pool size)
  uint32_t R;        // R_refine: row width
  uint32_t C;        // C_refine: candidates examined by the NSG prune
  float alpha;       // Vamana occlusion factor
  uint32_t entry_L;  // the index's L_refine member read by the entry search (0: ep_ = 0)
  LinkMode mode;
  float A = 0.f;     // SSG: angle bound in degrees
  // Vamana, clean mode: short prune pools sorted, the overflow re-prune of
  // InterInsert closest first against each candidate's own distance
  bool clean = false;
};

struct LinkStats {
  uint32_t ep = 0;
  uint32_t levels = 0;  // InterInsert dependency levels
  float ms = 0;
};

// Link on ctx->fg_* (candidate graph) -> ctx->fg_* (rows of width R, ep set)
int link_gpu(wv_ctx *c, const LinkParams &p, LinkStats *st);
// ComponentConnNSGDFS on ctx->fg_* (may widen the rows)
int conn_dfs_gpu(wv_ctx *c, uint32_t L_refine, uint32_t *added);
// ComponentConnSSGDFS on ctx->fg_* (rows keep width R): draws the n_try roots
// (eps) and links every node from them
int conn_ssg_gpu(wv_ctx *c, uint32_t n_try, uint32_t R, std::vector<uint32_t> &eps, uint32_t *added);

}  // namespace wv
