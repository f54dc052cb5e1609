#pragma once
#include <cstdint>

#include "wv_ctx.h"

namespace wv {
// sorts every segment keys[off[i], off[i] + cnt[i]) ascending, in place
int segsort_u64(wv_ctx *c, unsigned long long *keys, const uint32_t *off, const uint32_t *cnt, uint32_t nseg);
}  // namespace wv
