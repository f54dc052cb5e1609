// SEARCH_ENTRY_RAND seeds drawn on the device (wv_seeds.cu).
#pragma once
#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

struct wv_ctx;

namespace wv {

constexpr uint32_t SEED_MAX_L = 1536;

// shared memory of the seed kernel for beams up to Lmax
size_t seeds_rand_smem(uint32_t Lmax);
// seeds of nq queries (or of the first *d_nq, if d_nq is set) from their
// rand() values d_sv (one per query): query q gets L ids (d_L[q] if d_L is
// not null) at d_out + q * stride (a beam above Lmax or >= N sets
// DEV_OVERFLOW in *d_status and skips the query)
cudaError_t seeds_rand_launch(const uint32_t *d_sv, uint32_t nq, const uint32_t *d_nq, const uint32_t *d_L,
                              uint32_t L, uint32_t Lmax, uint32_t N, uint32_t *d_out, uint32_t stride, int *d_status,
                              cudaStream_t s);
// draws the nq rand() values from the context's stream (query order), copies
// them to the device and launches the seed kernel on the context's stream
int draw_seeds_rand_device(wv_ctx *c, uint32_t nq, const uint32_t *d_L, uint32_t L, uint32_t Lmax, uint32_t *d_out,
                           uint32_t stride);

// SearchEntrySubCentroid: the first n_eps seeds of every query (the first
// nq, or *d_nq) become the search graph's SSG roots (ctx->eps, uploaded here)
int put_roots_device(wv_ctx *c, uint32_t nq, const uint32_t *d_nq, uint32_t *d_out, uint32_t stride);

}  // namespace wv
