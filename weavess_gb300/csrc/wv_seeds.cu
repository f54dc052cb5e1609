// SEARCH_ENTRY_RAND seeds on the device.
//
// ComponentSearchEntryRand::SearchEntryInner (src/component_search_entry.cpp
// :9-30) seeds a std::mt19937 with one rand() per query and draws the query's
// L entry ids with GenRandom (include/weavess/util.h:13-27):
//   addr[i] = rng() % (N - L) for i < L; sort; addr[i] = max(addr[i],
//   addr[i-1] + 1); off = rng() % N; addr[i] = (addr[i] + off) % N.
// The host draws the rand() values in query order (the reference's shared
// stream) and ships 4 bytes per query; one warp per query then seeds its
// mt19937 (lane 0 runs the seeding recurrence), twists it as often as L + 1
// outputs need, sorts the L residues (bitonic, ints: any correct sort gives
// the same array), bumps duplicates with a prefix maximum of
// addr[i] - i, and writes the ids.  Identical to the host draw
// (wv_host.cpp gen_random) bit for bit.
#include <cstdint>
#include <algorithm>
#include <vector>

#include "wv_common.cuh"
#include "wv_ctx.h"
#include "wv_mt.cuh"
#include "wv_seeds.h"

namespace wv {
namespace {

constexpr int SEED_WARPS = 4;

__global__ void __launch_bounds__(SEED_WARPS * 32)
    k_seeds_rand(const uint32_t *sv, uint32_t nq, const uint32_t *nq_dev, const uint32_t *Lq, uint32_t L0,
                 uint32_t Lmax, uint32_t N, uint32_t *out, uint32_t stride, int *status) {
  const uint32_t Pmax = pow2_ge(Lmax);
  extern __shared__ uint32_t sm[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  uint32_t *mt = sm + (size_t)warp * (624 + Pmax + 1);
  uint32_t *key = mt + 624;
  const uint32_t q = blockIdx.x * SEED_WARPS + warp;
  if (q >= (nq_dev ? min(*nq_dev, nq) : nq)) return;  // warp-uniform
  const uint32_t L = Lq ? Lq[q] : L0;
  if (L > Lmax || L >= N) {  // the host checks; a device-side beam list may not
    if (lane == 0) set_err(status, DEV_OVERFLOW);
    return;
  }
  if (lane == 0) {
    uint32_t x = sv[q];
    mt[0] = x;
    for (uint32_t i = 1; i < 624; i++) {
      x = mt_seed_next(x, i);
      mt[i] = x;
    }
  }
  __syncwarp();
  // outputs 0..L-1 are the residues, output L the offset
  const uint32_t span = N - L;
  for (uint32_t base = 0; base <= L; base += 624) {
    mt_twist_warp(mt, lane);
    for (uint32_t i = lane; i < 624 && base + i <= L; i += 32) {
      const uint32_t v = mt_temper(mt[i]);
      key[base + i] = base + i < L ? v % span : v % N;
    }
    __syncwarp();
  }
  const uint32_t off = key[L];
  __syncwarp();
  warp_gen_random_tail(key, L, off, N, out + (size_t)q * stride, lane);
}

__global__ void k_put_roots(uint32_t nq, const uint32_t *d_nq, const uint32_t *roots, uint32_t nr, uint32_t *out,
                            uint32_t stride) {
  const uint32_t n = d_nq ? min(nq, *d_nq) : nq;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < (size_t)n * nr; t += (size_t)gridDim.x * blockDim.x)
    out[(t / nr) * stride + t % nr] = roots[t % nr];
}

}  // namespace

int put_roots_device(wv_ctx *c, uint32_t nq, const uint32_t *d_nq, uint32_t *d_out, uint32_t stride) {
  const uint32_t nr = (uint32_t)c->eps.size();
  WV_CHECK(c, nr > 0, WV_ERR_STATE, "the search graph has no SSG roots");
  WV_CHECK(c, nr <= stride, WV_ERR_ARG, "%u roots do not fit a seed row of %u", nr, stride);
  if (nq == 0) return WV_OK;
  cudaError_t e = cudaSuccess;
  uint32_t *d_roots = c->buf<uint32_t>("sd_roots", nr, &e);
  WV_CUDA(c, e);
  WV_CUDA(c, cudaMemcpyAsync(d_roots, c->eps.data(), (size_t)nr * 4, cudaMemcpyHostToDevice, c->stream));
  const size_t total = (size_t)nq * nr;
  const int blocks = (int)std::min<size_t>((total + 255) / 256, (size_t)c->sms * 8);
  k_put_roots<<<blocks, 256, 0, c->stream>>>(nq, d_nq, d_roots, nr, d_out, stride);
  WV_CUDA(c, cudaGetLastError());
  WV_CUDA(c, cudaStreamSynchronize(c->stream));  // the roots' host copy may change after this call
  return WV_OK;
}

size_t seeds_rand_smem(uint32_t Lmax) { return (size_t)SEED_WARPS * (624 + pow2_ge(Lmax) + 1) * 4; }

cudaError_t seeds_rand_launch(const uint32_t *d_sv, uint32_t nq, const uint32_t *d_nq, const uint32_t *d_L,
                              uint32_t L, uint32_t Lmax, uint32_t N, uint32_t *d_out, uint32_t stride, int *d_status,
                              cudaStream_t s) {
  if (nq == 0) return cudaSuccess;
  const size_t smem = seeds_rand_smem(Lmax);
  cudaError_t e = cudaFuncSetAttribute(k_seeds_rand, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  const uint32_t blocks = (nq + SEED_WARPS - 1) / SEED_WARPS;
  k_seeds_rand<<<blocks, SEED_WARPS * 32, smem, s>>>(d_sv, nq, d_nq, d_L, L, Lmax, N, d_out, stride, d_status);
  return cudaGetLastError();
}

// the per-query rand() values, drawn in query order, and the device draw
int draw_seeds_rand_device(wv_ctx *c, uint32_t nq, const uint32_t *d_L, uint32_t L, uint32_t Lmax, uint32_t *d_out,
                           uint32_t stride) {
  WV_CHECK(c, Lmax < c->n, WV_ERR_ARG, "L=%u must be smaller than n=%u", Lmax, c->n);
  WV_CHECK(c, Lmax <= SEED_MAX_L, WV_ERR_LIMIT, "L=%u above %u", Lmax, SEED_MAX_L);
  std::vector<uint32_t> sv(nq);
  for (uint32_t q = 0; q < nq; q++) sv[q] = (uint32_t)c->rnd.next();
  cudaError_t e = cudaSuccess;
  uint32_t *d_sv = c->buf<uint32_t>("sd_sv", nq, &e);
  WV_CUDA(c, e);
  WV_CUDA(c, cudaMemcpyAsync(d_sv, sv.data(), (size_t)nq * 4, cudaMemcpyHostToDevice, c->stream));
  WV_CUDA(c, cudaStreamSynchronize(c->stream));  // sv is consumed before it goes out of scope
  WV_CUDA(c, seeds_rand_launch(d_sv, nq, nullptr, d_L, L, Lmax, c->n, d_out, stride, c->d_status(), c->stream));
  return WV_OK;
}

}  // namespace wv
