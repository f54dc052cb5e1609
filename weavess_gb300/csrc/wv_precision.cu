// Low-precision copies of the base for candidate distances (bf16, fp8 e4m3
// with a per-row scale) and the diagnostic that reports their distances.
#include <cuda_bf16.h>
#include <cuda_fp8.h>

#include <vector>

#include "wv_common.cuh"
#include "wv_ctx.h"
#include "wv_lowp.cuh"

using namespace wv;

namespace {

__global__ void k_to_bf16(const float *x, size_t count, __nv_bfloat16 *out) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < count; i += (size_t)gridDim.x * blockDim.x)
    out[i] = __float2bfloat16_rn(x[i]);
}

// one warp per row: scale = max|x| / 448 (the largest finite e4m3 value)
__global__ void k_to_fp8(const float *x, uint32_t n, uint32_t d, __nv_fp8_storage_t *out, float *scale) {
  const int lane = threadIdx.x & 31;
  const uint32_t w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
  for (uint32_t r = w; r < n; r += nw) {
    const float *row = x + (size_t)r * d;
    float m = 0.f;
    for (uint32_t k = lane; k < d; k += 32) m = fmaxf(m, fabsf(row[k]));
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(FULL, m, o));
    const float sc = m > 0.f ? m / 448.f : 1.f;
    for (uint32_t k = lane; k < d; k += 32)
      out[(size_t)r * d + k] = __nv_cvt_float_to_fp8(row[k] / sc, __NV_SATFINITE, __NV_E4M3);
    if (lane == 0) scale[r] = sc;
  }
}

// squared norms of the stored low-precision rows, dequantised (warp per row)
__global__ void k_lowp_norms(const void *rows, const float *scale, int storage, uint32_t n, uint32_t d, float *out) {
  const int lane = threadIdx.x & 31;
  const uint32_t w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
  for (uint32_t r = w; r < n; r += nw) {
    float a = 0.f;
    for (uint32_t k = lane; k < d; k += 32) {
      float x;
      if (storage == 1) {
        x = __bfloat162float(reinterpret_cast<const __nv_bfloat16 *>(rows)[(size_t)r * d + k]);
      } else {
        const __half_raw h =
            __nv_cvt_fp8_to_halfraw(reinterpret_cast<const __nv_fp8_storage_t *>(rows)[(size_t)r * d + k], __NV_E4M3);
        x = scale[r] * __half2float(*reinterpret_cast<const __half *>(&h));
      }
      a = fmaf(x, x, a);
    }
    for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(FULL, a, o);
    if (lane == 0) out[r] = a;
  }
}

// out[q, j] = candidate distance of query q to base id ids[q, j]: fp32 in the
// reference's order, or the search kernel's low-precision distance (one warp
// per query and 32 ids, the same lowp_rows_dist the search calls)
__global__ void k_cand_dist(const float *base, LowpRows lp, int base_int, uint32_t d, const float *queries,
                            const uint32_t *ids, uint32_t nq, uint32_t m, float *out) {
  const int lane = threadIdx.x & 31;
  const size_t w = (blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5;
  const uint32_t chunks = (m + 31) / 32;
  if (w >= (size_t)nq * chunks) return;
  const uint32_t q = (uint32_t)(w / chunks), j0 = (uint32_t)(w % chunks) * 32;
  const int cnt = (int)min(32u, m - j0);
  const float *qv = queries + (size_t)q * d;
  const uint32_t my = lane < cnt ? ids[(size_t)q * m + j0 + lane] : 0u;
  float qn = 0.f;
  bool qint = true;
  for (uint32_t k = lane; k < d; k += 32) {
    qn = fmaf(qv[k], qv[k], qn);
    qint &= qv[k] >= 0.f && qv[k] <= 255.f && qv[k] == rintf(qv[k]);
  }
  for (int o = 16; o > 0; o >>= 1) qn += __shfl_xor_sync(FULL, qn, o);
  // as the search: the difference form for integer data at d > 128
  if (lp.norm && base_int && d > 128 && __all_sync(FULL, qint)) lp.norm = nullptr;
  float v;
  if (lp.storage == 0) {
    v = 0.f;
    if (lane < cnt) {
      const float4 *row = reinterpret_cast<const float4 *>(base + (size_t)my * d);
      const float4 *q4 = reinterpret_cast<const float4 *>(qv);
      for (uint32_t g = 0; g < d / 4; g++) v = __fadd_rn(v, group4(row[g], q4[g]));
    }
  } else {
    v = lowp_rows_dist(lp, my, cnt, qv, qn, lane);
  }
  if (lane < cnt) out[(size_t)q * m + j0 + lane] = v;
}

}  // namespace

extern "C" {

int wv_set_search_precision(wv_ctx *c, int storage, uint32_t rerank) {
  if (!c) return WV_ERR_ARG;
  WV_CHECK(c, storage >= 0 && storage <= 2, WV_ERR_ARG, "unknown storage %d", storage);
  WV_CHECK(c, c->n > 0, WV_ERR_STATE, "no base uploaded");
  WV_CHECK(c, c->d % 4 == 0, WV_ERR_LIMIT, "dimension %u is not a multiple of 4", c->d);
  WV_CUDA(c, cudaSetDevice(c->device));
  const size_t count = (size_t)c->n * c->d;
  if (storage == 1) {
    WV_CUDA(c, c->qbase.ensure(count * 2));
    k_to_bf16<<<c->sms * 16, 256, 0, c->stream>>>(c->base.as<float>(), count, c->qbase.as<__nv_bfloat16>());
  } else if (storage == 2) {
    WV_CUDA(c, c->qbase.ensure(count));
    WV_CUDA(c, c->qscale.ensure((size_t)c->n * 4));
    k_to_fp8<<<c->sms * 16, 256, 0, c->stream>>>(c->base.as<float>(), c->n, c->d,
                                                 c->qbase.as<__nv_fp8_storage_t>(), c->qscale.as<float>());
  }
  WV_CUDA(c, cudaGetLastError());
  if (storage != 0) {
    WV_CUDA(c, c->qnorm.ensure((size_t)c->n * 4));
    k_lowp_norms<<<c->sms * 8, 256, 0, c->stream>>>(c->qbase.p, c->qscale.as<float>(), storage, c->n, c->d,
                                                    c->qnorm.as<float>());
    WV_CUDA(c, cudaGetLastError());
  }
  WV_CUDA(c, cudaStreamSynchronize(c->stream));
  c->generation++;
  c->storage = storage;
  c->rerank = rerank;
  return WV_OK;
}

int wv_set_search_expansion(wv_ctx *c, uint32_t parents) {
  if (!c) return WV_ERR_ARG;
  WV_CHECK(c, parents <= BEAM_MAX_PARENTS, WV_ERR_ARG, "parents=%u (0 for the exact traversal, 1..%u)", parents,
           BEAM_MAX_PARENTS);
  c->generation++;
  c->parents = parents;
  return WV_OK;
}

int wv_candidate_distances(wv_ctx *c, const float *queries, uint32_t nq, const uint32_t *ids, uint32_t m,
                           float *out) {
  if (!c || !queries || !ids || !out) return WV_ERR_ARG;
  WV_CHECK(c, c->n > 0, WV_ERR_STATE, "no base uploaded");
  WV_CHECK(c, c->d % 4 == 0, WV_ERR_LIMIT, "dimension %u is not a multiple of 4", c->d);
  for (size_t i = 0; i < (size_t)nq * m; i++) WV_CHECK(c, ids[i] < c->n, WV_ERR_ARG, "id %u >= n", ids[i]);
  WV_CUDA(c, cudaSetDevice(c->device));
  cudaError_t e = cudaSuccess;
  float *dq = c->buf<float>("cd_q", (size_t)nq * c->d, &e);
  uint32_t *di = c->buf<uint32_t>("cd_i", (size_t)nq * m, &e);
  float *dout = c->buf<float>("cd_o", (size_t)nq * m, &e);
  WV_CUDA(c, e);
  WV_CUDA(c, cudaMemcpyAsync(dq, queries, (size_t)nq * c->d * 4, cudaMemcpyHostToDevice, c->stream));
  WV_CUDA(c, cudaMemcpyAsync(di, ids, (size_t)nq * m * 4, cudaMemcpyHostToDevice, c->stream));
  const size_t warps = (size_t)nq * ((m + 31) / 32);
  k_cand_dist<<<(unsigned)((warps * 32 + 255) / 256), 256, 0, c->stream>>>(
      c->base.as<float>(), LowpRows{c->qbase.p, c->qscale.as<float>(), c->qnorm.as<float>(), c->storage, c->d},
      c->base_int ? 1 : 0, c->d, dq, di, nq, m, dout);
  WV_CUDA(c, cudaGetLastError());
  WV_CUDA(c, cudaMemcpyAsync(out, dout, (size_t)nq * m * 4, cudaMemcpyDeviceToHost, c->stream));
  WV_CUDA(c, cudaStreamSynchronize(c->stream));
  return WV_OK;
}

}  // extern "C"
