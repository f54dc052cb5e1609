// Candidate distances from the low-precision copy of the base (bf16, or fp8
// e4m3 with one FP32 scale per row), FP32 accumulation.
//
// A warp computes the distances of up to 32 rows at once.  Each row is read
// in 16-byte chunks (8-byte or 4-byte when the row length is not a multiple
// of 16 bytes; d is a multiple of 4) by a group of G lanes, G the power of
// two (4 to 32) that covers the row's chunks, so 32 / G rows are read per
// pass; the loads of U passes are issued together, branch-free, before any
// of them is used, which keeps U chunk loads per lane in flight.  The order of the additions depends only on d and the
// storage, never on how many rows share the call, so the search kernel and
// the diagnostic (wv_candidate_distances) return the same values.
#pragma once
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_fp8.h>

#include "wv_common.cuh"

namespace wv {

struct LowpRows {
  const void *rows;    // n x d bf16 or fp8 values, row-major, no padding
  const float *scale;  // fp8: one scale per row
  const float *norm;   // squared norm of every stored row (dequantised), or null
  int storage;         // 1 bf16, 2 fp8
  uint32_t d;
};

namespace lowp_detail {

constexpr int U = 8;  // passes in flight

// the CB bytes of one chunk as 32-bit words
template <int CB>
struct Chunk {
  uint32_t w[CB / 4];
};
template <int CB>
__device__ __forceinline__ Chunk<CB> load_chunk(const uint8_t *p) {
  Chunk<CB> c;
  if (CB == 16) {
    const uint4 v = __ldg(reinterpret_cast<const uint4 *>(p));
    c.w[0] = v.x, c.w[1] = v.y, c.w[2] = v.z, c.w[3] = v.w;
  } else if (CB == 8) {
    const uint2 v = __ldg(reinterpret_cast<const uint2 *>(p));
    c.w[0] = v.x, c.w[1] = v.y;
  } else {
    c.w[0] = __ldg(reinterpret_cast<const uint32_t *>(p));
  }
  return c;
}

// contribution of one loaded chunk at element offset e0: the squared
// difference (DOT false) or the dot product with the query, fp8 values
// unscaled (DOT true)
template <int ST, int CB, bool DOT>
__device__ __forceinline__ float chunk_sq(const Chunk<CB> &c, const float *qv, uint32_t e0, float sc) {
  float acc = 0.f;
  const float4 *q4 = reinterpret_cast<const float4 *>(qv + e0);
  if (ST == 1) {
    constexpr int E = CB / 2;  // bf16 values per chunk
#pragma unroll
    for (int j = 0; j < E / 4; j++) {
      const float4 q = q4[j];
      // bf16 -> fp32: the 16 bits become the high half of the word
      const uint32_t w0 = c.w[2 * j], w1 = c.w[2 * j + 1];
      const float x0 = __uint_as_float(w0 << 16), x1 = __uint_as_float(w0 & 0xffff0000u);
      const float x2 = __uint_as_float(w1 << 16), x3 = __uint_as_float(w1 & 0xffff0000u);
      if (DOT) {
        acc = fmaf(q.x, x0, acc);
        acc = fmaf(q.y, x1, acc);
        acc = fmaf(q.z, x2, acc);
        acc = fmaf(q.w, x3, acc);
      } else {
        const float a0 = q.x - x0, a1 = q.y - x1, a2 = q.z - x2, a3 = q.w - x3;
        acc = fmaf(a0, a0, acc);
        acc = fmaf(a1, a1, acc);
        acc = fmaf(a2, a2, acc);
        acc = fmaf(a3, a3, acc);
      }
    }
  } else {
    constexpr int E = CB;  // fp8 values per chunk
#pragma unroll
    for (int j = 0; j < E / 4; j++) {
      const float4 q = q4[j];
      const __half2_raw h0 = __nv_cvt_fp8x2_to_halfraw2((__nv_fp8x2_storage_t)(c.w[j] & 0xffffu), __NV_E4M3);
      const __half2_raw h1 = __nv_cvt_fp8x2_to_halfraw2((__nv_fp8x2_storage_t)(c.w[j] >> 16), __NV_E4M3);
      const float2 x0 = __half22float2(*reinterpret_cast<const __half2 *>(&h0));
      const float2 x1 = __half22float2(*reinterpret_cast<const __half2 *>(&h1));
      if (DOT) {
        acc = fmaf(q.x, x0.x, acc);
        acc = fmaf(q.y, x0.y, acc);
        acc = fmaf(q.z, x1.x, acc);
        acc = fmaf(q.w, x1.y, acc);
      } else {
        const float a0 = q.x - sc * x0.x, a1 = q.y - sc * x0.y, a2 = q.z - sc * x1.x, a3 = q.w - sc * x1.y;
        acc = fmaf(a0, a0, acc);
        acc = fmaf(a1, a1, acc);
        acc = fmaf(a2, a2, acc);
        acc = fmaf(a3, a3, acc);
      }
    }
  }
  return acc;
}

template <int ST, int CB, int G, bool DOT>
__device__ __forceinline__ float rows_dist(const LowpRows &b, uint32_t my, int cnt, const float *qv, float qn,
                                           int lane) {
  constexpr int EPC = ST == 1 ? CB / 2 : CB;  // elements per chunk
  constexpr int RPP = 32 / G;                 // rows per pass
  const uint32_t rb = ST == 1 ? b.d * 2 : b.d;
  const uint32_t ch = rb / CB;
  const int sub = lane & (G - 1), grp = lane / G;
  const uint8_t *base = reinterpret_cast<const uint8_t *>(b.rows);
  const float xn = (DOT && lane < cnt) ? __ldg(b.norm + my) : 0.f;
  const float xs = (DOT && ST == 2 && lane < cnt) ? __ldg(b.scale + my) : 1.f;
  float out = 0.f;
  for (int p0 = 0; p0 * RPP < cnt; p0 += U) {
    float part[U], sc[U];
    const uint8_t *row[U];
    bool live[U];
#pragma unroll
    for (int u = 0; u < U; u++) {
      const int r = (p0 + u) * RPP + grp;
      const uint32_t id = __shfl_sync(FULL, my, r & 31);
      live[u] = r < cnt;
      part[u] = 0.f;
      // dead rows read row 0 (in bounds) and are ignored: no branch keeps the
      // U loads from issuing together
      row[u] = base + (size_t)(live[u] ? id : 0u) * rb;
      sc[u] = (ST == 2 && !DOT) ? __ldg(b.scale + (live[u] ? id : 0u)) : 1.f;
    }
    // chunk-major: all U rows' loads of one step are issued before any math
    for (uint32_t k = sub; k < ch; k += G) {
      Chunk<CB> c[U];
#pragma unroll
      for (int u = 0; u < U; u++) c[u] = load_chunk<CB>(row[u] + (size_t)k * CB);
#pragma unroll
      for (int u = 0; u < U; u++) part[u] += chunk_sq<ST, CB, DOT>(c[u], qv, k * EPC, sc[u]);
    }
#pragma unroll
    for (int u = 0; u < U; u++) {
      float v = live[u] ? part[u] : 0.f;
#pragma unroll
      for (int o = G >> 1; o > 0; o >>= 1) v += __shfl_xor_sync(FULL, v, o);
      // row `lane` sits in pass lane / RPP, group lane % RPP
      const float t = __shfl_sync(FULL, v, (lane % RPP) * G);
      if (lane / RPP == p0 + u) out = t;
    }
  }
  // |q|^2 + |x|^2 - 2 q.x with the stored row's norm (fp8: q.x = scale * q.h)
  if (DOT && lane < cnt) out = fmaxf(qn + xn - 2.f * xs * out, 0.f);
  return out;
}

// the dot product of one loaded bf16 chunk with the query, added to a packed
// pair of accumulators (two values per FMA instruction)
template <int CB>
__device__ __forceinline__ void chunk_dot2_bf16(const Chunk<CB> &c, const float *qv, uint32_t e0,
                                                unsigned long long &acc) {
  const float4 *q4 = reinterpret_cast<const float4 *>(qv + e0);
#pragma unroll
  for (int j = 0; j < CB / 8; j++) {
    const float4 q = q4[j];
    const uint32_t w0 = c.w[2 * j], w1 = c.w[2 * j + 1];
    fma2(acc, q.x, q.y, __uint_as_float(w0 << 16), __uint_as_float(w0 & 0xffff0000u));
    fma2(acc, q.z, q.w, __uint_as_float(w1 << 16), __uint_as_float(w1 & 0xffff0000u));
  }
}

// a warp per row (rows of at least 24 chunks): 8 rows per batch, their loads
// issued together, the 8 partial sums reduced across the warp by a transpose
// reduction (lanes swap halves at distances 16, 8, 4, then add over 2, 1:
// 10 shuffles for 8 rows); lane l ends with row 4 bit4(l) + 2 bit3(l) + bit2(l)
template <int ST, int CB, bool DOT>
__device__ __forceinline__ float rows_dist_w(const LowpRows &b, uint32_t my, int cnt, const float *qv, float qn,
                                             int lane) {
  constexpr int EPC = ST == 1 ? CB / 2 : CB;
  const uint32_t rb = ST == 1 ? b.d * 2 : b.d;
  const uint32_t ch = rb / CB;
  const uint8_t *base = reinterpret_cast<const uint8_t *>(b.rows);
  // the lane's own row norm (and fp8 scale), loaded before the rows
  const float xn = (DOT && lane < cnt) ? __ldg(b.norm + my) : 0.f;
  const float xs = (DOT && ST == 2 && lane < cnt) ? __ldg(b.scale + my) : 1.f;
  float out = 0.f;
  for (int c0 = 0; c0 < cnt; c0 += 8) {
    float part[8], sc[8];
    const uint8_t *row[8];
#pragma unroll
    for (int g = 0; g < 8; g++) {
      const int r = c0 + g;
      const uint32_t id = __shfl_sync(FULL, my, r & 31);
      const bool live = r < cnt;
      part[g] = 0.f;
      row[g] = base + (size_t)(live ? id : 0u) * rb;  // dead rows read row 0 (in bounds), ignored
      sc[g] = (ST == 2 && !DOT) ? __ldg(b.scale + (live ? id : 0u)) : 1.f;
    }
    unsigned long long pacc[8];  // bf16 dot form: packed accumulators
#pragma unroll
    for (int g = 0; g < 8; g++) pacc[g] = 0ull;
    for (uint32_t k = lane; k < ch; k += 32) {
      Chunk<CB> c[8];
#pragma unroll
      for (int g = 0; g < 8; g++) c[g] = load_chunk<CB>(row[g] + (size_t)k * CB);
      if (ST == 1 && DOT && CB >= 8) {
#pragma unroll
        for (int g = 0; g < 8; g++) chunk_dot2_bf16<CB>(c[g], qv, k * EPC, pacc[g]);
      } else {
#pragma unroll
        for (int g = 0; g < 8; g++) part[g] += chunk_sq<ST, CB, DOT>(c[g], qv, k * EPC, sc[g]);
      }
    }
    if (ST == 1 && DOT && CB >= 8) {
#pragma unroll
      for (int g = 0; g < 8; g++) part[g] = sum2(pacc[g]);
    }
    const bool b16 = lane & 16, b8 = lane & 8, b4 = lane & 4;
    float w[4];
#pragma unroll
    for (int j = 0; j < 4; j++) {
      const float send = b16 ? part[j] : part[j + 4];
      w[j] = (b16 ? part[j + 4] : part[j]) + __shfl_xor_sync(FULL, send, 16);
    }
    float x2[2];
#pragma unroll
    for (int j = 0; j < 2; j++) {
      const float send = b8 ? w[j] : w[j + 2];
      x2[j] = (b8 ? w[j + 2] : w[j]) + __shfl_xor_sync(FULL, send, 8);
    }
    float y = (b4 ? x2[1] : x2[0]) + __shfl_xor_sync(FULL, b4 ? x2[0] : x2[1], 4);
    y += __shfl_xor_sync(FULL, y, 2);
    y += __shfl_xor_sync(FULL, y, 1);
    const int g = (lane - c0) & 7;
    const float t = __shfl_sync(FULL, y, ((g >> 2) << 4) | (((g >> 1) & 1) << 3) | ((g & 1) << 2));
    if (lane >= c0 && lane < c0 + 8) out = t;
  }
  if (DOT && lane < cnt) out = fmaxf(qn + xn - 2.f * xs * out, 0.f);
  return out;
}

template <int ST, int CB, bool DOT>
__device__ __forceinline__ float rows_dist_g(const LowpRows &b, uint32_t my, int cnt, const float *qv, float qn,
                                             int lane) {
  const uint32_t ch = (ST == 1 ? b.d * 2 : b.d) / CB;
  if (ch >= 24) return rows_dist_w<ST, CB, DOT>(b, my, cnt, qv, qn, lane);
  if (ch <= 4) return rows_dist<ST, CB, 4, DOT>(b, my, cnt, qv, qn, lane);
  if (ch <= 8) return rows_dist<ST, CB, 8, DOT>(b, my, cnt, qv, qn, lane);
  if (ch <= 16) return rows_dist<ST, CB, 16, DOT>(b, my, cnt, qv, qn, lane);
  return rows_dist<ST, CB, 32, DOT>(b, my, cnt, qv, qn, lane);
}
template <int ST, int CB>
__device__ __forceinline__ float rows_dist_n(const LowpRows &b, uint32_t my, int cnt, const float *qv, float qn,
                                             int lane) {
  return b.norm ? rows_dist_g<ST, CB, true>(b, my, cnt, qv, qn, lane)
                : rows_dist_g<ST, CB, false>(b, my, cnt, qv, qn, lane);
}

}  // namespace lowp_detail

// distances of `cnt` rows (ids in lanes 0..cnt-1 of `my`; cnt <= 32) to the
// query `qv` (d floats, 16-byte aligned, any readable memory; d % 4 == 0;
// qn = |q|^2, used with b.norm); lane i returns row i's distance.  With row
// norms the distance is |q|^2 + |x|^2 - 2 q.x (one FMA per element; exact on
// integer data with d <= 128), else the sum of squared differences.
__device__ __forceinline__ float lowp_rows_dist(const LowpRows &b, uint32_t my, int cnt, const float *qv, float qn,
                                                int lane) {
  // chunk size: the largest that still gives a warp at least 24 chunks per
  // row (a warp per row), else the largest dividing the row (lane groups)
  // (a chunk holds at least 4 values: bf16 chunks are 8 or 16 bytes)
  const uint32_t rb = b.storage == 1 ? b.d * 2 : b.d;
  const uint32_t cmin = b.storage == 1 ? 8 : 4;
  const uint32_t cb = (rb % 16 == 0 && rb / 16 >= 24)               ? 16
                      : (rb % 8 == 0 && rb / 8 >= 24)               ? 8
                      : (cmin == 4 && rb % 4 == 0 && rb / 4 >= 24)  ? 4
                      : (rb % 16 == 0)                              ? 16
                      : (rb % 8 == 0 || cmin == 8)                  ? 8
                                                                    : 4;
  if (b.storage == 1) {
    if (cb == 16) return lowp_detail::rows_dist_n<1, 16>(b, my, cnt, qv, qn, lane);
    return lowp_detail::rows_dist_n<1, 8>(b, my, cnt, qv, qn, lane);  // d % 4 == 0: 8-byte multiples
  }
  if (cb == 16) return lowp_detail::rows_dist_n<2, 16>(b, my, cnt, qv, qn, lane);
  if (cb == 8) return lowp_detail::rows_dist_n<2, 8>(b, my, cnt, qv, qn, lane);
  return lowp_detail::rows_dist_n<2, 4>(b, my, cnt, qv, qn, lane);
}

}  // namespace wv
