// BF16 GEMM on the warp-level tensor-core instruction (mma.sync), the
// cross-check of the tcgen05 GEMM the MLP runs (see wv_mlp.cuh).
// 64 x 64 output tile per block, K in steps of 32, four warps of 32 x 32,
// each issuing m16n8k16 MMAs from shared-memory fragments.
#include "wv_common.cuh"
#include "wv_mlp.cuh"

namespace wv {
namespace {

constexpr int BM = 64, BN = 64, BK = 32;
constexpr int APAD = 8, BPAD = 8;

__device__ __forceinline__ uint32_t pack2(__nv_bfloat16 lo, __nv_bfloat16 hi) {
  return (uint32_t)__bfloat16_as_ushort(lo) | ((uint32_t)__bfloat16_as_ushort(hi) << 16);
}

__global__ void __launch_bounds__(128) k_gemm_bf16(GemmArgs g) {
  __shared__ __nv_bfloat16 As[BM][BK + APAD];
  __shared__ __nv_bfloat16 Bs[BK][BN + BPAD];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int gid = lane >> 2, tg = lane & 3;
  const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
  const int wm = (warp >> 1) * 32, wn = (warp & 1) * 32;
  float acc[2][4][4];
#pragma unroll
  for (int i = 0; i < 2; i++)
#pragma unroll
    for (int j = 0; j < 4; j++)
#pragma unroll
      for (int r = 0; r < 4; r++) acc[i][j][r] = 0.f;
  const __nv_bfloat16 zero = __float2bfloat16(0.f);
  for (int k0 = 0; k0 < g.K; k0 += BK) {
    for (int e = tid; e < BM * BK; e += 128) {
      const int r = e / BK, c = e % BK;
      const int m = m0 + r, k = k0 + c;
      As[r][c] = (m < g.M && k < g.K) ? g.A[(long long)m * g.sam + (long long)k * g.sak] : zero;
    }
    for (int e = tid; e < BK * BN; e += 128) {
      const int r = e / BN, c = e % BN;
      const int k = k0 + r, n = n0 + c;
      Bs[r][c] = (k < g.K && n < g.N) ? g.B[(long long)k * g.sbk + (long long)n * g.sbn] : zero;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < BK; kk += 16) {
      uint32_t af[2][4], bf[4][2];
#pragma unroll
      for (int i = 0; i < 2; i++) {
        const int r = wm + i * 16 + gid;
        const int c = kk + tg * 2;
        af[i][0] = pack2(As[r][c], As[r][c + 1]);
        af[i][1] = pack2(As[r + 8][c], As[r + 8][c + 1]);
        af[i][2] = pack2(As[r][c + 8], As[r][c + 9]);
        af[i][3] = pack2(As[r + 8][c + 8], As[r + 8][c + 9]);
      }
#pragma unroll
      for (int j = 0; j < 4; j++) {
        const int n = wn + j * 8 + gid;
        const int k = kk + tg * 2;
        bf[j][0] = pack2(Bs[k][n], Bs[k + 1][n]);
        bf[j][1] = pack2(Bs[k + 8][n], Bs[k + 9][n]);
      }
#pragma unroll
      for (int i = 0; i < 2; i++)
#pragma unroll
        for (int j = 0; j < 4; j++)
          asm volatile(
              "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
              "{%0,%1,%2,%3};\n"
              : "+f"(acc[i][j][0]), "+f"(acc[i][j][1]), "+f"(acc[i][j][2]), "+f"(acc[i][j][3])
              : "r"(af[i][0]), "r"(af[i][1]), "r"(af[i][2]), "r"(af[i][3]), "r"(bf[j][0]), "r"(bf[j][1]));
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 2; i++)
#pragma unroll
    for (int j = 0; j < 4; j++)
#pragma unroll
      for (int r = 0; r < 4; r++) {
        const int m = m0 + wm + i * 16 + gid + (r >= 2 ? 8 : 0);
        const int n = n0 + wn + j * 8 + tg * 2 + (r & 1);
        if (m < g.M && n < g.N) {
          float v = acc[i][j][r];
          if (g.bias) v += g.bias[n];
          if (g.relu) v = fmaxf(v, 0.f);
          if (g.C) g.C[(long long)m * g.ldc + n] = v;
          if (g.Cb) g.Cb[(long long)m * g.ldc + n] = __float2bfloat16_rn(v);
        }
      }
}

}  // namespace

cudaError_t gemm_bf16(const GemmArgs &g, cudaStream_t s) {
  dim3 grid((g.N + BN - 1) / BN, (g.M + BM - 1) / BM);
  k_gemm_bf16<<<grid, 128, 0, s>>>(g);
  return cudaGetLastError();
}

}  // namespace wv
