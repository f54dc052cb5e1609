// BF16 GEMM on Blackwell's 5th-generation tensor cores (tcgen05), FP32
// accumulation in tensor memory: C = A (M x K) B (K x N) [+ bias] [ReLU],
// with arbitrary element strides for A and B (the MLP's forward pass, weight
// gradients and input gradients all use it).
//
// One CTA (4 warps) computes a 128 x 128 tile of C:
//  * the K dimension goes in steps of 64 through two shared-memory stages;
//    the 4 warps stage A (128 rows) and B (128 columns) of a step in the
//    canonical no-swizzle K-major layout -- 8 x 8 core matrices of 16-byte
//    rows, core matrices adjacent in K 128 bytes apart (the descriptor's
//    leading offset), 8-row groups 1024 bytes apart (its stride offset) --
//    with 16-byte loads where K is contiguous in memory, element loads
//    otherwise, zeros past the edges;
//  * one thread issues four tcgen05.mma (M = 128, N = 128, K = 16 each) per
//    step and tcgen05.commit, which arrives on the stage's mbarrier once they
//    complete; a stage is refilled only after its previous commit arrived;
//  * the accumulator (128 lanes x 128 FP32 columns of tensor memory, taken
//    with tcgen05.alloc) is read back by the 4 warps with tcgen05.ld (warp w
//    owns lanes 32w..32w+31 = rows of the tile) and turned through shared
//    memory so that the epilogue (bias, ReLU, FP32 / BF16 stores) writes
//    whole rows with the lanes along the columns.
// Every mbarrier wait is bounded: on time-out the kernel sets an error flag,
// waits (bounded) for its outstanding MMAs, frees its tensor memory and
// returns.
#include <cuda_bf16.h>

#include <cstdint>

#include "wv_common.cuh"
#include "wv_mlp.cuh"
#include "wv_umma.cuh"

namespace wv {
namespace {

constexpr int TM = 128, TN = 128, TK = 64;          // tile
constexpr int STAGE_A = TM * TK * 2, STAGE_B = TN * TK * 2;  // bytes per stage
constexpr uint32_t LBO = 128;                        // K-adjacent core matrices
constexpr uint32_t SBO = (TK / 8) * 128;             // 8-row groups
constexpr uint32_t TMEM_COLS = 128;

using umma::mbar_init;
using umma::mbar_wait;
using umma::smem_u32;

__device__ __forceinline__ uint64_t umma_desc(uint32_t saddr) { return umma::desc(saddr, LBO, SBO); }
__host__ __device__ constexpr uint32_t umma_idesc(int M, int N) { return umma::idesc(M, N); }

// the byte offset of element (row, k) of a staged operand
__device__ __forceinline__ uint32_t core_off(int row, int k) {
  return (uint32_t)((row >> 3) * SBO + (k >> 3) * LBO + (row & 7) * 16 + (k & 7) * 2);
}

// stages rows [r0, r0 + 128) x k [k0, k0 + 64) of a strided operand X(row, k)
// = X[row * s_row + k * s_k] (rows >= R or k >= K read as zero)
__device__ __forceinline__ void stage_operand(uint8_t *dst, const __nv_bfloat16 *X, long long s_row, long long s_k,
                                              int R, int K, int r0, int k0, int tid) {
  const bool vec = s_k == 1 && (s_row % 8) == 0 && ((reinterpret_cast<uintptr_t>(X) & 15) == 0);
  if (vec) {
    // one 16-byte core-matrix row (8 consecutive k) per step: 128 x 8 of them
    for (int e = tid; e < TM * (TK / 8); e += 128) {
      const int r = e / (TK / 8), kc = (e % (TK / 8)) * 8;
      const int gr = r0 + r, gk = k0 + kc;
      uint4 v = make_uint4(0, 0, 0, 0);
      if (gr < R) {
        if (gk + 8 <= K) {
          v = __ldg(reinterpret_cast<const uint4 *>(X + (long long)gr * s_row + gk));
        } else if (gk < K) {
          uint16_t t[8];
          for (int j = 0; j < 8; j++)
            t[j] = gk + j < K ? __bfloat16_as_ushort(X[(long long)gr * s_row + gk + j]) : (uint16_t)0;
          v = make_uint4(t[0] | (t[1] << 16), t[2] | (t[3] << 16), t[4] | (t[5] << 16), t[6] | (t[7] << 16));
        }
      }
      *reinterpret_cast<uint4 *>(dst + core_off(r, kc)) = v;
    }
  } else {
    // element loads, consecutive threads along the row index (coalesced when
    // the rows are contiguous)
    for (int e = tid; e < TM * TK; e += 128) {
      const int k = e / TM, r = e % TM;
      const int gr = r0 + r, gk = k0 + k;
      const uint16_t v =
          (gr < R && gk < K) ? __bfloat16_as_ushort(X[(long long)gr * s_row + (long long)gk * s_k]) : (uint16_t)0;
      *reinterpret_cast<uint16_t *>(dst + core_off(r, k)) = v;
    }
  }
}

__global__ void __launch_bounds__(128) k_gemm_umma(GemmArgs g, int *status) {
  extern __shared__ __align__(1024) uint8_t smem[];
  uint8_t *stA[2] = {smem, smem + STAGE_A + STAGE_B};
  uint8_t *stB[2] = {smem + STAGE_A, smem + 2 * STAGE_A + STAGE_B};
  __shared__ __align__(8) uint64_t bar[2];
  __shared__ uint32_t tmem_base;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int m0 = blockIdx.y * TM, n0 = blockIdx.x * TN;

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base)),
                 "r"(TMEM_COLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    asm volatile("fence.mbarrier_init.release.cluster;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = tmem_base;

  const int nk = (g.K + TK - 1) / TK;
  constexpr uint32_t idesc = umma_idesc(TM, TN);
  bool ok = true;
  for (int kt = 0; kt < nk && ok; kt++) {
    const int s = kt & 1;
    // the stage's previous MMAs are done (every thread polls; the verdict is
    // made uniform so that no thread skips a barrier the others reach)
    if (kt >= 2) ok = __syncthreads_and(mbar_wait(&bar[s], ((kt - 2) >> 1) & 1)) != 0;
    if (!ok) break;
    // A(m, k) rows of C; B as B^T(n, k)
    stage_operand(stA[s], g.A, g.sam, g.sak, g.M, g.K, m0, kt * TK, tid);
    stage_operand(stB[s], g.B, g.sbn, g.sbk, g.N, g.K, n0, kt * TK, tid);
    asm volatile("fence.proxy.async.shared::cta;");  // generic stores -> tensor core reads
    __syncthreads();
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;");
      const uint32_t a0 = smem_u32(stA[s]), b0 = smem_u32(stB[s]);
#pragma unroll
      for (int kk = 0; kk < TK / 16; kk++) {
        // K slice kk: two core matrices along K, 2 * LBO bytes further
        const uint64_t ad = umma_desc(a0 + kk * 2 * LBO), bd = umma_desc(b0 + kk * 2 * LBO);
        const uint32_t acc = (kt > 0 || kk > 0) ? 1u : 0u;
        asm volatile(
            "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
            " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
            "l"(ad), "l"(bd), "r"(idesc), "r"(acc));
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          smem_u32(&bar[s])));
    }
  }
  // all MMAs done: the last commit covers every earlier one
  if (ok && nk > 0) ok = __syncthreads_and(mbar_wait(&bar[(nk - 1) & 1], ((nk - 1) >> 1) & 1)) != 0;
  if (!ok && tid == 0) set_err(status, DEV_TIMEOUT);
  asm volatile("tcgen05.fence::after_thread_sync;");
  if (ok) {
    // epilogue: warp w reads lanes 32w.. (its 32 tile rows), 16 columns at a
    // time, into its own slice of shared memory (the stages are free now;
    // rows TN + 1 floats apart, so both the column writes here and the row
    // reads below avoid bank conflicts), then writes the rows out with the
    // lanes along the columns (coalesced), adding the bias and the ReLU
    float *ot = reinterpret_cast<float *>(smem) + (size_t)warp * 32 * (TN + 1);
    for (int c0 = 0; c0 < TN; c0 += 16) {
      uint32_t v[16];
      const uint32_t addr = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0;
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
          : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
            "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
          : "r"(addr));
      asm volatile("tcgen05.wait::ld.sync.aligned;");
#pragma unroll
      for (int j = 0; j < 16; j++) ot[lane * (TN + 1) + c0 + j] = __uint_as_float(v[j]);
    }
    __syncwarp();
    for (int r = 0; r < 32; r++) {
      const int row = m0 + warp * 32 + r;
      if (row >= g.M) break;
      for (int cb = 0; cb < TN; cb += 32) {
        const int col = n0 + cb + lane;
        if (col < g.N) {
          float x = ot[r * (TN + 1) + cb + lane];
          if (g.bias) x += g.bias[col];
          if (g.relu) x = fmaxf(x, 0.f);
          if (g.C) g.C[(long long)row * g.ldc + col] = x;
          if (g.Cb) g.Cb[(long long)row * g.ldc + col] = __float2bfloat16_rn(x);
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS));
}

}  // namespace

// the two operand stages, or the epilogue's row buffers if larger
size_t gemm_umma_smem() {
  const size_t stages = 2 * (size_t)(STAGE_A + STAGE_B), out = 4 * 32 * (size_t)(TN + 1) * sizeof(float);
  return stages > out ? stages : out;
}

cudaError_t gemm_bf16_umma(const GemmArgs &g, int *status, cudaStream_t s) {
  if (g.M <= 0 || g.N <= 0) return cudaSuccess;
  if (g.K <= 0) return cudaErrorInvalidValue;  // the accumulator would never be written
  const size_t smem = gemm_umma_smem();
  cudaError_t e = cudaFuncSetAttribute(k_gemm_umma, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  dim3 grid((g.N + TN - 1) / TN, (g.M + TM - 1) / TM);
  k_gemm_umma<<<grid, 128, smem, s>>>(g, status);
  return cudaGetLastError();
}

}  // namespace wv
