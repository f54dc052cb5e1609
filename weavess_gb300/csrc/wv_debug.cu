// Diagnostic entry point: runs the device sort replicas on caller arrays so
// tests can compare them with the host's std::sort.
#include <cuda_bf16.h>

#include "warp_sort.cuh"
#include "wv_common.cuh"
#include "wv_ctx.h"
#include "wv_mlp.cuh"

using namespace wv;

namespace {

constexpr int DBG_CAP = 4096;

// one warp per array; mode 0: warp_std_sort, mode 1: one-lane stl::sort
__global__ void k_debug_sort(DI *data, const uint32_t *off, uint32_t narr, int mode) {
  extern __shared__ __align__(16) uint8_t smem[];
  const uint32_t w = blockIdx.x;
  if (w >= narr) return;
  const int lane = threadIdx.x;
  DI *a = (DI *)smem;
  int *ap = (int *)(a + DBG_CAP);
  int *bp = ap + DBG_CAP;
  int *st = bp + DBG_CAP;
  int *lf = st + 3 * 64;
  const uint32_t f = off[w], n = off[w + 1] - f;
  for (uint32_t i = lane; i < n; i += 32) a[i] = data[f + i];
  __syncwarp();
  if (mode == 0) {
    warp_std_sort(a, (int)n, DILess(), WarpSortScratch{ap, bp, st, lf}, lane);
  } else if (lane == 0) {
    stl::sort(a, (int)n, DILess());
  }
  __syncwarp();
  for (uint32_t i = lane; i < n; i += 32) data[f + i] = a[i];
}

}  // namespace

extern "C" int wv_debug_sort(wv_ctx *c, float *keys, uint32_t *vals, const uint32_t *offsets, uint32_t narr,
                             int mode) {
  if (!c || !keys || !vals || !offsets) return WV_ERR_ARG;
  WV_CUDA(c, cudaSetDevice(c->device));
  const uint32_t total = offsets[narr];
  for (uint32_t i = 0; i < narr; i++)
    WV_CHECK(c, offsets[i + 1] - offsets[i] <= (uint32_t)DBG_CAP, WV_ERR_LIMIT, "array longer than %d", DBG_CAP);
  std::vector<DI> h(total);
  for (uint32_t i = 0; i < total; i++) h[i] = DI{keys[i], vals[i]};
  cudaError_t e = cudaSuccess;
  DI *d = c->buf<DI>("dbg_sort", total + 1, &e);
  uint32_t *o = c->buf<uint32_t>("dbg_off", narr + 1, &e);
  WV_CUDA(c, e);
  WV_CUDA(c, cudaMemcpyAsync(d, h.data(), total * sizeof(DI), cudaMemcpyHostToDevice, c->stream));
  WV_CUDA(c, cudaMemcpyAsync(o, offsets, (narr + 1) * 4, cudaMemcpyHostToDevice, c->stream));
  const size_t smem = DBG_CAP * sizeof(DI) + 2 * DBG_CAP * 4 + (3 * 64 + 64) * 4;
  WV_CUDA(c, cudaFuncSetAttribute(k_debug_sort, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  k_debug_sort<<<narr, 32, smem, c->stream>>>(d, o, narr, mode);
  WV_CUDA(c, cudaGetLastError());
  WV_CUDA(c, cudaMemcpyAsync(h.data(), d, total * sizeof(DI), cudaMemcpyDeviceToHost, c->stream));
  WV_CUDA(c, cudaStreamSynchronize(c->stream));
  for (uint32_t i = 0; i < total; i++) {
    keys[i] = h[i].d;
    vals[i] = h[i].i;
  }
  return WV_OK;
}

// C (M x N, FP32) = A (M x K) B (K x N), bf16 operands given as their bit
// patterns with element strides; impl 0: mma.sync kernel, 1: tcgen05 kernel
extern "C" int wv_debug_gemm(wv_ctx *c, int impl, uint32_t M, uint32_t N, uint32_t K, const uint16_t *A,
                             long long sam, long long sak, const uint16_t *B, long long sbk, long long sbn,
                             float *C) {
  if (!c || !A || !B || !C || M == 0 || N == 0 || K == 0) return WV_ERR_ARG;
  WV_CHECK(c, impl == 0 || impl == 1, WV_ERR_ARG, "impl must be 0 or 1");
  WV_CUDA(c, cudaSetDevice(c->device));
  // extents of the strided operands
  const size_t na = (size_t)((M - 1) * sam + (K - 1) * sak + 1), nb = (size_t)((K - 1) * sbk + (N - 1) * sbn + 1);
  cudaError_t e = cudaSuccess;
  uint16_t *dA = c->buf<uint16_t>("dbg_gA", na, &e);
  uint16_t *dB = c->buf<uint16_t>("dbg_gB", nb, &e);
  float *dC = c->buf<float>("dbg_gC", (size_t)M * N, &e);
  WV_CUDA(c, e);
  WV_CUDA(c, cudaMemcpyAsync(dA, A, na * 2, cudaMemcpyHostToDevice, c->stream));
  WV_CUDA(c, cudaMemcpyAsync(dB, B, nb * 2, cudaMemcpyHostToDevice, c->stream));
  GemmArgs g{};
  g.A = reinterpret_cast<const __nv_bfloat16 *>(dA);
  g.sam = sam;
  g.sak = sak;
  g.B = reinterpret_cast<const __nv_bfloat16 *>(dB);
  g.sbk = sbk;
  g.sbn = sbn;
  g.C = dC;
  g.ldc = N;
  g.M = (int)M;
  g.N = (int)N;
  g.K = (int)K;
  WV_CUDA(c, impl == 0 ? gemm_bf16(g, c->stream) : gemm_bf16_umma(g, c->d_status(), c->stream));
  WV_CUDA(c, cudaMemcpyAsync(C, dC, (size_t)M * N * 4, cudaMemcpyDeviceToHost, c->stream));
  WV_CUDA(c, cudaStreamSynchronize(c->stream));
  return check_device_status(c, "gemm");
}
