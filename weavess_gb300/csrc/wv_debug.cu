// Diagnostic entry point: runs the device sort replicas on caller arrays so
// tests can compare them with the host's std::sort.
#include "warp_sort.cuh"
#include "wv_common.cuh"
#include "wv_ctx.h"

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
