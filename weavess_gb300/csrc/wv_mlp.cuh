// BF16 GEMM (FP32 accumulation) with arbitrary element strides for both
// operands, so one kernel serves the forward pass (X W), the weight gradients
// (X^T dY) and the input gradients (dY W^T) of the MLP.  Epilogue: + bias,
// ReLU, FP32 and/or BF16 store.  The MLP runs the tcgen05 form (wv_umma.cu);
// the mma.sync form (wv_gemm.cu) is kept as its cross-check.
#pragma once
#include <cuda_bf16.h>

#include <cstdint>

namespace wv {

struct GemmArgs {
  const __nv_bfloat16 *A;  // A(m, k) = A[m * sam + k * sak]
  long long sam, sak;
  const __nv_bfloat16 *B;  // B(k, n) = B[k * sbk + n * sbn]
  long long sbk, sbn;
  float *C;                // C(m, n) = C[m * ldc + n] (nullable)
  __nv_bfloat16 *Cb;       // bf16 copy of C (nullable)
  long long ldc;
  const float *bias;       // [N] (nullable)
  int relu;
  int M, N, K;
};

// mma.sync (m16n8k16) form
cudaError_t gemm_bf16(const GemmArgs &g, cudaStream_t s);
// tcgen05 form (wv_umma.cu): 128 x 128 tiles, accumulator in tensor memory;
// a bounded wait that gives up sets DEV_TIMEOUT in *status
cudaError_t gemm_bf16_umma(const GemmArgs &g, int *status, cudaStream_t s);

}  // namespace wv
