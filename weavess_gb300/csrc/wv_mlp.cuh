// BF16 GEMM on the tensor cores (mma.sync m16n8k16, FP32 accumulation) with
// arbitrary element strides for both operands, so one kernel serves the
// forward pass (X W), the weight gradients (X^T dY) and the input gradients
// (dY W^T) of the MLP.  Epilogue: + bias, ReLU, FP32 and/or BF16 store.
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

cudaError_t gemm_bf16(const GemmArgs &g, cudaStream_t s);

}  // namespace wv
