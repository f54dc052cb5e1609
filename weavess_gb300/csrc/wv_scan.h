#pragma once
#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

namespace wv {
// u32 words of scratch exclusive_scan_u32 needs for n inputs
size_t scan_scratch_words(size_t n);
// out[i] = sum(in[0..i)); in and out may not alias
cudaError_t exclusive_scan_u32(const uint32_t *in, uint32_t *out, size_t n, uint32_t *scratch, cudaStream_t s);
}  // namespace wv
