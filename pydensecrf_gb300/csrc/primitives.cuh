// primitives.cuh -- device-wide scan and stable radix sort (see primitives.cu).
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

namespace dcrf {

// Workspace (in 32-bit words) needed by scan_exclusive_u32 for n elements.
size_t scan_temp_words(size_t n);
// out[i] = sum(in[0..i)); in-place allowed; *d_total (device, may be NULL) = sum(in).
cudaError_t scan_exclusive_u32(const uint32_t *in, uint32_t *out, size_t n, uint32_t *d_total, uint32_t *temp,
                               cudaStream_t s);

// Workspace (in 32-bit words) needed by radix_sort_pairs_u32 for n elements.
size_t radix_temp_words(size_t n);
// Stable sort of (keys, vals) by the low `bits` bits of keys, ping-ponging with
// (keys_alt, vals_alt); *result_in_alt tells which pair holds the result.
cudaError_t radix_sort_pairs_u32(uint32_t *keys, uint32_t *vals, uint32_t *keys_alt, uint32_t *vals_alt, size_t n,
                                 int bits, uint32_t *temp, cudaStream_t s, int *result_in_alt);

}  // namespace dcrf
