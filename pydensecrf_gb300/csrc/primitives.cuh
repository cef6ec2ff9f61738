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

// Two independent scans of arrays of the same length (one launch when they fit
// the single-block scan); temp as for scan_exclusive_u32 of n elements.
cudaError_t scan_exclusive_u32_pair(const uint32_t *in0, uint32_t *out0, uint32_t *total0, const uint32_t *in1,
                                    uint32_t *out1, uint32_t *total1, size_t n, uint32_t *temp, cudaStream_t s);

// Workspace (in 32-bit words) needed by radix_argsort_u32 for n elements.
size_t radix_temp_words(size_t n);
// Stable argsort by the low `bits` bits of keys[0..n): vals_out[j] = the index
// of the j-th item in key order (ties in index order).  k0, v0, k1, v1 are n-word
// work arrays; keys is only read.
cudaError_t radix_argsort_u32(const uint32_t *keys, size_t n, int bits, uint32_t *vals_out, uint32_t *k0, uint32_t *v0,
                              uint32_t *k1, uint32_t *v1, uint32_t *temp, cudaStream_t s);

}  // namespace dcrf
