// primitives.cuh -- device-wide scan and stable radix sort (see primitives.cu).
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include "dcrf_common.cuh"

namespace dcrf {

// ---- single-pass exclusive scan (decoupled look-back) ----------------------
// One launch scans up to two u32 arrays of the same length: each CTA takes
// tiles in ticket order (an atomic counter, so that every tile it waits on
// belongs to a CTA that is already running), scans its tile, publishes the
// tile's sum, and looks back over its predecessors' published sums and
// prefixes.  The look-back wait is bounded: a CTA that gives up records
// DCRF_ERR_TIMEOUT in `st` and leaves its outputs unwritten.
constexpr int LB_THREADS = 256, LB_ITEMS = 16, LB_TILE = LB_THREADS * LB_ITEMS;

struct LBScanArgs {
    int narr = 1;             // arrays in this launch (1 or 2)
    size_t n = 0;             // items per array
    const uint32_t *in[2] = {nullptr, nullptr};
    uint32_t *out[2] = {nullptr, nullptr};        // exclusive prefix sums (in place allowed)
    uint32_t *total[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};  // the sum, to each non-null place
    // flag mode (in[0] == null): item k of array 0 is 1 when table[slot[k]] == k
    const uint32_t *table = nullptr, *slot = nullptr;
    unsigned long long *state = nullptr;  // lb_state_words(n) words, zero before the launch
    DevStatus *st = nullptr;
};

// 64-bit words of tile state a launch over n items per array needs (tile
// descriptors of both arrays plus the two tickets); they must be zero when the
// launch starts (a preceding kernel clears them, see ClearList).
size_t lb_state_words(size_t n);
cudaError_t lb_scan(const LBScanArgs &a, cudaStream_t s);

// Ranges of 32-bit words that a kernel sets (grid-stride) before later kernels
// of the same stream use them: hash tables, scan states, counters.
struct ClearList {
    int n = 0;
    uint32_t *p[6];
    size_t words[6];
    uint32_t val[6];
    void add(void *ptr, size_t nwords, uint32_t v) {
        p[n] = static_cast<uint32_t *>(ptr);
        words[n] = nwords;
        val[n] = v;
        n++;
    }
};

__device__ __forceinline__ void clear_words(const ClearList &c, size_t tid, size_t stride) {
    for (int j = 0; j < c.n; j++)
        for (size_t w = tid; w < c.words[j]; w += stride) c.p[j][w] = c.val[j];
}

// Workspace (in 32-bit words) needed by scan_exclusive_u32 for n elements.
size_t scan_temp_words(size_t n);
// out[i] = sum(in[0..i)); in-place allowed; *d_total (device, may be NULL) = sum(in).
cudaError_t scan_exclusive_u32(const uint32_t *in, uint32_t *out, size_t n, uint32_t *d_total, uint32_t *temp,
                               cudaStream_t s);

// Workspace (in 32-bit words) needed by radix_argsort_u32 for n elements.
size_t radix_temp_words(size_t n);
// Stable argsort by the low `bits` bits of keys[0..n): vals_out[j] = the index
// of the j-th item in key order (ties in index order).  k0, v0, k1, v1 are n-word
// work arrays; keys is only read.
cudaError_t radix_argsort_u32(const uint32_t *keys, size_t n, int bits, uint32_t *vals_out, uint32_t *k0, uint32_t *v0,
                              uint32_t *k1, uint32_t *v1, uint32_t *temp, cudaStream_t s);

}  // namespace dcrf
