// primitives.cu -- device-wide exclusive scan and stable LSD radix sort.
//
// Used by the lattice build: compaction of first-occurrence corners into
// vertex ids (the reference assigns ids in hash-insertion order,
// permutohedral.cpp:105-111) and the grouping of per-tile splat partials by
// vertex.  Both are deterministic: no float math, and the sort is stable.
#include "dcrf_common.cuh"
#include "primitives.cuh"

#include <algorithm>

namespace dcrf {

constexpr int SCAN_THREADS = 256;
constexpr int SCAN_ITEMS = 4;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;

// Block-wide exclusive scan of one value per thread; returns the block total.
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t *s_warp, uint32_t &total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) s_warp[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = lane < (SCAN_THREADS / 32) ? s_warp[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        if (lane < (SCAN_THREADS / 32)) s_warp[lane] = w;
    }
    __syncthreads();
    total = s_warp[SCAN_THREADS / 32 - 1];
    uint32_t before = warp ? s_warp[warp - 1] : 0;
    return before + x - v;
}

__global__ void scan_reduce_kernel(const uint32_t *__restrict__ in, size_t n, uint32_t *__restrict__ sums) {
    __shared__ uint32_t s_warp[SCAN_THREADS / 32];
    size_t base = (size_t)blockIdx.x * SCAN_TILE + (size_t)threadIdx.x * SCAN_ITEMS;
    uint32_t s = 0;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; k++)
        if (base + k < n) s += in[base + k];
    uint32_t total;
    block_exclusive_scan(s, s_warp, total);
    if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

// Exclusive scan of one tile plus the tile's offset; in-place safe.
__global__ void scan_tile_kernel(const uint32_t *in, uint32_t *out, size_t n, const uint32_t *__restrict__ offsets,
                                 uint32_t *__restrict__ d_total) {
    __shared__ uint32_t s_warp[SCAN_THREADS / 32];
    size_t base = (size_t)blockIdx.x * SCAN_TILE + (size_t)threadIdx.x * SCAN_ITEMS;
    uint32_t v[SCAN_ITEMS];
    uint32_t s = 0;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; k++) {
        v[k] = base + k < n ? in[base + k] : 0;
        s += v[k];
    }
    uint32_t total;
    uint32_t pre = block_exclusive_scan(s, s_warp, total);
    uint32_t off = offsets ? offsets[blockIdx.x] : 0;
    uint32_t run = off + pre;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; k++) {
        if (base + k < n) out[base + k] = run;
        run += v[k];
    }
    if (d_total && threadIdx.x == 0) *d_total = off + total;
}

// Exclusive scan of up to a few 16384-element chunks by one block of 1024
// threads (16 consecutive items each), carrying the running total across
// chunks: one launch instead of the three of the multi-block scan.
constexpr int SMALL_THREADS = 1024, SMALL_ITEMS = 16, SMALL_CHUNK = SMALL_THREADS * SMALL_ITEMS;
constexpr size_t SCAN_SMALL_MAX = 4 * (size_t)SMALL_CHUNK;

// Up to two independent arrays of the same length per launch: block b scans
// array b.
struct SmallScan {
    const uint32_t *in[2];
    uint32_t *out[2];
    uint32_t *total[2];
};

__global__ void __launch_bounds__(SMALL_THREADS) scan_small_kernel(const __grid_constant__ SmallScan a, size_t n) {
    const uint32_t *in = a.in[blockIdx.x];
    uint32_t *out = a.out[blockIdx.x];
    uint32_t *d_total = a.total[blockIdx.x];
    __shared__ uint32_t s_warp[SMALL_THREADS / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t carry = 0;
    for (size_t c0 = 0; c0 < n; c0 += SMALL_CHUNK) {
        const size_t base = c0 + (size_t)threadIdx.x * SMALL_ITEMS;
        uint32_t v[SMALL_ITEMS];
        uint32_t sum = 0;
#pragma unroll
        for (int k = 0; k < SMALL_ITEMS; k++) {
            v[k] = base + k < n ? in[base + k] : 0u;
            sum += v[k];
        }
        uint32_t x = sum;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) s_warp[warp] = x;
        __syncthreads();
        if (warp == 0) {
            uint32_t w = s_warp[lane];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
                if (lane >= o) w += y;
            }
            s_warp[lane] = w;
        }
        __syncthreads();
        uint32_t run = carry + (warp ? s_warp[warp - 1] : 0u) + x - sum;
#pragma unroll
        for (int k = 0; k < SMALL_ITEMS; k++) {
            if (base + k < n) out[base + k] = run;
            run += v[k];
        }
        carry += s_warp[SMALL_THREADS / 32 - 1];
        __syncthreads();  // s_warp is rewritten by the next chunk
    }
    if (d_total && threadIdx.x == 0) *d_total = carry;
}

size_t scan_temp_words(size_t n) {
    size_t w = 0;
    while (n > (size_t)SCAN_TILE) {
        n = (n + SCAN_TILE - 1) / SCAN_TILE;
        w += (n + 63) / 64 * 64;
    }
    return w + 64;
}

static cudaError_t scan_rec(const uint32_t *in, uint32_t *out, size_t n, uint32_t *d_total, uint32_t *temp,
                            cudaStream_t s) {
    size_t nb = (n + SCAN_TILE - 1) / SCAN_TILE;
    if (nb <= 1) {
        DCRF_LAUNCH(scan_tile_kernel<<<1, SCAN_THREADS, 0, s>>>(in, out, n, nullptr, d_total));
        return cudaGetLastError();
    }
    if (n <= SCAN_SMALL_MAX) {
        const SmallScan a = {{in, nullptr}, {out, nullptr}, {d_total, nullptr}};
        DCRF_LAUNCH(scan_small_kernel<<<1, SMALL_THREADS, 0, s>>>(a, n));
        return cudaGetLastError();
    }
    uint32_t *sums = temp;
    temp += (nb + 63) / 64 * 64;
    DCRF_LAUNCH(scan_reduce_kernel<<<(unsigned)nb, SCAN_THREADS, 0, s>>>(in, n, sums));
    cudaError_t e = scan_rec(sums, sums, nb, d_total, temp, s);
    if (e != cudaSuccess) return e;
    DCRF_LAUNCH(scan_tile_kernel<<<(unsigned)nb, SCAN_THREADS, 0, s>>>(in, out, n, sums, nullptr));
    return cudaGetLastError();
}

cudaError_t scan_exclusive_u32(const uint32_t *in, uint32_t *out, size_t n, uint32_t *d_total, uint32_t *temp,
                               cudaStream_t s) {
    if (n == 0) {
        if (d_total) return cudaMemsetAsync(d_total, 0, sizeof(uint32_t), s);
        return cudaSuccess;
    }
    return scan_rec(in, out, n, d_total, temp, s);
}

// ---------------------------------------------------------------------------
// Single-pass exclusive scan with decoupled look-back.
// ---------------------------------------------------------------------------
// A tile descriptor holds its kind in the top two bits (0: nothing yet, 1: the
// tile's own sum, 2: the inclusive prefix through the tile) and the value below.
constexpr unsigned long long LB_AGG = 1ull << 62, LB_INC = 2ull << 62, LB_VAL = (1ull << 62) - 1;
constexpr int LB_SPINS = 1 << 20;  // polls of one look-back window before giving up

static unsigned lb_tiles(size_t n) { return (unsigned)std::max<size_t>(1, (n + LB_TILE - 1) / LB_TILE); }

size_t lb_state_words(size_t n) { return 2 * (size_t)lb_tiles(n) + 1; }

__device__ __forceinline__ unsigned long long lb_load(const unsigned long long *p) {
    return *reinterpret_cast<const volatile unsigned long long *>(p);
}

__global__ void __launch_bounds__(LB_THREADS) lb_scan_kernel(const __grid_constant__ LBScanArgs a, unsigned ntiles) {
    __shared__ unsigned s_tile;
    __shared__ uint32_t s_warp[LB_THREADS / 32];
    __shared__ unsigned long long s_prefix;
    __shared__ int s_ok;
    const int arr = blockIdx.x >= ntiles ? 1 : 0;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    unsigned *tickets = reinterpret_cast<unsigned *>(a.state + 2 * (size_t)ntiles);
    if (tid == 0) s_tile = atomicAdd(tickets + arr, 1u);
    __syncthreads();
    const unsigned tile = s_tile;
    unsigned long long *desc = a.state + (size_t)arr * ntiles;
    const size_t n = a.n;
    const size_t base = (size_t)tile * LB_TILE + (size_t)tid * LB_ITEMS;
    const uint32_t *in = a.in[arr];
    uint32_t v[LB_ITEMS];
    const bool full = base + LB_ITEMS <= n;
    if (in) {
        if (full && ((reinterpret_cast<uintptr_t>(in) & 15) == 0)) {
            const uint4 *q = reinterpret_cast<const uint4 *>(in + base);
#pragma unroll
            for (int c = 0; c < LB_ITEMS / 4; c++) {
                const uint4 x = q[c];
                v[4 * c] = x.x, v[4 * c + 1] = x.y, v[4 * c + 2] = x.z, v[4 * c + 3] = x.w;
            }
        } else {
#pragma unroll
            for (int j = 0; j < LB_ITEMS; j++) v[j] = base + j < n ? in[base + j] : 0u;
        }
    } else {  // flag mode: first occurrences of the hash table's keys
        uint32_t sl[LB_ITEMS];
        if (full && ((reinterpret_cast<uintptr_t>(a.slot) & 15) == 0)) {
            const uint4 *q = reinterpret_cast<const uint4 *>(a.slot + base);
#pragma unroll
            for (int c = 0; c < LB_ITEMS / 4; c++) {
                const uint4 x = q[c];
                sl[4 * c] = x.x, sl[4 * c + 1] = x.y, sl[4 * c + 2] = x.z, sl[4 * c + 3] = x.w;
            }
        } else {
#pragma unroll
            for (int j = 0; j < LB_ITEMS; j++) sl[j] = base + j < n ? a.slot[base + j] : 0u;
        }
#pragma unroll
        for (int j = 0; j < LB_ITEMS; j++) v[j] = (base + j < n && a.table[sl[j]] == (uint32_t)(base + j)) ? 1u : 0u;
    }
    // block-wide exclusive scan of the thread sums
    uint32_t tsum = 0;
#pragma unroll
    for (int j = 0; j < LB_ITEMS; j++) tsum += v[j];
    uint32_t x = tsum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) s_warp[warp] = x;
    __syncthreads();
    uint32_t wpre = 0, agg = 0;
#pragma unroll
    for (int w = 0; w < LB_THREADS / 32; w++) {
        const uint32_t c = s_warp[w];
        wpre += w < warp ? c : 0u;
        agg += c;
    }
    const uint32_t texcl = wpre + x - tsum;
    // the tile's prefix: publish the own sum, then look back (warp 0)
    if (warp == 0) {
        unsigned long long prefix = 0;
        int ok = 1;
        if (tile == 0) {
            if (lane == 0) atomicExch(desc, LB_INC | (unsigned long long)agg);
        } else {
            if (lane == 0) atomicExch(desc + tile, LB_AGG | (unsigned long long)agg);
            long long pred = (long long)tile - 1;
            int spins = 0;
            for (;;) {
                const long long idx = pred - lane;
                const unsigned long long d = idx >= 0 ? lb_load(desc + idx) : LB_INC;
                if (__all_sync(0xffffffffu, (d >> 62) != 0)) {
                    const unsigned inc = __ballot_sync(0xffffffffu, (d >> 62) == 2);
                    const int stop = inc ? __ffs(inc) - 1 : 31;
                    unsigned long long val = lane <= stop ? (d & LB_VAL) : 0ull;
#pragma unroll
                    for (int o = 16; o > 0; o >>= 1) val += __shfl_xor_sync(0xffffffffu, val, o);
                    prefix += val;
                    if (inc) break;
                    pred -= 32;
                    spins = 0;
                    continue;
                }
                if (++spins > LB_SPINS) {
                    ok = 0;
                    break;
                }
                if (spins > 32) __nanosleep(64);
            }
            if (lane == 0 && ok) atomicExch(desc + tile, LB_INC | ((prefix + agg) & LB_VAL));
        }
        if (lane == 0) {
            s_prefix = prefix;
            s_ok = ok;
        }
    }
    __syncthreads();
    if (!s_ok) {
        if (tid == 0) dcrf_set_error(a.st, DCRF_ERR_TIMEOUT, (int)tile);
        return;
    }
    const unsigned long long prefix = s_prefix;
    uint32_t run = (uint32_t)prefix + texcl;
    uint32_t *out = a.out[arr];
    if (full && ((reinterpret_cast<uintptr_t>(out) & 15) == 0)) {
        uint32_t o[LB_ITEMS];
#pragma unroll
        for (int j = 0; j < LB_ITEMS; j++) {
            o[j] = run;
            run += v[j];
        }
        uint4 *q = reinterpret_cast<uint4 *>(out + base);
#pragma unroll
        for (int c = 0; c < LB_ITEMS / 4; c++) q[c] = make_uint4(o[4 * c], o[4 * c + 1], o[4 * c + 2], o[4 * c + 3]);
    } else {
#pragma unroll
        for (int j = 0; j < LB_ITEMS; j++) {
            if (base + j < n) out[base + j] = run;
            run += v[j];
        }
    }
    if (tile == ntiles - 1 && tid == 0) {
        const uint32_t total = (uint32_t)(prefix + agg);
        if (a.total[arr][0]) *a.total[arr][0] = total;
        if (a.total[arr][1]) *a.total[arr][1] = total;
    }
}

cudaError_t lb_scan(const LBScanArgs &a, cudaStream_t s) {
    if (a.narr < 1 || a.narr > 2 || !a.state || (!a.in[0] && (!a.table || !a.slot || a.narr != 1)))
        return cudaErrorInvalidValue;
    const unsigned nt = lb_tiles(a.n);
    DCRF_LAUNCH(lb_scan_kernel<<<nt * (unsigned)a.narr, LB_THREADS, 0, s>>>(a, nt));
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Stable LSD radix sort of (key, value) uint32 pairs, 8-bit digits.
// ---------------------------------------------------------------------------
constexpr int RADIX_THREADS = 256;
constexpr int RADIX_ROUNDS = 8;
constexpr int RADIX_TILE = RADIX_THREADS * RADIX_ROUNDS;
constexpr int RADIX_WARPS = RADIX_THREADS / 32;

__global__ void radix_hist_kernel(const uint32_t *__restrict__ keys, size_t n, int shift, uint32_t *__restrict__ hist,
                                  unsigned nblocks) {
    __shared__ uint32_t cnt[256];
    cnt[threadIdx.x] = 0;
    __syncthreads();
    size_t base = (size_t)blockIdx.x * RADIX_TILE;
#pragma unroll
    for (int r = 0; r < RADIX_ROUNDS; r++) {
        size_t i = base + (size_t)r * RADIX_THREADS + threadIdx.x;
        if (i < n) atomicAdd(&cnt[(keys[i] >> shift) & 255u], 1u);
    }
    __syncthreads();
    hist[(size_t)threadIdx.x * nblocks + blockIdx.x] = cnt[threadIdx.x];
}

// vals == nullptr: the value of item i is i (first pass of an argsort)
__global__ void radix_scatter_kernel(const uint32_t *__restrict__ keys, const uint32_t *__restrict__ vals, size_t n,
                                     int shift, const uint32_t *__restrict__ hist, unsigned nblocks,
                                     uint32_t *__restrict__ keys_out, uint32_t *__restrict__ vals_out) {
    __shared__ uint32_t s_wcnt[RADIX_WARPS][257];
    __shared__ uint32_t s_run[256];
    __shared__ uint32_t s_base[256];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    s_run[threadIdx.x] = 0;
    s_base[threadIdx.x] = hist[(size_t)threadIdx.x * nblocks + blockIdx.x];
    size_t base = (size_t)blockIdx.x * RADIX_TILE;
    for (int r = 0; r < RADIX_ROUNDS; r++) {
        for (int w = 0; w < RADIX_WARPS; w++) s_wcnt[w][threadIdx.x] = 0;
        __syncthreads();
        size_t i = base + (size_t)r * RADIX_THREADS + threadIdx.x;
        bool valid = i < n;
        uint32_t key = valid ? keys[i] : 0u;
        uint32_t val = valid ? (vals ? vals[i] : (uint32_t)i) : 0u;
        uint32_t digit = valid ? ((key >> shift) & 255u) : 256u;
        uint32_t peers = __match_any_sync(0xffffffffu, digit);
        int leader = __ffs(peers) - 1;
        uint32_t rank = __popc(peers & ((1u << lane) - 1u));
        if (lane == leader && valid) s_wcnt[warp][digit] = __popc(peers);
        __syncthreads();
        {
            uint32_t run = s_run[threadIdx.x];
            for (int w = 0; w < RADIX_WARPS; w++) {
                uint32_t c = s_wcnt[w][threadIdx.x];
                s_wcnt[w][threadIdx.x] = run;
                run += c;
            }
            s_run[threadIdx.x] = run;
        }
        __syncthreads();
        if (valid) {
            // s_wcnt now holds, per (warp, digit), the count of earlier items of that digit
            // in this tile (earlier rounds plus earlier warps of this round)
            uint32_t pos = s_base[digit] + s_wcnt[warp][digit] + rank;
            keys_out[pos] = key;
            vals_out[pos] = val;
        }
        __syncthreads();
    }
}

size_t radix_temp_words(size_t n) {
    size_t nb = (n + RADIX_TILE - 1) / RADIX_TILE;
    size_t h = 256 * nb;
    return (h + 63) / 64 * 64 + scan_temp_words(h);
}

cudaError_t radix_argsort_u32(const uint32_t *keys, size_t n, int bits, uint32_t *vals_out, uint32_t *k0, uint32_t *v0,
                              uint32_t *k1, uint32_t *v1, uint32_t *temp, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    unsigned nb = (unsigned)((n + RADIX_TILE - 1) / RADIX_TILE);
    size_t h = 256 * (size_t)nb;
    uint32_t *hist = temp;
    uint32_t *stemp = temp + (h + 63) / 64 * 64;
    int passes = (bits + 7) / 8;
    if (passes < 1) passes = 1;
    const uint32_t *kin = keys, *vin = nullptr;
    for (int p = 0; p < passes; p++) {
        const int shift = 8 * p;
        // ping-pong between (k1, v1) and (k0, v0); the last pass writes the values out
        uint32_t *kout = (p & 1) ? k0 : k1;
        uint32_t *vout = p == passes - 1 ? vals_out : (p & 1) ? v0 : v1;
        DCRF_LAUNCH(radix_hist_kernel<<<nb, RADIX_THREADS, 0, s>>>(kin, n, shift, hist, nb));
        cudaError_t e = scan_exclusive_u32(hist, hist, h, nullptr, stemp, s);
        if (e != cudaSuccess) return e;
        DCRF_LAUNCH(radix_scatter_kernel<<<nb, RADIX_THREADS, 0, s>>>(kin, vin, n, shift, hist, nb, kout, vout));
        e = cudaGetLastError();
        if (e != cudaSuccess) return e;
        kin = kout;
        vin = vout;
    }
    return cudaSuccess;
}

}  // namespace dcrf
