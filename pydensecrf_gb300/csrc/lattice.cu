// lattice.cu -- GPU build of the permutohedral lattice (the device form of
// Permutohedral::init, pydensecrf/densecrf/src/permutohedral.cpp:140-474).
//
// Pipeline (one launch each, all on the caller's stream):
//   1. embed      thread per point: elevate, round to the 0-coloured simplex,
//                 rank, wrap, barycentric weights and the d+1 corner keys
//                 (P:191-275 on x86, P:359-435 scalar).  Keys are packed
//                 16-bit fields (image id, d coordinates) in 64-bit words.
//   2. insert     thread per corner: open-addressing hash on the packed key;
//                 each slot keeps the SMALLEST corner index holding its key
//                 (CAS then atomicMin), i.e. the key's first occurrence.
//   3. compact    flag first occurrences, exclusive scan -> vertex id.  The
//                 reference numbers vertices in hash-insertion order, which
//                 is first-occurrence order, so the ids match the
//                 reference's exactly -- no relabelling is needed.
//   4. offsets    corner -> vertex id (offset_), vertex -> key.
//   5. neighbours thread per (axis, vertex): look up key -1/+1 with +d/-d on
//                 the axis.
//   6. tiles      per splat tile (a set of up to SPLAT_TILE points), the
//                 corners grouped by vertex in corner order without a sort
//                 (shared-memory hash, first-occurrence numbering, stable
//                 warp-sequential ranking): the tile's distinct vertices
//                 ("partials"), the member lists and splat tasks of the
//                 in-kernel splat, and per corner the index of its vertex among
//                 the tile's partials (the tile-local slice table).
//   7. reduce     the tiles' partials grouped by vertex, each vertex's in tile
//                 order: the order in which its partial sums are added (a
//                 counting placement and a rank within each vertex's range; a
//                 stable radix sort when vertices have very many partials).
// Bounded probing everywhere: a full table sets DCRF_ERR_HASH_FULL and the
// host retries with a larger table; no kernel waits on another thread.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>

#include "lattice.cuh"
#include "primitives.cuh"

namespace dcrf {

static thread_local std::string g_msg;
const char *lattice_last_message() { return g_msg.c_str(); }

constexpr uint32_t EMPTY = 0xFFFFFFFFu;

template <int D>
struct KeyW {
    static constexpr int KW = (D + 4) / 4;  // ceil((D+1)/4) 64-bit words of 16-bit fields
};

__device__ __forceinline__ uint64_t mix64(uint64_t x) {
    x ^= x >> 33;
    x *= 0xff51afd7ed558ccdULL;
    x ^= x >> 33;
    x *= 0xc4ceb9fe1a85ec53ULL;
    x ^= x >> 33;
    return x;
}

template <int KW>
__device__ __forceinline__ uint32_t key_hash(const uint64_t *k) {
    uint64_t h = 0x9E3779B97F4A7C15ULL;
#pragma unroll
    for (int w = 0; w < KW; w++) h = mix64(h ^ k[w]) + 0x632BE59BD9B4E019ULL * (w + 1);
    return (uint32_t)(h ^ (h >> 32));
}

struct EmbedArgs {
    const float *feat;  // [d][N]
    int N;
    int n_ph;
    const int *ph_img;     // [n_ph] image of each padding point
    const int *seg_start;  // [nseg+1]
    int nseg;
    float sf[DCRF_MAX_D];
    float invdp1, dp1, alpha;
    int variant;
    float *bary;
    float *wslice;
    uint8_t *rank;
    uint64_t *keys;  // [(N+n_ph)*(d+1)][KW]
    DevStatus *st;
    ClearList clr;   // set before the build's later kernels run: hash table, scan states, counts
};

template <int D>
__global__ void __launch_bounds__(128) embed_kernel(EmbedArgs a) {
    constexpr int KW = KeyW<D>::KW;
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    clear_words(a.clr, (size_t)p, (size_t)gridDim.x * blockDim.x);
    if (p >= a.N + a.n_ph) return;
    int img;
    float f[D];
    if (p < a.N) {
        int lo = 0, hi = a.nseg - 1;
        while (lo < hi) {
            int mid = (lo + hi + 1) >> 1;
            if (a.seg_start[mid] <= p)
                lo = mid;
            else
                hi = mid - 1;
        }
        img = lo;
#pragma unroll
        for (int j = 0; j < D; j++) f[j] = a.feat[(size_t)j * a.N + p];
    } else {
        img = a.ph_img ? a.ph_img[p - a.N] : 0;
#pragma unroll
        for (int j = 0; j < D; j++) f[j] = 0.f;
    }
    // Elevate (P:201-207 / P:364-370)
    float el[D + 1], rem0[D + 1];
    int rank[D + 1];
    float sm = 0.f;
#pragma unroll
    for (int j = D; j > 0; j--) {
        float cf = fmul(f[j - 1], a.sf[j - 1]);
        el[j] = fsub(sm, fmul((float)j, cf));
        sm = fadd(sm, cf);
    }
    el[0] = sm;
#pragma unroll
    for (int i = 0; i <= D; i++) rank[i] = 0;
    if (a.variant == DCRF_VARIANT_SSE) {
        // round-to-nearest-even of el/(d+1), float rank arithmetic
        float sum = 0.f;
#pragma unroll
        for (int i = 0; i <= D; i++) {
            float v = rintf(fmul(a.invdp1, el[i]));
            rem0[i] = fmul(v, a.dp1);
            sum = fadd(sum, v);
        }
#pragma unroll
        for (int i = 0; i < D; i++) {
            float di = fsub(el[i], rem0[i]);
#pragma unroll
            for (int j = i + 1; j <= D; j++) {
                float dj = fsub(el[j], rem0[j]);
                if (di < dj)
                    rank[i]++;
                else
                    rank[j]++;
            }
        }
        int isum = (int)sum;
#pragma unroll
        for (int i = 0; i <= D; i++) {
            rank[i] += isum;
            float add = rank[i] < 0 ? a.dp1 : 0.f;
            float sub = rank[i] >= D + 1 ? a.dp1 : 0.f;
            float adj = fsub(add, sub);
            rank[i] += (int)adj;
            rem0[i] = fadd(rem0[i], adj);
        }
    } else {
        // distance-compared rounding (ties down), int sum that
        // truncates on every add, short ranks
        int sum = 0;
#pragma unroll
        for (int i = 0; i <= D; i++) {
            float v = fmul(a.invdp1, el[i]);
            float up = fmul(ceilf(v), a.dp1);
            float down = fmul(floorf(v), a.dp1);
            int rd2 = (fsub(up, el[i]) < fsub(el[i], down)) ? (int)(short)(int)up : (int)(short)(int)down;
            rem0[i] = (float)rd2;
            sum = __float2int_rz(fadd((float)sum, fmul((float)rd2, a.invdp1)));
        }
#pragma unroll
        for (int i = 0; i < D; i++) {
            float di = fsub(el[i], rem0[i]);
#pragma unroll
            for (int j = i + 1; j <= D; j++) {
                if (di < fsub(el[j], rem0[j]))
                    rank[i]++;
                else
                    rank[j]++;
            }
        }
#pragma unroll
        for (int i = 0; i <= D; i++) {
            rank[i] = (short)(rank[i] + sum);
            if (rank[i] < 0) {
                rank[i] += D + 1;
                rem0[i] = fadd(rem0[i], a.dp1);
            } else if (rank[i] > D) {
                rank[i] -= D + 1;
                rem0[i] = fsub(rem0[i], a.dp1);
            }
        }
    }
    // Barycentric coordinates (P:244-263 / P:417-426), same operation order
    float bary[D + 2];
#pragma unroll
    for (int q = 0; q < D + 2; q++) bary[q] = 0.f;
#pragma unroll
    for (int i = 0; i <= D; i++) {
        float v = fmul(fsub(el[i], rem0[i]), a.invdp1);
        int pidx = D - rank[i];
#pragma unroll
        for (int q = 0; q < D + 2; q++) {
            if (q == pidx) bary[q] = fadd(bary[q], v);
            if (q == pidx + 1) bary[q] = fsub(bary[q], v);
        }
    }
    if (a.variant == DCRF_VARIANT_SSE)
        bary[0] = fadd(bary[0], fadd(1.0f, bary[D + 1]));
    else
        bary[0] = __double2float_rn(__dadd_rn((double)bary[0], __dadd_rn(1.0, (double)bary[D + 1])));
    if (p < a.N) {
#pragma unroll
        for (int r = 0; r <= D; r++) {
            a.bary[(size_t)r * a.N + p] = bary[r];
            a.wslice[(size_t)r * a.N + p] = fmul(bary[r], a.alpha);
            a.rank[(size_t)r * a.N + p] = (uint8_t)rank[r];
        }
    }
    // Corner keys (P:268-272 / P:429-432): rem0 + canonical simplex coordinate
    bool overflow = false;
#pragma unroll
    for (int r = 0; r <= D; r++) {
        uint64_t w[KW];
#pragma unroll
        for (int q = 0; q < KW; q++) w[q] = 0;
        w[0] = (uint64_t)(uint16_t)img;
#pragma unroll
        for (int q = 0; q < D; q++) {
            int canon = rank[q] <= D - r ? r : r - (D + 1);
            int c = (int)fadd(rem0[q], (float)canon);
            overflow |= (c < -32768 || c > 32767);
            const int field = q + 1;
            w[field >> 2] |= (uint64_t)(uint16_t)(short)c << (16 * (field & 3));
        }
        uint64_t *dst = a.keys + ((size_t)p * (D + 1) + r) * KW;
#pragma unroll
        for (int q = 0; q < KW; q++) dst[q] = w[q];
    }
    if (overflow) dcrf_set_error(a.st, DCRF_ERR_KEY_OVERFLOW, p);
}

template <int KW>
__device__ __forceinline__ bool key_eq(const uint64_t *__restrict__ a, const uint64_t *b) {
    bool eq = true;
#pragma unroll
    for (int w = 0; w < KW; w++) eq &= (a[w] == b[w]);
    return eq;
}

// Lanes of a warp holding the same key insert it once: the lowest such lane
// (the smallest corner index among them, the only one that can matter to the
// first-occurrence minimum) probes, the others take its slot.  Neighbouring
// points share most lattice vertices, so a warp of 32 corners holds only a
// few distinct keys.
template <int KW>
__global__ void insert_kernel(const uint64_t *__restrict__ keys, size_t E, uint32_t *table, uint32_t mask,
                              uint32_t *__restrict__ slot, DevStatus *st) {
    const size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const unsigned active = __ballot_sync(0xffffffffu, k < E);
    if (k >= E) return;
    uint64_t key[KW];
#pragma unroll
    for (int w = 0; w < KW; w++) key[w] = keys[k * KW + w];
    unsigned peers = active;
#pragma unroll
    for (int w = 0; w < KW; w++) peers &= __match_any_sync(active, key[w]);
    const int lane = (int)(threadIdx.x & 31u), leader = __ffs(peers) - 1;
    uint32_t h = key_hash<KW>(key) & mask;
    if (lane == leader) {
        bool done = false;
        for (uint32_t probe = 0; probe <= mask && !done; probe++) {
            uint32_t e = __ldcg(&table[h]);
            if (e == EMPTY) {
                e = atomicCAS(&table[h], EMPTY, (uint32_t)k);
                if (e == EMPTY) {
                    done = true;
                    break;
                }
            }
            if (key_eq<KW>(keys + (size_t)e * KW, key)) {
                atomicMin(&table[h], (uint32_t)k);
                done = true;
                break;
            }
            h = (h + 1) & mask;
        }
        if (!done) dcrf_set_error(st, DCRF_ERR_HASH_FULL, 0);
    }
    slot[k] = __shfl_sync(peers, h, leader);
}

template <int D>
__global__ void offsets_kernel(const uint64_t *__restrict__ keys, const uint32_t *__restrict__ table,
                               const uint32_t *__restrict__ slot, const uint32_t *__restrict__ vid, size_t E,
                               int N, int *__restrict__ off, uint16_t *__restrict__ vkeys,
                               uint32_t *__restrict__ vcount) {
    constexpr int KW = KeyW<D>::KW;
    size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= E) return;
    uint32_t rep = table[slot[k]];
    // a corner whose insert failed (hash table full, reported by the insert)
    // maps to vertex 0 until the host sees the status and drops the build
    if (rep >= (uint32_t)E) rep = (uint32_t)k;
    uint32_t v = vid[rep];
    if (k < (size_t)N * (D + 1)) {
        size_t i = k / (D + 1);
        int r = (int)(k - i * (D + 1));
        off[(size_t)r * N + i] = (int)v;
    }
    if (rep == (uint32_t)k) {
        vcount[v] = 0;  // partials per vertex, counted by the tile placement
#pragma unroll
        for (int q = 0; q <= D; q++) vkeys[(size_t)v * (D + 1) + q] = (uint16_t)(keys[k * KW + (q >> 2)] >> (16 * (q & 3)));
    }
}

template <int D>
__device__ __forceinline__ int lookup(const uint64_t *__restrict__ keys, const uint32_t *__restrict__ table,
                                      uint32_t mask, const uint32_t *__restrict__ vid, const uint16_t *fields) {
    constexpr int KW = KeyW<D>::KW;
    uint64_t key[KW];
#pragma unroll
    for (int w = 0; w < KW; w++) key[w] = 0;
#pragma unroll
    for (int q = 0; q <= D; q++) key[q >> 2] |= (uint64_t)fields[q] << (16 * (q & 3));
    uint32_t h = key_hash<KW>(key) & mask;
    for (uint32_t probe = 0; probe <= mask; probe++) {
        uint32_t e = table[h];
        if (e == EMPTY) return -1;
        if (key_eq<KW>(keys + (size_t)e * KW, key)) return (int)vid[e];
        h = (h + 1) & mask;
    }
    return -1;
}

// Neighbours of vertex v along axis j: the keys one step down and
// up the axis; nbr = (index + 1) of each, 0 when absent.
template <int D>
__device__ __forceinline__ void neighbors_of(const uint64_t *__restrict__ keys, const uint32_t *__restrict__ table,
                                             uint32_t mask, const uint32_t *__restrict__ vid,
                                             const uint16_t *__restrict__ vkeys, int v, int j, int2 *out) {
    uint16_t kf[D + 1], n1[D + 1], n2[D + 1];
#pragma unroll
    for (int q = 0; q <= D; q++) kf[q] = vkeys[(size_t)v * (D + 1) + q];
    n1[0] = n2[0] = kf[0];
#pragma unroll
    for (int q = 0; q < D; q++) {
        short c = (short)kf[q + 1];
        short a = (short)(c - 1), b = (short)(c + 1);
        if (q == j) {
            a = (short)(c + D);
            b = (short)(c - D);
        }
        n1[q + 1] = (uint16_t)a;
        n2[q + 1] = (uint16_t)b;
    }
    const int i1 = lookup<D>(keys, table, mask, vid, n1);
    const int i2 = lookup<D>(keys, table, mask, vid, n2);
    *out = make_int2(i1 + 1, i2 + 1);
}

// The vertex count L is read on the device (the host learns it later), so the
// launch covers an upper bound with a grid-stride loop.
template <int D>
__global__ void neighbors_kernel(const uint64_t *__restrict__ keys, const uint32_t *__restrict__ table, uint32_t mask,
                                 const uint32_t *__restrict__ vid, const uint16_t *__restrict__ vkeys,
                                 const uint32_t *__restrict__ d_L, int2 *__restrict__ nbr) {
    const int L = (int)*d_L;
    for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < (size_t)L * (D + 1);
         t += (size_t)gridDim.x * blockDim.x) {
        const int j = (int)(t / L);
        const int v = (int)(t - (size_t)j * L);
        neighbors_of<D>(keys, table, mask, vid, vkeys, v, j, nbr + t);
    }
}


// Block bitonic sort of one tile's corners by (vertex, corner) and count of
// distinct vertices.  Corner idx = slot*(D+1) + r of the tile's slot.
// ---- sort-free tile grouping ---------------------------------------------------
// A tile's corners c = li*(d+1)+r (point slot li, corner r) are grouped by
// vertex into "partials" numbered in first-occurrence order; the members of a
// partial stay in corner order.  tile_group finds the partials with a
// shared-memory hash (first corner by atomicMin, numbering by a block scan) and
// counts their members; tile_place, after the tiles' partial and task counts
// are scanned, lays out the member lists (stable, warp-sequential ranking),
// the tile-local slice tables and the splat tasks.
// Sentinel rows of a lattice's two value buffers (lattice_v1_offset, chunk_offset).
__device__ __forceinline__ void zero_value_rows(float *V0, float *V1, size_t L, int MP, int tid, int nthreads) {
    const int nc = MP <= DCRF_LCHUNK ? 1 : (MP + DCRF_LCHUNK - 1) / DCRF_LCHUNK;
    for (int e = tid; e < nc * DCRF_LCHUNK; e += nthreads) {
        const int c = e / DCRF_LCHUNK, m = e - c * DCRF_LCHUNK;
        const int w = MP <= DCRF_LCHUNK ? MP : min(DCRF_LCHUNK, MP - DCRF_LCHUNK * c);
        if (m < w) {
            const size_t o = (size_t)DCRF_LCHUNK * c * (L + 1) + m;
            V0[o] = 0.f;
            V1[o] = 0.f;
        }
    }
    if (tid == 0 && MP > 1) {
        const size_t o = (L + 1) * (size_t)(MP - 1);
        V0[o] = 0.f;
        V1[o] = 0.f;
    }
}

constexpr int TG_THREADS = 256;

template <int D>
struct TG {
    static constexpr int C = SPLAT_TILE * (D + 1);      // corners of a tile
    static constexpr int HT = C <= 1024 ? 2048 : C <= 2048 ? 4096 : C <= 4096 ? 8192 : 16384;
    static constexpr int PER = C / TG_THREADS;          // corners per thread (d+1)
};

__device__ __forceinline__ uint32_t tg_hash(uint32_t v) {
    v ^= v >> 16;
    v *= 0x7feb352dU;
    v ^= v >> 15;
    v *= 0x846ca68bU;
    v ^= v >> 16;
    return v;
}

template <int D>
__global__ void __launch_bounds__(TG_THREADS) tile_group_kernel(const int *__restrict__ off, int N,
                                                               const int *__restrict__ slot_pt, int task_len,
                                                               uint16_t *__restrict__ cl, int *__restrict__ pvx,
                                                               int *__restrict__ pcnt, uint32_t *__restrict__ tile_np,
                                                               uint32_t *__restrict__ tile_nt,
                                                               uint32_t *__restrict__ maxes, DevStatus *st) {
    constexpr int C = TG<D>::C, HT = TG<D>::HT, PER = TG<D>::PER;
    extern __shared__ int tg_smem[];
    int *hkey = tg_smem;            // [HT] vertex id or -1
    int *hfirst = hkey + HT;        // [HT] first corner of the vertex, then its partial id
    int *cnt = hfirst + HT;         // [C] members per partial
    __shared__ int swarp[TG_THREADS / 32];
    __shared__ uint32_t s_np, s_nt;
    const int t = blockIdx.x, tid = threadIdx.x;
    for (int e = tid; e < HT; e += TG_THREADS) {
        hkey[e] = -1;
        hfirst[e] = 0x7FFFFFFF;
    }
    for (int e = tid; e < C; e += TG_THREADS) cnt[e] = 0;
    if (tid == 0) s_nt = 0;
    __syncthreads();
    // 1. insert this thread's corners c = tid*PER + k (point li = tid, corners in order)
    int vtx[PER], hs[PER];
    const int pt = slot_pt[(size_t)t * SPLAT_TILE + tid];
#pragma unroll
    for (int k = 0; k < PER; k++) {
        vtx[k] = pt >= 0 ? off[(size_t)k * N + pt] : -1;
        hs[k] = -1;
        if (vtx[k] < 0) continue;
        uint32_t h = tg_hash((uint32_t)vtx[k]) & (HT - 1);
        for (int probe = 0; probe < HT; probe++, h = (h + 1) & (HT - 1)) {
            const int prev = atomicCAS(hkey + h, -1, vtx[k]);
            if (prev == -1 || prev == vtx[k]) {
                hs[k] = (int)h;
                break;
            }
        }
        if (hs[k] < 0) {  // cannot happen (HT >= 2 C); reported rather than assumed
            dcrf_set_error(st, DCRF_ERR_HASH_FULL, t);
            continue;
        }
        atomicMin(hfirst + hs[k], tid * PER + k);
    }
    __syncthreads();
    // 2. number the first occurrences in corner order (block exclusive scan)
    int nf = 0;
#pragma unroll
    for (int k = 0; k < PER; k++) nf += (hs[k] >= 0 && hfirst[hs[k]] == tid * PER + k) ? 1 : 0;
    const int lane = tid & 31, warp = tid >> 5;
    int x = nf;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) swarp[warp] = x;
    __syncthreads();
    int before = 0;
    for (int w = 0; w < warp; w++) before += swarp[w];
    if (tid == TG_THREADS - 1) s_np = (uint32_t)(before + x);
    int run = before + x - nf;
    int firstp[PER];
#pragma unroll
    for (int k = 0; k < PER; k++) {
        firstp[k] = -1;
        if (hs[k] >= 0 && hfirst[hs[k]] == tid * PER + k) {
            firstp[k] = run;
            pvx[(size_t)t * C + run] = vtx[k];
            run++;
        }
    }
    __syncthreads();  // every first corner has been identified: hfirst becomes the partial id
#pragma unroll
    for (int k = 0; k < PER; k++)
        if (firstp[k] >= 0) hfirst[hs[k]] = firstp[k];
    __syncthreads();
    // 3. each corner's partial; members per partial
#pragma unroll
    for (int k = 0; k < PER; k++) {
        uint16_t p = 0xFFFF;
        if (hs[k] >= 0) {
            p = (uint16_t)hfirst[hs[k]];
            atomicAdd(cnt + p, 1);
        }
        cl[(size_t)t * C + tid * PER + k] = p;
    }
    __syncthreads();
    const int np = (int)s_np;
    uint32_t ntask = 0;
    for (int p = tid; p < np; p += TG_THREADS) {
        const int c = cnt[p];
        pcnt[(size_t)t * C + p] = c;
        ntask += (uint32_t)((c + task_len - 1) / task_len);
    }
    atomicAdd(&s_nt, ntask);
    __syncthreads();
    if (tid == 0) {
        tile_np[t] = (uint32_t)np;
        tile_nt[t] = s_nt;
        atomicMax(maxes + 0, (uint32_t)np);
        atomicMax(maxes + 1, s_nt);
    }
}

// Block exclusive scan of v over 256 threads; returns the prefix, *total the sum.
__device__ __forceinline__ int block_exscan256(int v, int *swarp, int *total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    __syncthreads();
    if (lane == 31) swarp[warp] = x;
    __syncthreads();
    int before = 0, all = 0;
    for (int w = 0; w < TG_THREADS / 32; w++) {
        if (w < warp) before += swarp[w];
        all += swarp[w];
    }
    *total = all;
    return before + x - v;
}

template <int D>
__global__ void __launch_bounds__(TG_THREADS) tile_place_kernel(const uint16_t *__restrict__ cl,
                                                               const int *__restrict__ pvx,
                                                               const int *__restrict__ pcnt,
                                                               const float *__restrict__ bary, int N,
                                                               const int *__restrict__ slot_pt,
                                                               const uint32_t *__restrict__ tile_pbeg,
                                                               const uint32_t *__restrict__ tile_tbeg, int task_len,
                                                               int *__restrict__ part_v, int *__restrict__ part_mend,
                                                               uint16_t *__restrict__ mem_pt, float *__restrict__ mem_w,
                                                               uint16_t *__restrict__ tl_loc, float *__restrict__ tl_w,
                                                               uint32_t *__restrict__ task, uint32_t *__restrict__ tsched,
                                                               uint32_t *__restrict__ vcount,
                                                               int L, int P, int T, const __grid_constant__ ClearList clr,
                                                               float *V0, float *V1, int MP, DevStatus *st) {
    constexpr int C = TG<D>::C, NW = TG_THREADS / 32;
    constexpr int SEG = C / NW;  // corners per warp segment (a multiple of 32)
    extern __shared__ int tp_smem[];
    int *moff = tp_smem;            // [C] member offset of each partial
    int *toff = moff + C;           // [C] task offset of each partial
    uint16_t *wc = reinterpret_cast<uint16_t *>(toff + C);  // [NW][C] per-warp counts, then bases
    __shared__ int swarp[NW];
    const int t = blockIdx.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const uint32_t pb = tile_pbeg[t], np = tile_pbeg[t + 1] - pb, tb = tile_tbeg[t];
    const size_t base = (size_t)t * C;
    // member and task offsets of the partials (partials split among threads in order)
    const int chunk = ((int)np + TG_THREADS - 1) / TG_THREADS;
    const int p0 = min((int)np, tid * chunk), p1 = min((int)np, p0 + chunk);
    int mloc = 0, tloc = 0;
    for (int p = p0; p < p1; p++) {
        const int c = pcnt[base + p];
        mloc += c;
        tloc += (c + task_len - 1) / task_len;
    }
    int mtot, ttot;
    int mrun = block_exscan256(mloc, swarp, &mtot);
    int trun = block_exscan256(tloc, swarp, &ttot);
    // block 0: the padding after the partial and task tables, and the ranges
    // the reduce-list kernels need cleared (scan state, sentinel rows)
    if (t == 0) {
        if (tid < 8) {
            part_mend[P + tid] = 0;
            task[T + tid] = 0;
            tsched[T + tid] = 0;
        }
        clear_words(clr, (size_t)tid, TG_THREADS);
        zero_value_rows(V0, V1, (size_t)L, MP, tid, TG_THREADS);
    }
    for (int p = p0; p < p1; p++) {
        const int c = pcnt[base + p];
        const int v = pvx[base + p];
        moff[p] = mrun;
        toff[p] = trun;
        part_v[pb + p] = v;
        // partials per vertex (the reduce lists' sizes); an id outside [0, L)
        // is reported, never used as an index
        if (v >= 0 && v < L)
            atomicAdd(vcount + v, 1u);
        else
            dcrf_set_error(st, DCRF_ERR_CUDA, (int)(pb + p));
        part_mend[pb + p] = mrun + c;  // tile-relative end of the partial's members
        for (int q = 0; q < c; q += task_len)
            task[tb + trun++] = ((uint32_t)p << 19) | ((uint32_t)(mrun + q) << 6) | (uint32_t)min(task_len, c - q);
        mrun += c;
    }
    for (int e = tid; e < NW * C; e += TG_THREADS) wc[e] = 0;
    __syncthreads();  // the tile's tasks are written
    // the schedule: task indices by descending length, ties in task order, so
    // that the lane groups of one warp get tasks of similar length
    for (int j = tid; j < ttot; j += TG_THREADS) {
        const uint32_t lj = task[tb + j] & 63u;
        int rank = 0;
        for (int i = 0; i < ttot; i++) {
            const uint32_t li = task[tb + i] & 63u;
            rank += (li > lj || (li == lj && i < j)) ? 1 : 0;
        }
        tsched[tb + rank] = (uint32_t)j;
    }
    // members past the tile's last one, and the corners of empty slots: index 0, weight 0
    for (int e = mtot + tid; e < C; e += TG_THREADS) {
        mem_pt[base + e] = 0;
        mem_w[base + e] = 0.f;
    }
    if (slot_pt[(size_t)t * SPLAT_TILE + tid] < 0)
        for (int r = 0; r <= D; r++) {
            const size_t tl = ((size_t)t * (D + 1) + r) * SPLAT_TILE + tid;
            tl_loc[tl] = 0;
            tl_w[tl] = 0.f;
        }
    __syncthreads();
    // stable member ranks: warps own consecutive corner segments; each warp
    // counts its segment's corners per partial in order, then ranks them
    const int s0 = warp * SEG;
    for (int c0 = s0; c0 < s0 + SEG; c0 += 32) {
        const uint16_t p = cl[base + c0 + lane];
        const unsigned peers = __match_any_sync(0xffffffffu, (unsigned)p);
        if (p != 0xFFFF && (__ffs(peers) - 1) == lane) wc[warp * C + p] += (uint16_t)__popc(peers);
        __syncwarp();
    }
    __syncthreads();
    for (int p = tid; p < (int)np; p += TG_THREADS) {  // per partial: exclusive prefix over the warps
        int acc = 0;
        for (int w = 0; w < NW; w++) {
            const int c = wc[w * C + p];
            wc[w * C + p] = (uint16_t)acc;
            acc += c;
        }
    }
    __syncthreads();
    const unsigned lt = (1u << lane) - 1u;
    for (int c0 = s0; c0 < s0 + SEG; c0 += 32) {
        const int c = c0 + lane;
        const uint16_t p = cl[base + c];
        const unsigned peers = __match_any_sync(0xffffffffu, (unsigned)p);
        if (p != 0xFFFF) {
            const int li = c / (D + 1), r = c - li * (D + 1);
            const int pos = moff[p] + (int)wc[warp * C + p] + __popc(peers & lt);
            const float w = bary[(size_t)r * N + slot_pt[(size_t)t * SPLAT_TILE + li]];
            mem_pt[base + pos] = (uint16_t)li;
            mem_w[base + pos] = w;
            const size_t tl = ((size_t)t * (D + 1) + r) * SPLAT_TILE + li;
            tl_loc[tl] = p;
            tl_w[tl] = w;
        }
        __syncwarp();
        if (p != 0xFFFF && (__ffs(peers) - 1) == lane) wc[warp * C + p] += (uint16_t)__popc(peers);
        __syncwarp();
    }
}


// Reduce lists without a sort.  place: partial p takes a position in its
// vertex's range [red_beg[v], red_beg[v+1]) by counting that vertex's
// remaining count down (positions in arbitrary order); rank: the partial at
// position j moves to the position given by its rank among the range's
// partials -- the number of smaller partial indices, i.e. tile order, since the
// partials are numbered tile by tile -- so every vertex's list comes out in
// tile order, deterministically.  Work per partial is the length of its
// vertex's list (short: a vertex touches few tiles of a 16x16-pixel grid).
__global__ void red_place_kernel(const int *__restrict__ part_v, int P, int L, const int *__restrict__ red_beg,
                                 uint32_t *__restrict__ vcount, int *__restrict__ lst, DevStatus *st) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P) return;
    const int v = part_v[p];
    if (v < 0 || v >= L) return;  // reported by the tile placement
    const uint32_t left = atomicSub(vcount + v, 1u);
    const int pos = red_beg[v] + (int)left - 1;
    if (left == 0 || pos >= red_beg[v + 1]) {
        dcrf_set_error(st, DCRF_ERR_CUDA, p);
        return;
    }
    lst[pos] = p;
}

__global__ void red_rank_kernel(const int *__restrict__ part_v, int P, int L, const int *__restrict__ red_beg,
                                const int *__restrict__ lst, int *__restrict__ red_list, int *__restrict__ ppos) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= P) return;
    const int p = lst[j];
    if (p < 0 || p >= P) return;
    const int v = part_v[p];
    if (v < 0 || v >= L) return;
    const int s0 = red_beg[v], s1 = red_beg[v + 1];
    int rank = 0;
    for (int q = s0; q < s1; q++) rank += __ldg(lst + q) < p ? 1 : 0;
    red_list[s0 + rank] = p;
    ppos[p] = s0 + rank;
}

__global__ void zero_value_rows_kernel(float *V0, float *V1, size_t L, int MP) {
    zero_value_rows(V0, V1, L, MP, threadIdx.x, blockDim.x);
}

cudaError_t launch_lattice_zero_rows(float *V0, float *V1, size_t L, int MP, cudaStream_t s) {
    DCRF_LAUNCH(zero_value_rows_kernel<<<1, 256, 0, s>>>(V0, V1, L, MP));
    return cudaGetLastError();
}

// inv[list[i]] = i for a permutation list of [0, n)
__global__ void invert_kernel(const int *__restrict__ list, int n, int *__restrict__ inv) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) inv[list[i]] = i;
}

// ---------------------------------------------------------------------------
namespace {

// Stream-ordered bump allocation from a few pool blocks.  reserve(b) takes one
// block for the buffers that follow; get() carves 256-byte aligned pieces from
// it and falls back to a block of its own when the reservation is used up (a
// reservation that is too small costs an allocation, never correctness).
struct Arena {
    cudaStream_t s;
    std::vector<void *> blocks;
    char *cur = nullptr;
    size_t left = 0, bytes = 0;
    bool failed = false;
    static size_t rnd(size_t b) { return (std::max<size_t>(b, 16) + 255) & ~(size_t)255; }
    template <class T>
    static size_t sz(size_t n) {
        return rnd(n * sizeof(T));
    }
    void *block(size_t b) {
        void *p = nullptr;
        if (pool_malloc_async(&p, b, s) != cudaSuccess) {
            failed = true;
            return nullptr;
        }
        blocks.push_back(p);
        bytes += b;
        return p;
    }
    void reserve(size_t b) {
        cur = static_cast<char *>(block(b));
        left = cur ? b : 0;
    }
    template <class T>
    T *get(size_t n) {
        const size_t b = rnd(n * sizeof(T));
        if (b > left) return static_cast<T *>(block(b));
        T *p = reinterpret_cast<T *>(cur);
        cur += b;
        left -= b;
        return p;
    }
    void release() {
        for (void *p : blocks) cudaFreeAsync(p, s);
        blocks.clear();
        cur = nullptr;
        left = bytes = 0;
    }
};

// The tile kernels' exact dynamic shared memory, set once per device (the 48 KB
// default leaves no room for their static shared memory at d = 7, where the
// placement kernel's dynamic part is exactly 48 KB).
template <int D>
cudaError_t tile_kernels_optin(size_t smem_g, size_t smem_p) {
    static std::atomic<uint64_t> done{0};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    const uint64_t bit = dev < 64 ? (1ull << dev) : 0;
    if (bit && (done.load() & bit)) return cudaSuccess;
    e = cudaFuncSetAttribute(tile_group_kernel<D>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_g);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(tile_place_kernel<D>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_p);
    if (e == cudaSuccess && bit) done.fetch_or(bit);
    return e;
}

int fail(int code, const std::string &m) {
    g_msg = m;
    return code;
}

// Device counts of a build, read back at its single synchronisation.
enum : int { BI_L = 0, BI_P = 1, BI_T = 2, BI_MAXNP = 3, BI_MAXNT = 4, BI_WORDS = 8 };

template <int D>
int build_d(const float *feat, int N, const Segments &seg, const TileMapDev &tm, int variant, float load,
            int task_len, int MP, int nslots, cudaStream_t s, DevStatus *status, LatticeDev *out) {
    constexpr int KW = KeyW<D>::KW;
    LatticeDev L{};
    L.d = D;
    L.N = N;
    L.variant = variant;
    const int nseg = (int)seg.start.size() - 1;
    if (nseg > 65536) return fail(DCRF_ERR_INVALID_ARG, "at most 65536 images per lattice (16-bit image field)");
    // padding points of the x86 build: each image's N_img rounded up to 4
    std::vector<int> ph_img;
    if (variant == DCRF_VARIANT_SSE)
        for (int b = 0; b < nseg; b++) {
            int nb = seg.start[b + 1] - seg.start[b];
            for (int q = nb; q % 4 != 0; q++) ph_img.push_back(b);
        }
    const int n_ph = (int)ph_img.size();
    // one image: its padding points are image 0 and need no table
    const bool ph_table = n_ph > 0 && nseg > 1;
    const size_t E = (size_t)(N + n_ph) * (D + 1);
    const size_t Ereal = (size_t)N * (D + 1);
    if (E >= 0xFFFFFFF0ull) return fail(DCRF_ERR_INVALID_ARG, "lattice too large (more than 2^32 simplex corners)");

    size_t cap = 1024;
    while ((double)cap < (double)load * (double)E && cap < (1ull << 31)) cap <<= 1;
    const size_t ntl = (size_t)tm.ntiles * (D + 1) * SPLAT_TILE;
    const size_t vid_state = lb_state_words(E), tile_state = lb_state_words((size_t)tm.ntiles);
    // The vertex count L is needed on the host only to size the neighbour and
    // key tables.  When their upper bound (L <= E) is small, they are reserved
    // at that size and the build runs on to its single synchronisation (L comes
    // back with the tile counts); otherwise the host waits for L first.
    const bool learn_L_first = (size_t)10 * E * (D + 1) > ((size_t)256 << 20);
    // temporaries and the lattice's own tables come from one block per build
    // stage (sizes known at the start of each stage)
    Arena tmp{s}, per{s};
    tmp.reserve(Arena::sz<uint64_t>(E * KW) + 2 * Arena::sz<uint32_t>(E) + Arena::sz<uint32_t>(E + 1) +
                Arena::sz<uint32_t>(BI_WORDS) + Arena::sz<int>(n_ph + 1) + Arena::sz<uint32_t>(cap) +
                Arena::sz<unsigned long long>(vid_state) + Arena::sz<unsigned long long>(tile_state) +
                Arena::sz<uint16_t>(ntl) + 2 * Arena::sz<int>(ntl) + 2 * Arena::sz<uint32_t>(tm.ntiles + 1));
    uint64_t *keys = tmp.get<uint64_t>(E * KW);
    uint32_t *slot = tmp.get<uint32_t>(E);
    uint32_t *vid = tmp.get<uint32_t>(E);
    uint32_t *vcount = tmp.get<uint32_t>(E + 1);  // partials per vertex (indexed by vertex id < L <= E)
    uint32_t *info = tmp.get<uint32_t>(BI_WORDS);
    int *d_ph = tmp.get<int>(n_ph + 1);
    uint32_t *table = tmp.get<uint32_t>(cap);
    unsigned long long *st_vid = tmp.get<unsigned long long>(vid_state);
    unsigned long long *st_tile = tmp.get<unsigned long long>(tile_state);
    uint16_t *cl = tmp.get<uint16_t>(ntl);
    int *pvx = tmp.get<int>(ntl);
    int *pcnt = tmp.get<int>(ntl);
    uint32_t *tile_np = tmp.get<uint32_t>(tm.ntiles + 1);
    uint32_t *tile_nt = tmp.get<uint32_t>(tm.ntiles + 1);
    if (tmp.failed) {
        tmp.release();
        return fail(DCRF_ERR_OOM, "device allocation failed in lattice build");
    }
    auto bail = [&](int code, const std::string &m) {
        tmp.release();
        per.release();
        cudaMemsetAsync(status, 0, sizeof(DevStatus), s);  // the reported status is consumed
        return fail(code, m);
    };
    // device status of the build after a synchronisation: 0, or the error to return
    auto status_error = [&](const DevStatus &st) -> int {
        if (st.code == DCRF_ERR_KEY_OVERFLOW)
            return bail(DCRF_ERR_KEY_OVERFLOW,
                        "a lattice coordinate of point " + std::to_string(st.detail) +
                            " leaves the int16 key range of the reference (features too large)");
        if (st.code == DCRF_ERR_HASH_FULL) return bail(DCRF_ERR_HASH_FULL, "lattice hash table full");
        if (st.code != 0) return bail(st.code, "lattice build failed");
        return 0;
    };
    if (ph_table) cudaMemcpyAsync(d_ph, ph_img.data(), sizeof(int) * n_ph, cudaMemcpyHostToDevice, s);

    const size_t Lcap0 = learn_L_first ? 0 : E;  // rows reserved for the neighbour and key tables before L is known
    per.reserve(Arena::sz<int>(Ereal) + 2 * Arena::sz<float>(Ereal) + Arena::sz<uint8_t>(Ereal) +
                Arena::sz<int2>(Lcap0 * (D + 1)) + Arena::sz<uint16_t>(Lcap0 * (D + 1)) +
                2 * Arena::sz<int>(tm.ntiles + 1) + 2 * (Arena::sz<uint16_t>(ntl) + Arena::sz<float>(ntl)));
    L.off = per.get<int>(Ereal);
    L.bary = per.get<float>(Ereal);
    L.wslice = per.get<float>(Ereal);
    L.rank = per.get<uint8_t>(Ereal);
    if (per.failed) return bail(DCRF_ERR_OOM, "device allocation failed (lattice)");

    EmbedArgs ea{};
    ea.feat = feat;
    ea.N = N;
    ea.n_ph = n_ph;
    ea.ph_img = ph_table ? d_ph : nullptr;
    ea.seg_start = seg.dev_start;
    ea.nseg = nseg;
    {
        // float(sqrt(2/3)*(d+1)), scale = float(1/sqrt((i+2)(i+1)) * inv_std_dev)
        float inv_std_dev = (float)(std::sqrt(2.0 / 3.0) * (D + 1));
        for (int i = 0; i < D; i++) ea.sf[i] = (float)(1.0 / std::sqrt((double)((i + 2) * (i + 1))) * (double)inv_std_dev);
    }
    ea.invdp1 = 1.0f / (float)(D + 1);
    ea.dp1 = (float)(D + 1);
    ea.alpha = 1.0f / (1.0f + std::pow(2.0f, (float)-D));
    L.alpha = ea.alpha;
    ea.variant = variant;
    ea.bary = L.bary;
    ea.wslice = L.wslice;
    ea.rank = L.rank;
    ea.keys = keys;
    ea.st = status;
    // cleared by the embed launch, before the kernels that use them
    ea.clr.add(table, cap, EMPTY);
    ea.clr.add(info, BI_WORDS, 0u);
    ea.clr.add(st_vid, 2 * vid_state, 0u);
    ea.clr.add(st_tile, 2 * tile_state, 0u);
    const int npts = N + n_ph;
    DCRF_LAUNCH(embed_kernel<D><<<std::max(1u, ceil_div_u(npts, 128)), 128, 0, s>>>(ea));
    if (E > 0) DCRF_LAUNCH(insert_kernel<KW><<<ceil_div_u(E, 256), 256, 0, s>>>(keys, E, table, (uint32_t)(cap - 1), slot, status));
    {  // vertex ids: first occurrences, numbered in corner order (one launch)
        LBScanArgs sa;
        sa.n = E;
        sa.out[0] = vid;
        sa.total[0][0] = info + BI_L;
        sa.table = table;
        sa.slot = slot;
        sa.state = st_vid;
        sa.st = status;
        if (lb_scan(sa, s) != cudaSuccess) return bail(DCRF_ERR_CUDA, "scan failed");
    }
    uint32_t hinfo[BI_WORDS] = {};
    DevStatus hst{};
    cudaError_t ce = cudaSuccess;
    if (learn_L_first) {
        cudaMemcpyAsync(hinfo, info, sizeof(hinfo), cudaMemcpyDeviceToHost, s);
        cudaMemcpyAsync(&hst, status, sizeof(DevStatus), cudaMemcpyDeviceToHost, s);
        ce = cudaStreamSynchronize(s);
        if (ce != cudaSuccess) return bail(DCRF_ERR_CUDA, std::string("lattice build: ") + cudaGetErrorString(ce));
        if (int rc = status_error(hst)) return rc;
        L.L = (int)hinfo[BI_L];
        per.reserve(Arena::sz<int2>((size_t)L.L * (D + 1)) + Arena::sz<uint16_t>((size_t)L.L * (D + 1)));
    }
    const size_t Lcap = learn_L_first ? (size_t)L.L : E;
    L.nbr = per.get<int2>(Lcap * (D + 1));
    L.vkeys = per.get<uint16_t>(Lcap * (D + 1));
    if (per.failed) return bail(DCRF_ERR_OOM, "device allocation failed (neighbours)");
    if (E > 0)
        DCRF_LAUNCH(offsets_kernel<D><<<ceil_div_u(E, 256), 256, 0, s>>>(keys, table, slot, vid, E, N, L.off, L.vkeys,
                                                                         vcount));
    if (Lcap > 0) {
        const unsigned nb = (unsigned)std::min<size_t>(ceil_div_u(Lcap * (D + 1), 256), 4096);
        DCRF_LAUNCH(neighbors_kernel<D><<<nb, 256, 0, s>>>(keys, table, (uint32_t)(cap - 1), vid, L.vkeys,
                                                            info + BI_L, L.nbr));
    }
    // ---- splat tiles: partials, member lists, slice tables, tasks ----------------
    L.ntiles = tm.ntiles;
    L.tile_pbeg = per.get<int>(L.ntiles + 1);
    L.tile_tbeg = per.get<int>(L.ntiles + 1);
    L.mem_pt = per.get<uint16_t>(ntl);
    L.mem_w = per.get<float>(ntl);
    L.tl_loc = per.get<uint16_t>(ntl);
    L.tl_w = per.get<float>(ntl);
    if (per.failed) return bail(DCRF_ERR_OOM, "device allocation failed (tiles)");
    const size_t smem_g = (2 * (size_t)TG<D>::HT + TG<D>::C) * sizeof(int);
    const size_t smem_p = 2 * (size_t)TG<D>::C * sizeof(int) + (TG_THREADS / 32) * (size_t)TG<D>::C * sizeof(uint16_t);
    if (tile_kernels_optin<D>(smem_g, smem_p) != cudaSuccess)
        return bail(DCRF_ERR_CUDA, "tile kernels: shared-memory opt-in failed");
    if (L.ntiles > 0) {
        DCRF_LAUNCH(tile_group_kernel<D><<<L.ntiles, TG_THREADS, smem_g, s>>>(L.off, N, tm.slot_pt, task_len, cl, pvx,
                                                                             pcnt, tile_np, tile_nt, info + BI_MAXNP,
                                                                             status));
        // a launch that did not start must not leave its outputs to the next kernels
        if ((ce = cudaGetLastError()) != cudaSuccess)
            return bail(DCRF_ERR_CUDA, std::string("tile grouping launch: ") + cudaGetErrorString(ce));
    }
    {  // partial and task ranges of the tiles (one launch, both arrays)
        LBScanArgs sa;
        sa.narr = 2;
        sa.n = (size_t)L.ntiles;
        sa.in[0] = tile_np;
        sa.in[1] = tile_nt;
        sa.out[0] = (uint32_t *)L.tile_pbeg;
        sa.out[1] = (uint32_t *)L.tile_tbeg;
        sa.total[0][0] = (uint32_t *)L.tile_pbeg + L.ntiles;
        sa.total[0][1] = info + BI_P;
        sa.total[1][0] = (uint32_t *)L.tile_tbeg + L.ntiles;
        sa.total[1][1] = info + BI_T;
        sa.state = st_tile;
        sa.st = status;
        if (lb_scan(sa, s) != cudaSuccess) return bail(DCRF_ERR_CUDA, "scan failed");
    }
    cudaMemcpyAsync(hinfo, info, sizeof(hinfo), cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(&hst, status, sizeof(DevStatus), cudaMemcpyDeviceToHost, s);
    ce = cudaStreamSynchronize(s);
    if (ce != cudaSuccess) return bail(DCRF_ERR_CUDA, std::string("lattice tiles: ") + cudaGetErrorString(ce));
    if (int rc = status_error(hst)) return rc;
    L.L = (int)hinfo[BI_L];
    L.P = (int)hinfo[BI_P];
    const int T = (int)hinfo[BI_T];
    L.max_np = (int)hinfo[BI_MAXNP];
    L.max_nt = (int)hinfo[BI_MAXNT];
    // ---- partial tables, reduce lists and the value buffers --------------------
    const size_t Pn = (size_t)L.P + 1, Ln = (size_t)L.L + 1;
    const size_t red_state = lb_state_words(Ln - 1);
    // a vertex shared by very many tiles on average makes the rank counting
    // quadratic in its list length: such lattices take the radix sort
    const bool radix = (size_t)L.P > 64 * std::max<size_t>(1, (size_t)L.L);
    const size_t radix_words = radix ? radix_temp_words((size_t)L.P) : 0;
    per.reserve(3 * Arena::sz<int>(Pn) + Arena::sz<int>((size_t)L.P + 8) + Arena::sz<int>(Ln) +
                2 * Arena::sz<uint32_t>((size_t)T + 8) + 2 * Arena::sz<float>(Ln * MP) + 2 * Arena::sz<float>(Pn * MP) +
                Arena::sz<float>((size_t)nslots) + Arena::sz<float>(ntl));
    L.part_v = per.get<int>(Pn);
    L.red_beg = per.get<int>(Ln);
    L.red_list = per.get<int>(Pn);
    L.ppos = per.get<int>(Pn);
    L.part_mend = per.get<int>((size_t)L.P + 8);
    L.task = per.get<uint32_t>((size_t)T + 8);
    L.tsched = per.get<uint32_t>((size_t)T + 8);
    L.V0 = per.get<float>(Ln * MP);
    L.V1 = per.get<float>(Ln * MP);
    L.pv = per.get<float>(Pn * MP);
    L.pout = per.get<float>(Pn * MP);
    L.norm = per.get<float>((size_t)nslots);
    L.mem_wn = per.get<float>(ntl);
    if (per.failed) return bail(DCRF_ERR_OOM, "device allocation failed (partials)");
    Arena red{s};
    red.reserve(Arena::sz<unsigned long long>(red_state) + Arena::sz<int>(Pn) +
                (radix ? 4 * Arena::sz<uint32_t>(Pn) + Arena::sz<uint32_t>(radix_words) : 0));
    unsigned long long *st_red = red.get<unsigned long long>(red_state);
    int *lst = red.get<int>(Pn);
    if (red.failed) {
        red.release();
        return bail(DCRF_ERR_OOM, "device allocation failed (reduce lists)");
    }
    if (L.ntiles > 0) {
        // also cleared there: the reduce-list scan's state, and the sentinel rows
        // of both value buffers
        ClearList clr;
        clr.add(st_red, 2 * red_state, 0u);
        DCRF_LAUNCH(tile_place_kernel<D><<<L.ntiles, TG_THREADS, smem_p, s>>>(
            cl, pvx, pcnt, L.bary, N, tm.slot_pt, (const uint32_t *)L.tile_pbeg, (const uint32_t *)L.tile_tbeg,
            task_len, L.part_v, L.part_mend, L.mem_pt, L.mem_w, L.tl_loc, L.tl_w, L.task, L.tsched, vcount, L.L, L.P,
            T, clr,
            L.V0, L.V1, MP, status));
        if ((ce = cudaGetLastError()) != cudaSuccess) {
            red.release();
            return bail(DCRF_ERR_CUDA, std::string("tile placement launch: ") + cudaGetErrorString(ce));
        }
    }
    {  // red_beg = exclusive scan of the partials per vertex; red_beg[L] = P
        LBScanArgs sa;
        sa.n = (size_t)L.L;
        sa.in[0] = vcount;
        sa.out[0] = (uint32_t *)L.red_beg;
        sa.total[0][0] = (uint32_t *)L.red_beg + L.L;
        sa.state = st_red;
        sa.st = status;
        if (L.ntiles > 0 && lb_scan(sa, s) != cudaSuccess) {
            red.release();
            return bail(DCRF_ERR_CUDA, "scan failed");
        }
    }
    if (L.P > 0) {
        if (!radix) {
            DCRF_LAUNCH(red_place_kernel<<<ceil_div_u(L.P, 256), 256, 0, s>>>(L.part_v, L.P, L.L, L.red_beg, vcount,
                                                                              lst, status));
            DCRF_LAUNCH(red_rank_kernel<<<ceil_div_u(L.P, 256), 256, 0, s>>>(L.part_v, L.P, L.L, L.red_beg, lst,
                                                                             L.red_list, L.ppos));
        } else {
            uint32_t *k0 = red.get<uint32_t>(Pn), *v0 = red.get<uint32_t>(Pn);
            uint32_t *k1 = red.get<uint32_t>(Pn), *v1 = red.get<uint32_t>(Pn);
            uint32_t *rtemp = red.get<uint32_t>(radix_words);
            int bits = 1;
            while (bits < 32 && ((uint64_t)1 << bits) <= (uint64_t)L.L) bits++;
            if (red.failed || radix_argsort_u32((const uint32_t *)L.part_v, (size_t)L.P, bits, (uint32_t *)L.red_list,
                                                k0, v0, k1, v1, rtemp, s) != cudaSuccess) {
                red.release();
                return bail(DCRF_ERR_CUDA, "radix sort failed");
            }
            DCRF_LAUNCH(invert_kernel<<<ceil_div_u(L.P, 256), 256, 0, s>>>(L.red_list, L.P, L.ppos));
        }
    }
    // no synchronisation here: the temporaries go back to the pool in stream
    // order, and the caller checks the device status block (the placement's
    // consistency checks included) at its next synchronisation
    red.release();
    tmp.release();
    ce = cudaGetLastError();
    if (ce != cudaSuccess) {
        per.release();
        return fail(DCRF_ERR_CUDA, std::string("lattice build launch: ") + cudaGetErrorString(ce));
    }
    L.bytes = per.bytes;
    L.blocks = per.blocks;
    *out = L;
    return DCRF_OK;
}

}  // namespace

void lattice_free(LatticeDev *L, cudaStream_t s) {
    for (void *p : L->blocks) cudaFreeAsync(p, s);
    *L = LatticeDev{};
}

int lattice_build(const float *feat, int d, int N, const Segments &seg, const TileMapDev &tm, int variant, float load,
                  int task_len, int MP, int nslots, cudaStream_t s, DevStatus *status, LatticeDev *out) {
    if (task_len < 1 || task_len > 63) return fail(DCRF_ERR_INVALID_ARG, "splat task length must be in [1, 63]");
    if (N < 0 || seg.start.size() < 2 || !seg.dev_start) return fail(DCRF_ERR_INVALID_ARG, "bad point segmentation");
    if (MP < 1 || nslots < 0) return fail(DCRF_ERR_INVALID_ARG, "bad value-buffer sizes");
    switch (d) {
#define DCRF_CASE(D) \
    case D:          \
        return build_d<D>(feat, N, seg, tm, variant, load, task_len, MP, nslots, s, status, out);
        DCRF_CASE(1) DCRF_CASE(2) DCRF_CASE(3) DCRF_CASE(4) DCRF_CASE(5) DCRF_CASE(6) DCRF_CASE(7) DCRF_CASE(8)
        DCRF_CASE(9) DCRF_CASE(10) DCRF_CASE(11) DCRF_CASE(12) DCRF_CASE(13) DCRF_CASE(14) DCRF_CASE(15)
        DCRF_CASE(16)
#undef DCRF_CASE
        default:
            return fail(DCRF_ERR_INVALID_ARG, "feature dimension must be in [1, 16], got " + std::to_string(d));
    }
}

}  // namespace dcrf
