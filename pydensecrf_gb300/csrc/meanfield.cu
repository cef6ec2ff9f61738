// meanfield.cu -- the kernels of one mean-field iteration on the device.
//
// One iteration of DenseCRF::inference (pydensecrf/densecrf/src/densecrf.cpp:
// 122-129) for all pairwise terms at once is three phases:
//
//   reduce  per vertex: sum its per-tile splat partials (which the splat
//           wrote as one contiguous run of rows per vertex) into V[v] -- the
//           end of the splat of Permutohedral::compute (permutohedral.cpp:
//           545-553);
//   blur    per axis j = 0..d (d..0 for the transpose): V' = V + 1/2 (V[n1] +
//           V[n2]) with the zero sentinel row (permutohedral.cpp:556-569), two
//           axes per launch; terms of smaller d drop out of the later
//           launches.  The last axis also scatters every vertex's value to the
//           partials that reference it (tile-partial order), so each tile's
//           inputs of the next phase are one contiguous block;
//   point   one CTA per tile of 256 points (a 16x16 pixel block of a
//           DenseCRF2D): an elected thread prefetches the tile's tables and
//           blurred values with cp.async.bulk (TMA bulk copies) behind one
//           mbarrier while every thread loads its unary; then per point:
//           slice every term (permutohedral.cpp:574-584), normalise
//           (pairwise.cpp:78-79), label compatibility
//           (labelcompatibility.cpp:46-48,66-68,82-84), subtract from -U,
//           softmax (densecrf.cpp:98-106); then, in the same CTA, splat the
//           tile's new Q into each term's per-(tile, vertex) partials from
//           shared memory.  Q never makes a round trip through memory between
//           iterations.
//
// Deterministic: a tile's corners are grouped by vertex at lattice-build time
// (point order), every partial is a fixed-order sum, and the reduce adds a
// vertex's partials in an order fixed by its own list; no float atomics.  Products and sums are
// rounded separately like the reference's x86 build; the value-size <= 2
// arithmetic of seqCompute (double blur, (w*v)*alpha slice) is kept where the
// reference uses it.
#include <math.h>

#include <algorithm>
#include <atomic>

#include "meanfield.cuh"
#include "pointpass.cuh"
#include "labelprod.cuh"

namespace dcrf {

// ---------------------------------------------------------------------------
// More than 32 labels: the update chunk by chunk (a thread per point)
// ---------------------------------------------------------------------------
constexpr int WC = DCRF_LCHUNK;

// acc = slice of term T's blurred partial rows (chunk c, w labels) at the
// point of slot li of tile t (permutohedral.cpp:574-584 / 513-521)
__device__ __forceinline__ void wide_slice(const TermDev &T, long long pv_chunk, int t, int li, int c, int w,
                                           float (&acc)[WC]) {
#pragma unroll
    for (int e = 0; e < WC; e++) acc[e] = 0.f;
    const int pb = T.tile_pbeg[t];
    const size_t tb = (size_t)t * SPLAT_TILE * (T.d + 1);
    const float *pv = T.pv + pv_chunk * c;
    for (int r = 0; r <= T.d; r++) {
        const int loc = T.tl_loc[tb + (size_t)r * SPLAT_TILE + li];
        const float bw = T.tl_w[tb + (size_t)r * SPLAT_TILE + li];
        const float *row = pv + (size_t)(pb + loc) * w;
        const float wa = fmul(bw, T.alpha);
#pragma unroll
        for (int q = 0; q < WC / 4; q++) {
            if (4 * q >= w) break;
            const float4 v4 = __ldg(reinterpret_cast<const float4 *>(row) + q);
            const float v[4] = {v4.x, v4.y, v4.z, v4.w};
#pragma unroll
            for (int u = 0; u < 4; u++) {
                const int e = 4 * q + u;
                if (T.seq)  // (w * v) * alpha (permutohedral.cpp:520)
                    acc[e] = fmaf(fmul(bw, v[u]), T.alpha, acc[e]);
                else  // (w * alpha) * v (permutohedral.cpp:579-581)
                    acc[e] = fmaf(wa, v[u], acc[e]);
            }
        }
    }
}

__device__ __forceinline__ void wide_load(const float *row, int w, float (&x)[WC]) {
#pragma unroll
    for (int q = 0; q < WC / 4; q++) {
        if (4 * q >= w) break;
        const float4 v4 = *reinterpret_cast<const float4 *>(row + 4 * q);
        x[4 * q] = v4.x, x[4 * q + 1] = v4.y, x[4 * q + 2] = v4.z, x[4 * q + 3] = v4.w;
    }
}

__device__ __forceinline__ void wide_store(float *row, int w, const float (&x)[WC]) {
#pragma unroll
    for (int q = 0; q < WC / 4; q++) {
        if (4 * q >= w) break;
        *reinterpret_cast<float4 *>(row + 4 * q) = make_float4(x[4 * q], x[4 * q + 1], x[4 * q + 2], x[4 * q + 3]);
    }
}

// One CTA per tile, one thread per point.  The operations and their order
// are those of the point pass: per chunk, x = -U (or the given marginals),
// then per term in order x -= compatibility(post-normalised slice) -- a
// Matrix sums over all labels in label order from the term's sliced rows,
// stored first -- then the softmax over all chunks (maximum, exponentials
// summed in label order, one reciprocal) (densecrf.cpp:98-129).
__global__ void __launch_bounds__(SPLAT_TILE) wide_kernel(const __grid_constant__ WideArgs a) {
    __shared__ double sKL[SPLAT_TILE / 32];
    const int t = blockIdx.x, li = threadIdx.x, lane = li & 31, warp = li >> 5;
    const size_t s = (size_t)t * SPLAT_TILE + li;
    const int i = a.slot_pt[s];
    const int M = a.M, MP = a.MP, ns = a.nslots, mode = a.mode;
    const int nc = (MP + WC - 1) / WC;
    const bool kl_mode = (mode & WP_KL) != 0;
    const bool en_mode = (mode & WP_ENERGY) != 0;
    // the point's label and its pairwise energy (densecrf.cpp:160-177)
    const int lab = (en_mode && i >= 0) ? (int)a.labels[i] : -1;
    float energy = 0.f;
    double kl = 0.0;
    if (i >= 0) {
        if (mode & WP_MSG) {  // Matrix terms: every chunk of their post-normalised slice first
            int j = 0;
            for (int k = 0; k < a.ts.n; k++) {
                const TermDev &T = a.ts.t[k];
                if (T.ckind != DCRF_COMPAT_MATRIX) continue;
                float *Fj = a.F + (size_t)j * ns * MP;
                for (int c = 0; c < nc; c++) {
                    const int w = min(WC, MP - WC * c);
                    float acc[WC];
                    wide_slice(T, a.pv_chunk[k], t, li, c, w, acc);
                    if (T.post_norm) {
                        const float nn = T.norm[s];
#pragma unroll
                        for (int e = 0; e < WC; e++) acc[e] = fmul(acc[e], nn);
                    }
                    wide_store(Fj + (size_t)WC * c * ns + s * w, w, acc);
                }
                j++;
            }
        }
        float mx = -INFINITY;
        for (int c = 0; c < nc; c++) {
            const int w = min(WC, MP - WC * c), m0 = WC * c;
            const size_t ro = (size_t)WC * c * ns + s * w;
            float x[WC];
#pragma unroll
            for (int e = 0; e < WC; e++) x[e] = 0.f;
            if (mode & WP_LOAD_Q) {
                wide_load(a.Qin + ro, w, x);
            } else if (a.U) {
                wide_load(a.U + ro, w, x);
#pragma unroll
                for (int e = 0; e < WC; e++) x[e] = -x[e];
            }
            if (mode & WP_MSG) {
                int j = 0;
                for (int k = 0; k < a.ts.n; k++) {
                    const TermDev &T = a.ts.t[k];
                    float cc[WC];
                    if (T.ckind == DCRF_COMPAT_MATRIX) {
                        const float *Fj = a.F + (size_t)j * ns * MP;
#pragma unroll
                        for (int e = 0; e < WC; e++) cc[e] = 0.f;
                        for (int kk = 0; kk < M; kk++) {
                            const float f = Fj[chunk_offset((size_t)ns, MP, s, kk)];
#pragma unroll
                            for (int e = 0; e < WC; e++)
                                if (e < w && m0 + e < M) cc[e] = fmaf(__ldg(T.compat + (size_t)(m0 + e) * M + kk), f, cc[e]);
                        }
                        j++;
                    } else {
                        float acc[WC];
                        wide_slice(T, a.pv_chunk[k], t, li, c, w, acc);
                        if (T.post_norm) {
                            const float nn = T.norm[s];
#pragma unroll
                            for (int e = 0; e < WC; e++) acc[e] = fmul(acc[e], nn);
                        }
                        if (T.ckind == DCRF_COMPAT_POTTS) {
                            const float nw = -T.potts_w;
#pragma unroll
                            for (int e = 0; e < WC; e++) cc[e] = fmul(nw, acc[e]);
                        } else {
#pragma unroll
                            for (int e = 0; e < WC; e++) cc[e] = (e < w && m0 + e < M) ? fmul(__ldg(T.compat + m0 + e), acc[e]) : 0.f;
                        }
                    }
#pragma unroll
                    for (int e = 0; e < WC; e++) {
                        if (e >= w || m0 + e >= M) continue;
                        if (kl_mode)
                            kl += (double)fmul(x[e], cc[e]);
                        else
                            x[e] = fsub(x[e], cc[e]);
                        // r += -0.5 * tmp(l, i) per term, in term order (densecrf.cpp:172-174)
                        if (en_mode && m0 + e == lab && lab < M) energy = fadd(energy, fmul(-0.5f, cc[e]));
                    }
                }
            }
            if (en_mode) continue;  // no softmax: only the energy is wanted
            if (kl_mode) {  // entropy and unary parts (densecrf.cpp:216-226)
                float u[WC];
#pragma unroll
                for (int e = 0; e < WC; e++) u[e] = 0.f;
                if (a.U) wide_load(a.U + ro, w, u);
#pragma unroll
                for (int e = 0; e < WC; e++)
                    if (e < w && m0 + e < M) {
                        kl += (double)x[e] * log((double)fmaxf(x[e], 1e-20f));
                        kl += (double)fmul(u[e], x[e]);
                    }
            } else {
#pragma unroll
                for (int e = 0; e < WC; e++) {
                    if (m0 + e >= M) x[e] = -INFINITY;
                    mx = fmaxf(mx, x[e]);
                }
                wide_store(a.Qout + ro, w, x);  // the logits, until the softmax below
            }
        }
        if (!kl_mode && (mode & (WP_WRITE_Q | WP_MAP))) {
            float sum = 0.f;
            for (int c = 0; c < nc; c++) {
                const int w = min(WC, MP - WC * c);
                float *row = a.Qout + (size_t)WC * c * ns + s * w;
                float x[WC];
                wide_load(row, w, x);
#pragma unroll
                for (int e = 0; e < WC; e++) {
                    if (e >= w) break;
                    x[e] = __expf(fsub(x[e], mx));
                    sum = fadd(sum, x[e]);
                }
                wide_store(row, w, x);
            }
            const float rs = __frcp_rn(sum);
            int best = 0;
            float bv = -1.f;
            for (int c = 0; c < nc; c++) {
                const int w = min(WC, MP - WC * c), m0 = WC * c;
                float *row = a.Qout + (size_t)WC * c * ns + s * w;
                float x[WC];
                wide_load(row, w, x);
#pragma unroll
                for (int e = 0; e < WC; e++) {
                    x[e] = fmul(x[e], rs);
                    if (e < w && m0 + e < M && x[e] > bv) {  // first maximum (densecrf.cpp:132-137)
                        bv = x[e];
                        best = m0 + e;
                    }
                }
                if (mode & WP_WRITE_Q) wide_store(row, w, x);
            }
            if (mode & WP_MAP) a.map_out[i] = (int16_t)best;
        }
        if (en_mode) a.energy[i] = energy;
    }
    if (kl_mode) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) kl += __shfl_down_sync(0xffffffffu, kl, o);
        if (lane == 0) sKL[warp] = kl;
        __syncthreads();
        if (li == 0) {
            double ssum = 0.0;
            for (int w = 0; w < SPLAT_TILE / 32; w++) ssum += sKL[w];
            a.kl_part[t] = ssum;
        }
    }
}

cudaError_t launch_wide(const WideArgs &a, cudaStream_t s) {
    if (a.ntiles <= 0) return cudaSuccess;
    DCRF_LAUNCH(wide_kernel<<<a.ntiles, SPLAT_TILE, 0, s>>>(a));
    return cudaGetLastError();
}

// The reference evaluates the norms in double and rounds to float
// (pairwise.cpp:54-61: 1.0 / sqrt(n + 1e-20), 1.0 / (n + 1e-20) with n float);
// double arithmetic is slow on this GPU, so they are evaluated in float here.
// For n > 1e-4 (a lattice norm includes the point's own weight, so it is far
// larger), n + 1e-20 is n in double.  1/n: float division rounds the exact
// quotient once, as the double route does.  1/sqrt(n): the square root and
// its reciprocal are carried as float pairs (hi + lo, the low parts from exact
// fused multiply-add residuals) and rounded once; over 6 M random n this gave
// the double route's float in all cases but one, which was 1 ulp away.
__device__ __forceinline__ float norm_symmetric(float n) {
    if (!(n > 1e-4f)) return __double2float_rn(__ddiv_rn(1.0, __dsqrt_rn(__dadd_rn((double)n, 1e-20))));
    const float sh = __fsqrt_rn(n);
    const float sl = __fdiv_rn(fmaf(-sh, sh, n), fmul(2.f, sh));  // sqrt(n) = sh + sl
    const float r = __frcp_rn(sh);
    const float t = fmaf(-r, sh, 1.f);                           // 1 - r sh, exact
    return fadd(r, fmul(r, fsub(t, fmul(r, sl))));               // 1 / (sh + sl)
}

__device__ __forceinline__ float norm_one_sided(float n) {
    if (!(n > 1e-4f)) return __double2float_rn(__ddiv_rn(1.0, __dadd_rn((double)n, 1e-20)));
    return __fdiv_rn(1.f, n);
}

// Value-size-1 normalisation slice and raw lattice filter (point-order gather
// from the vertex-order blurred values; used off the iteration loop).
template <int MP>
__global__ void __launch_bounds__(256) slice_kernel(const __grid_constant__ PPArgs a) {
    __shared__ __align__(16) float sCT[(MP % 4 == 0) ? MP * MP : 4];
    const bool stage = a.Gacc && a.ts.t[0].ckind == DCRF_COMPAT_MATRIX && MP % 4 == 0;
    if (stage) {  // the adjoint epilogue's Matrix, [k][MP] (its transpose equals it)
        for (int e = threadIdx.x; e < MP * MP; e += blockDim.x) {
            const int k = e / MP, m = e - k * MP;
            sCT[e] = (k < a.M && m < a.M) ? a.ts.t[0].compat[(size_t)m * a.M + k] : 0.f;
        }
        __syncthreads();
    }
    const size_t s = (size_t)blockIdx.x * SPLAT_TILE + threadIdx.x;
    const int i = a.slot_pt[s];
    const int N = a.N, M = a.M;
    if (a.mode & PP_NORM) {
        // value size 1, seqCompute slice: out += (w * v) * alpha (permutohedral.cpp:513-521);
        // then, per term that folds its norm into the splat, the tile's member
        // weights times their point's norm (from this tile's norms in shared memory)
        __shared__ float sNorm[SPLAT_TILE];
        for (int k = 0; k < a.ts.n; k++) {
            const TermDev &T = a.ts.t[k];
            float out = 0.f;
            if (i >= 0) {
                float n = 0.f;
                for (int r = 0; r <= T.d; r++) {
                    int o = T.off[(size_t)r * N + i] + 1;
                    float w = T.bary[(size_t)r * N + i];
                    n = fadd(n, fmul(fmul(w, __ldg(T.V + o)), T.alpha));
                }
                if (a.ntype[k] == DCRF_NORMALIZE_SYMMETRIC)  // pairwise.cpp:54-57
                    out = norm_symmetric(n);
                else if (a.ntype[k] == DCRF_NO_NORMALIZATION)
                    out = n;  // raw K*1; the host derives the mean (pairwise.cpp:46-53)
                else  // pairwise.cpp:58-61
                    out = norm_one_sided(n);
            }
            a.norm_out[k][s] = out;
            if (a.wn_out[k]) {  // the block's threads are its tile's slots
                sNorm[threadIdx.x] = out;
                __syncthreads();
                const size_t base = (size_t)blockIdx.x * SPLAT_TILE * (T.d + 1);
                for (int e = threadIdx.x; e < SPLAT_TILE * (T.d + 1); e += blockDim.x)
                    a.wn_out[k][base + e] = fmul(T.mem_w[base + e], sNorm[T.mem_pt[base + e]]);
                __syncthreads();
            }
        }
        return;
    }
    if (i < 0) return;
    // PP_FILTER: raw K v of term 0
    const TermDev &T = a.ts.t[0];
    float acc[MP];
#pragma unroll
    for (int m = 0; m < MP; m++) acc[m] = 0.f;
    for (int r = 0; r <= T.d; r++) {
        const int o = T.off[(size_t)r * N + i] + 1;
        float v[MP];
        load_row<MP>(T.V + (size_t)o * MP, v);
        if (T.seq) {
            const float w = T.bary[(size_t)r * N + i];
#pragma unroll
            for (int m = 0; m < MP; m++) acc[m] = fadd(acc[m], fmul(fmul(w, v[m]), T.alpha));
        } else {
            const float w = T.wslice[(size_t)r * N + i];
#pragma unroll
            for (int m = 0; m < MP; m++) acc[m] = fadd(acc[m], fmul(w, v[m]));
        }
    }
#pragma unroll
    for (int m = 0; m < MP; m++)
        if (m >= M) acc[m] = 0.f;
    if (a.Qout) store_row<MP>(a.Qout + s * MP, acc);
    if (!a.Fpost && !a.Gacc) return;
    if (T.post_norm) {
        const float nn = T.norm[s];
#pragma unroll
        for (int m = 0; m < MP; m++) acc[m] = fmul(acc[m], nn);
    }
    if (a.Fpost) store_row<MP>(a.Fpost + s * MP, acc);
    if (a.Gacc) {  // Gacc += compat(F'); the compatibilities are symmetric (W = (m + m^T) / 2)
        float gv[MP];
        load_row<MP>(a.Gacc + s * MP, gv);
        double unused = 0.0;
        float neg[MP];
#pragma unroll
        for (int m = 0; m < MP; m++) neg[m] = -gv[m];
        fold_compat<MP>(T, stage ? sCT : nullptr, acc, neg, M, false, unused);  // neg -= compat(F')
#pragma unroll
        for (int m = 0; m < MP; m++) gv[m] = m < M ? -neg[m] : 0.f;
        store_row<MP>(a.Gacc + s * MP, gv);
    }
}

// See AdjArgs.  Dynamic shared memory: the tile's Q_t rows and F' rows
// (SPLAT_TILE x MP each), the products' group sums, and every Matrix term's
// compatibility as [k][MP].
// Floats of the products' group sums, rounded up to 16 bytes: the Matrix
// compatibilities after them are read as float4 rows.
__host__ __device__ inline int adj_group_words(int M) {
    const int w0 = block_label_products_words(M, 0), w1 = block_label_products_words(M, 1);
    return ((w0 > w1 ? w0 : w1) + 3) & ~3;
}

template <int MP>
// (three CTAs per SM at 16 labels or more, where each thread holds long rows;
// measured: the same bound at 4 labels made the 96^3 volumes' backward 20 % slower)
__global__ void __launch_bounds__(SPLAT_TILE, MP >= 16 ? 3 : 1) adjoint_tile_kernel(const __grid_constant__ AdjArgs a) {
    extern __shared__ __align__(16) float adj_smem[];
    float *sQ = adj_smem, *sF = sQ + SPLAT_TILE * MP, *sG = sF + SPLAT_TILE * MP;
    float *sCT = sG + adj_group_words(a.M);
    const int M = a.M;
    {  // Matrix compatibilities, transposed into [k][MP] (zero padded); symmetric, so equal
        int j = 0;
        for (int k = 0; k < a.ts.n; k++) {
            const TermDev &T = a.ts.t[k];
            if (T.ckind != DCRF_COMPAT_MATRIX) continue;
            for (int e = threadIdx.x; e < MP * MP; e += blockDim.x) {
                const int kk = e / MP, m = e - kk * MP;
                sCT[j * MP * MP + e] = (kk < M && m < M) ? T.compat[(size_t)m * M + kk] : 0.f;
            }
            j++;
        }
    }
    const size_t s = (size_t)blockIdx.x * SPLAT_TILE + threadIdx.x;
    const int i = a.slot_pt[s];
    const bool ok = i >= 0;
    {  // Q_t's row goes to shared memory (the products read it; the softmax adjoint re-reads it)
        float q[MP];
        if (ok)
            load_row<MP>(a.Qt + s * MP, q);
        else
#pragma unroll
            for (int m = 0; m < MP; m++) q[m] = 0.f;
        store_row<MP>(sQ + threadIdx.x * MP, q);
    }
    float x[MP];  // -g: x -= C F' per term
#pragma unroll
    for (int m = 0; m < MP; m++) x[m] = 0.f;
    __syncthreads();
    int jm = 0;
    constexpr int VW = MP % 4 == 0 ? 4 : 1;
    for (int k = 0; k < a.ts.n; k++) {
        const TermDev &T = a.ts.t[k];
        const AdjArgs::T &A = a.a[k];
        float acc[MP];
#pragma unroll
        for (int m = 0; m < MP; m++) acc[m] = 0.f;
        if (ok) {
            // the point-order gather from A (vertex order), each row streamed in vectors
            for (int r = 0; r <= T.d; r++) {
                const float *row = A.A + (size_t)(T.off[(size_t)r * a.N + i] + 1) * MP;
                const float w = T.seq ? T.bary[(size_t)r * a.N + i] : T.wslice[(size_t)r * a.N + i];
#pragma unroll
                for (int c = 0; c < MP / VW; c++) {
                    float v[VW];
                    vload_g<VW>(row + c * VW, v);
#pragma unroll
                    for (int e = 0; e < VW; e++) {
                        const int m = c * VW + e;
                        if (T.seq)  // (w * v) * alpha, then the sum (permutohedral.cpp:513-521)
                            acc[m] = fadd(acc[m], fmul(fmul(w, v[e]), T.alpha));
                        else  // (w * alpha) * v (permutohedral.cpp:579-581)
                            acc[m] = fadd(acc[m], fmul(w, v[e]));
                    }
                }
            }
#pragma unroll
            for (int m = 0; m < MP; m++)
                if (m >= M) acc[m] = 0.f;
            if (A.Fraw) store_row<MP>(A.Fraw + s * MP, acc);
            if (A.post) {
                const float nn = T.norm[s];
#pragma unroll
                for (int m = 0; m < MP; m++) acc[m] = fmul(acc[m], nn);
            }
            double unused = 0.0;
            const bool mat = T.ckind == DCRF_COMPAT_MATRIX && MP % 4 == 0;
            fold_compat<MP>(T, mat ? sCT + jm * MP * MP : nullptr, acc, x, M, false, unused);
        }
        if (T.ckind == DCRF_COMPAT_MATRIX) jm++;
        if (A.lp) {  // sum over the tile of F' (x) Q_t (labelcompatibility.cpp:57-61,76-78,101-107)
            store_row<MP>(sF + threadIdx.x * MP, acc);
            __syncthreads();
            const int K = A.lp_mode == 0 ? M : M * M;
            block_label_products(sF, sQ, SPLAT_TILE, MP, M, A.lp_mode, sG, A.lp + (size_t)blockIdx.x * K, a.lp_accum);
        }
    }
    if (!ok) return;
    // b_next = softmax adjoint of g = -x at Q_t (densecrf.cpp:107-114, 290)
    float q[MP];
    load_row_s<MP>(sQ + threadIdx.x * MP, q);
    float dot = 0.f;
#pragma unroll
    for (int m = 0; m < MP; m++)
        if (m < M) dot = fmaf(-x[m], q[m], dot);
    float o[MP];
#pragma unroll
    for (int m = 0; m < MP; m++) o[m] = m < M ? fmaf(q[m], dot, x[m] * q[m]) : 0.f;
    store_row<MP>(a.b_next + s * MP, o);
    if (a.du) {
        float u[MP];
        load_row<MP>(a.du + s * MP, u);
#pragma unroll
        for (int m = 0; m < MP; m++) u[m] += o[m];
        store_row<MP>(a.du + s * MP, u);
    }
}

template <int MP>
static cudaError_t adj_launch(const AdjArgs &a, cudaStream_t s) {
    int nmat = 0;
    for (int k = 0; k < a.ts.n; k++) nmat += a.ts.t[k].ckind == DCRF_COMPAT_MATRIX ? 1 : 0;
    const size_t words = 2 * (size_t)SPLAT_TILE * MP + adj_group_words(a.M) + (size_t)nmat * MP * MP;
    const size_t smem = words * sizeof(float);
    static std::atomic<uint64_t> opted{0};
    int dev = 0;
    cudaGetDevice(&dev);
    const uint64_t bit = dev < 64 ? 1ull << dev : 0;
    if (smem > 48 * 1024 && !(opted.load() & bit)) {
        cudaError_t e = cudaFuncSetAttribute(adjoint_tile_kernel<MP>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             POINTPASS_SMEM_MAX);
        if (e != cudaSuccess) return e;
        opted.fetch_or(bit);
    }
    if (smem > (size_t)POINTPASS_SMEM_MAX) return cudaErrorInvalidValue;
    DCRF_LAUNCH(adjoint_tile_kernel<MP><<<a.ntiles, SPLAT_TILE, smem, s>>>(a));
    return cudaGetLastError();
}

cudaError_t launch_adjoint_tile(const AdjArgs &a, int MP, cudaStream_t s) {
    if (a.ntiles <= 0) return cudaSuccess;
    switch (MP) {
        case 4: return adj_launch<4>(a, s);
        case 8: return adj_launch<8>(a, s);
        case 12: return adj_launch<12>(a, s);
        case 16: return adj_launch<16>(a, s);
        case 20: return adj_launch<20>(a, s);
        case 24: return adj_launch<24>(a, s);
        case 28: return adj_launch<28>(a, s);
        case 32: return adj_launch<32>(a, s);
        default: return cudaErrorInvalidValue;
    }
}

// Sum of each vertex's tile partials, which the splat wrote as one contiguous
// run of rows per vertex (in tile order).  A vertex gets G lanes per row (CH
// labels each) times R row slots; slot r sums rows r*G..r*G+G-1 of every batch
// of G*R rows in order (independent loads), and the slots' sums combine in a
// fixed pairwise tree, so the result depends only on the vertex's own rows.
// Terms whose vertices average many partials (large spatial bandwidths) take
// R = 32/G to shorten their longest chains.
template <int MP>
__global__ void __launch_bounds__(256) reduce_kernel(const __grid_constant__ ReduceArgs a) {
    constexpr int G = Grp<MP>::G, CH = Grp<MP>::CH;
    pdl_trigger();
    const long long gt = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (gt >= a.begin[a.n]) return;
    int k = 0;
    while (gt >= a.begin[k + 1]) k++;
    const ReduceArgs::T &T = a.t[k];
    const int GR = G * a.rs[k];
    const long long loc = gt - a.begin[k];
    const int v = (int)(loc / GR);
    if (v >= T.L) return;  // the whole group: groups never straddle terms or warps
    const int l = (int)(loc - (long long)v * GR);
    const int lgi = l % G, r0 = l - lgi;  // r0 = slot * G
    const unsigned lane = threadIdx.x & 31u;
    const unsigned gmask = GR == 32 ? 0xffffffffu : (((1u << GR) - 1u) << (lane & ~(unsigned)(GR - 1)));
    const int s0 = T.red_beg[v], s1 = T.red_beg[v + 1];
    float acc[CH];
#pragma unroll
    for (int c = 0; c < CH; c++) acc[c] = 0.f;
    pdl_wait();  // the partials come from the previous kernel
    for (int b = s0; b < s1; b += GR) {
        const int cnt = min(GR, s1 - b) - r0;  // rows of this slot in the batch (may be <= 0)
        const float *rows = T.partial + (size_t)(b + r0) * MP + lgi;
        float rowv[G][CH];
#pragma unroll
        for (int j = 0; j < G; j++)
#pragma unroll
            for (int c = 0; c < CH; c++) rowv[j][c] = j < cnt ? rows[(size_t)j * MP + c * G] : 0.f;
#pragma unroll
        for (int j = 0; j < G; j++)
            if (j < cnt) {
#pragma unroll
                for (int c = 0; c < CH; c++) acc[c] = fadd(acc[c], rowv[j][c]);
            }
    }
    for (int o = G; o < GR; o <<= 1)
#pragma unroll
        for (int c = 0; c < CH; c++) acc[c] = fadd(acc[c], __shfl_xor_sync(gmask, acc[c], o, GR));
    if (r0 != 0) return;
    float *dst = T.V + (size_t)(v + 1) * MP + lgi;
#pragma unroll
    for (int c = 0; c < CH; c++) dst[c * G] = acc[c];
}

// Copies a vertex's VEC values y into its partial rows pv[list[q]] for q in
// [s0, s1) (the scatter of the filter's last blur pass).  Eight indices are
// fetched before their stores, so a vertex with many partials (a large
// spatial bandwidth: over a hundred) costs a few load round trips, not one
// per partial.
template <int MP, int VEC>
__device__ __forceinline__ void scatter_partials(float *__restrict__ pv, const int *__restrict__ list, int s0, int s1,
                                                 int col, const float (&y)[VEC]) {
    auto put = [&](int p) {
        float *dst = pv + (size_t)p * MP + col;
        if constexpr (VEC == 4) {
            *reinterpret_cast<float4 *>(dst) = make_float4(y[0], y[1], y[2], y[3]);
        } else {
#pragma unroll
            for (int e = 0; e < VEC; e++) dst[e] = y[e];
        }
    };
    int q = s0;
    for (; q + 8 <= s1; q += 8) {
        int idx[8];
#pragma unroll
        for (int u = 0; u < 8; u++) idx[u] = __ldg(list + q + u);
#pragma unroll
        for (int u = 0; u < 8; u++) put(idx[u]);
    }
    for (; q < s1; q++) put(__ldg(list + q));
}

// One blur step at a vertex: y = x0 + 0.5 * (x1 + x2) over VEC labels.
// sseCompute evaluates it in float (permutohedral.cpp:566), seqCompute as
// old + 0.5 * (n1 + n2) in double with the float sum n1 + n2 (permutohedral.cpp:
// 505).  Both give the same float: x0 and 0.5 * (n1 + n2) are floats, whose
// sum is exact in double unless their exponents differ by more than 29 bits,
// and then both roundings give the larger operand (checked on 8 M random
// pairs, extreme magnitude ratios and near-cancellations included).  So one
// float evaluation serves both (double arithmetic is slow on this GPU); SEQ
// keeps the two instantiations apart for the other arithmetic that differs.
template <int VEC, bool SEQ>
__device__ __forceinline__ void blur_step(const float (&x0)[VEC], const float (&x1)[VEC], const float (&x2)[VEC],
                                          float (&y)[VEC]) {
#pragma unroll
    for (int e = 0; e < VEC; e++) y[e] = fadd(x0[e], fmul(0.5f, fadd(x1[e], x2[e])));
}

template <int VEC>
__device__ __forceinline__ void load_vec(const float *p, float (&x)[VEC]) {
    if constexpr (VEC == 4) {
        const float4 q = *reinterpret_cast<const float4 *>(p);
        x[0] = q.x, x[1] = q.y, x[2] = q.z, x[3] = q.w;
    } else {
#pragma unroll
        for (int e = 0; e < VEC; e++) x[e] = p[e];
    }
}

// One pass along an axis at lattice row `row` (1-based; its neighbours nb are
// rows, 0 = the zero sentinel), VEC labels from column col.
template <int MP, int VEC, bool SEQ>
__device__ __forceinline__ void blur_at(const float *Vin, int row, int2 nb, int col, float (&y)[VEC]) {
    float x0[VEC], x1[VEC], x2[VEC];
    load_vec<VEC>(Vin + (size_t)row * MP + col, x0);
    load_vec<VEC>(Vin + (size_t)nb.x * MP + col, x1);
    load_vec<VEC>(Vin + (size_t)nb.y * MP + col, x2);
    blur_step<VEC, SEQ>(x0, x1, x2, y);
}

// One launch = one or two consecutive axis passes for every listed term.  Two
// passes (axis2 >= 0) recompute the first pass at the vertex and at its two
// neighbours along axis2 (a missing neighbour is the zero sentinel row of the
// intermediate buffer, so 0) and apply the second: the same arithmetic as two
// launches through an intermediate buffer, one launch and one global round
// trip fewer.
template <int MP, bool SEQ>
__global__ void __launch_bounds__(256) blur_kernel(const __grid_constant__ BlurArgs a) {
    constexpr int VEC = (MP % 4 == 0) ? 4 : (MP % 2 == 0) ? 2 : 1;
    constexpr int NV = MP / VEC;
    pdl_trigger();
    const long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= a.begin[a.n]) return;
    int k = 0;
    while (g >= a.begin[k + 1]) k++;
    const BlurArgs::T &T = a.t[k];
    const long long local = g - a.begin[k];
    const int v = (int)(local / NV);
    const int c = (int)(local - (long long)v * NV);
    const int col = c * VEC;
    // neighbour tables are fixed since the build: read before the wait
    const int2 nb = __ldg(T.nbr + (size_t)T.axis * T.L + v);
    int2 nb2 = make_int2(0, 0), na = make_int2(0, 0), nbb = make_int2(0, 0);
    const bool two = T.axis2 >= 0;
    if (two) {
        nb2 = __ldg(T.nbr + (size_t)T.axis2 * T.L + v);
        if (nb2.x) na = __ldg(T.nbr + (size_t)T.axis * T.L + (nb2.x - 1));
        if (nb2.y) nbb = __ldg(T.nbr + (size_t)T.axis * T.L + (nb2.y - 1));
    }
    pdl_wait();  // the values come from the previous kernel
    float y[VEC];
    blur_at<MP, VEC, SEQ>(T.Vin, v + 1, nb, col, y);
    if (two) {
        float ya[VEC], yb[VEC], y2[VEC];
#pragma unroll
        for (int e = 0; e < VEC; e++) ya[e] = yb[e] = 0.f;
        if (nb2.x) blur_at<MP, VEC, SEQ>(T.Vin, nb2.x, na, col, ya);
        if (nb2.y) blur_at<MP, VEC, SEQ>(T.Vin, nb2.y, nbb, col, yb);
        blur_step<VEC, SEQ>(y, ya, yb, y2);
#pragma unroll
        for (int e = 0; e < VEC; e++) y[e] = y2[e];
    }
    const size_t o0 = (size_t)(v + 1) * MP + col;
    if (T.Vout) {
        if constexpr (VEC == 4) {
            *reinterpret_cast<float4 *>(T.Vout + o0) = make_float4(y[0], y[1], y[2], y[3]);
        } else {
#pragma unroll
            for (int e = 0; e < VEC; e++) T.Vout[o0 + e] = y[e];
        }
    }
    if (T.pv) scatter_partials<MP, VEC>(T.pv, T.red_list, T.red_beg[v], T.red_beg[v + 1], col, y);
}

// Bounded grid barrier of a cooperative launch: the last CTA to arrive resets
// the arrival count and advances the generation; the others wait for the new
// generation at most ~2^22 polls, then record DCRF_ERR_TIMEOUT and report
// failure (the caller returns; the barrier of the next launch starts from a
// cleared state).
__device__ __forceinline__ bool grid_barrier(unsigned *bar, unsigned nblocks, DevStatus *st) {
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile unsigned *vgen = bar + 1;
        const unsigned gen = *vgen;
        __threadfence();
        const unsigned arrived = atomicAdd(bar, 1u) + 1u;
        int ok = 1;
        if (arrived == nblocks) {
            atomicExch(bar, 0u);
            __threadfence();
            atomicAdd(bar + 1, 1u);
        } else {
            ok = 0;
            for (int it = 0; it < (1 << 22); it++) {
                if (*vgen != gen) {
                    ok = 1;
                    break;
                }
                if (it > 32) __nanosleep(64);
            }
            if (!ok) dcrf_set_error(st, DCRF_ERR_TIMEOUT, (int)blockIdx.x);
        }
        __threadfence();
        s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}

template <int MP, bool SEQ>
__global__ void __launch_bounds__(256) blur_chains_kernel(const __grid_constant__ BlurChainArgs a) {
    constexpr int VEC = (MP % 4 == 0) ? 4 : (MP % 2 == 0) ? 2 : 1;
    constexpr int NV = MP / VEC;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (int p = 0; p < a.npass; p++) {
        long long total = 0;
        for (int k = 0; k < a.n; k++)
            if (p <= a.c[k].d) total += (long long)a.c[k].L * NV;
        for (long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x; g < total; g += stride) {
            int k = 0;
            long long local = g;
            for (;; k++) {
                if (p > a.c[k].d) continue;
                const long long w = (long long)a.c[k].L * NV;
                if (local < w) break;
                local -= w;
            }
            const BlurChainArgs::C &C = a.c[k];
            const int v = (int)(local / NV);
            const int c = (int)(local - (long long)v * NV);
            const int axis = C.reverse ? C.d - p : p;
            const float *Vin = p == 0 ? C.S : C.buf[(p - 1) & 1];
            const bool last = p == C.d;
            float *Vout = last ? C.Out : C.buf[p & 1];
            const int2 nb = __ldg(C.nbr + (size_t)axis * C.L + v);
            const size_t o0 = (size_t)(v + 1) * MP + c * VEC, o1 = (size_t)nb.x * MP + c * VEC,
                         o2 = (size_t)nb.y * MP + c * VEC;
            float x0[VEC], x1[VEC], x2[VEC], y[VEC];
            // values written by other CTAs in the previous pass: read through L2 (ld.global.cg)
            if constexpr (VEC == 4) {
                const float4 q0 = __ldcg(reinterpret_cast<const float4 *>(Vin + o0));
                const float4 q1 = __ldcg(reinterpret_cast<const float4 *>(Vin + o1));
                const float4 q2 = __ldcg(reinterpret_cast<const float4 *>(Vin + o2));
                x0[0] = q0.x, x0[1] = q0.y, x0[2] = q0.z, x0[3] = q0.w;
                x1[0] = q1.x, x1[1] = q1.y, x1[2] = q1.z, x1[3] = q1.w;
                x2[0] = q2.x, x2[1] = q2.y, x2[2] = q2.z, x2[3] = q2.w;
            } else {
#pragma unroll
                for (int e = 0; e < VEC; e++) {
                    x0[e] = __ldcg(Vin + o0 + e);
                    x1[e] = __ldcg(Vin + o1 + e);
                    x2[e] = __ldcg(Vin + o2 + e);
                }
            }
            // seqCompute and sseCompute give the same float here (see blur_step)
            blur_step<VEC, SEQ>(x0, x1, x2, y);
            if (Vout) {
                if constexpr (VEC == 4) {
                    *reinterpret_cast<float4 *>(Vout + o0) = make_float4(y[0], y[1], y[2], y[3]);
                } else {
#pragma unroll
                    for (int e = 0; e < VEC; e++) Vout[o0 + e] = y[e];
                }
            }
            if (last && C.pv) scatter_partials<MP, VEC>(C.pv, C.red_list, C.red_beg[v], C.red_beg[v + 1], c * VEC, y);
        }
        if (p + 1 < a.npass && !grid_barrier(a.bar, gridDim.x, a.status)) return;
    }
}

// Image of point p: the b with seg[b] <= p < seg[b+1].
__device__ __forceinline__ int image_of(const int *__restrict__ seg, int nseg, int p) {
    int lo = 0, hi = nseg - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldg(seg + mid) <= p)
            lo = mid;
        else
            hi = mid - 1;
    }
    return lo;
}

// Offset of (label m, point p) in a caller's buffer: point-major [N][M], or
// label-major per image (image b's M x N_b block after those of images < b;
// with one image simply [M][N]).
__device__ __forceinline__ size_t user_offset(int point_major, int M, int N, const int *__restrict__ seg, int nseg,
                                              int p, int m) {
    if (point_major) return (size_t)p * M + m;
    if (nseg == 1) return (size_t)m * N + p;
    const int b = image_of(seg, nseg, p);
    const int s0 = __ldg(seg + b), nb = __ldg(seg + b + 1) - s0;
    return (size_t)s0 * M + (size_t)m * nb + (p - s0);
}

// Caller-layout <-> slot-row copies, one tile of SPLAT_TILE slots per block.
// The tile passes through shared memory (row pitch ld + 1, conflict-free), so
// that the caller's buffer is read or written with consecutive threads on
// consecutive addresses -- labels of a point for point-major buffers, points
// of a label for label-major ones -- and the tile's slot rows, one contiguous
// block of SPLAT_TILE * ld floats, with coalesced stores or loads.
constexpr int SLOT_PITCH_MAX = DCRF_MAX_MP + 1;

struct SlotTile {
    float rows[SPLAT_TILE * SLOT_PITCH_MAX];
    size_t o0[SPLAT_TILE], step[SPLAT_TILE];  // caller offset of label 0, stride between labels
    int pt[SPLAT_TILE];
};

__device__ __forceinline__ void slot_tile_points(SlotTile &st, int point_major, int M, int Mu, int m0, int N,
                                                 const int *seg, int nseg, const int *slot_pt) {
    const int li = threadIdx.x;
    const int p = slot_pt[(size_t)blockIdx.x * SPLAT_TILE + li];
    size_t o0 = 0, step = 0;
    if (p >= 0) {
        o0 = user_offset(point_major, Mu, N, seg, nseg, p, m0);
        step = M > 1 ? user_offset(point_major, Mu, N, seg, nseg, p, m0 + 1) - o0 : 0;
    }
    st.pt[li] = p;
    st.o0[li] = o0;
    st.step[li] = step;
}

// A thread's walk over the elements f = li, li + SPLAT_TILE, ... of a tile
// laid out as rows of w values: (row, column) = (f / w, f % w), advanced
// without a division per element.
struct TileWalk {
    int row, col, drow, dcol, w;
    __device__ __forceinline__ TileWalk(int f, int w_) : w(w_) {
        row = f / w;
        col = f - row * w;
        drow = SPLAT_TILE / w;
        dcol = SPLAT_TILE - drow * w;
    }
    __device__ __forceinline__ void next() {
        row += drow;
        col += dcol;
        if (col >= w) {
            col -= w;
            row++;
        }
    }
};

// the tile's caller-side walk from element f = li: (slot q, label m) --
// labels of a point for point-major buffers, points of a label otherwise
struct CallerWalk {
    TileWalk t;
    int point_major;
    __device__ __forceinline__ CallerWalk(int point_major_, int M) : t(threadIdx.x, point_major_ ? M : SPLAT_TILE),
                                                                     point_major(point_major_) {}
    __device__ __forceinline__ int q() const { return point_major ? t.row : t.col; }
    __device__ __forceinline__ int m() const { return point_major ? t.col : t.row; }
    __device__ __forceinline__ void next() { t.next(); }
};

// out[slot][m] = in(m0 + m, slot_pt[slot]) for m < M (Mu: the caller's label
// count); 0 for padding labels m < ld and for empty slots
__global__ void __launch_bounds__(SPLAT_TILE) to_slots_kernel(const float *__restrict__ in, int point_major, int M,
                                                              int Mu, int m0, int ld, int N,
                                                              const int *__restrict__ seg, int nseg,
                                                              const int *__restrict__ slot_pt,
                                                              float *__restrict__ out) {
    __shared__ SlotTile st;
    const int li = threadIdx.x, pitch = ld + 1;
    slot_tile_points(st, point_major, M, Mu, m0, N, seg, nseg, slot_pt);
    __syncthreads();
    // eight independent loads in flight per thread
    CallerWalk cw(point_major, M);
#pragma unroll 8
    for (int f = li; f < SPLAT_TILE * M; f += SPLAT_TILE, cw.next()) {
        const int q = cw.q(), m = cw.m();
        st.rows[q * pitch + m] = st.pt[q] >= 0 ? in[st.o0[q] + (size_t)m * st.step[q]] : 0.f;
    }
    __syncthreads();
    float *dst = out + (size_t)blockIdx.x * SPLAT_TILE * ld;
    TileWalk tw(li, ld);
    for (int f = li; f < SPLAT_TILE * ld; f += SPLAT_TILE, tw.next())
        dst[f] = tw.col < M ? st.rows[tw.row * pitch + tw.col] : 0.f;
}

// out(m, pt) = in[pt_slot[pt]][m], one thread per point: label-major output is
// written a whole image row at a time (consecutive points on consecutive
// addresses for every label)
__global__ void from_slots_lm_kernel(const float *__restrict__ in, int M, int Mu, int m0, int ld, int N,
                                     const int *__restrict__ seg, int nseg, const int *__restrict__ pt_slot,
                                     float *__restrict__ out) {
    const int pt = blockIdx.x * blockDim.x + threadIdx.x;
    if (pt >= N) return;
    const float *src = in + (size_t)pt_slot[pt] * ld;
    const size_t o0 = user_offset(0, Mu, N, seg, nseg, pt, m0);
    const size_t step = M > 1 ? user_offset(0, Mu, N, seg, nseg, pt, m0 + 1) - o0 : 0;
    for (int m = 0; m < M; m++) out[o0 + m * step] = src[m];
}

// out(m, pt) = in[slot of pt][m] through a shared-memory tile (point-major output)
__global__ void __launch_bounds__(SPLAT_TILE) from_slots_kernel(const float *__restrict__ in, int M, int Mu, int m0,
                                                                int ld, int N, const int *__restrict__ seg, int nseg,
                                                                const int *__restrict__ slot_pt, int point_major,
                                                                float *__restrict__ out) {
    __shared__ SlotTile st;
    const int li = threadIdx.x, pitch = ld + 1;
    slot_tile_points(st, point_major, M, Mu, m0, N, seg, nseg, slot_pt);
    const float *src = in + (size_t)blockIdx.x * SPLAT_TILE * ld;
    TileWalk tw(li, ld);
#pragma unroll 8
    for (int f = li; f < SPLAT_TILE * ld; f += SPLAT_TILE, tw.next())
        if (tw.col < M) st.rows[tw.row * pitch + tw.col] = src[f];
    __syncthreads();
    CallerWalk cw(point_major, M);
    for (int f = li; f < SPLAT_TILE * M; f += SPLAT_TILE, cw.next()) {
        const int q = cw.q(), m = cw.m();
        if (st.pt[q] >= 0) out[st.o0[q] + (size_t)m * st.step[q]] = st.rows[q * pitch + m];
    }
}

// DenseCRF2D features (densecrf.cpp:61-81) of every image of the handle:
// (x/sx, y/sy[, r/sr, g/sg, b/sb]) with (x, y) the pixel within its own image;
// rgb holds the images' H x W x 3 bytes one after another.
__global__ void features_2d_kernel(int N, const int *__restrict__ seg, const int *__restrict__ imgW, int nseg,
                                   float sx, float sy, const uint8_t *__restrict__ rgb, float sr, float sg, float sb,
                                   float *__restrict__ feat) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= N) return;
    const int b = image_of(seg, nseg, p);
    const int q = p - __ldg(seg + b), Wb = __ldg(imgW + b);
    const int j = q / Wb, i = q - j * Wb;
    feat[p] = __fdiv_rn((float)i, sx);
    feat[(size_t)N + p] = __fdiv_rn((float)j, sy);
    if (rgb) {
        feat[(size_t)2 * N + p] = __fdiv_rn((float)rgb[(size_t)p * 3 + 0], sr);
        feat[(size_t)3 * N + p] = __fdiv_rn((float)rgb[(size_t)p * 3 + 1], sg);
        feat[(size_t)4 * N + p] = __fdiv_rn((float)rgb[(size_t)p * 3 + 2], sb);
    }
}

// DIAG: out[j] = p[j]*f[j]; FULL: out[j] = sum_k P[j][k] f[k] (pairwise.cpp:140-151)
__global__ void scale_features_kernel(const float *__restrict__ in, float *__restrict__ out,
                                      const float *__restrict__ P, int d, int N, int full) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= N) return;
    for (int j = 0; j < d; j++) {
        float s;
        if (full) {
            s = 0.f;
            for (int k = 0; k < d; k++) s = fadd(s, fmul(P[j * d + k], in[(size_t)k * N + p]));
        } else {
            s = fmul(P[j], in[(size_t)j * N + p]);
        }
        out[(size_t)j * N + p] = s;
    }
}

// ---------------------------------------------------------------------------
int pointpass_smem_budget(int MP) { return MP <= 20 ? 72 * 1024 : 108 * 1024; }

template <int MP>
static cudaError_t slice_launch(const PPArgs &a, cudaStream_t s) {
    DCRF_LAUNCH(slice_kernel<MP><<<a.ntiles, SPLAT_TILE, 0, s>>>(a));
    return cudaGetLastError();
}

cudaError_t launch_slice(const PPArgs &a, int MP, cudaStream_t s) {
    if (a.ntiles <= 0) return cudaSuccess;
    switch (MP) {
        case 1: return slice_launch<1>(a, s);
        case 2: return slice_launch<2>(a, s);
        case 4: return slice_launch<4>(a, s);
        case 8: return slice_launch<8>(a, s);
        case 12: return slice_launch<12>(a, s);
        case 16: return slice_launch<16>(a, s);
        case 20: return slice_launch<20>(a, s);
        case 24: return slice_launch<24>(a, s);
        case 28: return slice_launch<28>(a, s);
        case 32: return slice_launch<32>(a, s);
        default: return cudaErrorInvalidValue;
    }
}

template <int MP>
static cudaError_t red_launch(ReduceArgs a, cudaStream_t s) {
    constexpr int G = Grp<MP>::G;
    long long threads = 0;
    for (int k = 0; k < a.n; k++) {
        // more than 4 partials per vertex on average: a full warp per vertex
        const bool wide = a.t[k].L > 0 && a.t[k].P > 4ll * a.t[k].L;
        a.rs[k] = wide ? 32 / G : 1;
        a.begin[k] = threads;
        threads += ((long long)a.t[k].L * G * a.rs[k] + 31) / 32 * 32;
    }
    a.begin[a.n] = threads;
    if (threads > 0) return launch_pdl(reduce_kernel<MP>, dim3((unsigned)((threads + 255) / 256)), dim3(256), 0, s, a);
    return cudaGetLastError();
}

cudaError_t launch_reduce(const ReduceArgs &a, int MP, cudaStream_t s) {
    switch (MP) {
        case 1: return red_launch<1>(a, s);
        case 2: return red_launch<2>(a, s);
        case 4: return red_launch<4>(a, s);
        case 8: return red_launch<8>(a, s);
        case 12: return red_launch<12>(a, s);
        case 16: return red_launch<16>(a, s);
        case 20: return red_launch<20>(a, s);
        case 24: return red_launch<24>(a, s);
        case 28: return red_launch<28>(a, s);
        case 32: return red_launch<32>(a, s);
        default: return cudaErrorInvalidValue;
    }
}

template <int MP, bool SEQ>
static cudaError_t blur_launch(const BlurArgs &a, cudaStream_t s) {
    long long threads = a.begin[a.n];
    if (threads > 0) return launch_pdl(blur_kernel<MP, SEQ>, dim3((unsigned)((threads + 255) / 256)), dim3(256), 0, s, a);
    return cudaGetLastError();
}

cudaError_t launch_blur(const BlurArgs &a, int MP, bool seq, cudaStream_t s) {
#define DCRF_BL(X) \
    case X:        \
        return seq ? blur_launch<X, true>(a, s) : blur_launch<X, false>(a, s);
    switch (MP) {
        DCRF_BL(1) DCRF_BL(2) DCRF_BL(4) DCRF_BL(8) DCRF_BL(12) DCRF_BL(16) DCRF_BL(20) DCRF_BL(24) DCRF_BL(28)
        DCRF_BL(32)
        default: return cudaErrorInvalidValue;
    }
#undef DCRF_BL
}

template <int MP, bool SEQ>
static cudaError_t chains_launch(const BlurChainArgs &a, cudaStream_t s) {
    // co-resident CTAs of this instance, queried once per device
    static std::atomic<int> grids[64];
    int dev = 0;
    cudaGetDevice(&dev);
    int grid = dev >= 0 && dev < 64 ? grids[dev].load() : 0;
    if (grid == 0) {
        int nsm = 0, per = 0;
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, blur_chains_kernel<MP, SEQ>, 256, 0);
        grid = std::max(1, nsm * std::max(1, per));
        if (dev >= 0 && dev < 64) grids[dev].store(grid);
    }
    long long work = 0;
    for (int k = 0; k < a.n; k++) work += (long long)a.c[k].L * (MP % 4 == 0 ? MP / 4 : MP % 2 == 0 ? MP / 2 : MP);
    const int blocks = (int)std::max<long long>(1, std::min<long long>(grid, (work + 255) / 256));
    cudaError_t e = cudaMemsetAsync(a.bar, 0, 2 * sizeof(unsigned), s);
    if (e != cudaSuccess) return e;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(blocks);
    cfg.blockDim = dim3(256);
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeCooperative;
    at[0].val.cooperative = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    note_launch();
    return cudaLaunchKernelEx(&cfg, blur_chains_kernel<MP, SEQ>, a);
}

cudaError_t launch_blur_chains(const BlurChainArgs &a, int MP, bool seq, cudaStream_t s) {
    if (a.n <= 0) return cudaSuccess;
#define DCRF_BC(X) \
    case X:        \
        return seq ? chains_launch<X, true>(a, s) : chains_launch<X, false>(a, s);
    switch (MP) {
        DCRF_BC(1) DCRF_BC(2) DCRF_BC(4) DCRF_BC(8) DCRF_BC(12) DCRF_BC(16) DCRF_BC(20) DCRF_BC(24) DCRF_BC(28)
        DCRF_BC(32)
        default: return cudaErrorInvalidValue;
    }
#undef DCRF_BC
}

cudaError_t launch_to_slots(const float *in, int point_major, int M, int Mu, int m0, int ld, int N, const int *seg,
                            int nseg, const int *slot_pt, int nslots, float *out, cudaStream_t s) {
    if (ld < M || ld > DCRF_MAX_MP || nslots % SPLAT_TILE != 0 || m0 + M > Mu) return cudaErrorInvalidValue;
    if (nslots > 0)
        DCRF_LAUNCH(to_slots_kernel<<<nslots / SPLAT_TILE, SPLAT_TILE, 0, s>>>(in, point_major, M, Mu, m0, ld, N, seg,
                                                                               nseg, slot_pt, out));
    return cudaGetLastError();
}

cudaError_t launch_from_slots(const float *in, int M, int Mu, int m0, int ld, int N, const int *seg, int nseg,
                              const int *slot_pt, int nslots, const int *pt_slot, int point_major, float *out,
                              cudaStream_t s) {
    if (ld < M || ld > DCRF_MAX_MP || nslots % SPLAT_TILE != 0 || m0 + M > Mu) return cudaErrorInvalidValue;
    if (N <= 0) return cudaGetLastError();
    if (point_major) {
        if (nslots > 0)
            DCRF_LAUNCH(from_slots_kernel<<<nslots / SPLAT_TILE, SPLAT_TILE, 0, s>>>(in, M, Mu, m0, ld, N, seg, nseg,
                                                                                     slot_pt, point_major, out));
    } else {
        DCRF_LAUNCH(from_slots_lm_kernel<<<(N + 255) / 256, 256, 0, s>>>(in, M, Mu, m0, ld, N, seg, nseg, pt_slot,
                                                                         out));
    }
    return cudaGetLastError();
}

cudaError_t launch_features_2d(int N, const int *seg, const int *imgW, int nseg, float sx, float sy,
                               const uint8_t *rgb, float sr, float sg, float sb, float *feat, cudaStream_t s) {
    if (N > 0)
        DCRF_LAUNCH(features_2d_kernel<<<(N + 255) / 256, 256, 0, s>>>(N, seg, imgW, nseg, sx, sy, rgb, sr, sg, sb,
                                                                       feat));
    return cudaGetLastError();
}

cudaError_t launch_scale_features(const float *in, float *out, const float *P, int d, int N, int full,
                                  cudaStream_t s) {
    if (N > 0) DCRF_LAUNCH(scale_features_kernel<<<(N + 255) / 256, 256, 0, s>>>(in, out, P, d, N, full));
    return cudaGetLastError();
}

}  // namespace dcrf
