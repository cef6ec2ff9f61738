// pointpass.cuh -- the mean-field point pass (see meanfield.cu for the
// iteration it belongs to) and the device helpers it shares with the other
// mean-field kernels: TMA bulk copies and mbarriers, row loads and stores,
// label compatibilities.  Included by meanfield.cu and pointpass.cu (which
// holds the point pass's launchers, so its many instances compile apart).
#pragma once
#include <math.h>

#include "meanfield.cuh"

namespace dcrf {

// ---------------------------------------------------------------------------
// TMA bulk copies and mbarriers (inline PTX)
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// 1-D bulk copy global -> shared; 16-byte aligned addresses, size a multiple of 16.
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}

// Bounded wait on phase `parity`: returns false after ~2^22 polls (seconds).
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity) {
    for (int it = 0; it < (1 << 22); it++) {
        if (mbar_try_wait(bar, parity)) return true;
        if (it > 16) __nanosleep(128);
    }
    return false;
}

template <int MP>
struct Grp {
    // lanes per splat/reduce group: the largest power of two <= 32 dividing MP
    static constexpr int G = (MP % 32 == 0) ? 32 : (MP % 16 == 0) ? 16 : (MP % 8 == 0) ? 8 : (MP % 4 == 0) ? 4
                             : (MP % 2 == 0)  ? 2
                                              : 1;
    static constexpr int CH = MP / G;
};

template <int MP>
__device__ __forceinline__ void load_row(const float *__restrict__ row, float (&v)[MP]) {
    if constexpr (MP % 4 == 0) {
        const float4 *r4 = reinterpret_cast<const float4 *>(row);
#pragma unroll
        for (int c = 0; c < MP / 4; c++) {
            float4 x = __ldg(r4 + c);
            v[4 * c + 0] = x.x;
            v[4 * c + 1] = x.y;
            v[4 * c + 2] = x.z;
            v[4 * c + 3] = x.w;
        }
    } else if constexpr (MP == 2) {
        float2 x = __ldg(reinterpret_cast<const float2 *>(row));
        v[0] = x.x;
        v[1] = x.y;
    } else {
#pragma unroll
        for (int m = 0; m < MP; m++) v[m] = __ldg(row + m);
    }
}

template <int MP>
__device__ __forceinline__ void load_row_s(const float *row, float (&v)[MP]) {
    if constexpr (MP % 4 == 0) {
#pragma unroll
        for (int c = 0; c < MP / 4; c++) {
            const float4 x = reinterpret_cast<const float4 *>(row)[c];
            v[4 * c + 0] = x.x, v[4 * c + 1] = x.y, v[4 * c + 2] = x.z, v[4 * c + 3] = x.w;
        }
    } else {
#pragma unroll
        for (int m = 0; m < MP; m++) v[m] = row[m];
    }
}

template <int MP>
__device__ __forceinline__ void store_row(float *row, const float (&v)[MP]) {
    if constexpr (MP % 4 == 0) {
#pragma unroll
        for (int c = 0; c < MP / 4; c++)
            reinterpret_cast<float4 *>(row)[c] = make_float4(v[4 * c], v[4 * c + 1], v[4 * c + 2], v[4 * c + 3]);
    } else {
#pragma unroll
        for (int m = 0; m < MP; m++) row[m] = v[m];
    }
}

// Point groups of the point pass: a point's MP labels are spread over G lanes
// of VW consecutive labels each (one float4 for MP >= 4), so every row access
// of a point -- unary, marginals, blurred vertex rows, splat rows -- is one
// contiguous, conflict-free vector access of the group.
template <int MP>
struct PG {
    static constexpr int VW = MP >= 4 ? 4 : MP;             // labels per lane
    static constexpr int G = MP / VW;                       // lanes per point
    static constexpr int GPW = 32 / G;                      // groups per warp
    static constexpr int NG = (SPLAT_TILE / 32) * GPW;      // groups per CTA
    static constexpr int PPG = (SPLAT_TILE + NG - 1) / NG;  // points per group
};

template <int VW>
__device__ __forceinline__ void vload(const float *p, float (&v)[VW]) {
    if constexpr (VW % 4 == 0) {
#pragma unroll
        for (int c = 0; c < VW / 4; c++) {
            const float4 x = *reinterpret_cast<const float4 *>(p + 4 * c);
            v[4 * c] = x.x, v[4 * c + 1] = x.y, v[4 * c + 2] = x.z, v[4 * c + 3] = x.w;
        }
    } else if constexpr (VW == 2) {
        const float2 x = *reinterpret_cast<const float2 *>(p);
        v[0] = x.x, v[1] = x.y;
    } else {
        v[0] = *p;
    }
}

template <int VW>
__device__ __forceinline__ void vload_g(const float *__restrict__ p, float (&v)[VW]) {
    if constexpr (VW == 4) {
        const float4 x = __ldg(reinterpret_cast<const float4 *>(p));
        v[0] = x.x, v[1] = x.y, v[2] = x.z, v[3] = x.w;
    } else if constexpr (VW == 2) {
        const float2 x = __ldg(reinterpret_cast<const float2 *>(p));
        v[0] = x.x, v[1] = x.y;
    } else {
        v[0] = __ldg(p);
    }
}

template <int VW>
__device__ __forceinline__ void vstore(float *p, const float (&v)[VW]) {
    if constexpr (VW % 4 == 0) {
#pragma unroll
        for (int c = 0; c < VW / 4; c++)
            *reinterpret_cast<float4 *>(p + 4 * c) = make_float4(v[4 * c], v[4 * c + 1], v[4 * c + 2], v[4 * c + 3]);
    } else if constexpr (VW == 2) {
        *reinterpret_cast<float2 *>(p) = make_float2(v[0], v[1]);
    } else {
        *p = v[0];
    }
}

// x -= compatibility(acc) (mean-field update), or, with kl_mode, kl += sum q *
// compatibility(acc) where x holds q.  Potts: -w acc; Diagonal: v * acc;
// Matrix: W acc with the sum over k in label order (labelcompatibility.cpp:
// 46-48,66-68,82-84); the Matrix comes from shared memory transposed to
// [k][MP] (sCT, broadcast row reads) or, without it, from global memory.
template <int MP>
__device__ __forceinline__ void fold_compat(const TermDev &T, const float *sCT, const float (&acc)[MP], float (&x)[MP],
                                            int M, bool kl_mode, double &kl) {
    float c[MP];
    if (T.ckind == DCRF_COMPAT_POTTS) {
        const float nw = -T.potts_w;
#pragma unroll
        for (int m = 0; m < MP; m++) c[m] = fmul(nw, acc[m]);
    } else if (T.ckind == DCRF_COMPAT_DIAGONAL) {
#pragma unroll
        for (int m = 0; m < MP; m++) c[m] = m < M ? fmul(__ldg(T.compat + m), acc[m]) : 0.f;
    } else {
#pragma unroll
        for (int m = 0; m < MP; m++) c[m] = 0.f;
        // products contracted into FMAs, as the reference's aarch64 build (Eigen's
        // fused multiply-add) computes W Q
        if (sCT && MP % 4 == 0) {
#pragma unroll
            for (int k = 0; k < MP; k++)
                if (k < M) {
                    float w[MP];
                    load_row_s<MP>(sCT + k * MP, w);
#pragma unroll
                    for (int m = 0; m < MP; m++) c[m] = fmaf(w[m], acc[k], c[m]);
                }
        } else {
#pragma unroll
            for (int m = 0; m < MP; m++)
                if (m < M) {
                    const float *row = T.compat + (size_t)m * M;
#pragma unroll
                    for (int k = 0; k < MP; k++)
                        if (k < M) c[m] = fmaf(__ldg(row + k), acc[k], c[m]);
                }
        }
    }
#pragma unroll
    for (int m = 0; m < MP; m++) {
        if (m >= M) continue;
        if (kl_mode)
            kl += (double)fmul(x[m], c[m]);
        else
            x[m] = fsub(x[m], c[m]);
    }
}

// Partial and task ranges of term T in tile t, and the 16-byte aligned window
// of its tasks that the prefetch copies.
struct TileBlocks {
    int pb, np;       // partials [pb, pb+np)
    int tb, nt;       // tasks [tb, tb+nt)
    int a0, nwin;     // task window [a0, a0+nwin), a0 = tb rounded down to 4
    int vp_staged;
};

__device__ __forceinline__ TileBlocks tile_blocks(const TermDev &T, int t) {
    TileBlocks b;
    b.pb = T.tile_pbeg[t];
    b.np = T.tile_pbeg[t + 1] - b.pb;
    b.tb = T.tile_tbeg[t];
    b.nt = T.tile_tbeg[t + 1] - b.tb;
    b.a0 = b.tb & ~3;
    b.nwin = ((b.tb + b.nt + 3) & ~3) - b.a0;
    b.vp_staged = b.np <= T.vcap;
    return b;
}

// Thread shape of the point pass: SPLIT threads per point (each owning H =
// MP / SPLIT consecutive labels), SPLAT_TILE * SPLIT threads per tile.  Two
// threads per point halve the registers a point needs (2 CTAs of 16 warps per
// SM instead of 2 CTAs of 8).
template <int MP, int S>
struct PPT {
    static constexpr int SPLIT = S;
    static constexpr int H = MP / SPLIT;
    static constexpr int NT = SPLAT_TILE * SPLIT;
    static constexpr int MINB = (SPLIT == 2 && MP > 24) ? 1 : 2;  // 32 labels: registers over CTAs
};

// x -= compatibility(acc) on the thread's labels l0..l0+H-1 (or kl += q .
// compatibility(acc) in kl_mode), the point's other labels coming from the
// partner thread (pair mask pm).  Potts: -w acc; Diagonal: v * acc; Matrix:
// W acc summed over k in label order with fused multiply-adds (the reference's
// aarch64 build, Eigen's FMA) (labelcompatibility.cpp:46-48,66-68,82-84).
template <int MP, int S>
__device__ __forceinline__ void fold_compat_h(const TermDev &T, const float *sCT, const float (&acc)[PPT<MP, S>::H],
                                              float (&x)[PPT<MP, S>::H], int M, int l0, int h, unsigned pm,
                                              bool kl_mode, double &kl) {
    constexpr int H = PPT<MP, S>::H, SPLIT = PPT<MP, S>::SPLIT;
    float c[H];
    if (T.ckind == DCRF_COMPAT_POTTS) {
        const float nw = -T.potts_w;
#pragma unroll
        for (int e = 0; e < H; e++) c[e] = fmul(nw, acc[e]);
    } else if (T.ckind == DCRF_COMPAT_DIAGONAL) {
#pragma unroll
        for (int e = 0; e < H; e++) c[e] = l0 + e < M ? fmul(__ldg(T.compat + l0 + e), acc[e]) : 0.f;
    } else {
#pragma unroll
        for (int e = 0; e < H; e++) c[e] = 0.f;
#pragma unroll
        for (int b = 0; b < SPLIT; b++) {
#pragma unroll
            for (int j = 0; j < H; j++) {
                float a = acc[j];
                if constexpr (SPLIT == 2) {
                    const float other = __shfl_xor_sync(pm, acc[j], 1);
                    a = b == h ? acc[j] : other;
                }
                const int k = b * H + j;
                if (k >= M) continue;
                if (sCT) {
                    float w[H];
                    load_row_s<H>(sCT + k * MP + l0, w);
#pragma unroll
                    for (int e = 0; e < H; e++) c[e] = fmaf(w[e], a, c[e]);
                } else {
#pragma unroll
                    for (int e = 0; e < H; e++)
                        if (l0 + e < M) c[e] = fmaf(__ldg(T.compat + (size_t)(l0 + e) * M + k), a, c[e]);
                }
            }
        }
    }
    // padding labels have c = 0 (their filtered values and compatibility
    // entries are 0), so no label mask is needed here
#pragma unroll
    for (int e = 0; e < H; e++) {
        if (kl_mode)
            kl += (double)fmul(x[e], c[e]);
        else
            x[e] = fsub(x[e], c[e]);
    }
}

// One CTA per tile of SPLAT_TILE points; marginals and unaries are slot rows
// of MP floats ([nslots][MP]).  MODE != 0 fixes the mode bits at compile time
// (the iteration passes: fewer live registers and no untaken paths); MODE == 0
// reads them from the arguments.
template <int MP, int S, int MODE = 0>
__global__ void __launch_bounds__(PPT<MP, S>::NT, PPT<MP, S>::MINB) pointpass_kernel(const __grid_constant__ PPArgs a) {
    constexpr int SPLIT = PPT<MP, S>::SPLIT, H = PPT<MP, S>::H, NT = PPT<MP, S>::NT;
    using P = PG<MP>;
    constexpr int VW = P::VW, G = P::G, GPW = P::GPW;
    constexpr int NG = (NT / 32) * GPW;  // splat groups per CTA
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ uint64_t mbar;
    __shared__ double sKL[NT / 32];
    __shared__ TileBlocks sTB[DCRF_MAX_TERMS];

    const int t = blockIdx.x;
    const int li = threadIdx.x;
    const int lane = li & 31, warp = li >> 5;
    const int pi = li / SPLIT;               // point of the tile
    const int h = li - pi * SPLIT;           // which labels of it
    const int l0 = h * H;
    const unsigned pm = SPLIT == 2 ? (3u << (lane & ~1)) : (1u << lane);
    const int g = lane / G;                  // splat group within the warp
    const bool gactive = g < GPW;            // lanes past the last full group idle
    const int gc = gactive ? g : GPW - 1;
    const int c = lane - gc * G;             // lane within the group
    const int gid = warp * GPW + gc;         // group within the CTA
    const int m0 = c * VW;                   // first label of the lane in the splat
    const int M = a.M, mode = MODE ? MODE : a.mode;
    pdl_trigger();

    // ---- 1. prefetch the tile's tables (TMA bulk copies, one elected thread):
    // the lattice tables first, the blurred rows once the previous kernel is done
    bool any_staged = false;
    for (int k = 0; k < a.ts.n; k++) any_staged |= a.ts.t[k].staged != 0;
    if (li < a.ts.n) sTB[li] = tile_blocks(a.ts.t[li], t);
    if (any_staged && li == 0) {
        mbar_init(&mbar, 1);
        fence_mbar_init();
    }
    __syncthreads();
    if (any_staged && li == 0) {
        uint32_t total = 0;
        for (int k = 0; k < a.ts.n; k++) {
            const TermDev &T = a.ts.t[k];
            const TileBlocks b = sTB[k];
            if (!T.staged) continue;
            const uint32_t d1 = T.d + 1;
            total += 1024u + (uint32_t)b.nwin * 8u + d1 * SPLAT_TILE * 6u;  // norm, tasks, schedule, members
            if (mode & PP_MSG) {
                total += d1 * SPLAT_TILE * 6u;                                // corner tables
                if (b.vp_staged) total += (uint32_t)b.np * MP * 4u;           // blurred rows
            }
        }
        mbar_arrive_expect_tx(&mbar, total);
        for (int k = 0; k < a.ts.n; k++) {
            const TermDev &T = a.ts.t[k];
            if (!T.staged) continue;
            const TileBlocks b = sTB[k];
            const size_t d1 = T.d + 1;
            const size_t tb = (size_t)t * SPLAT_TILE * d1;
            bulk_g2s(smem + T.sm_norm, T.norm + (size_t)t * SPLAT_TILE, 1024u, &mbar);
            bulk_g2s(smem + T.sm_task, T.task + b.a0, (uint32_t)b.nwin * 4u, &mbar);
            bulk_g2s(smem + T.sm_sched, T.tsched + b.a0, (uint32_t)b.nwin * 4u, &mbar);
            bulk_g2s(smem + T.sm_mpt, T.mem_pt + tb, (uint32_t)(d1 * SPLAT_TILE * 2), &mbar);
            bulk_g2s(smem + T.sm_mw, T.mem_w + tb, (uint32_t)(d1 * SPLAT_TILE * 4), &mbar);
            if (mode & PP_MSG) {
                bulk_g2s(smem + T.sm_loc, T.tl_loc + tb, (uint32_t)(d1 * SPLAT_TILE * 2), &mbar);
                bulk_g2s(smem + T.sm_w, T.tl_w + tb, (uint32_t)(d1 * SPLAT_TILE * 4), &mbar);
            }
        }
        pdl_wait();
        for (int k = 0; k < a.ts.n && (mode & PP_MSG); k++) {
            const TermDev &T = a.ts.t[k];
            const TileBlocks b = sTB[k];
            if (T.staged && b.vp_staged && b.np > 0)
                bulk_g2s(smem + T.sm_vp, T.pv + (size_t)b.pb * MP, (uint32_t)(b.np * MP * 4), &mbar);
        }
    }
    // Matrix compatibilities, transposed into [k][MP] (zero padded), by every thread
    if (mode & PP_MSG) {
        for (int k = 0; k < a.ts.n; k++) {
            const TermDev &T = a.ts.t[k];
            if (T.ckind != DCRF_COMPAT_MATRIX || T.sm_cmp < 0) continue;
            float *sCT = reinterpret_cast<float *>(smem + T.sm_cmp);
            for (int e = li; e < MP * MP; e += NT) {
                const int kk = e / MP, m = e - kk * MP;
                sCT[e] = (kk < M && m < M) ? T.compat[(size_t)m * M + kk] : 0.f;
            }
        }
    }

    // the point's own inputs, overlapping the copies
    const size_t s = (size_t)t * SPLAT_TILE + pi;
    const int i = a.slot_pt[s];
    const bool valid = i >= 0;
    const bool given = (mode & (PP_LOAD_Q | PP_ONES)) != 0;
    double kl = 0.0;
    // x: the logits of the update, or the given marginals (LOAD_Q / ONES); q after the softmax
    float x[H];
#pragma unroll
    for (int e = 0; e < H; e++) x[e] = 0.f;
    if (valid && !(mode & (PP_ONES | PP_LOAD_Q)) && a.U) {  // the unary is fixed during inference
        load_row<H>(a.U + s * MP + l0, x);
#pragma unroll
        for (int e = 0; e < H; e++) x[e] = -x[e];
    }
    pdl_wait();
    if (valid) {
        if (mode & PP_ONES) {
            if (h == 0) x[0] = 1.f;
        } else if (mode & PP_LOAD_Q) {
            load_row<H>(a.Qin + s * MP + l0, x);
        }
    }
    // ---- 2. wait for the copies (bounded; a timeout is reported, never a hang)
    if (any_staged) {
        const bool ok = mbar_wait_bounded(&mbar, 0);
        if (__syncthreads_or(!ok)) {
            if (li == 0) dcrf_set_error(a.status, DCRF_ERR_TIMEOUT, t);
            mbar_wait_bounded(&mbar, 0);  // let this CTA's own copies land before it exits
            return;
        }
    } else {
        __syncthreads();
    }

    // ---- 3. per point: messages of every term, softmax, outputs (the two
    // threads of a point share `valid`, so their pair shuffles converge)
    if ((mode & PP_MSG) && valid) {
        for (int k = 0; k < a.ts.n; k++) {
            const TermDev &T = a.ts.t[k];
            const TileBlocks b = sTB[k];
            float acc[H];
#pragma unroll
            for (int e = 0; e < H; e++) acc[e] = 0.f;
            const size_t tb = (size_t)t * SPLAT_TILE * (T.d + 1);
            const uint16_t *locs = T.staged ? reinterpret_cast<const uint16_t *>(smem + T.sm_loc) : T.tl_loc + tb;
            const float *ws = T.staged ? reinterpret_cast<const float *>(smem + T.sm_w) : T.tl_w + tb;
            const float *vps = reinterpret_cast<const float *>(smem + T.sm_vp);
            const bool rows_smem = T.staged && b.vp_staged;
            const float alpha = T.alpha;
            if (rows_smem && !T.seq) {
                // the common case on its own loop: rows staged in shared memory,
                // the x86 slice (w * alpha) * v (permutohedral.cpp:579-581); no
                // per-corner branches (measured: 7.7 % fewer instructions, -2.4 us)
                const float *vrow = vps + l0;
                const uint16_t *lp = locs + pi;
                const float *wp = ws + pi;
                for (int r = 0; r <= T.d; r++, lp += SPLAT_TILE, wp += SPLAT_TILE) {
                    float v[H];
                    load_row_s<H>(vrow + *lp * MP, v);
                    const float w = fmul(*wp, alpha);
#pragma unroll
                    for (int e = 0; e < H; e++) acc[e] = fmaf(w, v[e], acc[e]);
                }
            } else {
                for (int r = 0; r <= T.d; r++) {
                    const int loc = locs[r * SPLAT_TILE + pi];
                    const float bw = ws[r * SPLAT_TILE + pi];
                    float v[H];
                    if (rows_smem)
                        load_row_s<H>(vps + loc * MP + l0, v);
                    else
                        load_row<H>(T.pv + (size_t)(b.pb + loc) * MP + l0, v);
                    if (T.seq) {  // seqCompute slice: (w * v) * alpha (permutohedral.cpp:520)
#pragma unroll
                        for (int e = 0; e < H; e++) acc[e] = fmaf(fmul(bw, v[e]), alpha, acc[e]);
                    } else {  // sseCompute slice: (w * alpha) * v (permutohedral.cpp:579-581)
                        const float w = fmul(bw, alpha);
#pragma unroll
                        for (int e = 0; e < H; e++) acc[e] = fmaf(w, v[e], acc[e]);
                    }
                }
            }
            if (a.ckY[k]) store_row<H>(a.ckY[k] + s * MP + l0, acc);
            if (T.post_norm) {
                const float nn = T.staged ? reinterpret_cast<const float *>(smem + T.sm_norm)[pi] : T.norm[s];
#pragma unroll
                for (int e = 0; e < H; e++) acc[e] = fmul(acc[e], nn);
            }
            // with given marginals this is the pairwise part of klDivergence
            // (densecrf.cpp:229-233): sum Q * compat(K Q)
            fold_compat_h<MP, S>(T, T.sm_cmp >= 0 ? reinterpret_cast<const float *>(smem + T.sm_cmp) : nullptr, acc, x,
                              M, l0, h, pm, given, kl);
        }
    }
    if (valid && !given) {  // softmax over the point's labels (densecrf.cpp:98-106)
        // padding labels at -inf: their exponentials are exact zeros, so the
        // loops below need no label masks and the sums are unchanged
#pragma unroll
        for (int e = 0; e < H; e++)
            if (l0 + e >= M) x[e] = -INFINITY;
        float mx = -INFINITY;
#pragma unroll
        for (int e = 0; e < H; e++) mx = fmaxf(mx, x[e]);
        if constexpr (SPLIT == 2) mx = fmaxf(mx, __shfl_xor_sync(pm, mx, 1));
        // exponentials through the fast hardware path: __expf is within a few
        // ulp for arguments near 0, where the marginals' mass is, and its larger
        // error at very negative arguments scales values below 1e-30 of the sum
        float part = 0.f;
#pragma unroll
        for (int e = 0; e < H; e++) {
            x[e] = __expf(fsub(x[e], mx));
            part = fadd(part, x[e]);
        }
        float sum = part;
        if constexpr (SPLIT == 2) {
            // one sum in label order, as with one thread per point: the upper
            // thread continues from the lower thread's partial sum
            float full = __shfl_sync(pm, part, lane & ~1);
            if (h == 1) {
#pragma unroll
                for (int e = 0; e < H; e++) full = fadd(full, x[e]);
            }
            sum = __shfl_sync(pm, full, lane | 1);
        }
        const float rs = __frcp_rn(sum);
#pragma unroll
        for (int e = 0; e < H; e++) x[e] = fmul(x[e], rs);
    }
    float(&q)[H] = x;
    if (valid) {
        if (mode & PP_KL) {
            // entropy and unary parts (densecrf.cpp:216-226); log() there is the double overload
            float u[H];
#pragma unroll
            for (int e = 0; e < H; e++) u[e] = 0.f;
            if (a.U) load_row<H>(a.U + s * MP + l0, u);
#pragma unroll
            for (int e = 0; e < H; e++)
                if (l0 + e < M) {
                    kl += (double)q[e] * log((double)fmaxf(q[e], 1e-20f));
                    kl += (double)fmul(u[e], q[e]);
                }
        }
        if (mode & PP_WRITE_Q) store_row<H>(a.Qout + s * MP + l0, q);
        if (mode & PP_MAP) {  // first maximum (densecrf.cpp:132-137)
            int best = l0;
            float bv = q[0];
#pragma unroll
            for (int e = 1; e < H; e++)
                if (l0 + e < M && q[e] > bv) {
                    bv = q[e];
                    best = l0 + e;
                }
            if constexpr (SPLIT == 2) {
                const float ov = __shfl_xor_sync(pm, bv, 1);
                const int ob = __shfl_xor_sync(pm, best, 1);
                if (h == 0 && ob < M && ov > bv) best = ob;
            }
            if (h == 0) a.map_out[i] = (int16_t)best;
        }
    }
    if (mode & PP_KL) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) kl += __shfl_down_sync(0xffffffffu, kl, o);
        if (lane == 0) sKL[warp] = kl;
        __syncthreads();
        if (li == 0) {
            double ssum = 0.0;
            for (int w = 0; w < NT / 32; w++) ssum += sKL[w];
            a.kl_part[t] = ssum;
        }
    }

    // ---- 4. splat the tile's q into each term's partials.  Each task sums at
    // most SPLAT_TASK members of one partial in member order; a partial made of
    // several tasks adds the task sums in task order.  A group of lanes takes
    // one task at a time, each lane its own labels; the tasks are dealt in the
    // tile's schedule (descending length), so that the groups of one warp,
    // which run in lock step, get tasks of similar length.
    if (mode & PP_SPLAT) {
        float *sQ = reinterpret_cast<float *>(smem + a.sm_q);
        float *sRes = reinterpret_cast<float *>(smem + a.sm_res);
        __syncthreads();  // the message phase is done with the regions sQ aliases
        store_row<H>(sQ + pi * MP + l0, q);
        __syncthreads();
        for (int k = 0; k < a.ts.n; k++) {
            // the normalisation before the filter (pairwise.cpp:65-66) is folded into
            // the member weights of the term (w * norm of the member's point)
            const TermDev &T = a.ts.t[k];
            const TileBlocks b = sTB[k];
            const size_t tbm = (size_t)t * SPLAT_TILE * (T.d + 1);
            const uint32_t *tasks = T.staged ? reinterpret_cast<const uint32_t *>(smem + T.sm_task) + (b.tb - b.a0)
                                             : T.task + b.tb;
            const uint32_t *sched = T.staged ? reinterpret_cast<const uint32_t *>(smem + T.sm_sched) + (b.tb - b.a0)
                                             : T.tsched + b.tb;
            const uint16_t *mpt = T.staged ? reinterpret_cast<const uint16_t *>(smem + T.sm_mpt) : T.mem_pt + tbm;
            const float *mw = T.staged ? reinterpret_cast<const float *>(smem + T.sm_mw) : T.mem_w + tbm;
            // every partial of this term in this tile is one task: no combine phase
            const bool whole = b.nt == b.np;
            if (gactive) {
                for (int sj = gid; sj < b.nt; sj += NG) {
                    const int j = (int)sched[sj];
                    const uint32_t tk = tasks[j];
                    const int pl = (int)(tk >> 19), e0 = (int)((tk >> 6) & 0x1FFFu), len = (int)(tk & 63u);
                    // the partial's output row, fetched before the member loop hides its latency
                    const int prow = __ldg(T.ppos + b.pb + pl);
                    float acc[VW];
#pragma unroll
                    for (int e = 0; e < VW; e++) acc[e] = 0.f;
                    // two members per trip: their loads overlap (measured 4% on
                    // the point pass at 21 labels; wider unrolls lose it again)
#pragma unroll 2
                    for (int e = e0; e < e0 + len; e++) {
                        const float w = mw[e];
                        float v[VW];
                        vload<VW>(sQ + mpt[e] * MP + m0, v);
#pragma unroll
                        for (int f = 0; f < VW; f++) acc[f] = fmaf(w, v[f], acc[f]);
                    }
                    const bool first = whole || j == 0 || (int)(tasks[j - 1] >> 19) != pl;
                    const bool last = whole || j == b.nt - 1 || (int)(tasks[j + 1] >> 19) != pl;
                    float *dst = (first && last) ? T.pout + (size_t)prow * MP : sRes + (size_t)j * MP;
                    vstore<VW>(dst + m0, acc);
                }
            }
            if (whole) continue;  // nothing went to sRes (the flag is uniform over the CTA)
            __syncthreads();
            if (gactive) {
                for (int j = gid; j < b.nt; j += NG) {
                    const int pl = (int)(tasks[j] >> 19);
                    const bool first = j == 0 || (int)(tasks[j - 1] >> 19) != pl;
                    const bool last = j == b.nt - 1 || (int)(tasks[j + 1] >> 19) != pl;
                    if (!first || last) continue;
                    const int prow = __ldg(T.ppos + b.pb + pl);
                    float acc[VW];
                    vload<VW>(sRes + (size_t)j * MP + m0, acc);
                    for (int jj = j + 1; jj < b.nt && (int)(tasks[jj] >> 19) == pl; jj++) {
                        float v[VW];
                        vload<VW>(sRes + (size_t)jj * MP + m0, v);
#pragma unroll
                        for (int f = 0; f < VW; f++) acc[f] = fadd(acc[f], v[f]);
                    }
                    vstore<VW>(T.pout + (size_t)prow * MP + m0, acc);
                }
            }
            if (k + 1 < a.ts.n) __syncthreads();  // the next term reuses sRes
        }
    }
}

}  // namespace dcrf
