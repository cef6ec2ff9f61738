// meanfield.cu -- the kernels of one mean-field iteration on the device.
//
// One iteration of DenseCRF::inference (pydensecrf/densecrf/src/densecrf.cpp:
// 122-129) for all pairwise terms at once is three phases:
//
//   reduce  per vertex: sum the per-tile splat partials (in tile order) into
//           V[v] -- the end of the splat of Permutohedral::compute
//           (permutohedral.cpp:545-553);
//   blur    per axis j = 0..d (d..0 for the transpose): V' = V + 1/2 (V[n1] +
//           V[n2]) with the zero sentinel row (permutohedral.cpp:556-569);
//           terms of smaller d drop out of the later axis launches;
//   point   thread per point (tile of 256 points per CTA): slice every term
//           (permutohedral.cpp:574-584), apply the normalisation
//           (pairwise.cpp:78-79) and the label compatibility
//           (labelcompatibility.cpp:46-48,66-68,82-84), subtract from -U,
//           softmax (densecrf.cpp:98-106) -- and then, still in the same CTA,
//           splat the new Q of the tile into each term's per-(tile, vertex)
//           partials from shared memory, so Q never makes a round trip
//           through memory between iterations.
//
// The splat is deterministic: a tile's corners are grouped by vertex at
// lattice-build time (in point order), so every partial is a fixed-order sum,
// and the reduce adds a vertex's partials in tile order.  There are no float
// atomics anywhere.  Products and sums are rounded separately like the
// reference's x86 build; the value-size <= 2 arithmetic of seqCompute (double
// blur, (w*v)*alpha slice) is kept where the reference uses it.
#include <math.h>

#include "meanfield.cuh"

namespace dcrf {

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

// x -= compatibility(acc) (mean-field update), or, with kl_mode, kl += sum q * compatibility(acc)
// where x holds q.  Potts: -w acc; Diagonal: v * acc; Matrix: W acc (labelcompatibility.cpp:46-48,66-68,82-84).
template <int MP>
__device__ __forceinline__ void fold_compat(const TermDev &T, const float (&acc)[MP], float (&x)[MP], int M,
                                            bool kl_mode, double &kl) {
    if (T.ckind == DCRF_COMPAT_POTTS) {
        const float nw = -T.potts_w;
#pragma unroll
        for (int m = 0; m < MP; m++) {
            const float c = fmul(nw, acc[m]);
            if (kl_mode) {
                if (m < M) kl += (double)fmul(x[m], c);
            } else {
                x[m] = fsub(x[m], c);
            }
        }
    } else if (T.ckind == DCRF_COMPAT_DIAGONAL) {
#pragma unroll
        for (int m = 0; m < MP; m++)
            if (m < M) {
                const float c = fmul(__ldg(T.compat + m), acc[m]);
                if (kl_mode)
                    kl += (double)fmul(x[m], c);
                else
                    x[m] = fsub(x[m], c);
            }
    } else {
#pragma unroll
        for (int m = 0; m < MP; m++)
            if (m < M) {
                const float *row = T.compat + (size_t)m * M;
                float c = 0.f;
#pragma unroll
                for (int k = 0; k < MP; k++)
                    if (k < M) c = fadd(c, fmul(__ldg(row + k), acc[k]));
                if (kl_mode)
                    kl += (double)fmul(x[m], c);
                else
                    x[m] = fsub(x[m], c);
            }
    }
}

// Shared-memory budget of the point pass: a union of the vertex-row stage
// (slice phase) and the q rows + member lists (splat phase).
template <int MP>
struct PPSmem {
    static constexpr int MCAP = SPLAT_TILE * 6;  // staged members (corners of d <= 5)
    static constexpr int SPLAT_BYTES = SPLAT_TILE * MP * 4 + MCAP * 6 + (MCAP + 1) * 4;
    static constexpr int SV_ROWS = (SPLAT_BYTES / (MP * 4)) < 128 ? 128 : (SPLAT_BYTES / (MP * 4));
    static constexpr int BYTES = (SV_ROWS * MP * 4 > SPLAT_BYTES ? SV_ROWS * MP * 4 : SPLAT_BYTES);
};

// Slice of term T for the calling thread's point (tile-local tables), from the
// staged rows when the tile's vertex rows fit in shared memory.
template <int MP>
__device__ __forceinline__ void slice_tiled(const TermDev &T, int t, int li, bool staged, int pb,
                                            const float *__restrict__ sV, float (&acc)[MP]) {
#pragma unroll
    for (int m = 0; m < MP; m++) acc[m] = 0.f;
    const size_t tbase = (size_t)t * (T.d + 1) * SPLAT_TILE + li;
    for (int r = 0; r <= T.d; r++) {
        const int loc = T.tl_loc[tbase + (size_t)r * SPLAT_TILE];
        const float b = T.tl_w[tbase + (size_t)r * SPLAT_TILE];
        float v[MP];
        if (staged) {
            if constexpr (MP % 4 == 0) {
                const float4 *r4 = reinterpret_cast<const float4 *>(sV + loc * MP);
#pragma unroll
                for (int c = 0; c < MP / 4; c++) {
                    float4 x = r4[c];
                    v[4 * c] = x.x, v[4 * c + 1] = x.y, v[4 * c + 2] = x.z, v[4 * c + 3] = x.w;
                }
            } else {
#pragma unroll
                for (int m = 0; m < MP; m++) v[m] = sV[loc * MP + m];
            }
        } else {
            load_row<MP>(T.V + (size_t)(T.part_v[pb + loc] + 1) * MP, v);
        }
        if (T.seq) {  // seqCompute slice: (w * v) * alpha (permutohedral.cpp:520)
#pragma unroll
            for (int m = 0; m < MP; m++) acc[m] = fadd(acc[m], fmul(fmul(b, v[m]), T.alpha));
        } else {  // sseCompute slice: (w * alpha) * v (permutohedral.cpp:579-581)
            const float w = fmul(b, T.alpha);
#pragma unroll
            for (int m = 0; m < MP; m++) acc[m] = fadd(acc[m], fmul(w, v[m]));
        }
    }
}

template <int MP>
__global__ void __launch_bounds__(SPLAT_TILE, (MP <= 20 ? 3 : 2)) pointpass_kernel(const __grid_constant__ PPArgs a) {
    using SM = PPSmem<MP>;
    __shared__ __align__(16) unsigned char smem[SM::BYTES];
    __shared__ double sKL[SPLAT_TILE / 32];
    float *sV = reinterpret_cast<float *>(smem);
    float *sQ = reinterpret_cast<float *>(smem);
    float *sMw = reinterpret_cast<float *>(smem + SPLAT_TILE * MP * 4);
    int *sPmb = reinterpret_cast<int *>(smem + SPLAT_TILE * MP * 4 + SM::MCAP * 4);
    uint16_t *sMpt = reinterpret_cast<uint16_t *>(smem + SPLAT_TILE * MP * 4 + SM::MCAP * 4 + (SM::MCAP + 1) * 4);

    const int t = blockIdx.x;
    const int li = threadIdx.x;
    const int i = a.slot_pt[(size_t)t * SPLAT_TILE + li];
    const bool valid = i >= 0;
    const int N = a.N, M = a.M, mode = a.mode;
    // x: the logits of the update, or the given marginals (LOAD_Q / ONES); q after the softmax
    float x[MP];
#pragma unroll
    for (int m = 0; m < MP; m++) x[m] = 0.f;
    double kl = 0.0;
    const bool given = (mode & (PP_LOAD_Q | PP_ONES)) != 0;
    if (mode & PP_ONES) {
        if (valid) x[0] = 1.f;
    } else if (mode & PP_LOAD_Q) {
        if (valid) {
#pragma unroll
            for (int m = 0; m < MP; m++)
                if (m < M) x[m] = a.Qin[(size_t)m * N + i];
        }
    } else {
#pragma unroll
        for (int m = 0; m < MP; m++) x[m] = (valid && m < M && a.U) ? -a.U[(size_t)m * N + i] : 0.f;
    }
    if (mode & PP_MSG) {
        for (int k = 0; k < a.ts.n; k++) {
            const TermDev &T = a.ts.t[k];
            const int pb = T.tile_pbeg[t], np = T.tile_pbeg[t + 1] - pb;
            const bool staged = np <= SM::SV_ROWS;
            if (staged) {
                // stage the tile's vertex rows: row p = V[part_v[pb + p] + 1]
                if constexpr (MP % 4 == 0) {
                    constexpr int C4 = MP / 4;
                    float4 *d4 = reinterpret_cast<float4 *>(sV);
                    for (int x = li; x < np * C4; x += SPLAT_TILE) {
                        const int p = x / C4, c = x - p * C4;
                        d4[x] = __ldg(reinterpret_cast<const float4 *>(T.V + (size_t)(T.part_v[pb + p] + 1) * MP) + c);
                    }
                } else {
                    for (int x = li; x < np * MP; x += SPLAT_TILE) {
                        const int p = x / MP, c = x - p * MP;
                        sV[x] = __ldg(T.V + (size_t)(T.part_v[pb + p] + 1) * MP + c);
                    }
                }
            }
            __syncthreads();
            if (valid) {
                float acc[MP];
                slice_tiled<MP>(T, t, li, staged, pb, sV, acc);
                if (T.post_norm) {
                    const float nn = T.norm[i];
#pragma unroll
                    for (int m = 0; m < MP; m++) acc[m] = fmul(acc[m], nn);
                }
                // with given marginals this is the pairwise part of klDivergence
                // (densecrf.cpp:229-233): sum Q * compat(K Q)
                fold_compat<MP>(T, acc, x, M, given, kl);
            }
            __syncthreads();
        }
    }
    if (valid && !given) {
        // softmax (densecrf.cpp:98-106)
        float mx = x[0];
#pragma unroll
        for (int m = 1; m < MP; m++)
            if (m < M) mx = fmaxf(mx, x[m]);
        float s = 0.f;
#pragma unroll
        for (int m = 0; m < MP; m++)
            if (m < M) {
                x[m] = expf(fsub(x[m], mx));
                s = fadd(s, x[m]);
            }
#pragma unroll
        for (int m = 0; m < MP; m++) x[m] = m < M ? __fdiv_rn(x[m], s) : 0.f;
    }
    float (&q)[MP] = x;
    if (valid) {
        if (mode & PP_KL) {
            // entropy and unary parts (densecrf.cpp:216-226); log() there is the double overload
#pragma unroll
            for (int m = 0; m < MP; m++)
                if (m < M) {
                    kl += (double)q[m] * log((double)fmaxf(q[m], 1e-20f));
                    if (a.U) kl += (double)fmul(a.U[(size_t)m * N + i], q[m]);
                }
        }
        if (mode & PP_WRITE_Q) {
#pragma unroll
            for (int m = 0; m < MP; m++)
                if (m < M) a.Qout[(size_t)m * N + i] = q[m];
        }
        if (mode & PP_MAP) {
            int best = 0;
            float bv = q[0];
#pragma unroll
            for (int m = 1; m < MP; m++)
                if (m < M && q[m] > bv) {
                    bv = q[m];
                    best = m;
                }
            a.map_out[i] = (int16_t)best;
        }
    }
    if (mode & PP_KL) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) kl += __shfl_down_sync(0xffffffffu, kl, o);
        if ((li & 31) == 0) sKL[li >> 5] = kl;
        __syncthreads();
        if (li == 0) {
            double s = 0.0;
            for (int w = 0; w < SPLAT_TILE / 32; w++) s += sKL[w];
            a.kl_part[t] = s;
        }
    }
    if (mode & PP_SPLAT) {
        // splat the tile's q into each term's partials (every thread takes part)
        constexpr int G = Grp<MP>::G, CH = Grp<MP>::CH, NG = SPLAT_TILE / G;
        const int lg_ = li % G, gid = li / G;
        for (int k = 0; k < a.ts.n; k++) {
            const TermDev &T = a.ts.t[k];
            const float nn = (valid && T.pre_norm) ? T.norm[i] : 1.f;
#pragma unroll
            for (int m = 0; m < MP; m++) sQ[li * MP + m] = T.pre_norm ? fmul(q[m], nn) : q[m];
            const int pb = T.tile_pbeg[t], pe = T.tile_pbeg[t + 1];
            const int mbase = T.part_mbeg[pb], nmem = T.part_mbeg[pe] - mbase;
            const bool staged = nmem <= SM::MCAP;
            if (staged) {
                for (int x = li; x < nmem; x += SPLAT_TILE) {
                    sMpt[x] = T.mem_pt[mbase + x];
                    sMw[x] = T.mem_w[mbase + x];
                }
                for (int x = li; x <= pe - pb; x += SPLAT_TILE) sPmb[x] = T.part_mbeg[pb + x] - mbase;
            }
            __syncthreads();
            for (int p = pb + gid; p < pe; p += NG) {
                float acc[CH];
#pragma unroll
                for (int c = 0; c < CH; c++) acc[c] = 0.f;
                if (staged) {
                    const int mb = sPmb[p - pb], me = sPmb[p - pb + 1];
                    for (int e = mb; e < me; e++) {
                        const float w = sMw[e];
                        const float *row = sQ + sMpt[e] * MP + lg_;
#pragma unroll
                        for (int c = 0; c < CH; c++) acc[c] = fadd(acc[c], fmul(w, row[c * G]));
                    }
                } else {
                    const int mb = T.part_mbeg[p], me = T.part_mbeg[p + 1];
                    for (int e = mb; e < me; e++) {
                        const float w = T.mem_w[e];
                        const float *row = sQ + T.mem_pt[e] * MP + lg_;
#pragma unroll
                        for (int c = 0; c < CH; c++) acc[c] = fadd(acc[c], fmul(w, row[c * G]));
                    }
                }
                float *dst = T.partial + (size_t)p * MP + lg_;
#pragma unroll
                for (int c = 0; c < CH; c++) dst[c * G] = acc[c];
            }
            __syncthreads();
        }
    }
}

// Value-size-1 normalisation slice and raw lattice filter (point-order gather;
// used off the iteration loop).
template <int MP>
__global__ void __launch_bounds__(256) slice_kernel(const __grid_constant__ PPArgs a) {
    const int t = blockIdx.x;
    const int i = a.slot_pt[(size_t)t * SPLAT_TILE + threadIdx.x];
    if (i < 0) return;
    const int N = a.N, M = a.M;
    if (a.mode & PP_NORM) {
        // value size 1, seqCompute slice: out += (w * v) * alpha (permutohedral.cpp:513-521)
        for (int k = 0; k < a.ts.n; k++) {
            const TermDev &T = a.ts.t[k];
            float n = 0.f;
            for (int r = 0; r <= T.d; r++) {
                int o = T.off[(size_t)r * N + i] + 1;
                float w = T.bary[(size_t)r * N + i];
                n = fadd(n, fmul(fmul(w, __ldg(T.V + o)), T.alpha));
            }
            float out;
            if (a.ntype[k] == DCRF_NORMALIZE_SYMMETRIC)  // pairwise.cpp:54-57
                out = __double2float_rn(__ddiv_rn(1.0, __dsqrt_rn(__dadd_rn((double)n, 1e-20))));
            else if (a.ntype[k] == DCRF_NO_NORMALIZATION)
                out = n;  // raw K*1; the host derives the mean (pairwise.cpp:46-53)
            else  // pairwise.cpp:58-61
                out = __double2float_rn(__ddiv_rn(1.0, __dadd_rn((double)n, 1e-20)));
            a.norm_out[k][i] = out;
        }
        return;
    }
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
        if (m < M) a.Qout[(size_t)m * N + i] = acc[m];
}

template <int MP>
__global__ void __launch_bounds__(256) reduce_kernel(const __grid_constant__ ReduceArgs a) {
    constexpr int G = Grp<MP>::G, CH = Grp<MP>::CH;
    const long long gidx = ((long long)blockIdx.x * blockDim.x + threadIdx.x) / G;
    const int lg_ = threadIdx.x % G;
    if (gidx >= a.begin[a.n]) return;
    int k = 0;
    while (gidx >= a.begin[k + 1]) k++;
    const ReduceArgs::T &T = a.t[k];
    const int v = (int)(gidx - a.begin[k]);
    const int s0 = T.red_beg[v], s1 = T.red_beg[v + 1];
    float acc[CH];
#pragma unroll
    for (int c = 0; c < CH; c++) acc[c] = 0.f;
    // the group's lanes fetch G partial indices at a time; the rows are then
    // read back to back (independent loads), added in list order
    const unsigned gmask = (G == 32) ? 0xffffffffu : (((1u << G) - 1u) << ((threadIdx.x & 31) & ~(G - 1)));
    for (int b = s0; b < s1; b += G) {
        const int mine = (b + lg_ < s1) ? T.red_list[b + lg_] : 0;
        const int cnt = min(G, s1 - b);
        float rowv[G][CH];
#pragma unroll
        for (int j = 0; j < G; j++) {
            const int p = __shfl_sync(gmask, mine, j, G);
#pragma unroll
            for (int c = 0; c < CH; c++) rowv[j][c] = j < cnt ? T.partial[(size_t)p * MP + lg_ + c * G] : 0.f;
        }
#pragma unroll
        for (int j = 0; j < G; j++)
            if (j < cnt) {
#pragma unroll
                for (int c = 0; c < CH; c++) acc[c] = fadd(acc[c], rowv[j][c]);
            }
    }
    float *dst = T.V + (size_t)(v + 1) * MP + lg_;
#pragma unroll
    for (int c = 0; c < CH; c++) dst[c * G] = acc[c];
}

template <int MP, bool SEQ>
__global__ void __launch_bounds__(256) blur_kernel(const __grid_constant__ BlurArgs a) {
    constexpr int VEC = (MP % 4 == 0) ? 4 : (MP % 2 == 0) ? 2 : 1;
    constexpr int NV = MP / VEC;
    const long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= a.begin[a.n]) return;
    int k = 0;
    while (g >= a.begin[k + 1]) k++;
    const BlurArgs::T &T = a.t[k];
    const long long local = g - a.begin[k];
    const int v = (int)(local / NV);
    const int c = (int)(local - (long long)v * NV);
    const int2 nb = __ldg(T.nbr + (size_t)T.axis * T.L + v);
    const size_t o0 = (size_t)(v + 1) * MP + c * VEC, o1 = (size_t)nb.x * MP + c * VEC, o2 = (size_t)nb.y * MP + c * VEC;
    float x0[VEC], x1[VEC], x2[VEC], y[VEC];
    if constexpr (VEC == 4) {
        float4 p = *reinterpret_cast<const float4 *>(T.Vin + o0), q1 = *reinterpret_cast<const float4 *>(T.Vin + o1),
               q2 = *reinterpret_cast<const float4 *>(T.Vin + o2);
        x0[0] = p.x, x0[1] = p.y, x0[2] = p.z, x0[3] = p.w;
        x1[0] = q1.x, x1[1] = q1.y, x1[2] = q1.z, x1[3] = q1.w;
        x2[0] = q2.x, x2[1] = q2.y, x2[2] = q2.z, x2[3] = q2.w;
    } else {
#pragma unroll
        for (int e = 0; e < VEC; e++) {
            x0[e] = T.Vin[o0 + e];
            x1[e] = T.Vin[o1 + e];
            x2[e] = T.Vin[o2 + e];
        }
    }
#pragma unroll
    for (int e = 0; e < VEC; e++) {
        const float s = fadd(x1[e], x2[e]);
        if (SEQ)  // seqCompute: old + 0.5*(n1+n2) evaluated in double (permutohedral.cpp:505)
            y[e] = __double2float_rn(__dadd_rn((double)x0[e], 0.5 * (double)s));
        else  // sseCompute: float (permutohedral.cpp:566)
            y[e] = fadd(x0[e], fmul(0.5f, s));
    }
    if constexpr (VEC == 4) {
        *reinterpret_cast<float4 *>(T.Vout + o0) = make_float4(y[0], y[1], y[2], y[3]);
    } else {
#pragma unroll
        for (int e = 0; e < VEC; e++) T.Vout[o0 + e] = y[e];
    }
}

__global__ void transpose_kernel(const float *__restrict__ in, float *__restrict__ out, int rows, int cols) {
    __shared__ float tile[32][33];
    int c = blockIdx.x * 32 + threadIdx.x;
    int r0 = blockIdx.y * 32;
    for (int y = threadIdx.y; y < 32; y += blockDim.y) {
        int r = r0 + y;
        if (r < rows && c < cols) tile[y][threadIdx.x] = in[(size_t)r * cols + c];
    }
    __syncthreads();
    int oc = r0 + threadIdx.x;  // output column = input row
    for (int y = threadIdx.y; y < 32; y += blockDim.y) {
        int orow = blockIdx.x * 32 + y;  // output row = input column
        if (orow < cols && oc < rows) out[(size_t)orow * rows + oc] = tile[threadIdx.x][y];
    }
}

__global__ void features_2d_kernel(int W, int H, float sx, float sy, const uint8_t *__restrict__ rgb, float sr,
                                   float sg, float sb, float *__restrict__ feat) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    int N = W * H;
    if (p >= N) return;
    int j = p / W, i = p - j * W;
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

__global__ void argmax_kernel(const float *__restrict__ Q, int M, int N, int16_t *__restrict__ out) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= N) return;
    int best = 0;
    float bv = Q[p];
    for (int m = 1; m < M; m++) {
        float v = Q[(size_t)m * N + p];
        if (v > bv) {
            bv = v;
            best = m;
        }
    }
    out[p] = (int16_t)best;
}

// ---------------------------------------------------------------------------
template <int MP>
static cudaError_t pp_launch(const PPArgs &a, cudaStream_t s) {
    if (a.ntiles <= 0) return cudaSuccess;
    if (a.mode & (PP_NORM | PP_FILTER))
        DCRF_LAUNCH(slice_kernel<MP><<<a.ntiles, SPLAT_TILE, 0, s>>>(a));
    else
        DCRF_LAUNCH(pointpass_kernel<MP><<<a.ntiles, SPLAT_TILE, 0, s>>>(a));
    return cudaGetLastError();
}

cudaError_t launch_pointpass(const PPArgs &a, int MP, cudaStream_t s) {
    switch (MP) {
        case 1: return pp_launch<1>(a, s);
        case 2: return pp_launch<2>(a, s);
        case 4: return pp_launch<4>(a, s);
        case 8: return pp_launch<8>(a, s);
        case 12: return pp_launch<12>(a, s);
        case 16: return pp_launch<16>(a, s);
        case 20: return pp_launch<20>(a, s);
        case 24: return pp_launch<24>(a, s);
        case 28: return pp_launch<28>(a, s);
        case 32: return pp_launch<32>(a, s);
        default: return cudaErrorInvalidValue;
    }
}

template <int MP>
static cudaError_t red_launch(const ReduceArgs &a, cudaStream_t s) {
    long long threads = a.begin[a.n] * Grp<MP>::G;
    if (threads > 0) DCRF_LAUNCH(reduce_kernel<MP><<<(unsigned)((threads + 255) / 256), 256, 0, s>>>(a));
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
    if (threads > 0) DCRF_LAUNCH(blur_kernel<MP, SEQ><<<(unsigned)((threads + 255) / 256), 256, 0, s>>>(a));
    return cudaGetLastError();
}

cudaError_t launch_blur(const BlurArgs &a, int MP, bool seq, cudaStream_t s) {
#define DCRF_BL(X)                                                    \
    case X:                                                           \
        return seq ? blur_launch<X, true>(a, s) : blur_launch<X, false>(a, s);
    switch (MP) {
        DCRF_BL(1) DCRF_BL(2) DCRF_BL(4) DCRF_BL(8) DCRF_BL(12) DCRF_BL(16) DCRF_BL(20) DCRF_BL(24) DCRF_BL(28)
        DCRF_BL(32)
        default: return cudaErrorInvalidValue;
    }
#undef DCRF_BL
}

cudaError_t launch_transpose(const float *in, float *out, int rows, int cols, cudaStream_t s) {
    if (rows <= 0 || cols <= 0) return cudaSuccess;
    dim3 grid((cols + 31) / 32, (rows + 31) / 32), block(32, 8);
    DCRF_LAUNCH(transpose_kernel<<<grid, block, 0, s>>>(in, out, rows, cols));
    return cudaGetLastError();
}

cudaError_t launch_features_2d(int W, int H, float sx, float sy, const uint8_t *rgb, float sr, float sg, float sb,
                               float *feat, cudaStream_t s) {
    int N = W * H;
    if (N > 0) DCRF_LAUNCH(features_2d_kernel<<<(N + 255) / 256, 256, 0, s>>>(W, H, sx, sy, rgb, sr, sg, sb, feat));
    return cudaGetLastError();
}

cudaError_t launch_scale_features(const float *in, float *out, const float *P, int d, int N, int full,
                                  cudaStream_t s) {
    if (N > 0) DCRF_LAUNCH(scale_features_kernel<<<(N + 255) / 256, 256, 0, s>>>(in, out, P, d, N, full));
    return cudaGetLastError();
}

cudaError_t launch_argmax(const float *Q, int M, int N, int16_t *out, cudaStream_t s) {
    if (N > 0) DCRF_LAUNCH(argmax_kernel<<<(N + 255) / 256, 256, 0, s>>>(Q, M, N, out));
    return cudaGetLastError();
}

}  // namespace dcrf
