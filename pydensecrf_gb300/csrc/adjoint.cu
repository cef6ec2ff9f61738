// adjoint.cu -- device kernels of the hand-written adjoint of T mean-field
// iterations (the device form of DenseCRF::gradient,
// pydensecrf/densecrf/src/densecrf.cpp:238-297).
//
// All point quantities are slot-major [M][nslots] (empty slots hold zero).
// Reductions are two-level and deterministic: per-block partial sums in
// double, then one block adds them in block order.
#include <algorithm>

#include "adjoint.cuh"
#include "labelprod.cuh"

namespace dcrf {

// A row of MP floats from global memory (float4 loads when MP % 4 == 0).
template <int MP>
__device__ __forceinline__ void row_load(const float *__restrict__ p, float (&v)[MP]) {
    if constexpr (MP % 4 == 0) {
#pragma unroll
        for (int c = 0; c < MP / 4; c++) {
            const float4 q = __ldg(reinterpret_cast<const float4 *>(p) + c);
            v[4 * c] = q.x, v[4 * c + 1] = q.y, v[4 * c + 2] = q.z, v[4 * c + 3] = q.w;
        }
    } else {
#pragma unroll
        for (int m = 0; m < MP; m++) v[m] = __ldg(p + m);
    }
}

// All label-valued buffers here are slot rows [ns][ld] (ld = padded label
// count); labels m >= M and empty slots are written as 0.

// b = Q * sum(x .* Q) - x .* Q  per point: the softmax adjoint with the
// reference's sign (sumAndNormalize, densecrf.cpp:107-114, applied to x .* Q);
// with du, also du += b.  Rows are read and written as float4 vectors.
template <int MP>
__global__ void __launch_bounds__(256) softmax_adjoint_kernel(const float *__restrict__ Q, const float *__restrict__ x,
                                                              float *__restrict__ b, float *__restrict__ du, int M,
                                                              int ns, const int *__restrict__ slot_pt) {
    const size_t s = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= (size_t)ns) return;
    float q[MP], xx[MP], o[MP];
    const bool ok = slot_pt[s] >= 0;
#pragma unroll
    for (int c = 0; c < MP / 4; c++) {
        float4 a4 = make_float4(0.f, 0.f, 0.f, 0.f), b4 = a4;
        if (ok) {
            a4 = reinterpret_cast<const float4 *>(Q + s * MP)[c];
            b4 = reinterpret_cast<const float4 *>(x + s * MP)[c];
        }
        q[4 * c] = a4.x, q[4 * c + 1] = a4.y, q[4 * c + 2] = a4.z, q[4 * c + 3] = a4.w;
        xx[4 * c] = b4.x, xx[4 * c + 1] = b4.y, xx[4 * c + 2] = b4.z, xx[4 * c + 3] = b4.w;
    }
    float dot = 0.f;
#pragma unroll
    for (int m = 0; m < MP; m++)
        if (m < M) dot = fmaf(xx[m], q[m], dot);
#pragma unroll
    for (int m = 0; m < MP; m++) o[m] = (ok && m < M) ? fmaf(q[m], dot, -xx[m] * q[m]) : 0.f;
#pragma unroll
    for (int c = 0; c < MP / 4; c++) {
        const float4 v = make_float4(o[4 * c], o[4 * c + 1], o[4 * c + 2], o[4 * c + 3]);
        reinterpret_cast<float4 *>(b + s * MP)[c] = v;
        if (du) {
            float4 u = reinterpret_cast<const float4 *>(du + s * MP)[c];
            u.x += v.x, u.y += v.y, u.z += v.z, u.w += v.w;
            reinterpret_cast<float4 *>(du + s * MP)[c] = u;
        }
    }
}

// The same for M <= 2 (rows of M floats).
__global__ void softmax_adjoint_small_kernel(const float *__restrict__ Q, const float *__restrict__ x,
                                             float *__restrict__ b, float *__restrict__ du, int M, int ld, int ns,
                                             const int *__restrict__ slot_pt) {
    const size_t s = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= (size_t)ns) return;
    const float *q = Q + s * ld, *xx = x + s * ld;
    float *o = b + s * ld;
    if (slot_pt[s] < 0) {
        for (int m = 0; m < ld; m++) o[m] = 0.f;
        return;
    }
    float dot = 0.f;
    for (int m = 0; m < M; m++) dot = fmaf(xx[m], q[m], dot);
    for (int m = 0; m < ld; m++) {
        o[m] = m < M ? fmaf(q[m], dot, -xx[m] * q[m]) : 0.f;
        if (du) du[s * ld + m] += o[m];
    }
}

// y (+)= C x, or C^T x, per point (labelcompatibility.cpp:46-48,66-68,82-87).
// One thread per row; the row is read and written as float4 vectors and the
// Matrix is staged in shared memory (transposed when applying C).
template <int MP>
__global__ void __launch_bounds__(256) compat_kernel(const float *__restrict__ x, float *__restrict__ y, int M, int ns,
                                                     int kind, float potts_w, const float *__restrict__ C,
                                                     int transpose, int accumulate) {
    __shared__ float sC[MP * MP];  // sC[k][m]: weight of x_k in y_m
    if (kind == DCRF_COMPAT_MATRIX) {
        for (int e = threadIdx.x; e < MP * MP; e += blockDim.x) {
            const int k = e / MP, m = e - k * MP;
            sC[e] = (k < M && m < M) ? (transpose ? C[k * M + m] : C[m * M + k]) : 0.f;
        }
        __syncthreads();
    }
    const size_t s = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= (size_t)ns) return;
    float xv[MP], v[MP];
#pragma unroll
    for (int c = 0; c < MP / 4; c++) {
        const float4 q = reinterpret_cast<const float4 *>(x + s * MP)[c];
        xv[4 * c] = q.x, xv[4 * c + 1] = q.y, xv[4 * c + 2] = q.z, xv[4 * c + 3] = q.w;
    }
    if (kind == DCRF_COMPAT_POTTS) {
#pragma unroll
        for (int m = 0; m < MP; m++) v[m] = m < M ? -potts_w * xv[m] : 0.f;
    } else if (kind == DCRF_COMPAT_DIAGONAL) {
#pragma unroll
        for (int m = 0; m < MP; m++) v[m] = m < M ? __ldg(C + m) * xv[m] : 0.f;
    } else {
#pragma unroll
        for (int m = 0; m < MP; m++) v[m] = 0.f;
#pragma unroll
        for (int k = 0; k < MP; k++) {
            if (k >= M) continue;
#pragma unroll
            for (int m = 0; m < MP; m++) v[m] = fmaf(sC[k * MP + m], xv[k], v[m]);
        }
    }
    float4 *yr = reinterpret_cast<float4 *>(y + s * MP);
#pragma unroll
    for (int c = 0; c < MP / 4; c++) {
        float4 o = make_float4(v[4 * c], v[4 * c + 1], v[4 * c + 2], v[4 * c + 3]);
        if (accumulate) {
            const float4 p = yr[c];
            o.x += p.x, o.y += p.y, o.z += p.z, o.w += p.w;
        }
        yr[c] = o;
    }
}

// Labels M <= 2 (rows of 1 or 2 floats): the scalar form of the same.
__global__ void compat_small_kernel(const float *__restrict__ x, float *__restrict__ y, int M, int ld, int ns, int kind,
                                    float potts_w, const float *__restrict__ C, int transpose, int accumulate) {
    const size_t s = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= (size_t)ns) return;
    const float *xx = x + s * ld;
    float *yy = y + s * ld;
    float v[2] = {0.f, 0.f};
    for (int m = 0; m < M; m++) {
        if (kind == DCRF_COMPAT_POTTS)
            v[m] = -potts_w * xx[m];
        else if (kind == DCRF_COMPAT_DIAGONAL)
            v[m] = C[m] * xx[m];
        else
            for (int k = 0; k < M; k++) v[m] = fmaf(transpose ? C[k * M + m] : C[m * M + k], xx[k], v[m]);
    }
    for (int m = 0; m < ld; m++) yy[m] = accumulate ? yy[m] + v[m] : v[m];
}

// y = x .* norm^pw per point (pw in 1..3), one thread per float4 of a row (ld % 4 == 0)
// or per row (ld < 4)
__global__ void scale_norm_kernel(const float *__restrict__ x, float *__restrict__ y, const float *__restrict__ norm,
                                  int ld, int ns, int pw) {
    const int nv = ld % 4 == 0 ? ld / 4 : 1;
    const size_t gi = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (gi >= (size_t)ns * nv) return;
    const size_t s = gi / nv;
    const float n = norm[s];
    const float f = pw == 1 ? n : pw == 2 ? n * n : n * n * n;
    if (ld % 4 == 0) {
        float4 q = reinterpret_cast<const float4 *>(x)[gi];
        q.x *= f, q.y *= f, q.z *= f, q.w *= f;
        reinterpret_cast<float4 *>(y)[gi] = q;
    } else {
        for (int m = 0; m < ld; m++) y[s * ld + m] = x[s * ld + m] * f;
    }
}

// y = scale * (x1 .* x2 + x3 .* x4) .* norm^pw per point (x3/x4 may be null; norm null: pw ignored)
__global__ void prod_kernel(const float *__restrict__ x1, const float *__restrict__ x2, const float *__restrict__ x3,
                            const float *__restrict__ x4, float scale, const float *__restrict__ norm, int pw,
                            float *__restrict__ y, int ld, int ns) {
    const size_t o = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= (size_t)ns * ld) return;
    float f = scale;
    if (norm) {
        const float n = norm[o / ld];
        f *= pw == 1 ? n : pw == 2 ? n * n : n * n * n;
    }
    float v = x1[o] * x2[o];
    if (x3) v = fmaf(x3[o], x4[o], v);
    y[o] = v * f;
}

__global__ void fill_kernel(float *__restrict__ y, float v, int M, int ld, int ns, const int *__restrict__ slot_pt) {
    const size_t s = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= (size_t)ns) return;
    const float val = slot_pt[s] >= 0 ? v : 0.f;
    for (int m = 0; m < ld; m++) y[s * ld + m] = m < M ? val : 0.f;
}

// The normalisation's coefficients of the kernel-parameter gradient
// (DenseKernel::featureGradient, pairwise.cpp:87-114) in one pass per point:
//   ys = C Q (times norm when the forward filter starts with the norm)
//   x1 = sum over labels of c1, with
//     SYMMETRIC c1 = 1/2 (b . C y + F . C Q) norm^3
//     AFTER     c1 = (b . C y) norm^2
//     BEFORE    c1 = (F . C Q) norm^2
// (y = K_raw [norm] Q, F = K_raw^T x~); the compatibilities are symmetric.
template <int MP>
__global__ void __launch_bounds__(256) norm_terms_kernel(const float *__restrict__ b, const float *__restrict__ y,
                                                         const float *__restrict__ F, const float *__restrict__ Q,
                                                         const float *__restrict__ norm, int M, int ns, int ntype,
                                                         int kind, float potts_w, const float *__restrict__ C,
                                                         float *__restrict__ ys, float *__restrict__ x1) {
    __shared__ float sC[MP * MP];  // sC[k][m]
    if (kind == DCRF_COMPAT_MATRIX) {
        for (int e = threadIdx.x; e < MP * MP; e += blockDim.x) {
            const int k = e / MP, m = e - k * MP;
            sC[e] = (k < M && m < M) ? C[m * M + k] : 0.f;
        }
        __syncthreads();
    }
    const size_t s = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= (size_t)ns) return;
    auto apply = [&](const float (&x)[MP], float (&o)[MP]) {
        if (kind == DCRF_COMPAT_POTTS) {
#pragma unroll
            for (int m = 0; m < MP; m++) o[m] = m < M ? -potts_w * x[m] : 0.f;
        } else if (kind == DCRF_COMPAT_DIAGONAL) {
#pragma unroll
            for (int m = 0; m < MP; m++) o[m] = m < M ? __ldg(C + m) * x[m] : 0.f;
        } else {
#pragma unroll
            for (int m = 0; m < MP; m++) o[m] = 0.f;
#pragma unroll
            for (int k = 0; k < MP; k++) {
                if (k >= M) continue;
#pragma unroll
                for (int m = 0; m < MP; m++) o[m] = fmaf(sC[k * MP + m], x[k], o[m]);
            }
        }
    };
    const float n = norm[s];
    const bool pre = ntype == DCRF_NORMALIZE_SYMMETRIC || ntype == DCRF_NORMALIZE_BEFORE;
    float q[MP], cq[MP];
    row_load<MP>(Q + s * MP, q);
    apply(q, cq);
    float out[MP];
#pragma unroll
    for (int m = 0; m < MP; m++) out[m] = pre ? cq[m] * n : cq[m];
#pragma unroll
    for (int c = 0; c < MP / 4; c++)
        reinterpret_cast<float4 *>(ys + s * MP)[c] = make_float4(out[4 * c], out[4 * c + 1], out[4 * c + 2], out[4 * c + 3]);
    if (ntype == DCRF_NO_NORMALIZATION) return;
    float bb[MP], cy[MP], ff[MP];
    row_load<MP>(b + s * MP, bb);
    if (ntype != DCRF_NORMALIZE_BEFORE) {
        float yy[MP];
        row_load<MP>(y + s * MP, yy);
        apply(yy, cy);
    }
    if (ntype != DCRF_NORMALIZE_AFTER) row_load<MP>(F + s * MP, ff);
    float t = 0.f;
#pragma unroll
    for (int m = 0; m < MP; m++) {
        if (m >= M) continue;
        float c1;
        if (ntype == DCRF_NORMALIZE_SYMMETRIC)
            c1 = 0.5f * fmaf(ff[m], cq[m], bb[m] * cy[m]) * (n * n * n);
        else if (ntype == DCRF_NORMALIZE_AFTER)
            c1 = bb[m] * cy[m] * (n * n);
        else
            c1 = ff[m] * cq[m] * (n * n);
        t = fadd(t, c1);
    }
    x1[s] = t;
}

// One-hot rows of a labelling (densecrf.cpp:165-168): row s gets 1 at the
// label of its point when 0 <= label < M (else an all-zero row).
__global__ void onehot_kernel(const int16_t *__restrict__ labels, int M, int ld, int ns,
                              const int *__restrict__ slot_pt, float *__restrict__ out) {
    const size_t s = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= (size_t)ns) return;
    const int pt = slot_pt[s];
    const int l = pt >= 0 ? (int)labels[pt] : -1;
    for (int m = 0; m < ld; m++) out[s * ld + m] = (m == l && l < M) ? 1.f : 0.f;
}

// The same one-hot rows in the label-chunk layout of more than 32 labels
// (chunk_offset), all MP padded labels of every slot written.
__global__ void onehot_chunked_kernel(const int16_t *__restrict__ labels, int M, int MP, int ns,
                                      const int *__restrict__ slot_pt, float *__restrict__ out) {
    const size_t s = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= (size_t)ns) return;
    const int pt = slot_pt[s];
    const int l = pt >= 0 ? (int)labels[pt] : -1;
    for (int m = 0; m < MP; m++) out[chunk_offset((size_t)ns, MP, s, m)] = (m == l && l < M) ? 1.f : 0.f;
}

// energy[pt] (+)= scale * x[slot of pt][label of pt] for 0 <= label < M, else
// (+)= 0 (densecrf.cpp:146-150, 169-174)
__global__ void label_energy_kernel(const float *__restrict__ x, const int16_t *__restrict__ labels, int M, int ld,
                                    int ns, int N, const int *__restrict__ pt_slot, float scale, int accumulate,
                                    float *__restrict__ energy) {
    const int pt = blockIdx.x * blockDim.x + threadIdx.x;
    if (pt >= N) return;
    const int l = labels[pt];
    const float v = (x && l >= 0 && l < M) ? scale * x[chunk_offset((size_t)ns, ld, (size_t)pt_slot[pt], l)] : 0.f;
    energy[pt] = accumulate ? energy[pt] + v : v;
}

// out[s] = sum over labels of x (one value per slot)
__global__ void row_sum_kernel(const float *__restrict__ x, float *__restrict__ out, int M, int ld, int ns) {
    const size_t s = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= (size_t)ns) return;
    float t = 0.f;
    for (int m = 0; m < M; m++) t = fadd(t, x[s * ld + m]);
    out[s] = t;
}

// Label products of slot rows a, b over the slots, per block of LP_ROWS slots
// (staged in shared memory):
//  mode 0 (per label):  part[blk][m]      (+)= sum_s a[s][m] * b[s][m]
//  mode 1 (outer):      part[blk][m*M+k]  (+)= sum_s a[s][m] * b[s][k]
// (block_label_products); the block's result is stored (or added, accumulate)
// block-major, so that the block's writes are contiguous.  Padding slots
// (slot_pt < 0) are left out whatever they contain.
constexpr int LP_ROWS = 128;

__global__ void __launch_bounds__(256) label_products_kernel(const float *__restrict__ a, const float *__restrict__ b,
                                                             int M, int ld, int ns, const int *__restrict__ slot_pt,
                                                             int mode, int accumulate, double *__restrict__ part) {
    extern __shared__ float sab[];  // [LP_ROWS][ld] of a, then of b; the groups' sums after them
    float *sa = sab, *sb = sab + LP_ROWS * ld;
    const int K = mode == 0 ? M : M * M;
    const size_t r0 = (size_t)blockIdx.x * LP_ROWS;
    for (int e = threadIdx.x; e < LP_ROWS * ld; e += blockDim.x) {
        const int r = e / ld;
        const size_t sl = r0 + r;
        const bool ok = sl < (size_t)ns && slot_pt[sl] >= 0;
        sa[e] = ok ? a[r0 * ld + e] : 0.f;
        sb[e] = ok ? b[r0 * ld + e] : 0.f;
    }
    __syncthreads();
    block_label_products(sa, sb, LP_ROWS, ld, M, mode, sb + LP_ROWS * ld, part + (size_t)blockIdx.x * K, accumulate);
}

// out[k] (+)= sum over blocks of part[blk][k] (block-major partials): one warp
// per output, lanes striding over the blocks, then a fixed shuffle tree
__global__ void sum_parts_bm_kernel(const double *__restrict__ part, int nblk, int K, double *__restrict__ out,
                                    int accumulate) {
    const int k = blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (k >= K) return;
    double t = 0.0;
    for (int b = lane; b < nblk; b += 32) t += part[(size_t)b * K + k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
    if (lane == 0) out[k] = accumulate ? out[k] + t : t;
}

cudaError_t launch_sum_parts_bm(const double *part, int nblk, int K, double *out, int accumulate, cudaStream_t s) {
    DCRF_LAUNCH(sum_parts_bm_kernel<<<(K + 7) / 8, 256, 0, s>>>(part, nblk, K, out, accumulate));
    return cudaGetLastError();
}

// out[k] (+)= sum over blocks of part[k][blk] (output-major partials): one
// warp per output, lanes striding over the blocks, then a fixed shuffle tree
__global__ void sum_parts_kernel(const double *__restrict__ part, int nblk, int K, double *__restrict__ out,
                                 int accumulate) {
    const int k = blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (k >= K) return;
    double t = 0.0;
    for (int b = lane; b < nblk; b += 32) t += part[(size_t)k * nblk + b];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
    if (lane == 0) out[k] = accumulate ? out[k] + t : t;
}

// Feature gradient of the slice (the per-point part of Permutohedral::gradient,
// permutohedral.cpp:660-690): with V the blurred lattice of one direction and
// z the contraction values, df[i][j-1] += sum_k z[k] * sf[j-1] * (sm_k - j * ra_j[k]),
// ra_j = alpha/(d+1) * (V[off[r0]] - V[off[r1]]), r0 = d - rank_j, r1 = r0+1 mod (d+1),
// sm the running sum of ra_0..ra_{j-1}.  Summed over the labels first:
//   D_j = sum_k z[k] ra_j[k] = alpha * sum_k z[k] (V[r0][k] - V[r1][k])
//   df[i][j-1] += sf[j-1] * (D_0 + ... + D_{j-1} - j D_j)
// (the per-label differences are taken first, as in the per-label form), so a
// thread keeps only the point's z row and streams the corner rows through it.
// (zrow null: z = 1 for every label; M: the labels of this pair)
template <int MP>
__device__ __forceinline__ void slice_grad_pair(const SliceGradArgs &a, const float *V, const float *zrow, float alpha,
                                                const float *zscale, int M, size_t s, int i,
                                                float (&grad)[DCRF_MAX_D]) {
    constexpr int VW = MP % 4 == 0 ? 4 : 1;
    const int d = a.d, N = a.N;
    float z[MP];
    if (zrow) {
        row_load<MP>(zrow + s * MP, z);
    } else {
#pragma unroll
        for (int m = 0; m < MP; m++) z[m] = 1.f;
    }
    if (zscale) {
        const float f = zscale[s];
#pragma unroll
        for (int m = 0; m < MP; m++) z[m] = z[m] * f;
    }
#pragma unroll
    for (int m = 0; m < MP; m++)
        if (m >= M) z[m] = 0.f;
    // the row of corner r (row 0 is the zero sentinel)
    auto row = [&](int r) -> const float * { return V + (size_t)(a.off[(size_t)r * N + i] + 1) * MP; };
    float S = 0.f;  // D_0 + ... + D_{j-1}
    // unrolled over the largest d so that grad[] stays in registers
#pragma unroll
    for (int j = 0; j <= DCRF_MAX_D; j++) {
        if (j > d) break;
        const int r0 = d - (int)a.rank[(size_t)j * N + i];
        const int r1 = r0 + 1 > d ? 0 : r0 + 1;
        const float *p0 = row(r0), *p1 = row(r1);
        float dot = 0.f;
#pragma unroll
        for (int c = 0; c < MP / VW; c++) {
            float v0[VW], v1[VW];
            row_load<VW>(p0 + c * VW, v0);
            row_load<VW>(p1 + c * VW, v1);
#pragma unroll
            for (int e = 0; e < VW; e++) dot = fmaf(z[c * VW + e], v0[e] - v1[e], dot);
        }
        const float Dj = alpha * dot;
        if (j > 0) grad[j - 1] += a.sf[j - 1] * (S - (float)j * Dj);
        S += Dj;
    }
}

template <int MP>
__global__ void __launch_bounds__(256, 4) slice_grad_kernel(SliceGradArgs a) {
    const size_t s = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= (size_t)a.nslots) return;
    const int i = a.slot_pt[s];
    if (i < 0) return;
    float grad[DCRF_MAX_D];
#pragma unroll
    for (int j = 0; j < DCRF_MAX_D; j++) grad[j] = 0.f;
    slice_grad_pair<MP>(a, a.V, a.z, a.alpha, nullptr, a.M, s, i, grad);
    if (a.V2) slice_grad_pair<MP>(a, a.V2, a.z2, a.alpha2, a.z2scale, a.M, s, i, grad);
    if (a.V3) slice_grad_pair<1>(a, a.V3, nullptr, a.alpha3, nullptr, 1, s, i, grad);
    if (a.V4) slice_grad_pair<1>(a, a.V4, a.z4, a.alpha4, nullptr, 1, s, i, grad);
#pragma unroll
    for (int j = 0; j < DCRF_MAX_D; j++)
        if (j < a.d) a.df[(size_t)i * a.d + j] += grad[j];
}

// Kernel-parameter gradient from the feature gradient: DIAG g[j] = sum_n f[j][n] fg[n][j];
// FULL g[j + d*j'] = sum_n fg[n][j] f[j'][n] (pairwise.cpp:152-163).  Per-block partials.
__global__ void __launch_bounds__(256) kernel_param_grad_kernel(const float *__restrict__ f, const float *__restrict__ fg,
                                                                int d, int N, int full, double *__restrict__ part) {
    extern __shared__ double sred[];
    const int K = full ? d * d : d;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const size_t n = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const bool ok = n < (size_t)N;
    for (int kk = 0; kk < K; kk++) {
        const int j = full ? kk % d : kk, jj = full ? kk / d : kk;
        double v = ok ? (double)fg[n * d + j] * (double)f[(size_t)jj * N + n] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0) sred[warp * K + kk] = v;
    }
    __syncthreads();
    for (int kk = threadIdx.x; kk < K; kk += blockDim.x) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x / 32); w++) t += sred[w * K + kk];
        part[(size_t)kk * gridDim.x + blockIdx.x] = t;
    }
}

// ---------------------------------------------------------------------------
static unsigned blocks(size_t n) { return (unsigned)((n + 255) / 256); }

cudaError_t launch_softmax_adjoint(const float *Q, const float *x, float *b, float *du, int M, int ns,
                                   const int *slot_pt, cudaStream_t s) {
    switch (pad_labels(M)) {
#define DCRF_SA(X) \
    case X: DCRF_LAUNCH(softmax_adjoint_kernel<X><<<blocks(ns), 256, 0, s>>>(Q, x, b, du, M, ns, slot_pt)); break;
        DCRF_SA(4) DCRF_SA(8) DCRF_SA(12) DCRF_SA(16) DCRF_SA(20) DCRF_SA(24) DCRF_SA(28) DCRF_SA(32)
#undef DCRF_SA
        default:
            DCRF_LAUNCH(softmax_adjoint_small_kernel<<<blocks(ns), 256, 0, s>>>(Q, x, b, du, M, pad_labels(M), ns,
                                                                                slot_pt));
    }
    return cudaGetLastError();
}

template <int MP>
static cudaError_t compat_launch(const float *x, float *y, int M, int ns, int kind, float potts_w, const float *C,
                                 int transpose, int accumulate, cudaStream_t s) {
    DCRF_LAUNCH(compat_kernel<MP><<<blocks(ns), 256, 0, s>>>(x, y, M, ns, kind, potts_w, C, transpose, accumulate));
    return cudaGetLastError();
}

cudaError_t launch_compat(const float *x, float *y, int M, int ns, int kind, float potts_w, const float *C,
                          int transpose, int accumulate, cudaStream_t s) {
    switch (pad_labels(M)) {
        case 4: return compat_launch<4>(x, y, M, ns, kind, potts_w, C, transpose, accumulate, s);
        case 8: return compat_launch<8>(x, y, M, ns, kind, potts_w, C, transpose, accumulate, s);
        case 12: return compat_launch<12>(x, y, M, ns, kind, potts_w, C, transpose, accumulate, s);
        case 16: return compat_launch<16>(x, y, M, ns, kind, potts_w, C, transpose, accumulate, s);
        case 20: return compat_launch<20>(x, y, M, ns, kind, potts_w, C, transpose, accumulate, s);
        case 24: return compat_launch<24>(x, y, M, ns, kind, potts_w, C, transpose, accumulate, s);
        case 28: return compat_launch<28>(x, y, M, ns, kind, potts_w, C, transpose, accumulate, s);
        case 32: return compat_launch<32>(x, y, M, ns, kind, potts_w, C, transpose, accumulate, s);
        default:
            DCRF_LAUNCH(compat_small_kernel<<<blocks(ns), 256, 0, s>>>(x, y, M, pad_labels(M), ns, kind, potts_w, C,
                                                                       transpose, accumulate));
            return cudaGetLastError();
    }
}

cudaError_t launch_scale_norm(const float *x, float *y, const float *norm, int M, int ns, int pw, cudaStream_t s) {
    const int ld = pad_labels(M);
    const size_t n = (size_t)ns * (ld % 4 == 0 ? ld / 4 : 1);
    DCRF_LAUNCH(scale_norm_kernel<<<blocks(n), 256, 0, s>>>(x, y, norm, ld, ns, pw));
    return cudaGetLastError();
}

cudaError_t launch_prod(const float *x1, const float *x2, const float *x3, const float *x4, float scale,
                        const float *norm, int pw, float *y, int M, int ns, cudaStream_t s) {
    const int ld = pad_labels(M);
    DCRF_LAUNCH(prod_kernel<<<blocks((size_t)ns * ld), 256, 0, s>>>(x1, x2, x3, x4, scale, norm, pw, y, ld, ns));
    return cudaGetLastError();
}

cudaError_t launch_fill(float *y, float v, int M, int ns, const int *slot_pt, cudaStream_t s) {
    DCRF_LAUNCH(fill_kernel<<<blocks(ns), 256, 0, s>>>(y, v, M, pad_labels(M), ns, slot_pt));
    return cudaGetLastError();
}

cudaError_t launch_row_sum(const float *x, float *out, int M, int ns, cudaStream_t s) {
    DCRF_LAUNCH(row_sum_kernel<<<blocks(ns), 256, 0, s>>>(x, out, M, pad_labels(M), ns));
    return cudaGetLastError();
}

cudaError_t launch_norm_terms(const float *b, const float *y, const float *F, const float *Q, const float *norm,
                              int M, int ns, int ntype, int kind, float potts_w, const float *C, float *ys,
                              float *x1, cudaStream_t s) {
    switch (pad_labels(M)) {
#define DCRF_NT(X)                                                                                               \
    case X:                                                                                                      \
        DCRF_LAUNCH(norm_terms_kernel<X><<<blocks(ns), 256, 0, s>>>(b, y, F, Q, norm, M, ns, ntype, kind, potts_w, \
                                                                    C, ys, x1));                                 \
        break;
        DCRF_NT(4) DCRF_NT(8) DCRF_NT(12) DCRF_NT(16) DCRF_NT(20) DCRF_NT(24) DCRF_NT(28) DCRF_NT(32)
#undef DCRF_NT
        default: return cudaErrorInvalidValue;  // M <= 2 takes the unfused path
    }
    return cudaGetLastError();
}

cudaError_t launch_onehot_chunked(const int16_t *labels, int M, int MP, int ns, const int *slot_pt, float *out,
                                  cudaStream_t s) {
    DCRF_LAUNCH(onehot_chunked_kernel<<<blocks(ns), 256, 0, s>>>(labels, M, MP, ns, slot_pt, out));
    return cudaGetLastError();
}

cudaError_t launch_onehot(const int16_t *labels, int M, int ns, const int *slot_pt, float *out, cudaStream_t s) {
    DCRF_LAUNCH(onehot_kernel<<<blocks(ns), 256, 0, s>>>(labels, M, pad_labels(M), ns, slot_pt, out));
    return cudaGetLastError();
}

cudaError_t launch_label_energy(const float *x, const int16_t *labels, int M, int ns, int N, const int *pt_slot,
                                float scale, int accumulate, float *energy, cudaStream_t s) {
    DCRF_LAUNCH(label_energy_kernel<<<blocks(N), 256, 0, s>>>(x, labels, M, pad_labels(M), ns, N, pt_slot, scale,
                                                               accumulate, energy));
    return cudaGetLastError();
}

int label_products_blocks(int ns) { return (ns + LP_ROWS - 1) / LP_ROWS; }

cudaError_t launch_sum_parts(const double *part, int nblk, int K, double *out, int accumulate, cudaStream_t s) {
    DCRF_LAUNCH(sum_parts_kernel<<<(K + 7) / 8, 256, 0, s>>>(part, nblk, K, out, accumulate));
    return cudaGetLastError();
}

static cudaError_t sum_parts(const double *part, int nblk, int K, double *out, int accumulate, cudaStream_t s) {
    DCRF_LAUNCH(sum_parts_kernel<<<(K + 7) / 8, 256, 0, s>>>(part, nblk, K, out, accumulate));
    return cudaGetLastError();
}

cudaError_t launch_label_products_part(const float *a, const float *b, int M, int ns, const int *slot_pt, int mode,
                                       double *part, int accumulate, cudaStream_t s) {
    const int ld = pad_labels(M);
    const unsigned nb = (unsigned)label_products_blocks(ns);
    const size_t smem = (2 * (size_t)LP_ROWS * ld + block_label_products_words(M, mode)) * sizeof(float);
    if (smem > 48 * 1024) return cudaErrorInvalidValue;
    DCRF_LAUNCH(label_products_kernel<<<nb, 256, smem, s>>>(a, b, M, ld, ns, slot_pt, mode, accumulate, part));
    return cudaGetLastError();
}

template <int MP>
static cudaError_t sg_launch(const SliceGradArgs &a, cudaStream_t s) {
    DCRF_LAUNCH(slice_grad_kernel<MP><<<blocks(a.nslots), 256, 0, s>>>(a));
    return cudaGetLastError();
}

cudaError_t launch_slice_grad(const SliceGradArgs &a, int MP, cudaStream_t s) {
    switch (MP) {
        case 1: return sg_launch<1>(a, s);
        case 2: return sg_launch<2>(a, s);
        case 4: return sg_launch<4>(a, s);
        case 8: return sg_launch<8>(a, s);
        case 12: return sg_launch<12>(a, s);
        case 16: return sg_launch<16>(a, s);
        case 20: return sg_launch<20>(a, s);
        case 24: return sg_launch<24>(a, s);
        case 28: return sg_launch<28>(a, s);
        case 32: return sg_launch<32>(a, s);
        default: return cudaErrorInvalidValue;
    }
}

int kernel_param_blocks(int N) { return (int)blocks(N); }

cudaError_t launch_kernel_param_grad(const float *f, const float *fg, int d, int N, int full, double *part,
                                     double *out, int accumulate, cudaStream_t s) {
    const int K = full ? d * d : d;
    const unsigned nb = blocks(N);
    DCRF_LAUNCH(kernel_param_grad_kernel<<<nb, 256, 8 * K * sizeof(double), s>>>(f, fg, d, N, full, part));
    return sum_parts(part, (int)nb, K, out, accumulate, s);
}

}  // namespace dcrf
