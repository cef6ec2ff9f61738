// adjoint.cu -- device kernels of the hand-written adjoint of T mean-field
// iterations (the device form of DenseCRF::gradient,
// pydensecrf/densecrf/src/densecrf.cpp:238-297).
//
// All point quantities are slot-major [M][nslots] (empty slots hold zero).
// Reductions are two-level and deterministic: per-block partial sums in
// double, then one block adds them in block order.
#include "adjoint.cuh"

namespace dcrf {

// All label-valued buffers here are slot rows [ns][ld] (ld = padded label
// count); labels m >= M and empty slots are written as 0.

// b = Q * sum(x .* Q) - x .* Q  per point: the softmax adjoint with the
// reference's sign (sumAndNormalize, densecrf.cpp:107-114, applied to x .* Q).
__global__ void softmax_adjoint_kernel(const float *__restrict__ Q, const float *__restrict__ x, float *__restrict__ b,
                                       int M, int ld, int ns, const int *__restrict__ slot_pt) {
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
    for (int m = 0; m < ld; m++) o[m] = m < M ? fmaf(q[m], dot, -xx[m] * q[m]) : 0.f;
}

// y (+)= C x, or C^T x, per point (labelcompatibility.cpp:46-48,66-68,82-87)
__global__ void compat_kernel(const float *__restrict__ x, float *__restrict__ y, int M, int ld, int ns, int kind,
                              float potts_w, const float *__restrict__ C, int transpose, int accumulate) {
    const size_t s = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= (size_t)ns) return;
    const float *xx = x + s * ld;
    float *yy = y + s * ld;
    for (int m = 0; m < ld; m++) {
        float v = 0.f;
        if (m < M) {
            if (kind == DCRF_COMPAT_POTTS) {
                v = -potts_w * xx[m];
            } else if (kind == DCRF_COMPAT_DIAGONAL) {
                v = C[m] * xx[m];
            } else {
                for (int k = 0; k < M; k++) v = fmaf(transpose ? C[k * M + m] : C[m * M + k], xx[k], v);
            }
        }
        if (accumulate)
            yy[m] += v;
        else
            yy[m] = v;
    }
}

// y = x .* norm^pw per point (pw in 1..3)
__global__ void scale_norm_kernel(const float *__restrict__ x, float *__restrict__ y, const float *__restrict__ norm,
                                  int ld, int ns, int pw) {
    const size_t s = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= (size_t)ns) return;
    const float n = norm[s];
    const float f = pw == 1 ? n : pw == 2 ? n * n : n * n * n;
    for (int m = 0; m < ld; m++) y[s * ld + m] = x[s * ld + m] * f;
}

// y = scale * (x1 .* x2 + x3 .* x4) .* norm^pw per point (x3/x4 may be null; norm null: pw ignored)
__global__ void prod_kernel(const float *__restrict__ x1, const float *__restrict__ x2, const float *__restrict__ x3,
                            const float *__restrict__ x4, float scale, const float *__restrict__ norm, int pw,
                            float *__restrict__ y, int ld, int ns) {
    const size_t s = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= (size_t)ns) return;
    float f = scale;
    if (norm) {
        const float n = norm[s];
        f *= pw == 1 ? n : pw == 2 ? n * n : n * n * n;
    }
    for (int m = 0; m < ld; m++) {
        const size_t o = s * ld + m;
        float v = x1[o] * x2[o];
        if (x3) v = fmaf(x3[o], x4[o], v);
        y[o] = v * f;
    }
}

__global__ void add_kernel(const float *__restrict__ x, float *__restrict__ y, size_t n) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) y[i] += x[i];
}

__global__ void fill_kernel(float *__restrict__ y, float v, int M, int ld, int ns, const int *__restrict__ slot_pt) {
    const size_t s = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= (size_t)ns) return;
    const float val = slot_pt[s] >= 0 ? v : 0.f;
    for (int m = 0; m < ld; m++) y[s * ld + m] = m < M ? val : 0.f;
}

// Per-block partial sums of the label products over the occupied slots:
//  mode 0 (per label):  part[blk][m]      = sum_s a[m][s] * b[m][s]
//  mode 1 (outer):      part[blk][m*M+k]  = sum_s a[m][s] * b[k][s]
// Padding slots (slot_pt < 0) hold no point and are left out whatever they contain.
__global__ void __launch_bounds__(256) label_products_kernel(const float *__restrict__ a, const float *__restrict__ b,
                                                             int M, int ld, int ns, const int *__restrict__ slot_pt,
                                                             int mode, double *__restrict__ part) {
    extern __shared__ double sred[];  // [8 warps][K]
    const int K = mode == 0 ? M : M * M;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const size_t s = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const bool ok = s < (size_t)ns && slot_pt[s] >= 0;
    for (int kk = 0; kk < K; kk++) {
        const int m = mode == 0 ? kk : kk / M, k = mode == 0 ? kk : kk % M;
        double v = ok ? (double)a[s * ld + m] * (double)b[s * ld + k] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0) sred[warp * K + kk] = v;
    }
    __syncthreads();
    for (int kk = threadIdx.x; kk < K; kk += blockDim.x) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x / 32); w++) t += sred[w * K + kk];
        part[(size_t)blockIdx.x * K + kk] = t;
    }
}

// out[k] = sum over blocks (in block order) of part[blk][k]
__global__ void sum_parts_kernel(const double *__restrict__ part, int nblk, int K, double *__restrict__ out,
                                 int accumulate) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= K) return;
    double t = 0.0;
    for (int b = 0; b < nblk; b++) t += part[(size_t)b * K + k];
    out[k] = accumulate ? out[k] + t : t;
}

// Feature gradient of the slice (the per-point part of Permutohedral::gradient,
// permutohedral.cpp:660-690): with V the blurred lattice of one direction and
// z the contraction values, df[i][j-1] += sum_k z[k] * sf[j-1] * (sm_k - j * ra_j[k]),
// ra_j = alpha/(d+1) * (V[off[r0]] - V[off[r1]]), r0 = d - rank_j, r1 = r0+1 mod (d+1),
// sm the running sum of ra_0..ra_{j-1}.
template <int MP>
__global__ void __launch_bounds__(256) slice_grad_kernel(SliceGradArgs a) {
    const size_t s = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= (size_t)a.nslots) return;
    const int i = a.slot_pt[s];
    if (i < 0) return;
    const int d = a.d, N = a.N, M = a.M;
    float z[MP];
#pragma unroll
    for (int m = 0; m < MP; m++) z[m] = m < M ? a.z[s * MP + m] : 0.f;
    float sm[MP];
#pragma unroll
    for (int m = 0; m < MP; m++) sm[m] = 0.f;
    for (int j = 0; j <= d; j++) {
        const int r0 = d - (int)a.rank[(size_t)j * N + i];
        const int r1 = r0 + 1 > d ? 0 : r0 + 1;
        const float *v0 = a.V + (size_t)(a.off[(size_t)r0 * N + i] + 1) * MP;
        const float *v1 = a.V + (size_t)(a.off[(size_t)r1 * N + i] + 1) * MP;
        float grad = 0.f;
#pragma unroll
        for (int m = 0; m < MP; m++) {
            const float ra = a.alpha * (v0[m] - v1[m]);
            if (j > 0) grad = fmaf(z[m], a.sf[j - 1] * (sm[m] - (float)j * ra), grad);
            sm[m] += ra;
        }
        if (j > 0) a.df[(size_t)i * d + (j - 1)] += grad;
    }
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
        part[(size_t)blockIdx.x * K + kk] = t;
    }
}

// ---------------------------------------------------------------------------
static unsigned blocks(size_t n) { return (unsigned)((n + 255) / 256); }

cudaError_t launch_softmax_adjoint(const float *Q, const float *x, float *b, int M, int ns, const int *slot_pt,
                                   cudaStream_t s) {
    DCRF_LAUNCH(softmax_adjoint_kernel<<<blocks(ns), 256, 0, s>>>(Q, x, b, M, pad_labels(M), ns, slot_pt));
    return cudaGetLastError();
}

cudaError_t launch_compat(const float *x, float *y, int M, int ns, int kind, float potts_w, const float *C,
                          int transpose, int accumulate, cudaStream_t s) {
    DCRF_LAUNCH(compat_kernel<<<blocks(ns), 256, 0, s>>>(x, y, M, pad_labels(M), ns, kind, potts_w, C, transpose,
                                                         accumulate));
    return cudaGetLastError();
}

cudaError_t launch_scale_norm(const float *x, float *y, const float *norm, int M, int ns, int pw, cudaStream_t s) {
    DCRF_LAUNCH(scale_norm_kernel<<<blocks(ns), 256, 0, s>>>(x, y, norm, pad_labels(M), ns, pw));
    return cudaGetLastError();
}

cudaError_t launch_prod(const float *x1, const float *x2, const float *x3, const float *x4, float scale,
                        const float *norm, int pw, float *y, int M, int ns, cudaStream_t s) {
    DCRF_LAUNCH(prod_kernel<<<blocks(ns), 256, 0, s>>>(x1, x2, x3, x4, scale, norm, pw, y, pad_labels(M), ns));
    return cudaGetLastError();
}

cudaError_t launch_add(const float *x, float *y, size_t n, cudaStream_t s) {
    if (n) DCRF_LAUNCH(add_kernel<<<blocks(n), 256, 0, s>>>(x, y, n));
    return cudaGetLastError();
}

cudaError_t launch_fill(float *y, float v, int M, int ns, const int *slot_pt, cudaStream_t s) {
    DCRF_LAUNCH(fill_kernel<<<blocks(ns), 256, 0, s>>>(y, v, M, pad_labels(M), ns, slot_pt));
    return cudaGetLastError();
}

int label_products_blocks(int ns) { return (int)blocks(ns); }

cudaError_t launch_label_products(const float *a, const float *b, int M, int ns, const int *slot_pt, int mode,
                                  double *part, double *out, int accumulate, cudaStream_t s) {
    const int K = mode == 0 ? M : M * M;
    const unsigned nb = blocks(ns);
    const size_t smem = 8 * (size_t)K * sizeof(double);  // up to 64 KB for 32 x 32 labels
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(label_products_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem);
        if (e != cudaSuccess) return e;
    }
    DCRF_LAUNCH(label_products_kernel<<<nb, 256, smem, s>>>(a, b, M, pad_labels(M), ns, slot_pt, mode, part));
    DCRF_LAUNCH(sum_parts_kernel<<<blocks(K), 256, 0, s>>>(part, (int)nb, K, out, accumulate));
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
    DCRF_LAUNCH(sum_parts_kernel<<<blocks(K), 256, 0, s>>>(part, (int)nb, K, out, accumulate));
    return cudaGetLastError();
}

}  // namespace dcrf
