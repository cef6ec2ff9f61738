// unary.cu -- the logistic unary energy on the device (LogisticUnaryEnergy,
// pydensecrf/densecrf/src/unary.cpp:48-68): U = L f and its parameter
// gradient b f^T.
#include <algorithm>

#include "adjoint.cuh"

namespace dcrf {

// U (slot rows, chunk_offset layout) = L f: L is M x F (row-major), f is F x N
// (feature-major, the numpy (F, N) array).  One CTA per tile, a thread per
// slot; L is read through shared memory when it fits.  Every label's sum runs
// over the features in order (fused multiply-adds); padding labels and empty
// slots are 0.
constexpr int LU_SMEM_FLOATS = 12 * 1024;  // 48 KB of L in shared memory

__global__ void __launch_bounds__(256) logistic_unary_kernel(const float *__restrict__ L, const float *__restrict__ f,
                                                             int M, int MP, int F, int N, int ns,
                                                             const int *__restrict__ slot_pt, float *__restrict__ U) {
    __shared__ float sL[LU_SMEM_FLOATS];
    const bool staged = (size_t)M * F <= (size_t)LU_SMEM_FLOATS;
    if (staged)
        for (int e = threadIdx.x; e < M * F; e += blockDim.x) sL[e] = L[e];
    __syncthreads();
    const float *Lm = staged ? sL : L;
    const size_t s = (size_t)blockIdx.x * 256 + threadIdx.x;
    const int pt = slot_pt[s];
    const int nc = MP <= DCRF_LCHUNK ? 1 : (MP + DCRF_LCHUNK - 1) / DCRF_LCHUNK;
    for (int c = 0; c < nc; c++) {
        const int m0 = DCRF_LCHUNK * c;
        const int w = MP <= DCRF_LCHUNK ? MP : min(DCRF_LCHUNK, MP - m0);
        float acc[DCRF_LCHUNK];
#pragma unroll
        for (int e = 0; e < DCRF_LCHUNK; e++) acc[e] = 0.f;
        if (pt >= 0)
            for (int j = 0; j < F; j++) {
                const float fj = __ldg(f + (size_t)j * N + pt);
#pragma unroll
                for (int e = 0; e < DCRF_LCHUNK; e++)
                    if (e < w && m0 + e < M) acc[e] = fmaf(Lm[(size_t)(m0 + e) * F + j], fj, acc[e]);
            }
        float *row = U + chunk_offset((size_t)ns, MP, s, m0);
#pragma unroll
        for (int e = 0; e < DCRF_LCHUNK; e++)
            if (e < w) row[e] = acc[e];
    }
}

cudaError_t launch_logistic_unary(const float *L, const float *f, int M, int F, int N, int ns, const int *slot_pt,
                                  float *U, cudaStream_t s) {
    if (ns <= 0) return cudaSuccess;
    DCRF_LAUNCH(logistic_unary_kernel<<<ns / 256, 256, 0, s>>>(L, f, M, pad_labels(M), F, N, ns, slot_pt, U));
    return cudaGetLastError();
}

// part[o][blk] = sum over the block's PT slots of b[m][pt] * f[j][pt], o = m + M j
// (the column-major order of the reference's parameter vector); b are slot rows
// with M <= 32 labels.  Rows of b and f are staged in shared memory; each output
// sums its points in slot order, in double.
__global__ void logistic_grad_kernel(const float *__restrict__ b, const float *__restrict__ f, int M, int MP, int F,
                                     int N, int ns, int PT, const int *__restrict__ slot_pt, double *__restrict__ part) {
    extern __shared__ float lg_smem[];
    float *sb = lg_smem;             // [PT][M]
    float *sf = lg_smem + PT * M;    // [PT][F]
    const size_t s0 = (size_t)blockIdx.x * PT;
    for (int e = threadIdx.x; e < PT * M; e += blockDim.x) {
        const int q = e / M, m = e - q * M;
        const size_t s = s0 + q;
        sb[e] = (s < (size_t)ns && slot_pt[s] >= 0) ? b[s * MP + m] : 0.f;
    }
    for (int e = threadIdx.x; e < PT * F; e += blockDim.x) {
        const int j = e / PT, q = e - j * PT;
        const size_t s = s0 + q;
        const int pt = s < (size_t)ns ? slot_pt[s] : -1;
        sf[q * F + j] = pt >= 0 ? f[(size_t)j * N + pt] : 0.f;
    }
    __syncthreads();
    for (int o = threadIdx.x; o < M * F; o += blockDim.x) {
        const int j = o / M, m = o - j * M;
        double t = 0.0;
        for (int q = 0; q < PT; q++) t += (double)sb[q * M + m] * (double)sf[q * F + j];
        part[(size_t)o * gridDim.x + blockIdx.x] = t;
    }
}

int logistic_grad_points(int M, int F) {
    int PT = 256;
    while (PT > 8 && (size_t)PT * (M + F) * sizeof(float) > 96 * 1024) PT /= 2;
    return (size_t)PT * (M + F) * sizeof(float) > 96 * 1024 ? 0 : PT;
}

int logistic_grad_blocks(int ns, int M, int F) {
    const int PT = logistic_grad_points(M, F);
    return PT > 0 ? (ns + PT - 1) / PT : 0;
}

cudaError_t launch_logistic_grad(const float *b, const float *f, int M, int F, int N, int ns, const int *slot_pt,
                                 double *part, double *out, cudaStream_t s) {
    const int PT = logistic_grad_points(M, F);
    if (PT <= 0 || M > DCRF_MAX_MP) return cudaErrorInvalidValue;
    const int nb = (ns + PT - 1) / PT;
    const size_t smem = (size_t)PT * (M + F) * sizeof(float);
    static bool opted[64] = {};
    int dev = 0;
    cudaGetDevice(&dev);
    if (smem > 48 * 1024 && dev < 64 && !opted[dev]) {
        cudaError_t e = cudaFuncSetAttribute(logistic_grad_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 96 * 1024);
        if (e != cudaSuccess) return e;
        opted[dev] = true;
    }
    DCRF_LAUNCH(logistic_grad_kernel<<<nb, 256, smem, s>>>(b, f, M, pad_labels(M), F, N, ns, PT, slot_pt, part));
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    return launch_sum_parts(part, nb, M * F, out, 0, s);
}

}  // namespace dcrf
