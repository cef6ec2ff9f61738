// labelprod.cuh -- block-level label products of staged slot rows (the
// compatibility gradients of the adjoint, labelcompatibility.cpp:57-61,76-78,
// 101-107): per block, over `rows` rows of a and b (row pitch ld, labels < M):
//   mode 0: out[m]       = sum_r a[r][m] * b[r][m]
//   mode 1: out[m*M + k] = sum_r a[r][m] * b[r][k]
// Mode 0: 8 row groups, one warp each, lane m; mode 1: 3 x 3 output blocks per
// thread over the rows r = g, g + G, ... of its row group g.  The groups' float
// sums are added in group order, so the result depends only on the rows; it is
// stored (or, accumulate, added) as double at dst[0 .. K).  sg is shared scratch
// of block_label_products_words floats, which may alias a and b.  All threads
// of the block (256) call it.
#pragma once
#include "dcrf_common.cuh"

namespace dcrf {

constexpr int BLP_GROUPS = 8, BLP_TB = 3, BLP_THREADS = 256;

__host__ __device__ inline int block_label_products_words(int M, int mode) {
    const int K = mode == 0 ? M : M * M, TM = (M + BLP_TB - 1) / BLP_TB;
    const int G = BLP_THREADS / (TM * TM) > 0 ? BLP_THREADS / (TM * TM) : 1;
    return mode == 0 ? BLP_GROUPS * 32 : G * K;
}

__device__ __forceinline__ void block_label_products(const float *sa, const float *sb, int rows, int ld, int M,
                                                     int mode, float *sg, double *dst, int accumulate) {
    const int K = mode == 0 ? M : M * M;
    if (mode == 0) {
        const int g = threadIdx.x >> 5, m = threadIdx.x & 31;
        const int RG = (rows + BLP_GROUPS - 1) / BLP_GROUPS;
        float t = 0.f;
        if (m < M)
            for (int r = g * RG; r < min(rows, (g + 1) * RG); r++) t = fmaf(sa[r * ld + m], sb[r * ld + m], t);
        __syncthreads();  // sg may alias the rows
        sg[g * 32 + m] = t;
        __syncthreads();
        if ((int)threadIdx.x < M) {
            float u = 0.f;
            for (int q = 0; q < BLP_GROUPS; q++) u += sg[q * 32 + threadIdx.x];
            dst[threadIdx.x] = accumulate ? dst[threadIdx.x] + (double)u : (double)u;
        }
        __syncthreads();
        return;
    }
    const int TM = (M + BLP_TB - 1) / BLP_TB, tiles = TM * TM;
    const int G = BLP_THREADS / tiles > 0 ? BLP_THREADS / tiles : 1;
    const int tile = threadIdx.x % tiles, g = threadIdx.x / tiles;
    const int m0 = (tile / TM) * BLP_TB, k0 = (tile % TM) * BLP_TB;
    float t[BLP_TB][BLP_TB];
#pragma unroll
    for (int i = 0; i < BLP_TB; i++)
#pragma unroll
        for (int j = 0; j < BLP_TB; j++) t[i][j] = 0.f;
    if (g < G)
        for (int r = g; r < rows; r += G) {
            float va[BLP_TB], vb[BLP_TB];
#pragma unroll
            for (int i = 0; i < BLP_TB; i++) {
                va[i] = m0 + i < ld ? sa[r * ld + m0 + i] : 0.f;
                vb[i] = k0 + i < ld ? sb[r * ld + k0 + i] : 0.f;
            }
#pragma unroll
            for (int i = 0; i < BLP_TB; i++)
#pragma unroll
                for (int j = 0; j < BLP_TB; j++) t[i][j] = fmaf(va[i], vb[j], t[i][j]);
        }
    __syncthreads();  // sg may alias the rows
    if (g < G)
#pragma unroll
        for (int i = 0; i < BLP_TB; i++)
#pragma unroll
            for (int j = 0; j < BLP_TB; j++)
                if (m0 + i < M && k0 + j < M) sg[g * K + (m0 + i) * M + k0 + j] = t[i][j];
    __syncthreads();
    for (int kk = threadIdx.x; kk < K; kk += blockDim.x) {
        float u = 0.f;
        for (int q = 0; q < G; q++) u += sg[q * K + kk];
        dst[kk] = accumulate ? dst[kk] + (double)u : (double)u;
    }
    __syncthreads();
}

}  // namespace dcrf
