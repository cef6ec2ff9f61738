// dcrf_common.cuh -- shared definitions of the GB300 dense-CRF engine.
//
// Data layout in device memory (N points, M labels, MP = padded label count,
// d feature dims, L lattice vertices of one term, E = N*(d+1) simplex corners):
//   U, Q          float [M][N]        label-major (the numpy (M, N) layout)
//   feat          float [d][N]        feature-major (the numpy (d, N) layout)
//   off           int   [d+1][N]      vertex id of corner r of point i
//   bary          float [d+1][N]      barycentric weight of that corner
//   wslice        float [d+1][N]      bary*alpha rounded (x86 slice weight)
//   rank          uint8 [d+1][N]      rank of coordinate r (feature gradient)
//   nbr           int2  [d+1][L]      (n1+1, n2+1) of vertex v along axis j; 0 = none
//   V             float [L+1][MP]     lattice values, row 0 = zero sentinel
//   partial       float [P][MP]       per-(tile, vertex) splat partial sums
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "dcrf.h"

#define DCRF_MAX_TERMS 16
#define DCRF_MAX_D 16
#define DCRF_MAX_MP 32  // thread-per-point kernels keep MP labels in registers

namespace dcrf {
// Counts every kernel launch of the library (dcrf_launch_count).
void note_launch();
}  // namespace dcrf
#define DCRF_LAUNCH(...)      \
    do {                      \
        dcrf::note_launch();  \
        __VA_ARGS__;          \
    } while (0)

// Device status block: slot 0 = first error code (0 = fine), slot 1 = detail.
struct DevStatus {
    int code;
    int detail;
    int pad[2];
};

__device__ __forceinline__ void dcrf_set_error(DevStatus *st, int code, int detail) {
    if (atomicCAS(&st->code, 0, code) == 0) st->detail = detail;
}

// Explicitly rounded float arithmetic: the reference's x86 build rounds every
// product and sum separately (no FMA), and these keep nvcc from contracting.
__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fsub(float a, float b) { return __fsub_rn(a, b); }

static inline int pad_labels(int M) {
    if (M <= 2) return M;
    return (M + 3) / 4 * 4;
}

static inline unsigned ceil_div_u(size_t a, size_t b) { return (unsigned)((a + b - 1) / b); }

// Per-term descriptor handed to the mean-field kernels by value.
struct TermDev {
    int d;
    int L;
    int ckind;      // 0 Potts, 1 Diagonal, 2 Matrix
    int pre_norm;   // multiply Q by norm before splatting
    int post_norm;  // multiply the sliced value by norm
    int seq;        // seqCompute arithmetic (value size <= 2 or scalar build)
    float potts_w;
    float alpha;
    // point-order tables (normalisation and raw-filter paths)
    const int *off;       // [d+1][N]
    const float *bary;    // [d+1][N]
    const float *wslice;  // [d+1][N]
    const float *V;       // [L+1][MP] blurred values in vertex order
    // tile tables (mean-field point pass)
    const int *tile_pbeg;    // [ntiles+1] partial range of each tile
    const int *part_mend;    // [P+8] member end of each partial, tile-relative
    const uint16_t *mem_pt;  // [ntiles][SPLAT_TILE*(d+1)] member -> tile slot
    const float *mem_w;      // [ntiles][SPLAT_TILE*(d+1)] member weight
    const uint16_t *tl_loc;  // [ntiles][d+1][SPLAT_TILE] corner -> index among the tile's partials
    const float *tl_w;       // [ntiles][d+1][SPLAT_TILE] corner barycentric weight
    const uint32_t *task;    // splat tasks (see LatticeDev::task)
    const int *tile_tbeg;    // [ntiles+1] task range of each tile
    float *pv;               // [P][MP] blurred values in partial order (read), splat partials (written)
    const float *norm;       // [nslots]
    const float *compat;     // Diagonal [M] / Matrix [M][M] (symmetrised)
    // shared-memory plan of the point pass (byte offsets; staged = 0: global reads)
    int staged, vcap;
    int sm_loc, sm_w, sm_norm, sm_task, sm_mpt, sm_mw, sm_vp;
};

struct TermSet {
    int n;
    TermDev t[DCRF_MAX_TERMS];
};
