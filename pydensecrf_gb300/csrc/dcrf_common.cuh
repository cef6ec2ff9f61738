// dcrf_common.cuh -- shared definitions of the GB300 dense-CRF engine.
//
// Data layout in device memory (N points, M labels, MP = padded label count,
// d feature dims, L lattice vertices of one term, E = N*(d+1) simplex corners):
//   U, Q          float [nslots][MP]  slot rows: point slot_pt[s] of tile s/256,
//                                     labels m < M (padding labels and empty slots 0)
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
#define DCRF_MAX_MP 32  // labels one thread-per-point kernel keeps in registers (one label chunk)
#define DCRF_MAX_LABELS 4096  // labels of a handle (label ids are int16 in the MAP output)

// Label chunks.  Quantities with more than DCRF_MAX_MP labels are stored
// chunk-major: labels [32c, 32c + w_c) of every row form chunk c, a block of
// rows of w_c floats (w_c = 32 except the last), after the blocks of chunks
// < c.  With MP <= 32 there is one chunk and this is the plain row layout.
#define DCRF_LCHUNK 32
static inline int label_chunks(int MP) { return MP <= DCRF_LCHUNK ? 1 : (MP + DCRF_LCHUNK - 1) / DCRF_LCHUNK; }
static inline int chunk_width(int MP, int c) {
    return MP <= DCRF_LCHUNK ? MP : (MP - DCRF_LCHUNK * c < DCRF_LCHUNK ? MP - DCRF_LCHUNK * c : DCRF_LCHUNK);
}
// first float of chunk c in a buffer of `rows` rows
static inline size_t chunk_base(size_t rows, int c) { return (size_t)DCRF_LCHUNK * c * rows; }
// offset of (row r, label l) in such a buffer
__host__ __device__ __forceinline__ size_t chunk_offset(size_t rows, int MP, size_t r, int l) {
    if (MP <= DCRF_LCHUNK) return r * MP + l;
    const int c = l / DCRF_LCHUNK, w = MP - DCRF_LCHUNK * c < DCRF_LCHUNK ? MP - DCRF_LCHUNK * c : DCRF_LCHUNK;
    return (size_t)DCRF_LCHUNK * c * rows + r * w + (l - DCRF_LCHUNK * c);
}

namespace dcrf {
// Counts every kernel launch of the library (dcrf_launch_count).
void note_launch();
}  // namespace dcrf
#define DCRF_LAUNCH(...)      \
    do {                      \
        dcrf::note_launch();  \
        __VA_ARGS__;          \
    } while (0)

namespace dcrf {
// Programmatic dependent launch.  The mean-field kernels (point pass, reduce,
// blur) are launched so that the next one may start while its predecessor on
// the stream drains: each calls pdl_trigger() on entry and pdl_wait() before
// its first access to memory that a kernel of the launch sequence reads or
// writes; only tables fixed since the lattice build (and the unary) are read
// before the wait.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

// Whether launches use the programmatic-serialization attribute (default on;
// DCRF_PDL=0 in the environment turns it off).
bool pdl_enabled();

// Stream-ordered allocation from the library's memory pool of the current
// device.  The pool keeps freed blocks (release threshold: unlimited), so the
// per-term buffers of a rebuilt lattice come back without new mappings; the
// default pool would return them to the driver at every synchronisation.
cudaError_t pool_malloc_async(void **p, size_t bytes, cudaStream_t s);

template <typename... KArgs, typename... Args>
cudaError_t launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s,
                       Args &&...args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = pdl_enabled() ? 1 : 0;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    note_launch();
    return cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...);
}
}  // namespace dcrf

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
    const uint32_t *tsched;  // per tile, task indices by descending length (LatticeDev::tsched)
    const int *tile_tbeg;    // [ntiles+1] task range of each tile
    float *pv;               // [P][MP] blurred values in partial order (slice input)
    float *pout;             // [P][MP] splat partials, grouped by vertex (row ppos[p] for partial p)
    const int *ppos;         // [P] row of each partial in pout
    const float *norm;       // [nslots]
    const float *compat;     // Diagonal [M] / Matrix [M][M] (symmetrised)
    // shared-memory plan of the point pass (byte offsets; staged = 0: global reads)
    int staged, vcap;
    int sm_loc, sm_w, sm_norm, sm_task, sm_sched, sm_mpt, sm_mw, sm_vp;
    int sm_cmp;  // Matrix compatibility staged as [k][MP] (transposed, zero padded); -1: global reads
};

struct TermSet {
    int n;
    TermDev t[DCRF_MAX_TERMS];
};
