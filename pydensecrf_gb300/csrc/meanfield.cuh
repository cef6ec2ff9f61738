// meanfield.cuh -- kernels of one mean-field iteration (see meanfield.cu).
#pragma once
#include "dcrf_common.cuh"
#include "lattice.cuh"

namespace dcrf {

// point-pass mode bits
enum : int {
    PP_LOAD_Q = 1,   // q = Qin (label-major)
    PP_ONES = 2,     // q = 1 (value size 1: the normalisation pass)
    PP_MSG = 4,      // slice every term's blurred lattice into messages
    PP_WRITE_Q = 8,  // Qout = q
    PP_SPLAT = 16,   // splat q into every term's per-tile partials
    PP_MAP = 32,     // map_out = argmax q (first maximum)
    PP_KL = 64,      // per-block KL-divergence partial sums (needs LOAD_Q|MSG)
    PP_NORM = 128,   // slice (value size 1) and write each term's normalisation
    PP_FILTER = 256, // Qout = raw lattice filter of term 0 (no normalisation, compatibility or softmax)
    // the mean-field iteration's passes, compiled as their own instances
    PP_HOT_STEP = PP_MSG | PP_SPLAT,    // messages, softmax, splat of the new marginals
    PP_HOT_LAST = PP_MSG | PP_WRITE_Q,  // the last iteration: messages, softmax, marginals out
    PP_HOT_SPLAT = PP_LOAD_Q | PP_SPLAT,  // the adjoint's splat of given rows through every term
};

struct PPArgs {
    int N, M, mode;
    int ntiles, nslots;
    const int *slot_pt;  // [nslots] point of each tile slot, -1 = empty
    const float *U;      // [nslots][MP] slot rows, or nullptr (no unary: zero)
    const float *Qin;    // [nslots][MP]
    float *Qout;         // [nslots][MP]
    int16_t *map_out;    // [N] (point order)
    double *kl_part;     // [ntiles]
    DevStatus *status;
    int smem_bytes;      // dynamic shared memory of the point pass
    int split;           // threads per point of the point pass (1, or 2 when MP % 8 == 0)
    int sm_q;            // offset of the splat's q rows (aliases the slice-phase regions)
    int sm_res;          // offset of the splat's per-task results (after the q rows)
    // checkpoint (adjoint): per term, the sliced value before the term's
    // post-normalisation, K_raw [norm] Q, as slot rows (null: not kept)
    float *ckY[DCRF_MAX_TERMS];
    // PP_FILTER epilogue (adjoint): with F the raw filter of term 0 and
    // F' = F .* norm when term 0's post_norm is set (else F): Fpost = F' and
    // Gacc += compat(F') (rows; null to skip).  Qout (raw F) may be null.
    float *Fpost;
    float *Gacc;
    // PP_NORM outputs, per term ([nslots] each; empty slots get 0), and the
    // splat member weights times their point's norm (null: not wanted)
    float *norm_out[DCRF_MAX_TERMS];
    float *wn_out[DCRF_MAX_TERMS];
    int ntype[DCRF_MAX_TERMS];
    TermSet ts;
};

// The mean-field update for more than 32 labels (label chunks of 32, see
// chunk_offset): one CTA per tile, a thread per point walks the chunks.
enum : int {
    WP_MSG = 1,      // slice every term's blurred lattice (pv, chunk by chunk) into messages
    WP_LOAD_Q = 2,   // the marginals are given (Qin); with WP_KL: klDivergence's partial sums
    WP_WRITE_Q = 4,  // softmax, Qout = the new marginals
    WP_MAP = 8,      // softmax, map_out = argmax (first maximum)
    WP_KL = 16,
    WP_ENERGY = 32,  // with WP_MSG | WP_LOAD_Q (a one-hot labelling): energy[i] = the pairwise
                     // energy of the point's label, -1/2 * message, added term by term
};

struct WideArgs {
    int N, M, MP, mode;
    int ntiles, nslots;
    const int *slot_pt;
    const float *U;     // chunked slot rows, or nullptr (zero unary)
    const float *Qin;   // chunked slot rows (WP_LOAD_Q)
    float *Qout;        // chunked slot rows; also the logits' scratch of the softmax
    float *F;           // per Matrix term j (in term order), chunked slot rows of its sliced
                        // messages at F + j * nslots * MP
    int16_t *map_out;   // [N]
    double *kl_part;    // [ntiles]
    const int16_t *labels;  // [N] (WP_ENERGY)
    float *energy;          // [N] (WP_ENERGY)
    long long pv_chunk[DCRF_MAX_TERMS];  // floats between consecutive chunks of a term's pv (32 (P+1))
    TermSet ts;         // terms; pv, tile tables, norm and compatibility of chunk 0
};
cudaError_t launch_wide(const WideArgs &a, cudaStream_t s);

// One iteration of the adjoint's per-point work (DenseCRF::gradient,
// densecrf.cpp:271-290) for all terms, one CTA per tile (a thread per slot):
// per term F = the raw slice of its reverse-blurred splat A (vertex order,
// permutohedral.cpp:574-584), F' = [norm .*] F (the transpose's last
// normalisation, pairwise.cpp:78-79), g += C F' (C symmetric, so C^T = C), and
// the compatibility-gradient products sum F' (x) Q_t per tile; then
// b_next = the softmax adjoint of g at Q_t and du += b_next.
struct AdjArgs {
    int N, M, nslots, ntiles;
    const int *slot_pt;
    const float *Qt;    // [nslots][MP] the iterate Q_t
    float *b_next;      // [nslots][MP]
    float *du;          // [nslots][MP], += b_next
    int lp_accum;       // add to the products' partials (not the first iteration)
    int n;
    struct T {
        const float *A;  // [L+1][MP]
        int post;        // F' = norm .* F
        float *Fraw;     // F stored when non-null (kernel gradients)
        double *lp;      // [ntiles][K] products' partials, null: not wanted
        int lp_mode;     // 0: per label (Potts, Diagonal), 1: outer (Matrix)
    } a[DCRF_MAX_TERMS];
    TermSet ts;          // off, bary, wslice, alpha, seq, d, compatibility, norm of every term
};
cudaError_t launch_adjoint_tile(const AdjArgs &a, int MP, cudaStream_t s);

struct ReduceArgs {
    int n;  // number of terms
    struct T {
        const int *red_beg;   // [L+1] vertex v's partials are rows [red_beg[v], red_beg[v+1]) of partial
        const float *partial; // [P][MP] splat partials grouped by vertex
        float *V;             // [L+1][MP]
        int L, P;
    } t[DCRF_MAX_TERMS];
    // set by launch_reduce: row slots of a vertex's lane group, and the prefix
    // of threads over terms (each term's range starts on a warp boundary)
    int rs[DCRF_MAX_TERMS];
    long long begin[DCRF_MAX_TERMS + 1];
};

struct BlurArgs {
    int n;
    struct T {
        const float *Vin;
        float *Vout;          // vertex order output (may be null when only scattering)
        const int2 *nbr;      // [d+1][L]
        int L;
        int axis;
        int axis2;            // >= 0: a second pass along axis2 in the same launch (the first
                              // pass recomputed at the second's neighbours); -1: one pass
        const int *red_beg;   // scatter of the result into partial order (last pass of the
        const int *red_list;  // mean-field filter): pv[red_list[s]] = out[v], s in red_beg[v..v+1)
        float *pv;            // null: no scatter
    } t[DCRF_MAX_TERMS];
    long long begin[DCRF_MAX_TERMS + 1];  // prefix of (vertex, vector) work over terms
};

// Blur chains for the single-launch blur: each chain runs its d+1 axis passes
// (d..0 when reverse) from S, ping-ponging through buf[0], buf[1]; the last
// pass writes Out (may be null) and optionally scatters into pv in partial
// order.  All chains advance pass by pass together, separated by a bounded grid
// barrier (cooperative launch, so every CTA is resident).
struct BlurChainArgs {
    int n;      // chains
    int npass;  // max over chains of d+1
    struct C {
        const float *S;
        float *buf[2];
        float *Out;
        const int2 *nbr;
        int L, d, reverse;
        const int *red_beg;
        const int *red_list;
        float *pv;
    } c[2 * DCRF_MAX_TERMS];
    unsigned *bar;  // [2] grid-barrier state (arrivals, generation), zero before the launch
    DevStatus *status;
};

// Launchers; MP is the padded label count (1, 2, 4, 8, ..., 32).
cudaError_t launch_pointpass(const PPArgs &a, int MP, cudaStream_t s);
// the PP_NORM / PP_FILTER passes (point-order slice; launch_pointpass routes them here)
cudaError_t launch_slice(const PPArgs &a, int MP, cudaStream_t s);
cudaError_t launch_reduce(const ReduceArgs &a, int MP, cudaStream_t s);
cudaError_t launch_blur(const BlurArgs &a, int MP, bool seq, cudaStream_t s);
cudaError_t launch_blur_chains(const BlurChainArgs &a, int MP, bool seq, cudaStream_t s);

// Layout conversions between user layouts (point-major [N][M], or label-major:
// per image an M x N_b block, images one after another -- [M][N] for one image)
// and the device slot rows [nslots][ld] (ld >= M; padding labels and empty
// slots hold 0).  seg[0..nseg] are the images' point offsets on the device.
// Labels m0 .. m0+M-1 of a caller buffer with Mu labels (M <= ld <= 32).
cudaError_t launch_to_slots(const float *in, int point_major, int M, int Mu, int m0, int ld, int N, const int *seg,
                            int nseg, const int *slot_pt, int nslots, float *out, cudaStream_t s);
cudaError_t launch_from_slots(const float *in, int M, int Mu, int m0, int ld, int N, const int *seg, int nseg,
                              const int *slot_pt, int nslots, const int *pt_slot, int point_major, float *out,
                              cudaStream_t s);
// 2D features of DenseCRF2D (densecrf.cpp:61-81) of every image into [d][N]
cudaError_t launch_features_2d(int N, const int *seg, const int *imgW, int nseg, float sx, float sy,
                               const uint8_t *rgb, float sr, float sg, float sb, float *feat, cudaStream_t s);
cudaError_t launch_scale_features(const float *in, float *out, const float *scale_or_matrix, int d, int N, int full,
                                  cudaStream_t s);
// Opts every point-pass instantiation in to its dynamic shared-memory budget.
void prepare_pointpass_kernels();
// Largest dynamic shared memory the point pass may use per CTA.
// default shared-memory budget of a point-pass CTA (two CTAs per SM)
int pointpass_smem_budget(int MP);
constexpr int POINTPASS_SMEM_MAX = 224 * 1024;  // dynamic shared memory a point-pass CTA may plan

}  // namespace dcrf
