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
};

struct PPArgs {
    int N, M, mode;
    int ntiles;
    const int *slot_pt;  // [ntiles*SPLAT_TILE]
    const float *U;      // [M][N] or nullptr (no unary: zero)
    const float *Qin;    // [M][N]
    float *Qout;         // [M][N]
    int16_t *map_out;    // [N]
    double *kl_part;     // [ntiles]
    // PP_NORM outputs, per term
    float *norm_out[DCRF_MAX_TERMS];
    int ntype[DCRF_MAX_TERMS];
    TermSet ts;
};

struct ReduceArgs {
    int n;  // number of terms
    struct T {
        const int *red_beg;   // [L+1]
        const int *red_list;  // [P]
        const float *partial; // [P][MP]
        float *V;             // [L+1][MP]
        int L;
    } t[DCRF_MAX_TERMS];
    long long begin[DCRF_MAX_TERMS + 1];  // prefix of vertex work over terms
};

struct BlurArgs {
    int n;
    struct T {
        const float *Vin;
        float *Vout;
        const int2 *nbr;  // [d+1][L]
        int L;
        int axis;
    } t[DCRF_MAX_TERMS];
    long long begin[DCRF_MAX_TERMS + 1];  // prefix of (vertex, vector) work over terms
};

// Launchers; MP is the padded label count (1, 2, 4, 8, ..., 32).
cudaError_t launch_pointpass(const PPArgs &a, int MP, cudaStream_t s);
cudaError_t launch_reduce(const ReduceArgs &a, int MP, cudaStream_t s);
cudaError_t launch_blur(const BlurArgs &a, int MP, bool seq, cudaStream_t s);

// Layout conversions between the device's label-major [M][N] and a padded or
// point-major view.
cudaError_t launch_transpose(const float *in, float *out, int rows, int cols, cudaStream_t s);  // out[c][r] = in[r][c]
// 2D features of DenseCRF2D (densecrf.cpp:61-81) into [d][N]
cudaError_t launch_features_2d(int W, int H, float sx, float sy, const uint8_t *rgb, float sr, float sg, float sb,
                               float *feat, cudaStream_t s);
cudaError_t launch_scale_features(const float *in, float *out, const float *scale_or_matrix, int d, int N, int full,
                                  cudaStream_t s);
cudaError_t launch_argmax(const float *Q, int M, int N, int16_t *out, cudaStream_t s);

}  // namespace dcrf
