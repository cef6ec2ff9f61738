// adjoint.cuh -- device kernels of the mean-field adjoint (see adjoint.cu).
#pragma once
#include "dcrf_common.cuh"

// Label-valued buffers are slot rows [ns][pad_labels(M)].

namespace dcrf {

struct SliceGradArgs {
    int N, M, d, nslots;
    const int *slot_pt;   // [nslots]
    const int *off;       // [d+1][N]
    const uint8_t *rank;  // [d+1][N]
    const float *V;       // [L+1][MP] blurred values, vertex order
    const float *z;       // [nslots][MP] contraction values (slot rows)
    const float *V2;      // optional second (V, z) pair, added in the same pass (null: none)
    const float *z2;
    const float *z2scale; // optional [nslots]: the second pair's z is z2 .* z2scale
    float sf[DCRF_MAX_D];
    float alpha;          // sign / (1+2^-d) / (d+1) for the first pair
    float alpha2;         // and for the second
    // optional value-size-1 pairs in the same pass (the normalisation's terms):
    // V3 [L+1] with z = 1 everywhere, V4 [L+1] with z = z4 [nslots]
    const float *V3;
    const float *V4;
    const float *z4;
    float alpha3, alpha4;
    float *df;            // [N][d] accumulated feature gradient
};

// b = softmax adjoint of x at Q (slot rows); du += b when du is not null
cudaError_t launch_softmax_adjoint(const float *Q, const float *x, float *b, float *du, int M, int ns,
                                   const int *slot_pt, cudaStream_t s);
cudaError_t launch_compat(const float *x, float *y, int M, int ns, int kind, float potts_w, const float *C,
                          int transpose, int accumulate, cudaStream_t s);
cudaError_t launch_scale_norm(const float *x, float *y, const float *norm, int M, int ns, int pw, cudaStream_t s);
cudaError_t launch_prod(const float *x1, const float *x2, const float *x3, const float *x4, float scale,
                        const float *norm, int pw, float *y, int M, int ns, cudaStream_t s);
cudaError_t launch_fill(float *y, float v, int M, int ns, const int *slot_pt, cudaStream_t s);
cudaError_t launch_row_sum(const float *x, float *out, int M, int ns, cudaStream_t s);
// ys = [norm .*] C Q and x1 = sum of the normalisation coefficients c1 per point
// (see adjoint.cu); labels M > 2 only.
cudaError_t launch_norm_terms(const float *b, const float *y, const float *F, const float *Q, const float *norm,
                              int M, int ns, int ntype, int kind, float potts_w, const float *C, float *ys,
                              float *x1, cudaStream_t s);
// one-hot slot rows of a point-order labelling; per-point energy from slot rows
cudaError_t launch_onehot(const int16_t *labels, int M, int ns, const int *slot_pt, float *out, cudaStream_t s);
// the same for more than 32 labels, in the label-chunk layout (chunk_offset)
cudaError_t launch_onehot_chunked(const int16_t *labels, int M, int MP, int ns, const int *slot_pt, float *out,
                                  cudaStream_t s);
cudaError_t launch_label_energy(const float *x, const int16_t *labels, int M, int ns, int N, const int *pt_slot,
                                float scale, int accumulate, float *energy, cudaStream_t s);
int label_products_blocks(int ns);
// label products per block: mode 0: out[m] = sum a[m].*b[m]; mode 1: out[m*M+k] =
// sum a[m].*b[k]; the block partials are stored or added (accumulate) into part
// ([blocks][K] doubles), and launch_sum_parts_bm reduces such block-major partials
cudaError_t launch_label_products_part(const float *a, const float *b, int M, int ns, const int *slot_pt, int mode,
                                       double *part, int accumulate, cudaStream_t s);
cudaError_t launch_slice_grad(const SliceGradArgs &a, int MP, cudaStream_t s);
// out[k] (+)= sum over blocks of part[k][blk] (fixed order)
cudaError_t launch_sum_parts(const double *part, int nblk, int K, double *out, int accumulate, cudaStream_t s);
cudaError_t launch_sum_parts_bm(const double *part, int nblk, int K, double *out, int accumulate, cudaStream_t s);
// LogisticUnaryEnergy (unary.cpp:48-68): U = L f into slot rows (chunk_offset
// layout; L is M x F, f is F x N), and the parameter gradient b f^T summed over
// the points (M <= 32; out has M*F doubles, column-major in L; part holds
// logistic_grad_blocks * M * F doubles)
cudaError_t launch_logistic_unary(const float *L, const float *f, int M, int F, int N, int ns, const int *slot_pt,
                                  float *U, cudaStream_t s);
int logistic_grad_blocks(int ns, int M, int F);
cudaError_t launch_logistic_grad(const float *b, const float *f, int M, int F, int N, int ns, const int *slot_pt,
                                 double *part, double *out, cudaStream_t s);
int kernel_param_blocks(int N);
cudaError_t launch_kernel_param_grad(const float *f, const float *fg, int d, int N, int full, double *part,
                                     double *out, int accumulate, cudaStream_t s);

}  // namespace dcrf
