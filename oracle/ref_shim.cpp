// ref_shim.cpp -- test infrastructure, NOT part of the product.
//
// A thin extern "C" layer over the reference's own C++ classes (Krähenbühl's
// densecrf as vendored by pydensecrf), compiled together with the reference's
// unmodified sources by oracle/Makefile into oracle/_ref/libdcrf_ref.so.  Only
// the tests and tests/golden/make_golden.py load it, to pin the C restatement
// in oracle/dcrf_oracle.c and to produce golden fixtures.  Nothing here is
// shipped or timed as the product.
//
// Layout convention of every buffer crossing this boundary (same as the
// product's C-ABI): per-point-contiguous, i.e. element (label m, point n) of an
// M x N quantity lives at [n*M + m] -- exactly the memory of the reference's
// column-major Eigen MatrixXf (pydensecrf/densecrf/include/densecrf.h).
// Features are passed the same way: feature j of point n at [n*d + j].
#include <cstring>
#include <vector>
#include "densecrf.h"
#include "permutohedral.h"
#include "objective.h"

namespace {

// Exposes the protected lattice tables of Permutohedral
// (pydensecrf/densecrf/include/permutohedral.h:49-53).
struct DumpLattice : public Permutohedral {
    int vertices() const { return M_; }
    int dims() const { return d_; }
    const std::vector<int> &offsets() const { return offset_; }
    const std::vector<int> &ranks() const { return rank_; }
    const std::vector<float> &bary() const { return barycentric_; }
    int n1(int i) const { return blur_neighbors_[i].n1; }
    int n2(int i) const { return blur_neighbors_[i].n2; }
};

MatrixXf from_points(const float *p, int rows, int cols) {
    // p is per-point contiguous ([col*rows + row]) == column-major rows x cols
    MatrixXf m(rows, cols);
    std::memcpy(m.data(), p, sizeof(float) * (size_t)rows * cols);
    return m;
}

void to_points(const MatrixXf &m, float *p) {
    std::memcpy(p, m.data(), sizeof(float) * (size_t)m.rows() * m.cols());
}

LabelCompatibility *make_compat(int kind, const float *w, int M) {
    // kind 0: Potts(w[0]); 1: Diagonal(w[0..M)); 2: Matrix(w row-major M x M)
    if (kind == 0) return new PottsCompatibility(w[0]);
    if (kind == 1) {
        VectorXf v(M);
        for (int i = 0; i < M; i++) v[i] = w[i];
        return new DiagonalCompatibility(v);
    }
    MatrixXf m(M, M);
    for (int r = 0; r < M; r++)
        for (int c = 0; c < M; c++) m(r, c) = w[r * M + c];
    return new MatrixCompatibility(m);
}

}  // namespace

extern "C" {

// Lattice build over N points of dimension d; returns L (vertex count).
// offset/rank/bary: (d+1)*N each (the first N points; the reference allocates
// (d+1)*(N+16) on the SSE build); neighbors: 2*(d+1)*L ints (n1,n2 pairs,
// axis-major j*L+i) -- caller sizes it with ref_lattice_vertices first.
void *ref_lattice_new(const float *feat, int d, int N) {
    DumpLattice *lat = new DumpLattice();
    lat->init(from_points(feat, d, N));
    return lat;
}
int ref_lattice_vertices(void *h) { return static_cast<DumpLattice *>(h)->vertices(); }
void ref_lattice_dump(void *h, int N, int *offset, int *rank, float *bary, int *neighbors) {
    DumpLattice *lat = static_cast<DumpLattice *>(h);
    int d = lat->dims(), L = lat->vertices();
    size_t n = (size_t)(d + 1) * N;
    std::memcpy(offset, lat->offsets().data(), n * sizeof(int));
    std::memcpy(rank, lat->ranks().data(), n * sizeof(int));
    std::memcpy(bary, lat->bary().data(), n * sizeof(float));
    for (int i = 0; i < (d + 1) * L; i++) {
        neighbors[2 * i] = lat->n1(i);
        neighbors[2 * i + 1] = lat->n2(i);
    }
}
// out = lattice filter of `in` (value_size x N, per-point contiguous)
void ref_lattice_compute(void *h, const float *in, int value_size, int N, int reverse, float *out) {
    DumpLattice *lat = static_cast<DumpLattice *>(h);
    MatrixXf o;
    lat->compute(o, from_points(in, value_size, N), reverse != 0);
    to_points(o, out);
}
// df (N x d, per-point contiguous) = d/df a^T K b
void ref_lattice_gradient(void *h, const float *a, const float *b, int value_size, int N, float *df) {
    DumpLattice *lat = static_cast<DumpLattice *>(h);
    lat->gradient(df, a, b, value_size);
}
void ref_lattice_free(void *h) { delete static_cast<DumpLattice *>(h); }

// ---- DenseCRF / DenseCRF2D ------------------------------------------------
void *ref_crf_new(int N, int M) { return new DenseCRF(N, M); }
void *ref_crf2d_new(int W, int H, int M) { return new DenseCRF2D(W, H, M); }
void ref_crf_free(void *h) { delete static_cast<DenseCRF *>(h); }

// U: per-point contiguous M x N
void ref_crf_set_unary(void *h, const float *U, int M, int N) {
    static_cast<DenseCRF *>(h)->setUnaryEnergy(from_points(U, M, N));
}
// Logistic unary L (M x K) * f (K x N), both per-column contiguous
void ref_crf_set_unary_logistic(void *h, const float *Lmat, const float *f, int M, int K, int N) {
    static_cast<DenseCRF *>(h)->setUnaryEnergy(from_points(Lmat, M, K), from_points(f, K, N));
}
void ref_crf_add_pairwise(void *h, const float *feat, int d, int N, int compat_kind,
                          const float *compat, int M, int ktype, int ntype) {
    static_cast<DenseCRF *>(h)->addPairwiseEnergy(from_points(feat, d, N), make_compat(compat_kind, compat, M),
                                                  (KernelType)ktype, (NormalizationType)ntype);
}
void ref_crf2d_add_gaussian(void *h, float sx, float sy, int compat_kind, const float *compat, int M, int ktype,
                            int ntype) {
    static_cast<DenseCRF2D *>(h)->addPairwiseGaussian(sx, sy, make_compat(compat_kind, compat, M),
                                                      (KernelType)ktype, (NormalizationType)ntype);
}
void ref_crf2d_add_bilateral(void *h, float sx, float sy, float sr, float sg, float sb, const unsigned char *im,
                             int compat_kind, const float *compat, int M, int ktype, int ntype) {
    static_cast<DenseCRF2D *>(h)->addPairwiseBilateral(sx, sy, sr, sg, sb, im, make_compat(compat_kind, compat, M),
                                                       (KernelType)ktype, (NormalizationType)ntype);
}
void ref_crf_inference(void *h, int T, float *Q) { to_points(static_cast<DenseCRF *>(h)->inference(T), Q); }
void ref_crf_start(void *h, float *Q) { to_points(static_cast<DenseCRF *>(h)->startInference(), Q); }
void ref_crf_step(void *h, float *Q, int M, int N) {
    MatrixXf q = from_points(Q, M, N), t1, t2;
    static_cast<DenseCRF *>(h)->stepInference(q, t1, t2);
    to_points(q, Q);
}
double ref_crf_kl(void *h, const float *Q, int M, int N) {
    return static_cast<DenseCRF *>(h)->klDivergence(from_points(Q, M, N));
}
void ref_crf_map(void *h, int T, short *labels) {
    VectorXs r = static_cast<DenseCRF *>(h)->map(T);
    std::memcpy(labels, r.data(), sizeof(short) * r.size());
}
// DenseCRF::unaryEnergy / pairwiseEnergy (densecrf.cpp:141-177): per-point
// energies of the labelling l (N entries; labels outside [0, M) give 0);
// term -1 sums every pairwise term.
void ref_crf_unary_energy(void *h, const short *l, int N, float *out) {
    VectorXs v(N);
    for (int i = 0; i < N; i++) v[i] = l[i];
    VectorXf r = static_cast<DenseCRF *>(h)->unaryEnergy(v);
    std::memcpy(out, r.data(), sizeof(float) * r.size());
}
void ref_crf_pairwise_energy(void *h, const short *l, int N, int term, float *out) {
    VectorXs v(N);
    for (int i = 0; i < N; i++) v[i] = l[i];
    VectorXf r = static_cast<DenseCRF *>(h)->pairwiseEnergy(v, term);
    std::memcpy(out, r.data(), sizeof(float) * r.size());
}
// Parameter vectors: sizes via *_count
int ref_crf_compat_param_count(void *h) { return (int)static_cast<DenseCRF *>(h)->labelCompatibilityParameters().size(); }
int ref_crf_kernel_param_count(void *h) { return (int)static_cast<DenseCRF *>(h)->kernelParameters().size(); }
int ref_crf_unary_param_count(void *h) { return (int)static_cast<DenseCRF *>(h)->unaryParameters().size(); }
void ref_crf_set_kernel_params(void *h, const float *p, int n) {
    VectorXf v(n);
    for (int i = 0; i < n; i++) v[i] = p[i];
    static_cast<DenseCRF *>(h)->setKernelParameters(v);
}
void ref_crf_set_compat_params(void *h, const float *p, int n) {
    VectorXf v(n);
    for (int i = 0; i < n; i++) v[i] = p[i];
    static_cast<DenseCRF *>(h)->setLabelCompatibilityParameters(v);
}
// gradient of mean log-likelihood of gt after T iterations
// (pydensecrf/densecrf/src/densecrf.cpp:238-297 with objective.cpp:37-50).
double ref_crf_gradient(void *h, int T, const short *gt, int N, float *unary_grad, float *compat_grad,
                        float *kernel_grad) {
    DenseCRF *c = static_cast<DenseCRF *>(h);
    VectorXs g(N);
    for (int i = 0; i < N; i++) g[i] = gt[i];
    LogLikelihood obj(g, 0.f);
    VectorXf ug, cg, kg;
    double r = c->gradient(T, obj, unary_grad ? &ug : nullptr, compat_grad ? &cg : nullptr,
                           kernel_grad ? &kg : nullptr);
    if (unary_grad) std::memcpy(unary_grad, ug.data(), sizeof(float) * ug.size());
    if (compat_grad) std::memcpy(compat_grad, cg.data(), sizeof(float) * cg.size());
    if (kernel_grad) std::memcpy(kernel_grad, kg.data(), sizeof(float) * kg.size());
    return r;
}

}  // extern "C"
