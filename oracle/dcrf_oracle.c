/*
 * dcrf_oracle.c -- TEST INFRASTRUCTURE ONLY: the CPU oracle of the dense-CRF
 * hot path.  Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
 * arm may load it, and only as the checker / the timed CPU baseline; the
 * product (pydensecrf_gb300) never calls it.
 *
 * A plain-C restatement of the mean-field inference of Krähenbühl's densecrf
 * as vendored by lucasb-eyer/pydensecrf.  Every function names the reference
 * file:line it follows (paths relative to the pydensecrf project root,
 * abbreviated: P = pydensecrf/densecrf/src/permutohedral.cpp,
 * K = pydensecrf/densecrf/src/pairwise.cpp, D = pydensecrf/densecrf/src/densecrf.cpp,
 * C = pydensecrf/densecrf/src/labelcompatibility.cpp,
 * O = pydensecrf/densecrf/src/objective.cpp).
 *
 * The reference compiles two different lattice builds depending on the host
 * ISA, and both are restated here, selected by `variant`:
 *   ORC_VARIANT_SSE    (0) -- x86-64 builds (__SSE__ defined): P:140-321 and
 *                             the SSE filter P:529-589 for value_size > 2.
 *   ORC_VARIANT_SCALAR (1) -- builds without SSE (e.g. aarch64): P:323-474
 *                             and seqCompute P:476-527 for every value size.
 * Both are restated operation by operation in float (with the double-precision
 * steps where the reference has them), so that the lattice tables come out
 * bit-identical to the reference's, and Q agrees to the ulp level (the only
 * differences are libm expf vs Eigen's vectorised exp and the order of the
 * softmax / matrix-compatibility sums).
 *
 * A second, FP64 restatement of the same mean-field (same lattice structure,
 * every value in double) is provided as orc_crf_inference_f64 to state the
 * error of every float result against the exact-arithmetic limit.
 *
 * Layout of every buffer: per-point contiguous, element (m, n) of an M x N
 * quantity at [n*M + m] (the memory of the reference's column-major MatrixXf);
 * features: feature j of point n at [n*d + j].
 *
 * Build: gcc -O3 -ffp-contract=off -fPIC -shared (oracle/Makefile).  FP
 * contraction must stay off: the reference's x86 build has no FMA, and the
 * restatement must round every product and sum separately.  -O3 vectorises
 * only the element-wise loops over labels (each lane rounds exactly as the
 * scalar code does; without -ffast-math no sum is reassociated), which keeps
 * the results bit-identical to -O2 and the speed close to the reference's
 * SSE-packed loops, so that the oracle timed as the CPU baseline is not
 * slower than the code it restates.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define ORC_VARIANT_SSE 0
#define ORC_VARIANT_SCALAR 1

/* ------------------------------------------------------------------------ */
/* Hash table on int16 keys: linear probing, ids in insertion order.         */
/* Follows P:54-131 (hash r=(r+k)*1664525, capacity doubles at 50% load).    */
/* ------------------------------------------------------------------------ */
typedef struct {
    size_t key_size, filled, capacity;
    short *keys; /* (capacity/2+10)*key_size */
    int *table;  /* capacity */
} orc_hash;

static size_t orc_hash_fn(const orc_hash *h, const short *k) {
    size_t r = 0;
    for (size_t i = 0; i < h->key_size; i++) {
        r += (size_t)(long)k[i];
        r *= 1664525;
    }
    return r;
}

static void orc_hash_init(orc_hash *h, int key_size, size_t n_elements) {
    h->key_size = key_size;
    h->filled = 0;
    h->capacity = 2 * n_elements;
    if (h->capacity < 2) h->capacity = 2;
    h->keys = (short *)calloc((h->capacity / 2 + 10) * (key_size ? key_size : 1), sizeof(short));
    h->table = (int *)malloc(h->capacity * sizeof(int));
    for (size_t i = 0; i < h->capacity; i++) h->table[i] = -1;
}

static void orc_hash_free(orc_hash *h) {
    free(h->keys);
    free(h->table);
}

static void orc_hash_grow(orc_hash *h) {
    size_t old_cap = h->capacity;
    h->capacity *= 2;
    short *nk = (short *)calloc((h->capacity / 2 + 10) * (h->key_size ? h->key_size : 1), sizeof(short));
    memcpy(nk, h->keys, h->filled * h->key_size * sizeof(short));
    int *nt = (int *)malloc(h->capacity * sizeof(int));
    for (size_t i = 0; i < h->capacity; i++) nt[i] = -1;
    for (size_t i = 0; i < old_cap; i++) {
        int e = h->table[i];
        if (e >= 0) {
            size_t p = orc_hash_fn(h, nk + (size_t)e * h->key_size) % h->capacity;
            while (nt[p] >= 0) p = p < h->capacity - 1 ? p + 1 : 0;
            nt[p] = e;
        }
    }
    free(h->keys);
    free(h->table);
    h->keys = nk;
    h->table = nt;
}

static int orc_hash_find(orc_hash *h, const short *k, int create) {
    if (2 * h->filled >= h->capacity) orc_hash_grow(h);
    size_t p = orc_hash_fn(h, k) % h->capacity;
    for (;;) {
        int e = h->table[p];
        if (e == -1) {
            if (!create) return -1;
            memcpy(h->keys + h->filled * h->key_size, k, h->key_size * sizeof(short));
            h->table[p] = (int)h->filled;
            return (int)h->filled++;
        }
        if (memcmp(h->keys + (size_t)e * h->key_size, k, h->key_size * sizeof(short)) == 0) return e;
        p++;
        if (p == h->capacity) p = 0;
    }
}

/* ------------------------------------------------------------------------ */
/* Lattice                                                                   */
/* ------------------------------------------------------------------------ */
typedef struct {
    int N, d, L, variant;
    int n_phantom; /* zero-feature padding points inserted by the SSE build */
    int *offset;   /* (d+1)*N */
    int *rank;     /* (d+1)*N */
    float *bary;   /* (d+1)*N */
    int *nbr;      /* 2*(d+1)*L : (n1,n2) for axis j, vertex i at 2*(j*L+i) */
    short *keys;   /* L*d */
} orc_lattice;

/* scale factors of the elevation matrix, P:178-182 / P:352-356 */
static void orc_scale_factors(int d, float *sf) {
    float inv_std_dev = (float)(sqrt(2.0 / 3.0) * (d + 1));
    for (int i = 0; i < d; i++) sf[i] = (float)(1.0 / sqrt((double)((i + 2) * (i + 1))) * (double)inv_std_dev);
}

/* Per-point embedding of the SSE build (one lane of P:191-275). */
static void orc_embed_sse(int d, const float *f, const float *sf, float *elevated, float *rem0, float *rank,
                          float *bary) {
    const float invdp1 = 1.0f / (float)(d + 1);
    const float dp1 = (float)(d + 1);
    float sm = 0.0f;
    for (int j = d; j > 0; j--) {
        float cf = f[j - 1] * sf[j - 1];
        float t = (float)j * cf;
        elevated[j] = sm - t;
        sm += cf;
    }
    elevated[0] = sm;
    float sum = 0.0f;
    for (int i = 0; i <= d; i++) { /* cvtps under round-to-nearest-even */
        float v = invdp1 * elevated[i];
        v = rintf(v);
        rem0[i] = v * dp1;
        sum += v;
    }
    for (int i = 0; i <= d; i++) rank[i] = 0.0f;
    for (int i = 0; i < d; i++) {
        float di = elevated[i] - rem0[i];
        for (int j = i + 1; j <= d; j++) {
            float dj = elevated[j] - rem0[j];
            float c = (di < dj) ? 1.0f : 0.0f;
            rank[i] += c;
            rank[j] += 1.0f - c;
        }
    }
    for (int i = 0; i <= d; i++) {
        rank[i] += sum;
        float add = rank[i] < 0.0f ? dp1 : 0.0f;
        float sub = rank[i] >= dp1 ? dp1 : 0.0f;
        rank[i] += add - sub;
        rem0[i] += add - sub;
    }
    for (int i = 0; i < d + 2; i++) bary[i] = 0.0f;
    for (int i = 0; i <= d; i++) {
        float v = (elevated[i] - rem0[i]) * invdp1;
        int p = (int)((float)d - rank[i]);
        bary[p] += v;
        bary[p + 1] -= v;
    }
    bary[0] += 1.0f + bary[d + 1]; /* P:263, float */
}

/* Per-point embedding of the scalar build. rank returned as float
 * holding the short values. */
static void orc_embed_scalar(int d, const float *f, const float *sf, float *elevated, float *rem0, float *rankf,
                             float *bary) {
    short rank[64];
    float sm = 0.0f;
    for (int j = d; j > 0; j--) {
        float cf = f[j - 1] * sf[j - 1];
        float t = (float)j * cf;
        elevated[j] = sm - t;
        sm += cf;
    }
    elevated[0] = sm;
    const float down_factor = 1.0f / (float)(d + 1);
    const float up_factor = (float)(d + 1);
    int sum = 0;
    for (int i = 0; i <= d; i++) {
        int rd2;
        float v = down_factor * elevated[i];
        float up = ceilf(v) * up_factor;
        float down = floorf(v) * up_factor;
        if (up - elevated[i] < elevated[i] - down)
            rd2 = (short)up;
        else
            rd2 = (short)down;
        rem0[i] = (float)rd2;
        sum = (int)((float)sum + (float)rd2 * down_factor); /* int += float truncates */
    }
    for (int i = 0; i <= d; i++) rank[i] = 0;
    for (int i = 0; i < d; i++) {
        double di = elevated[i] - rem0[i];
        for (int j = i + 1; j <= d; j++)
            if (di < (double)(elevated[j] - rem0[j]))
                rank[i]++;
            else
                rank[j]++;
    }
    for (int i = 0; i <= d; i++) {
        rank[i] = (short)(rank[i] + sum);
        if (rank[i] < 0) {
            rank[i] = (short)(rank[i] + d + 1);
            rem0[i] += d + 1;
        } else if (rank[i] > d) {
            rank[i] = (short)(rank[i] - (d + 1));
            rem0[i] -= d + 1;
        }
    }
    for (int i = 0; i < d + 2; i++) bary[i] = 0.0f;
    for (int i = 0; i <= d; i++) {
        float v = (elevated[i] - rem0[i]) * down_factor;
        bary[d - rank[i]] += v;
        bary[d - rank[i] + 1] -= v;
    }
    bary[0] = (float)((double)bary[0] + (1.0 + (double)bary[d + 1])); /* P:426, double */
    for (int i = 0; i <= d; i++) rankf[i] = (float)rank[i];
}

void orc_lattice_free(void *hp);

/* Lattice build: P:140-321 (SSE) or P:323-474 (scalar). Returns NULL if d>62. */
void *orc_lattice_new(const float *feat, int d, int N, int variant) {
    if (d < 1 || d > 62 || N < 0) return NULL;
    orc_lattice *lat = (orc_lattice *)calloc(1, sizeof(orc_lattice));
    lat->N = N;
    lat->d = d;
    lat->variant = variant;
    int Npad = N;
    if (variant == ORC_VARIANT_SSE) Npad = (N + 3) / 4 * 4; /* P:191 blocks of 4, zero-padded */
    lat->n_phantom = Npad - N;
    size_t nn = (size_t)(d + 1) * N;
    lat->offset = (int *)malloc((nn ? nn : 1) * sizeof(int));
    lat->rank = (int *)malloc((nn ? nn : 1) * sizeof(int));
    lat->bary = (float *)malloc((nn ? nn : 1) * sizeof(float));
    orc_hash h;
    orc_hash_init(&h, d, variant == ORC_VARIANT_SSE ? (size_t)N : (size_t)N * (d + 1));
    float sf[64], el[64], rem0[64], rank[64], bary[66], zero[64];
    short key[64];
    memset(zero, 0, sizeof(zero));
    orc_scale_factors(d, sf);
    for (int k = 0; k < Npad; k++) {
        const float *f = k < N ? feat + (size_t)k * d : zero;
        if (variant == ORC_VARIANT_SSE)
            orc_embed_sse(d, f, sf, el, rem0, rank, bary);
        else
            orc_embed_scalar(d, f, sf, el, rem0, rank, bary);
        for (int r = 0; r <= d; r++) { /* P:268-275 / P:429-435 */
            for (int i = 0; i < d; i++) {
                int ri = (int)rank[i];
                short canon = (short)(ri <= d - r ? r : r - (d + 1)); /* canonical simplex */
                key[i] = (short)(int)(rem0[i] + (float)canon);
            }
            int id = orc_hash_find(&h, key, 1);
            if (k < N) {
                lat->offset[(size_t)k * (d + 1) + r] = id;
                lat->rank[(size_t)k * (d + 1) + r] = (int)rank[r];
                lat->bary[(size_t)k * (d + 1) + r] = bary[r];
            }
        }
    }
    int L = (int)h.filled;
    lat->L = L;
    lat->keys = (short *)malloc(((size_t)L * d + 1) * sizeof(short));
    memcpy(lat->keys, h.keys, (size_t)L * d * sizeof(short));
    lat->nbr = (int *)malloc(((size_t)2 * (d + 1) * L + 1) * sizeof(int));
    short n1[64], n2[64];
    for (int j = 0; j <= d; j++) {
        for (int i = 0; i < L; i++) {
            const short *kk = lat->keys + (size_t)i * d;
            for (int q = 0; q < d; q++) {
                n1[q] = (short)(kk[q] - 1);
                n2[q] = (short)(kk[q] + 1);
            }
            if (j < d) {
                n1[j] = (short)(kk[j] + d);
                n2[j] = (short)(kk[j] - d);
            }
            lat->nbr[2 * ((size_t)j * L + i)] = orc_hash_find(&h, n1, 0);
            lat->nbr[2 * ((size_t)j * L + i) + 1] = orc_hash_find(&h, n2, 0);
        }
    }
    orc_hash_free(&h);
    return lat;
}

int orc_lattice_vertices(void *hp) { return ((orc_lattice *)hp)->L; }
int orc_lattice_phantoms(void *hp) { return ((orc_lattice *)hp)->n_phantom; }

void orc_lattice_dump(void *hp, int *offset, int *rank, float *bary, int *nbr, short *keys) {
    orc_lattice *l = (orc_lattice *)hp;
    size_t nn = (size_t)(l->d + 1) * l->N;
    if (offset) memcpy(offset, l->offset, nn * sizeof(int));
    if (rank) memcpy(rank, l->rank, nn * sizeof(int));
    if (bary) memcpy(bary, l->bary, nn * sizeof(float));
    if (nbr) memcpy(nbr, l->nbr, (size_t)2 * (l->d + 1) * l->L * sizeof(int));
    if (keys) memcpy(keys, l->keys, (size_t)l->L * l->d * sizeof(short));
}

void orc_lattice_free(void *hp) {
    orc_lattice *l = (orc_lattice *)hp;
    if (!l) return;
    free(l->offset);
    free(l->rank);
    free(l->bary);
    free(l->nbr);
    free(l->keys);
    free(l);
}

/* seqCompute: float splat, double-rounded blur, (w*v)*alpha slice */
static void orc_seq_compute(const orc_lattice *l, float *out, const float *in, int vs, int reverse) {
    int d = l->d, L = l->L, N = l->N;
    float *values = (float *)calloc((size_t)(L + 2) * vs, sizeof(float));
    float *nv = (float *)calloc((size_t)(L + 2) * vs, sizeof(float));
    for (int i = 0; i < N; i++)
        for (int j = 0; j <= d; j++) {
            int o = l->offset[(size_t)i * (d + 1) + j] + 1;
            float w = l->bary[(size_t)i * (d + 1) + j];
            for (int k = 0; k < vs; k++) {
                float t = w * in[(size_t)i * vs + k];
                values[(size_t)o * vs + k] += t;
            }
        }
    for (int jj = 0; jj <= d; jj++) {
        int j = reverse ? d - jj : jj;
        for (int i = 0; i < L; i++) {
            const float *ov = values + (size_t)(i + 1) * vs;
            float *w = nv + (size_t)(i + 1) * vs;
            int n1 = l->nbr[2 * ((size_t)j * L + i)] + 1, n2 = l->nbr[2 * ((size_t)j * L + i) + 1] + 1;
            const float *a = values + (size_t)n1 * vs, *b = values + (size_t)n2 * vs;
            for (int k = 0; k < vs; k++) {
                float s = a[k] + b[k];
                w[k] = (float)((double)ov[k] + 0.5 * (double)s);
            }
        }
        float *t = values;
        values = nv;
        nv = t;
    }
    float alpha = 1.0f / (1.0f + powf(2.0f, (float)-d));
    for (int i = 0; i < N; i++) {
        for (int k = 0; k < vs; k++) out[(size_t)i * vs + k] = 0.0f;
        for (int j = 0; j <= d; j++) {
            int o = l->offset[(size_t)i * (d + 1) + j] + 1;
            float w = l->bary[(size_t)i * (d + 1) + j];
            for (int k = 0; k < vs; k++) {
                float t = w * values[(size_t)o * vs + k];
                t = t * alpha;
                out[(size_t)i * vs + k] += t;
            }
        }
    }
    free(values);
    free(nv);
}

/* sseCompute: float everywhere, slice weight w*alpha rounded first */
static void orc_sse_compute(const orc_lattice *l, float *out, const float *in, int vs, int reverse) {
    int d = l->d, L = l->L, N = l->N;
    float *values = (float *)calloc((size_t)(L + 2) * vs, sizeof(float));
    float *nv = (float *)calloc((size_t)(L + 2) * vs, sizeof(float));
    for (int i = 0; i < N; i++)
        for (int j = 0; j <= d; j++) {
            int o = l->offset[(size_t)i * (d + 1) + j] + 1;
            float w = l->bary[(size_t)i * (d + 1) + j];
            for (int k = 0; k < vs; k++) {
                float t = w * in[(size_t)i * vs + k];
                values[(size_t)o * vs + k] += t;
            }
        }
    for (int jj = 0; jj <= d; jj++) {
        int j = reverse ? d - jj : jj;
        for (int i = 0; i < L; i++) {
            const float *ov = values + (size_t)(i + 1) * vs;
            float *w = nv + (size_t)(i + 1) * vs;
            int n1 = l->nbr[2 * ((size_t)j * L + i)] + 1, n2 = l->nbr[2 * ((size_t)j * L + i) + 1] + 1;
            const float *a = values + (size_t)n1 * vs, *b = values + (size_t)n2 * vs;
            for (int k = 0; k < vs; k++) {
                float s = a[k] + b[k];
                float h = 0.5f * s;
                w[k] = ov[k] + h;
            }
        }
        float *t = values;
        values = nv;
        nv = t;
    }
    float alpha = 1.0f / (1.0f + powf(2.0f, (float)-d));
    float *acc = (float *)malloc((size_t)vs * sizeof(float));
    for (int i = 0; i < N; i++) {
        for (int k = 0; k < vs; k++) acc[k] = 0.0f;
        for (int j = 0; j <= d; j++) {
            int o = l->offset[(size_t)i * (d + 1) + j] + 1;
            float w = l->bary[(size_t)i * (d + 1) + j] * alpha;
            for (int k = 0; k < vs; k++) {
                float t = w * values[(size_t)o * vs + k];
                acc[k] += t;
            }
        }
        memcpy(out + (size_t)i * vs, acc, (size_t)vs * sizeof(float));
    }
    free(acc);
    free(values);
    free(nv);
}

/* Permutohedral::compute dispatch, P:596-604 (the scalar build maps sse to seq).
 * `out` may be `in`: the splat reads all of `in` before the slice writes `out`. */
void orc_lattice_compute(void *hp, const float *in, int vs, int reverse, float *out) {
    orc_lattice *l = (orc_lattice *)hp;
    if (vs <= 2 || l->variant == ORC_VARIANT_SCALAR)
        orc_seq_compute(l, out, in, vs, reverse);
    else
        orc_sse_compute(l, out, in, vs, reverse);
}

/* FP64 filter over the same lattice structure (no reference counterpart: the
 * exact-arithmetic limit of P:476-527). */
static void orc_compute_f64(const orc_lattice *l, double *out, const double *in, int vs, int reverse) {
    int d = l->d, L = l->L, N = l->N;
    double *values = (double *)calloc((size_t)(L + 2) * vs, sizeof(double));
    double *nv = (double *)calloc((size_t)(L + 2) * vs, sizeof(double));
    for (int i = 0; i < N; i++)
        for (int j = 0; j <= d; j++) {
            int o = l->offset[(size_t)i * (d + 1) + j] + 1;
            double w = l->bary[(size_t)i * (d + 1) + j];
            for (int k = 0; k < vs; k++) values[(size_t)o * vs + k] += w * in[(size_t)i * vs + k];
        }
    for (int jj = 0; jj <= d; jj++) {
        int j = reverse ? d - jj : jj;
        for (int i = 0; i < L; i++) {
            int n1 = l->nbr[2 * ((size_t)j * L + i)] + 1, n2 = l->nbr[2 * ((size_t)j * L + i) + 1] + 1;
            for (int k = 0; k < vs; k++)
                nv[(size_t)(i + 1) * vs + k] = values[(size_t)(i + 1) * vs + k] +
                                               0.5 * (values[(size_t)n1 * vs + k] + values[(size_t)n2 * vs + k]);
        }
        double *t = values;
        values = nv;
        nv = t;
    }
    double alpha = 1.0 / (1.0 + pow(2.0, -d));
    for (int i = 0; i < N; i++) {
        for (int k = 0; k < vs; k++) out[(size_t)i * vs + k] = 0.0;
        for (int j = 0; j <= d; j++) {
            int o = l->offset[(size_t)i * (d + 1) + j] + 1;
            double w = l->bary[(size_t)i * (d + 1) + j];
            for (int k = 0; k < vs; k++) out[(size_t)i * vs + k] += w * alpha * values[(size_t)o * vs + k];
        }
    }
    free(values);
    free(nv);
}

/* ------------------------------------------------------------------------ */
/* DenseCRF                                                                  */
/* ------------------------------------------------------------------------ */
enum { ORC_NO_NORMALIZATION = 0, ORC_NORMALIZE_BEFORE, ORC_NORMALIZE_AFTER, ORC_NORMALIZE_SYMMETRIC };
enum { ORC_CONST_KERNEL = 0, ORC_DIAG_KERNEL, ORC_FULL_KERNEL };
enum { ORC_POTTS = 0, ORC_DIAGONAL, ORC_MATRIX };

typedef struct {
    orc_lattice *lat;
    int d, ktype, ntype, ckind;
    float *feat;   /* N*d, unscaled features as given */
    float *norm;   /* N */
    double *norm64;
    float *compat; /* Potts: 1, Diagonal: M, Matrix: M*M symmetrised (row-major) */
} orc_term;

typedef struct {
    int N, M, variant, nterms, has_unary;
    float *unary; /* N*M */
    float *ws;    /* 3 x (N*M+1) floats of scratch, made on first use */
    orc_term terms[16];
} orc_crf;

/* Scratch buffer i (0..2) of N*M floats, kept for the CRF's lifetime so that
 * the iterations run on warm pages rather than on freshly mapped ones. */
static float *orc_scratch(const orc_crf *cc, int i) {
    orc_crf *c = (orc_crf *)cc;
    size_t stride = (size_t)c->N * c->M + 1;
    if (!c->ws) c->ws = (float *)malloc(3 * stride * sizeof(float));
    return c->ws + (size_t)i * stride;
}

void *orc_crf_new(int N, int M, int variant) {
    orc_crf *c = (orc_crf *)calloc(1, sizeof(orc_crf));
    c->N = N;
    c->M = M;
    c->variant = variant;
    c->unary = (float *)calloc((size_t)N * M + 1, sizeof(float));
    return c;
}

void orc_crf_free(void *cp) {
    orc_crf *c = (orc_crf *)cp;
    for (int t = 0; t < c->nterms; t++) {
        orc_lattice_free(c->terms[t].lat);
        free(c->terms[t].feat);
        free(c->terms[t].norm);
        free(c->terms[t].norm64);
        free(c->terms[t].compat);
    }
    free(c->unary);
    free(c->ws);
    free(c);
}

void orc_crf_set_unary(void *cp, const float *U) { /* D:89-91 */
    orc_crf *c = (orc_crf *)cp;
    memcpy(c->unary, U, (size_t)c->N * c->M * sizeof(float));
    c->has_unary = 1;
}

/* DenseKernel::initLattice, K:40-62 */
static void orc_term_init_lattice(orc_crf *c, orc_term *t, const float *f) {
    int N = c->N;
    if (t->lat) orc_lattice_free(t->lat);
    t->lat = (orc_lattice *)orc_lattice_new(f, t->d, N, c->variant);
    float *ones = (float *)malloc(((size_t)N + 1) * sizeof(float));
    for (int i = 0; i < N; i++) ones[i] = 1.0f;
    free(t->norm);
    t->norm = (float *)malloc(((size_t)N + 1) * sizeof(float));
    orc_seq_compute(t->lat, t->norm, ones, 1, 0); /* rows == 1 -> seqCompute */
    /* FP64 norm over the same structure */
    double *ones64 = (double *)malloc(((size_t)N + 1) * sizeof(double));
    for (int i = 0; i < N; i++) ones64[i] = 1.0;
    free(t->norm64);
    t->norm64 = (double *)malloc(((size_t)N + 1) * sizeof(double));
    orc_compute_f64(t->lat, t->norm64, ones64, 1, 0);
    if (t->ntype == ORC_NO_NORMALIZATION) {
        float mean_norm = 0.0f;
        for (int i = 0; i < N; i++) mean_norm += t->norm[i];
        mean_norm = (float)N / mean_norm;
        for (int i = 0; i < N; i++) t->norm[i] = mean_norm;
        double mn = 0.0;
        for (int i = 0; i < N; i++) mn += t->norm64[i];
        for (int i = 0; i < N; i++) t->norm64[i] = N / mn;
    } else if (t->ntype == ORC_NORMALIZE_SYMMETRIC) {
        for (int i = 0; i < N; i++) t->norm[i] = (float)(1.0 / sqrt((double)t->norm[i] + 1e-20));
        for (int i = 0; i < N; i++) t->norm64[i] = 1.0 / sqrt(t->norm64[i] + 1e-20);
    } else {
        for (int i = 0; i < N; i++) t->norm[i] = (float)(1.0 / ((double)t->norm[i] + 1e-20));
        for (int i = 0; i < N; i++) t->norm64[i] = 1.0 / (t->norm64[i] + 1e-20);
    }
    free(ones);
    free(ones64);
}

/* addPairwiseEnergy, D:54-57 + K:116-122 + compat ctors C:44-45,64-65,79-81.
 * Returns the term index, or -1. */
int orc_crf_add_pairwise(void *cp, const float *feat, int d, int ckind, const float *compat, int ktype, int ntype) {
    orc_crf *c = (orc_crf *)cp;
    if (c->nterms >= 16) return -1;
    orc_term *t = &c->terms[c->nterms];
    memset(t, 0, sizeof(*t));
    t->d = d;
    t->ktype = ktype;
    t->ntype = ntype;
    t->ckind = ckind;
    int M = c->M;
    t->feat = (float *)malloc(((size_t)c->N * d + 1) * sizeof(float));
    memcpy(t->feat, feat, (size_t)c->N * d * sizeof(float));
    if (ckind == ORC_POTTS) {
        t->compat = (float *)malloc(sizeof(float));
        t->compat[0] = compat[0];
    } else if (ckind == ORC_DIAGONAL) {
        t->compat = (float *)malloc((size_t)M * sizeof(float));
        memcpy(t->compat, compat, (size_t)M * sizeof(float));
    } else {
        t->compat = (float *)malloc((size_t)M * M * sizeof(float));
        for (int a = 0; a < M; a++)
            for (int b = 0; b < M; b++) {
                float s = compat[a * M + b] + compat[b * M + a];
                t->compat[a * M + b] = 0.5f * s;
            }
    }
    orc_term_init_lattice(c, t, feat);
    return c->nterms++;
}

/* DenseKernel::filter, K:63-80; then LabelCompatibility::apply (C:46-48,66-68,82-84) */
static void orc_term_apply(const orc_crf *c, const orc_term *t, float *out, const float *Q, int transpose) {
    int N = c->N, M = c->M;
    size_t NM = (size_t)N * M;
    float *tmp = orc_scratch(c, 2);
    int pre = t->ntype == ORC_NORMALIZE_SYMMETRIC || (t->ntype == ORC_NORMALIZE_BEFORE && !transpose) ||
              (t->ntype == ORC_NORMALIZE_AFTER && transpose);
    int post = t->ntype == ORC_NORMALIZE_SYMMETRIC || (t->ntype == ORC_NORMALIZE_BEFORE && transpose) ||
               (t->ntype == ORC_NORMALIZE_AFTER && !transpose);
    for (int n = 0; n < N; n++)
        for (int m = 0; m < M; m++) tmp[(size_t)n * M + m] = pre ? Q[(size_t)n * M + m] * t->norm[n] : Q[(size_t)n * M + m];
    orc_lattice_compute(t->lat, tmp, M, transpose, tmp);
    if (post)
        for (int n = 0; n < N; n++)
            for (int m = 0; m < M; m++) tmp[(size_t)n * M + m] = tmp[(size_t)n * M + m] * t->norm[n];
    if (t->ckind == ORC_POTTS) {
        float nw = -t->compat[0];
        for (size_t i = 0; i < NM; i++) out[i] = nw * tmp[i];
    } else if (t->ckind == ORC_DIAGONAL) {
        for (int n = 0; n < N; n++)
            for (int m = 0; m < M; m++) out[(size_t)n * M + m] = t->compat[m] * tmp[(size_t)n * M + m];
    } else {
        for (int n = 0; n < N; n++)
            for (int m = 0; m < M; m++) {
                float s = 0.0f;
                for (int k = 0; k < M; k++) {
                    float p = (transpose ? t->compat[k * M + m] : t->compat[m * M + k]) * tmp[(size_t)n * M + k];
                    s += p;
                }
                out[(size_t)n * M + m] = s;
            }
    }
}

/* expAndNormalize, D:98-106 */
static void orc_softmax(int N, int M, float *out, const float *in) {
    for (int n = 0; n < N; n++) {
        const float *b = in + (size_t)n * M;
        float mx = b[0];
        for (int m = 1; m < M; m++)
            if (b[m] > mx) mx = b[m];
        float e[4096];
        float s = 0.0f;
        for (int m = 0; m < M; m++) {
            e[m] = expf(b[m] - mx);
            s += e[m];
        }
        for (int m = 0; m < M; m++) out[(size_t)n * M + m] = e[m] / s;
    }
}

/* one mean-field update of Q in place, D:187-201 (the body of D:122-129) */
static void orc_step(const orc_crf *c, float *Q) {
    int N = c->N, M = c->M;
    size_t NM = (size_t)N * M;
    float *t1 = orc_scratch(c, 0);
    float *t2 = orc_scratch(c, 1);
    for (size_t i = 0; i < NM; i++) t1[i] = c->has_unary ? -c->unary[i] : 0.0f;
    for (int k = 0; k < c->nterms; k++) {
        orc_term_apply(c, &c->terms[k], t2, Q, 0);
        for (size_t i = 0; i < NM; i++) t1[i] -= t2[i];
    }
    orc_softmax(N, M, Q, t1);
}

/* inference, D:115-131 */
void orc_crf_inference(void *cp, int T, float *Q) {
    orc_crf *c = (orc_crf *)cp;
    size_t NM = (size_t)c->N * c->M;
    float *nu = (float *)malloc((NM + 1) * sizeof(float));
    for (size_t i = 0; i < NM; i++) nu[i] = c->has_unary ? -c->unary[i] : 0.0f;
    orc_softmax(c->N, c->M, Q, nu);
    free(nu);
    for (int it = 0; it < T; it++) orc_step(c, Q);
}

/* startInference, D:178-186 (zeros when no unary is set) */
void orc_crf_start(void *cp, float *Q) {
    orc_crf *c = (orc_crf *)cp;
    size_t NM = (size_t)c->N * c->M;
    if (!c->has_unary) {
        memset(Q, 0, NM * sizeof(float));
        return;
    }
    float *nu = (float *)malloc((NM + 1) * sizeof(float));
    for (size_t i = 0; i < NM; i++) nu[i] = -c->unary[i];
    orc_softmax(c->N, c->M, Q, nu);
    free(nu);
}

void orc_crf_step(void *cp, float *Q) { orc_step((orc_crf *)cp, Q); }

/* Float sum in the order of the reference's vectorised Eigen reduction
 * (pydensecrf/densecrf/include/Eigen/src/Core/Redux.h:215-254 with 4-lane SSE
 * packets): two interleaved 4-lane accumulators over blocks of 8, an optional
 * trailing packet, a horizontal (l0+l2)+(l1+l3) sum, then the scalar tail. */
static float orc_packet_sum(const float *x, size_t n) {
    size_t aligned = n / 4 * 4, aligned2 = n / 8 * 8;
    if (aligned == 0) {
        float r = n ? x[0] : 0.0f;
        for (size_t i = 1; i < n; i++) r += x[i];
        return r;
    }
    float a[4], b[4];
    for (int l = 0; l < 4; l++) a[l] = x[l];
    if (aligned > 4) {
        for (int l = 0; l < 4; l++) b[l] = x[4 + l];
        for (size_t i = 8; i < aligned2; i += 8)
            for (int l = 0; l < 4; l++) {
                a[l] += x[i + l];
                b[l] += x[i + 4 + l];
            }
        for (int l = 0; l < 4; l++) a[l] += b[l];
        if (aligned > aligned2)
            for (int l = 0; l < 4; l++) a[l] += x[aligned2 + l];
    }
    float r = (a[0] + a[2]) + (a[1] + a[3]);
    for (size_t i = aligned; i < n; i++) r += x[i];
    return r;
}

/* klDivergence, D:214-235 */
double orc_crf_kl(void *cp, const float *Q) {
    orc_crf *c = (orc_crf *)cp;
    int N = c->N, M = c->M;
    size_t NM = (size_t)N * M;
    double kl = 0.0;
    for (size_t i = 0; i < NM; i++) { /* unqualified log() resolves to log(double) */
        float q = Q[i];
        kl += (double)q * log((double)(q > 1e-20f ? q : 1e-20f));
    }
    if (c->has_unary)
        for (size_t i = 0; i < NM; i++) kl += (double)(c->unary[i] * Q[i]);
    float *tmp = orc_scratch(c, 0);
    for (int k = 0; k < c->nterms; k++) {
        orc_term_apply(c, &c->terms[k], tmp, Q, 0);
        for (size_t i = 0; i < NM; i++) tmp[i] = Q[i] * tmp[i];
        kl += (double)orc_packet_sum(tmp, NM);
    }
    return kl;
}

/* map / currentMap, D:132-137,202-211: first maximum */
void orc_crf_map(void *cp, int T, short *labels) {
    orc_crf *c = (orc_crf *)cp;
    size_t NM = (size_t)c->N * c->M;
    float *Q = (float *)malloc((NM + 1) * sizeof(float));
    orc_crf_inference(cp, T, Q);
    for (int n = 0; n < c->N; n++) {
        int best = 0;
        for (int m = 1; m < c->M; m++)
            if (Q[(size_t)n * c->M + m] > Q[(size_t)n * c->M + best]) best = m;
        labels[n] = (short)best;
    }
    free(Q);
}

/* ---- FP64 restatement of the same mean-field ---------------------------- */
static void orc_term_apply_f64(const orc_crf *c, const orc_term *t, double *out, const double *Q, int transpose) {
    int N = c->N, M = c->M;
    size_t NM = (size_t)N * M;
    double *tmp = (double *)malloc((NM + 1) * sizeof(double));
    int pre = t->ntype == ORC_NORMALIZE_SYMMETRIC || (t->ntype == ORC_NORMALIZE_BEFORE && !transpose) ||
              (t->ntype == ORC_NORMALIZE_AFTER && transpose);
    int post = t->ntype == ORC_NORMALIZE_SYMMETRIC || (t->ntype == ORC_NORMALIZE_BEFORE && transpose) ||
               (t->ntype == ORC_NORMALIZE_AFTER && !transpose);
    for (int n = 0; n < N; n++)
        for (int m = 0; m < M; m++) tmp[(size_t)n * M + m] = pre ? Q[(size_t)n * M + m] * t->norm64[n] : Q[(size_t)n * M + m];
    double *f = (double *)malloc((NM + 1) * sizeof(double));
    orc_compute_f64(t->lat, f, tmp, M, transpose);
    if (post)
        for (int n = 0; n < N; n++)
            for (int m = 0; m < M; m++) f[(size_t)n * M + m] *= t->norm64[n];
    for (int n = 0; n < N; n++)
        for (int m = 0; m < M; m++) {
            double v;
            if (t->ckind == ORC_POTTS)
                v = -(double)t->compat[0] * f[(size_t)n * M + m];
            else if (t->ckind == ORC_DIAGONAL)
                v = (double)t->compat[m] * f[(size_t)n * M + m];
            else {
                v = 0.0;
                for (int k = 0; k < M; k++) v += (double)t->compat[m * M + k] * f[(size_t)n * M + k];
            }
            out[(size_t)n * M + m] = v;
        }
    free(tmp);
    free(f);
}

static void orc_softmax_f64(int N, int M, double *out, const double *in) {
    for (int n = 0; n < N; n++) {
        const double *b = in + (size_t)n * M;
        double mx = b[0];
        for (int m = 1; m < M; m++)
            if (b[m] > mx) mx = b[m];
        double s = 0.0;
        for (int m = 0; m < M; m++) s += exp(b[m] - mx);
        for (int m = 0; m < M; m++) out[(size_t)n * M + m] = exp(b[m] - mx) / s;
    }
}

void orc_crf_inference_f64(void *cp, int T, double *Q) {
    orc_crf *c = (orc_crf *)cp;
    int N = c->N, M = c->M;
    size_t NM = (size_t)N * M;
    double *t1 = (double *)malloc((NM + 1) * sizeof(double));
    double *t2 = (double *)malloc((NM + 1) * sizeof(double));
    for (size_t i = 0; i < NM; i++) t1[i] = c->has_unary ? -(double)c->unary[i] : 0.0;
    orc_softmax_f64(N, M, Q, t1);
    for (int it = 0; it < T; it++) {
        for (size_t i = 0; i < NM; i++) t1[i] = c->has_unary ? -(double)c->unary[i] : 0.0;
        for (int k = 0; k < c->nterms; k++) {
            orc_term_apply_f64(c, &c->terms[k], t2, Q, 0);
            for (size_t i = 0; i < NM; i++) t1[i] -= t2[i];
        }
        orc_softmax_f64(N, M, Q, t1);
    }
    free(t1);
    free(t2);
}

/* accessors used by the tests */
int orc_crf_term_vertices(void *cp, int k) { return ((orc_crf *)cp)->terms[k].lat->L; }
void orc_crf_term_norm(void *cp, int k, float *norm) {
    orc_crf *c = (orc_crf *)cp;
    memcpy(norm, c->terms[k].norm, (size_t)c->N * sizeof(float));
}
void *orc_crf_term_lattice(void *cp, int k) { return ((orc_crf *)cp)->terms[k].lat; }
