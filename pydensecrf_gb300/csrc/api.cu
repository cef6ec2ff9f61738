// api.cu -- the C ABI of include/dcrf.h: handles, device memory, and the
// launch sequences of lattice build, normalisation and mean-field inference.
#include <algorithm>
#include <chrono>
#include <map>
#include <memory>
#include <atomic>
#include <cmath>
#include <mutex>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "adjoint.cuh"
#include "lattice.cuh"
#include "meanfield.cuh"

using namespace dcrf;

namespace dcrf {
static std::atomic<unsigned long long> g_launches{0};
void note_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
cudaError_t pool_malloc_async(void **p, size_t bytes, cudaStream_t s) {
    static std::mutex mu;
    static cudaMemPool_t pools[256] = {};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= 256) return cudaErrorInvalidDevice;
    cudaMemPool_t pool;
    {
        std::lock_guard<std::mutex> lk(mu);
        if (!pools[dev]) {
            cudaMemPoolProps props = {};
            props.allocType = cudaMemAllocationTypePinned;
            props.location.type = cudaMemLocationTypeDevice;
            props.location.id = dev;
            e = cudaMemPoolCreate(&pools[dev], &props);
            if (e != cudaSuccess) return e;
            uint64_t keep = ~0ull;
            cudaMemPoolSetAttribute(pools[dev], cudaMemPoolAttrReleaseThreshold, &keep);
        }
        pool = pools[dev];
    }
    return cudaMallocFromPoolAsync(p, bytes, pool, s);
}

bool pdl_enabled() {
    static const bool on = [] {
        const char *e = std::getenv("DCRF_PDL");
        return !(e && e[0] == '0');
    }();
    return on;
}
}  // namespace dcrf

namespace {

thread_local std::string g_err;
thread_local int g_code = DCRF_OK;

int set_err(int code, const std::string &msg) {
    g_err = msg;
    g_code = code;
    return code;
}

int ok() {
    g_code = DCRF_OK;
    return DCRF_OK;
}

#define CU(call)                                                                                  \
    do {                                                                                          \
        cudaError_t e_ = (call);                                                                  \
        if (e_ != cudaSuccess) return set_err(DCRF_ERR_CUDA, std::string(#call ": ") + cudaGetErrorString(e_)); \
    } while (0)

// stream-ordered allocations from the library's pool (released memory stays
// in the pool): creating, rebuilding and destroying handles does not
// synchronise the device
template <class T>
int dev_alloc_async(T **p, size_t n, cudaStream_t s) {
    void *q = nullptr;
    cudaError_t e = pool_malloc_async(&q, std::max<size_t>(n * sizeof(T), 16), s);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return set_err(DCRF_ERR_OOM, "stream-ordered allocation of " + std::to_string(n * sizeof(T)) + " bytes failed");
    }
    *p = static_cast<T *>(q);
    return DCRF_OK;
}

void dev_free_async(void *p, cudaStream_t s) {
    if (p) cudaFreeAsync(p, s);
}

struct Term {
    int d = 0, ktype = DCRF_DIAG_KERNEL, ntype = DCRF_NORMALIZE_SYMMETRIC, ckind = DCRF_COMPAT_POTTS;
    int variant = DCRF_VARIANT_SSE;
    float potts_w = 0.f;
    LatticeDev lat;
    float *feat = nullptr;  // [d][N] features as given (kernel parameters at identity)
    float *norm = nullptr;  // [N]
    float *V[2] = {nullptr, nullptr};  // [L+1][MP] blurred values, vertex order (ping-pong)
    float *pv = nullptr;               // [P][MP] blurred values in partial order (slice input)
    float *pout = nullptr;             // [P][MP] splat partials grouped by vertex (reduce input)
    float *compat = nullptr;  // device compat (Diagonal M / Matrix M*M symmetrised)
    float *mem_wn = nullptr;  // splat member weights times the members' norm (forward pre-normalisation)
    float *df = nullptr;      // [N][d] accumulated feature gradient (adjoint)
    // adjoint work lattices, vertex order with a zero row 0: [L+1][MP] x 9, [L+1] x 3
    float *bv[9] = {};
    float *b1[3] = {nullptr, nullptr, nullptr};
    bool r1_valid = false;  // b1[2] holds the reverse-blurred splat of ones
    std::vector<float> compat_h;
    std::vector<float> params;  // kernel parameters (DIAG d, FULL d*d row-major)
    bool params_set = false;    // the lattice uses params (else the features as given)
    bool norm_pending = false;  // built, normalisation not yet computed (see flush_norms)
};

// Knobs of the launch sequence that the autotuner picks per configuration.
struct TuneCfg {
    int split = 0;           // threads per point in the point pass (0: by rule, see pick_split)
    int smem_kb = 0;         // point-pass shared-memory budget per CTA (0: the default for MP)
    int task = SPLAT_TASK;   // most members of one splat task (lattice build)
    float hash_load = 2.0f;  // hash-table capacity factor (lattice build)
    int coop = 0;            // blur axes in one cooperative launch (1) or one launch per axis (0)
};

// Tile tables of one image-size list: slot -> point, point -> slot, and the
// prefix of valid slots per tile, on the host and -- made on first use, one
// allocation per device -- on the device, shared read-only by every handle of
// that size list and freed with the layout.
struct TileLayout {
    std::vector<int> slot, inv, vbase;
    mutable std::mutex dmu;
    mutable std::vector<std::pair<int, int *>> dev;  // (device, [slot | inv | vbase])
    int *device_tables(int device) const {
        std::lock_guard<std::mutex> lk(dmu);
        for (auto &d : dev)
            if (d.first == device) return d.second;
        std::vector<int> all(slot);
        all.push_back(0);
        all.insert(all.end(), inv.begin(), inv.end());
        all.push_back(0);
        all.insert(all.end(), vbase.begin(), vbase.end());
        all.push_back(0);
        int *p = nullptr;
        if (cudaMalloc(&p, all.size() * sizeof(int)) != cudaSuccess) {
            cudaGetLastError();
            return nullptr;
        }
        if (cudaMemcpy(p, all.data(), all.size() * sizeof(int), cudaMemcpyHostToDevice) != cudaSuccess) {
            cudaGetLastError();
            cudaFree(p);
            return nullptr;
        }
        dev.push_back({device, p});
        return p;
    }
    ~TileLayout() {
        int cur = 0;
        if (cudaGetDevice(&cur) != cudaSuccess) return;
        for (auto &d : dev) {
            cudaSetDevice(d.first);
            cudaFree(d.second);  // synchronises: no handle's work still reads the tables
        }
        cudaSetDevice(cur);
    }
};

}  // namespace

struct dcrf_crf {
    int N = 0, M = 0, MP = 0, W = 0, H = 0;
    // the images of the handle: point ranges seg[b]..seg[b+1] (one image for
    // DenseCRF/DenseCRF2D, several for a batch); grid2d with each image's W x H
    bool grid2d = false;
    std::vector<int> seg, imgW, imgH;
    int *d_seg = nullptr;   // [nimg+1] device copy of seg
    int *d_imgW = nullptr;  // [nimg] device copy of imgW (grid2d)
    int variant = DCRF_VARIANT_SSE;
    int device = 0;
    cudaStream_t own = nullptr, stream = nullptr;
    // orders work a caller queues on another stream (the allocation-free
    // filter) against the handle's stream in both directions; created once
    cudaEvent_t xorder = nullptr;
    DevStatus *status = nullptr;
    float *U = nullptr;  // [M][nslots] unary, slot-major
    bool has_unary = false;
    // logistic unary U = L f (unary.cpp:48-68): L [M][nfeat] (host copy and
    // device), f [nfeat][N] on the device; nfeat = 0 for a constant unary
    int nfeat = 0;
    std::vector<float> L_h;
    float *L_d = nullptr, *f_d = nullptr;
    float *Q = nullptr;      // [M][nslots] working marginals, slot-major
    float *tmp = nullptr;    // [M][nslots] scratch of the raw-filter path
    float *stage = nullptr;  // [N*M] user-layout staging of host copies
    int nslots = 0;
    int *pt_slot = nullptr;  // [N] slot of each point
    int16_t *map = nullptr;
    double *kl_part = nullptr;
    int ntiles = 0;
    int *slot_pt = nullptr;
    int *tile_vbase = nullptr;
    std::shared_ptr<const TileLayout> layout;  // owns slot_pt, pt_slot, tile_vbase
    std::vector<Term> terms;
    // model version (bumped by every change of unary, terms or parameters) and
    // the per-iteration checkpoints of the last dcrf_inference_checkpointed
    unsigned long long version = 0, ckpt_version = ~0ull;
    unsigned long long du_version = ~0ull;  // model version whose dL/dU bw[2] holds (after dcrf_backward)
    int ckpt_T = -1;
    float *ckpt = nullptr;  // [(T+1)][nslots][MP]; with an interval k > 1: Q_0, Q_k, Q_2k, ..., then Q_T
    size_t ckpt_cap = 0;
    // checkpoint interval (dcrf_set_checkpoint_interval) and the one the last
    // dcrf_inference_checkpointed used; with k > 1 the backward recomputes each
    // segment's iterates into segq ([k+1][nslots][MP]) and ckv / cky (k steps)
    int ckpt_every = 1, ckpt_every_used = 1;
    float *segq = nullptr;
    size_t segq_cap = 0;
    // per iteration t < T and term k: the forward's splat S and blurred lattice
    // B of Q_t, each [L_k+1][MP], at ckv + t * ckv_iter + ckv_off[k] (+ (L_k+1)*MP for B)
    float *ckv = nullptr;
    size_t ckv_cap = 0, ckv_iter = 0;
    // per term with kernel parameters (and a post-normalised forward): the
    // sliced values y_t = K_raw [norm] Q_t of every iterate, [T][nslots][MP]
    float *cky = nullptr;
    size_t cky_cap = 0;
    std::vector<long long> cky_off;  // per term, -1: not kept
    std::vector<size_t> ckv_off, ckv_layout;
    // per term with kernel gradients, the adjoint's raw slices F ([nslots][MP])
    // and, when the forward kept none, its sliced y = K_raw [norm] Q_t
    std::vector<float *> adjF, adjY;
    float *wideF = nullptr;  // more than 32 labels: the Matrix terms' sliced messages (WideArgs::F)
    size_t wideF_cap = 0;
    float *bw[14] = {};     // adjoint work buffers, [nslots][MP] each
    float *bw1[2] = {};     // adjoint work buffers, [nslots] each
    unsigned *bar = nullptr;  // grid-barrier state of the single-launch blur
    double *dpart = nullptr, *dacc = nullptr;
    size_t dpart_cap = 0, dacc_cap = 0;
    // CUDA graph of the last inference launch sequence (re-used through
    // cudaGraphExecUpdate while its topology stays the same); a handle's first
    // inference launches directly, since instantiating a graph costs more than
    // it saves on a one-shot solve
    bool use_graphs = true;
    int inference_runs = 0;
    // launch and build knobs (see the autotuner below)
    TuneCfg tune;
    bool autotune = false, tuned = false;
    cudaStream_t capture = nullptr;
    cudaGraphExec_t gexec = nullptr;
    // profiling: events bracketing launches, by kernel class
    bool profiling = false;
    int prof_class = -1;  // >= 0: every launch is counted in this kernel class (the normalisation: lattice)
    struct Mark {
        int cls;
        cudaEvent_t a, b;
    };
    std::vector<Mark> marks;
    std::vector<cudaEvent_t> event_pool;
};

namespace {

cudaEvent_t take_event(dcrf_crf *h) {
    if (!h->event_pool.empty()) {
        cudaEvent_t e = h->event_pool.back();
        h->event_pool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
}

// Brackets one or more launches of class `cls` with events when profiling.
struct ProfScope {
    dcrf_crf *h;
    int cls;
    cudaEvent_t a = nullptr;
    ProfScope(dcrf_crf *h_, int c) : h(h_), cls(h_->prof_class >= 0 ? h_->prof_class : c) {
        if (h->profiling) {
            a = take_event(h);
            cudaEventRecord(a, h->stream);
        }
    }
    ~ProfScope() {
        if (a) {
            cudaEvent_t b = take_event(h);
            cudaEventRecord(b, h->stream);
            h->marks.push_back({cls, a, b});
        }
    }
};

void release_marks(dcrf_crf *h) {
    for (auto &m : h->marks) {
        h->event_pool.push_back(m.a);
        h->event_pool.push_back(m.b);
    }
    h->marks.clear();
}

// Sets kernel attributes (dynamic shared memory opt-in) outside any capture,
// once per device (function attributes belong to the device's context).
void prepare_kernels() {
    static std::mutex mu;
    static uint64_t done = 0;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        return;
    }
    const uint64_t bit = dev < 64 ? 1ull << dev : 0;
    std::lock_guard<std::mutex> lk(mu);
    if (bit && (done & bit)) return;
    prepare_pointpass_kernels();
    done |= bit;
}

int check_handle(dcrf_crf *h) {
    if (!h) return set_err(DCRF_ERR_INVALID_ARG, "null handle");
    cudaError_t e = cudaSetDevice(h->device);
    if (e != cudaSuccess) return set_err(DCRF_ERR_CUDA, std::string("cudaSetDevice: ") + cudaGetErrorString(e));
    return DCRF_OK;
}

// Tiles of the in-kernel splat, image by image (no tile holds points of two
// images).  A 2D image uses 16x16 pixel blocks (the corners of a block share
// far more lattice vertices than a raster strip of the same size); a generic
// point set uses runs of 256 consecutive points.

// Host tables of a tile layout, computed once per image-size list for the
// process (handles are often created per image; the tables depend only on the
// sizes) and kept for the few most recent layouts.
std::shared_ptr<const TileLayout> tile_layout(const dcrf_crf *h) {
    static std::mutex mu;
    static std::vector<std::pair<std::vector<int>, std::shared_ptr<const TileLayout>>> cache;
    std::vector<int> key{h->grid2d ? 1 : 0, h->N};
    key.insert(key.end(), h->seg.begin(), h->seg.end());
    key.insert(key.end(), h->imgW.begin(), h->imgW.end());
    key.insert(key.end(), h->imgH.begin(), h->imgH.end());
    {
        std::lock_guard<std::mutex> lk(mu);
        for (size_t k = 0; k < cache.size(); k++)
            if (cache[k].first == key) {
                auto hit = cache[k].second;
                std::rotate(cache.begin(), cache.begin() + k, cache.begin() + k + 1);
                return hit;
            }
    }
    auto lay = std::make_shared<TileLayout>();
    std::vector<int> &slot = lay->slot, &vbase = lay->vbase;
    vbase.push_back(0);
    const int nimg = (int)h->seg.size() - 1;
    for (int b = 0; b < nimg; b++) {
        const int base = h->seg[b], nb = h->seg[b + 1] - h->seg[b];
        if (h->grid2d) {
            const int Wb = h->imgW[b], Hb = h->imgH[b];
            const int bx = (Wb + 15) / 16, by = (Hb + 15) / 16;
            for (int ty = 0; ty < by; ty++)
                for (int tx = 0; tx < bx; tx++) {
                    const size_t t0 = slot.size();
                    slot.resize(t0 + SPLAT_TILE, -1);
                    int cnt = 0;
                    for (int yy = 0; yy < 16; yy++)
                        for (int xx = 0; xx < 16; xx++) {
                            const int y = ty * 16 + yy, x = tx * 16 + xx;
                            if (y < Hb && x < Wb) {
                                slot[t0 + yy * 16 + xx] = base + y * Wb + x;
                                cnt++;
                            }
                        }
                    vbase.push_back(vbase.back() + cnt);
                }
        } else {
            for (int t0 = 0; t0 < nb; t0 += SPLAT_TILE) {
                const size_t o = slot.size();
                slot.resize(o + SPLAT_TILE, -1);
                const int cnt = std::min(SPLAT_TILE, nb - t0);
                for (int q = 0; q < cnt; q++) slot[o + q] = base + t0 + q;
                vbase.push_back(vbase.back() + cnt);
            }
        }
    }
    lay->inv.assign(h->N, 0);
    for (size_t sl = 0; sl < slot.size(); sl++)
        if (slot[sl] >= 0) lay->inv[slot[sl]] = (int)sl;
    std::lock_guard<std::mutex> lk(mu);
    cache.insert(cache.begin(), {key, lay});
    if (cache.size() > 8) cache.pop_back();
    return lay;
}

// Device tile tables of the handle (stream-ordered on the handle's own stream).
int build_tiles(dcrf_crf *h) {
    const std::shared_ptr<const TileLayout> lay = tile_layout(h);
    const cudaStream_t s = h->own;
    h->ntiles = (int)lay->vbase.size() - 1;
    h->nslots = h->ntiles * SPLAT_TILE;
    int rc;
    int *tables = lay->device_tables(h->device);
    if (!tables) return set_err(DCRF_ERR_OOM, "device allocation of the tile tables failed");
    h->layout = lay;
    h->slot_pt = tables;
    h->pt_slot = tables + lay->slot.size() + 1;
    h->tile_vbase = h->pt_slot + lay->inv.size() + 1;
    if ((rc = dev_alloc_async(&h->kl_part, (size_t)h->ntiles + 1, s))) return rc;
    if ((rc = dev_alloc_async(&h->d_seg, h->seg.size(), s))) return rc;
    if ((rc = dev_alloc_async(&h->d_imgW, h->seg.size(), s))) return rc;
    CU(cudaMemcpyAsync(h->d_seg, h->seg.data(), h->seg.size() * sizeof(int), cudaMemcpyHostToDevice, s));
    if (h->grid2d)
        CU(cudaMemcpyAsync(h->d_imgW, h->imgW.data(), h->imgW.size() * sizeof(int), cudaMemcpyHostToDevice, s));
    return DCRF_OK;
}

// A handle over one or more images: Ns[b] points each, and for a 2D handle
// Ws[b] x Hs[b] pixels (Ns[b] = Ws[b] * Hs[b]).  Points of image b are
// numbered after those of images 0..b-1.
int create(int M, const std::vector<int> &Ns, const std::vector<int> &Ws, const std::vector<int> &Hs,
           dcrf_crf **out) {
    if (!out) return set_err(DCRF_ERR_INVALID_ARG, "null output pointer");
    *out = nullptr;
    if (Ns.empty()) return set_err(DCRF_ERR_INVALID_ARG, "no images");
    long long total = 0;
    for (int n : Ns) {
        if (n <= 0) return set_err(DCRF_ERR_INVALID_ARG, "N and M must be positive");
        total += n;
    }
    if (total > 0x7FFFFFF0LL) return set_err(DCRF_ERR_INVALID_ARG, "too many points (more than 2^31)");
    const int N = (int)total;
    if (M <= 0) return set_err(DCRF_ERR_INVALID_ARG, "N and M must be positive");
    if (M > DCRF_MAX_LABELS)
        return set_err(DCRF_ERR_INVALID_ARG, "at most " + std::to_string(DCRF_MAX_LABELS) +
                                                 " labels are supported, got " + std::to_string(M));
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return set_err(DCRF_ERR_NO_DEVICE, "no CUDA device available");
    }
    dcrf_crf *h = new dcrf_crf();
    h->N = N;
    h->M = M;
    h->MP = pad_labels(M);
    h->grid2d = !Ws.empty();
    h->W = Ns.size() == 1 && h->grid2d ? Ws[0] : 0;
    h->H = Ns.size() == 1 && h->grid2d ? Hs[0] : 0;
    h->imgW = Ws;
    h->imgH = Hs;
    h->seg.assign(1, 0);
    for (int n : Ns) h->seg.push_back(h->seg.back() + n);
    cudaGetDevice(&h->device);
    int rc = DCRF_OK;
    auto fail = [&](int code) {
        dcrf_destroy(h);
        return code;
    };
    if (cudaStreamCreateWithFlags(&h->own, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&h->capture, cudaStreamNonBlocking) != cudaSuccess)
        return fail(set_err(DCRF_ERR_CUDA, "cudaStreamCreate failed"));
    if (cudaEventCreateWithFlags(&h->xorder, cudaEventDisableTiming) != cudaSuccess)
        return fail(set_err(DCRF_ERR_CUDA, "cudaEventCreate failed"));
    prepare_kernels();
    h->stream = h->own;
    // handle memory comes from the stream-ordered pool on the handle's own
    // stream (no device-wide synchronisation at creation or destruction);
    // work on another stream starts after dcrf_set_stream's synchronisation
    const cudaStream_t s = h->own;
    const size_t rows = (size_t)h->nslots * h->MP;
    if ((rc = dev_alloc_async(&h->status, 1, s))) return fail(rc);
    if ((rc = dev_alloc_async(&h->bar, 2, s))) return fail(rc);
    if ((rc = build_tiles(h))) return fail(rc);
    if ((rc = dev_alloc_async(&h->U, (size_t)h->nslots * h->MP, s))) return fail(rc);
    if ((rc = dev_alloc_async(&h->Q, (size_t)h->nslots * h->MP, s))) return fail(rc);
    if ((rc = dev_alloc_async(&h->stage, (size_t)N * M, s))) return fail(rc);
    if ((rc = dev_alloc_async(&h->map, (size_t)N, s))) return fail(rc);
    // pooled memory may hold an earlier handle's data: status, the grid
    // barrier and the slot rows (padding slots and labels included) start at 0
    if (cudaMemsetAsync(h->status, 0, sizeof(DevStatus), s) != cudaSuccess ||
        cudaMemsetAsync(h->bar, 0, 2 * sizeof(unsigned), s) != cudaSuccess ||
        cudaMemsetAsync(h->U, 0, rows * sizeof(float), s) != cudaSuccess ||
        cudaMemsetAsync(h->Q, 0, rows * sizeof(float), s) != cudaSuccess)
        return fail(set_err(DCRF_ERR_CUDA, "cudaMemsetAsync failed"));
    *out = h;
    return ok();
}

// Copies an M x N quantity from the caller (label- or point-major, host or
// device) into device slot rows dst [nslots][ld] (ld = MP, or 1 for M = 1),
// label chunk by label chunk when M > 32 (chunk_offset layout).
int load_mn(dcrf_crf *h, const float *src, int layout, int where, float *dst, int M = -1) {
    if (M < 0) M = h->M;
    const bool full = M == h->M;
    if (layout != DCRF_LAYOUT_LM && layout != DCRF_LAYOUT_PM) return set_err(DCRF_ERR_INVALID_ARG, "unknown layout");
    const float *dsrc = src;
    if (where != DCRF_DEVICE) {
        CU(cudaMemcpyAsync(h->stage, src, sizeof(float) * (size_t)h->N * M, cudaMemcpyHostToDevice, h->stream));
        dsrc = h->stage;
    }
    ProfScope ps(h, DCRF_KCLASS_OTHER);
    const int nc = full ? label_chunks(h->MP) : 1;
    for (int c = 0; c < nc; c++) {
        const int w = full ? chunk_width(h->MP, c) : M, m0 = DCRF_LCHUNK * c;
        CU(launch_to_slots(dsrc, layout == DCRF_LAYOUT_PM, std::min(w, M - m0), M, m0, w, h->N, h->d_seg,
                           (int)h->seg.size() - 1, h->slot_pt, h->nslots, dst + chunk_base(h->nslots, c), h->stream));
    }
    return DCRF_OK;
}

// Copies the slot rows src [nslots][ld] out to the caller's layout.
int store_mn(dcrf_crf *h, const float *src, float *dst, int layout, int where, int M = -1) {
    if (M < 0) M = h->M;
    const bool full = M == h->M;
    if (layout != DCRF_LAYOUT_LM && layout != DCRF_LAYOUT_PM) return set_err(DCRF_ERR_INVALID_ARG, "unknown layout");
    float *ddst = where == DCRF_DEVICE ? dst : h->stage;
    {
        ProfScope ps(h, DCRF_KCLASS_OTHER);
        const int nc = full ? label_chunks(h->MP) : 1;
        for (int c = 0; c < nc; c++) {
            const int w = full ? chunk_width(h->MP, c) : M, m0 = DCRF_LCHUNK * c;
            CU(launch_from_slots(src + chunk_base(h->nslots, c), std::min(w, M - m0), M, m0, w, h->N, h->d_seg,
                                 (int)h->seg.size() - 1, h->slot_pt, h->nslots, h->pt_slot, layout == DCRF_LAYOUT_PM,
                                 ddst, h->stream));
        }
    }
    if (where != DCRF_DEVICE)
        CU(cudaMemcpyAsync(dst, h->stage, sizeof(float) * (size_t)h->N * M, cudaMemcpyDeviceToHost, h->stream));
    return DCRF_OK;
}

// Value-size-1 rows live in the last L+1 floats of the term's lattice
// buffers (lattice_v1_offset): clear of every label chunk's zero row 0, their
// own zero row 0 cleared at the build.
float *v1_buffer(const dcrf_crf *h, const Term &T, float *V) {
    return V + lattice_v1_offset((size_t)T.lat.L, h->MP);
}

// Descriptor of a term for the forward filter (or its transpose).
TermDev term_dev(dcrf_crf *h, const Term &T, bool transpose, bool value1) {
    TermDev t{};
    t.d = T.d;
    t.L = T.lat.L;
    t.ckind = T.ckind;
    bool sym = T.ntype == DCRF_NORMALIZE_SYMMETRIC;
    bool before = T.ntype == DCRF_NORMALIZE_BEFORE, after = T.ntype == DCRF_NORMALIZE_AFTER;
    t.pre_norm = sym || (before && !transpose) || (after && transpose);   // pairwise.cpp:65
    t.post_norm = sym || (before && transpose) || (after && !transpose);  // pairwise.cpp:78
    int vs = value1 ? 1 : h->M;
    t.seq = (vs <= 2 || T.variant == DCRF_VARIANT_SCALAR) ? 1 : 0;  // permutohedral.cpp:600-603
    t.potts_w = T.potts_w;
    t.alpha = T.lat.alpha;
    t.off = T.lat.off;
    t.bary = T.lat.bary;
    t.wslice = T.lat.wslice;
    t.V = value1 ? v1_buffer(h, T, T.V[(T.d + 1) & 1]) : T.V[(T.d + 1) & 1];
    t.tile_pbeg = T.lat.tile_pbeg;
    t.part_mend = T.lat.part_mend;
    t.mem_pt = T.lat.mem_pt;
    // forward pre-normalisation is folded into the member weights; the
    // transpose (and terms without one) use the plain weights
    t.mem_w = (t.pre_norm && !transpose && !value1 && T.mem_wn) ? T.mem_wn : T.lat.mem_w;
    t.tl_loc = T.lat.tl_loc;
    t.tl_w = T.lat.tl_w;
    t.task = T.lat.task;
    t.tsched = T.lat.tsched;
    t.tile_tbeg = T.lat.tile_tbeg;
    t.pv = T.pv;
    t.pout = T.pout;
    t.ppos = T.lat.ppos;
    t.norm = T.norm;
    t.compat = T.compat;
    t.staged = 0;
    t.vcap = 0;
    t.sm_cmp = -1;
    return t;
}

size_t align128(size_t x) { return (x + 127) & ~(size_t)127; }

// Shared-memory plan of the point pass: per staged term its norm, member ends
// and members (live to the end), and -- only with messages -- its corner
// tables and blurred rows (dead once the slice is done; the splat's q rows
// alias them).  Tiles with more partials than a term's vcap read their rows
// from global memory; terms whose fixed blocks do not fit are not staged.
void plan_smem(dcrf_crf *h, PPArgs &a, const std::vector<int> &which, bool msg, int MP) {
    const int budget = h->tune.smem_kb > 0 ? std::min(h->tune.smem_kb * 1024, POINTPASS_SMEM_MAX)
                                           : pointpass_smem_budget(MP);
    const int n = (int)which.size();
    int max_nt = 0;
    for (int k = 0; k < n; k++) max_nt = std::max(max_nt, h->terms[which[k]].lat.max_nt);
    // splat phase: q rows + per-task results
    const size_t sq = align128((size_t)SPLAT_TILE * MP * 4) + (size_t)max_nt * MP * 4;
    a.sm_q = 0;
    a.sm_res = (int)align128((size_t)SPLAT_TILE * MP * 4);
    a.smem_bytes = (int)sq;
    if (MP % 4 != 0) return;  // bulk copies need 16-byte rows
    // Matrix compatibilities of the message pass, [k][MP] each (first, never aliased)
    size_t cmp_end = 0;
    for (int k = 0; k < n && msg; k++)
        if (h->terms[which[k]].ckind == DCRF_COMPAT_MATRIX) cmp_end = align128(cmp_end + (size_t)MP * MP * 4);
    if (cmp_end + sq > (size_t)budget) return;
    for (int k = 0, o = 0; k < n && msg; k++)
        if (h->terms[which[k]].ckind == DCRF_COMPAT_MATRIX) {
            a.ts.t[k].sm_cmp = o;
            o += (int)align128((size_t)MP * MP * 4);
        }
    a.sm_q = (int)cmp_end;
    a.sm_res = (int)(cmp_end + align128((size_t)SPLAT_TILE * MP * 4));
    a.smem_bytes = (int)(cmp_end + sq);
    std::vector<int> staged(n, 1), vcap(n, 0);
    for (int k = 0; k < n; k++) vcap[k] = msg ? h->terms[which[k]].lat.max_np : 0;
    for (int attempt = 0; attempt < 64; attempt++) {
        size_t off = cmp_end;
        for (int k = 0; k < n; k++) {
            if (!staged[k]) continue;
            const Term &T = h->terms[which[k]];
            const size_t d1 = T.d + 1;
            a.ts.t[k].sm_norm = (int)off;
            off = align128(off + 1024);
            a.ts.t[k].sm_task = (int)off;
            off = align128(off + ((size_t)T.lat.max_nt + 8) * 4);
            a.ts.t[k].sm_sched = (int)off;
            off = align128(off + ((size_t)T.lat.max_nt + 8) * 4);
            a.ts.t[k].sm_mpt = (int)off;
            off = align128(off + d1 * SPLAT_TILE * 2);
            a.ts.t[k].sm_mw = (int)off;
            off = align128(off + d1 * SPLAT_TILE * 4);
        }
        const size_t persist = off;
        for (int k = 0; k < n && msg; k++) {
            if (!staged[k]) continue;
            const Term &T = h->terms[which[k]];
            const size_t d1 = T.d + 1;
            a.ts.t[k].sm_loc = (int)off;
            off = align128(off + d1 * SPLAT_TILE * 2);
            a.ts.t[k].sm_w = (int)off;
            off = align128(off + d1 * SPLAT_TILE * 4);
            a.ts.t[k].sm_vp = (int)off;
            off = align128(off + (size_t)vcap[k] * MP * 4);
        }
        const size_t total = std::max(off, persist + sq);
        if (total <= (size_t)budget) {
            for (int k = 0; k < n; k++) {
                a.ts.t[k].staged = staged[k];
                a.ts.t[k].vcap = staged[k] ? vcap[k] : 0;
            }
            a.sm_q = (int)persist;
            a.sm_res = (int)(persist + align128((size_t)SPLAT_TILE * MP * 4));
            a.smem_bytes = (int)total;
            return;
        }
        // shrink: halve the largest row cache first, then drop the largest term
        int big = -1;
        for (int k = 0; k < n; k++)
            if (staged[k] && vcap[k] > 0 && (big < 0 || vcap[k] > vcap[big])) big = k;
        if (big >= 0) {
            vcap[big] = vcap[big] > 16 ? vcap[big] / 2 : 0;
            continue;
        }
        int drop = -1;
        for (int k = 0; k < n; k++)
            if (staged[k] && (drop < 0 || h->terms[which[k]].d > h->terms[which[drop]].d)) drop = k;
        if (drop < 0) break;
        staged[drop] = 0;
    }
    for (int k = 0; k < n; k++) a.ts.t[k].staged = 0;
    a.sm_q = (int)cmp_end;
    a.sm_res = (int)(cmp_end + align128((size_t)SPLAT_TILE * MP * 4));
    a.smem_bytes = (int)(cmp_end + sq);
}

cudaError_t pp(dcrf_crf *h, const PPArgs &a, int MP) {
    ProfScope ps(h, DCRF_KCLASS_POINT);
    return launch_pointpass(a, MP, h->stream);
}

// Threads per point of the point pass: the tuned value, else two for label
// rows of 8k floats without a Matrix compatibility (measured: two threads win
// for Potts/Diagonal, one for Matrix, whose products then need the partner's
// labels).
int pick_split(const dcrf_crf *h, bool value1, int MP) {
    if (value1 || MP % 8 != 0) return 1;
    if (h->tune.split == 1 || h->tune.split == 2) return h->tune.split;
    for (const Term &T : h->terms)
        if (T.ckind == DCRF_COMPAT_MATRIX) return 1;
    return 2;
}

// Point-pass arguments for the listed terms; `chunk` >= 0 selects one label
// chunk of a handle with more than 32 labels (its rows, its lattice rows).
PPArgs pp_args(dcrf_crf *h, int mode, const std::vector<int> &which, bool transpose, bool value1, int chunk = -1) {
    const int c = chunk < 0 || value1 ? 0 : chunk;
    const int MPc = value1 ? 1 : chunk_width(h->MP, c);
    const size_t so = chunk_base(h->nslots, c);
    PPArgs a{};
    a.N = h->N;
    a.M = value1 ? 1 : std::min(MPc, h->M - DCRF_LCHUNK * c);
    a.mode = mode;
    a.ntiles = h->ntiles;
    a.nslots = h->nslots;
    a.slot_pt = h->slot_pt;
    a.U = h->has_unary ? h->U + so : nullptr;
    a.Qin = h->Q + so;
    a.Qout = h->Q + so;
    a.map_out = h->map;
    a.kl_part = h->kl_part;
    a.status = h->status;
    a.ts.n = (int)which.size();
    for (size_t k = 0; k < which.size(); k++) {
        const Term &T = h->terms[which[k]];
        TermDev &t = a.ts.t[k];
        t = term_dev(h, T, transpose, value1);
        if (c > 0) {
            t.pv += chunk_base((size_t)T.lat.P + 1, c);
            t.pout += chunk_base((size_t)T.lat.P + 1, c);
            t.V += chunk_base((size_t)T.lat.L + 1, c);
        }
        a.ntype[k] = T.ntype;
        a.norm_out[k] = T.norm;
    }
    // without messages there is no compatibility product: two threads per
    // point give the splat twice the lane groups
    a.split = (mode & PP_MSG) || value1 || MPc % 8 != 0 ? pick_split(h, value1, MPc) : 2;
    plan_smem(h, a, which, (mode & PP_MSG) != 0, MPc);
    return a;
}

std::vector<int> all_terms(dcrf_crf *h) {
    std::vector<int> w(h->terms.size());
    for (size_t k = 0; k < w.size(); k++) w[k] = (int)k;
    return w;
}

// reduce + d+1 blur passes for the listed terms (after a splat point pass).
// partial_order: the last pass writes the result in tile-partial order (pv,
// input of the mean-field point pass) instead of vertex order (V, input of the
// point-order slice).
int filter_phase(dcrf_crf *h, const std::vector<int> &which, bool transpose, bool value1, bool partial_order,
                 float *const *S_out = nullptr, float *const *B_out = nullptr, int chunk = 0) {
    const int ch = value1 ? 0 : chunk;
    int MP = value1 ? 1 : chunk_width(h->MP, ch);
    bool seq = value1 || h->M <= 2;
    // lattice rows of label chunk ch (the whole rows when MP <= 32)
    auto Vb = [&](const Term &T, int j) {
        return value1 ? v1_buffer(h, T, T.V[j]) : T.V[j] + chunk_base((size_t)T.lat.L + 1, ch);
    };
    auto Pb = [&](const Term &T, float *p) { return p + (value1 ? 0 : chunk_base((size_t)T.lat.P + 1, ch)); };
    // Blur launches per term: passes 2i and 2i+1 share launch i (the last pass
    // alone when d+1 is odd).  Buffers are planned backwards from the final
    // output, alternating the term's two lattice buffers launch by launch, so
    // that no launch reads the buffer it writes; the reduce fills the first
    // launch's input.  (The cooperative blur keeps its pass-by-pass chain from
    // V[0].)
    struct Chain2 {
        int n;
        float *fin;
        float *x[DCRF_MAX_D + 2];
    };
    std::vector<Chain2> plan(which.size());
    ReduceArgs ra{};
    ra.n = (int)which.size();
    int maxd = 0;
    for (size_t k = 0; k < which.size(); k++) {
        Term &T = h->terms[which[k]];
        Chain2 &c = plan[k];
        c.n = (T.d + 2) / 2;
        c.fin = B_out ? B_out[k] : partial_order ? nullptr : Vb(T, (T.d + 1) & 1);
        c.x[c.n - 1] = c.fin == Vb(T, 0) ? Vb(T, 1) : Vb(T, 0);
        for (int i = c.n - 2; i >= 0; i--) c.x[i] = c.x[i + 1] == Vb(T, 0) ? Vb(T, 1) : Vb(T, 0);
        float *red_out = S_out ? S_out[k] : h->tune.coop ? Vb(T, 0) : c.x[0];
        ra.t[k] = {T.lat.red_beg, Pb(T, T.pout), red_out, T.lat.L, T.lat.P};
        maxd = std::max(maxd, T.d);
        if (T.variant == DCRF_VARIANT_SCALAR) seq = true;
    }
    if (which.empty()) return DCRF_OK;
    {
        ProfScope ps(h, DCRF_KCLASS_REDUCE);
        CU(launch_reduce(ra, MP, h->stream));
    }
    if (h->tune.coop) {  // every axis pass of every term in one launch
        BlurChainArgs ca{};
        ca.n = (int)which.size();
        ca.npass = maxd + 1;
        ca.bar = h->bar;
        ca.status = h->status;
        for (size_t k = 0; k < which.size(); k++) {
            Term &T = h->terms[which[k]];
            BlurChainArgs::C &c = ca.c[k];
            c.S = S_out ? S_out[k] : Vb(T, 0);
            c.buf[0] = Vb(T, 1);
            c.buf[1] = Vb(T, 0);
            c.Out = B_out ? B_out[k] : partial_order ? nullptr : Vb(T, (T.d + 1) & 1);
            c.nbr = T.lat.nbr;
            c.L = T.lat.L;
            c.d = T.d;
            c.reverse = transpose ? 1 : 0;
            c.red_beg = T.lat.red_beg;
            c.red_list = T.lat.red_list;
            c.pv = partial_order ? Pb(T, T.pv) : nullptr;
        }
        ProfScope ps(h, DCRF_KCLASS_BLUR);
        CU(launch_blur_chains(ca, MP, seq, h->stream));
        return DCRF_OK;
    }
    const int NV = MP % 4 == 0 ? MP / 4 : MP % 2 == 0 ? MP / 2 : MP;
    for (int i = 0; 2 * i <= maxd; i++) {
        BlurArgs ba{};
        ba.n = 0;
        ba.begin[0] = 0;
        for (size_t k = 0; k < which.size(); k++) {
            Term &T = h->terms[which[k]];
            const Chain2 &c = plan[k];
            if (i >= c.n) continue;
            const bool last = i == c.n - 1;
            const int p = 2 * i;
            BlurArgs::T &bt = ba.t[ba.n];
            bt.Vin = (i == 0 && S_out) ? S_out[k] : c.x[i];
            bt.Vout = last ? c.fin : c.x[i + 1];
            bt.nbr = T.lat.nbr;
            bt.L = T.lat.L;
            bt.axis = transpose ? T.d - p : p;  // reverse blur order for the transpose (permutohedral.cpp:556)
            bt.axis2 = p + 1 > T.d ? -1 : transpose ? T.d - (p + 1) : p + 1;
            bt.red_beg = T.lat.red_beg;
            bt.red_list = T.lat.red_list;
            bt.pv = (last && partial_order) ? Pb(T, T.pv) : nullptr;
            ba.begin[ba.n + 1] = ba.begin[ba.n] + (long long)T.lat.L * NV;
            ba.n++;
        }
        // All listed terms share the arithmetic flavour: the scalar build and
        // value size <= 2 use the double-precision blur.
        ProfScope ps(h, DCRF_KCLASS_BLUR);
        CU(launch_blur(ba, MP, seq, h->stream));
    }
    return DCRF_OK;
}

// The value-size-1 passes (normalisation, 1-row filters) use the lattice-value
// buffers at stride 1, which overwrites entries that the stride-MP passes read
// as the zero sentinel row (row 0).  Restore it afterwards.
int zero_sentinels(dcrf_crf *h, Term &T) {
    CU(launch_lattice_zero_rows(T.V[0], T.V[1], (size_t)T.lat.L, h->MP, h->stream));
    return DCRF_OK;
}

// Waits for the handle's stream and reports CUDA errors and the device status
// block (set by kernels whose bounded waits ran out or whose inputs failed a
// consistency check); a reported status is cleared.
int sync_check(dcrf_crf *h) {
    DevStatus st{};
    cudaError_t e = cudaMemcpyAsync(&st, h->status, sizeof(DevStatus), cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return set_err(DCRF_ERR_CUDA, std::string("device error: ") + cudaGetErrorString(e));
    e = cudaGetLastError();
    if (e != cudaSuccess) return set_err(DCRF_ERR_CUDA, std::string("launch error: ") + cudaGetErrorString(e));
    if (st.code != 0) {
        cudaMemsetAsync(h->status, 0, sizeof(DevStatus), h->stream);
        return set_err(st.code, "device status " + std::to_string(st.code) + " (detail " + std::to_string(st.detail) +
                                    ")");
    }
    return DCRF_OK;
}

void free_term_lattice(dcrf_crf *h, Term &T) {
    // norm, V, pv, pout and mem_wn are carved from the lattice's memory
    dev_free_async(T.df, h->stream);
    T.norm_pending = false;
    T.norm = T.V[0] = T.V[1] = T.pv = T.pout = T.mem_wn = T.df = nullptr;
    for (float *&b : T.bv) {
        dev_free_async(b, h->stream);
        b = nullptr;
    }
    for (float *&b : T.b1) {
        dev_free_async(b, h->stream);
        b = nullptr;
    }
    T.r1_valid = false;
    lattice_free(&T.lat, h->stream);
}

void free_term(dcrf_crf *h, Term &T) {
    free_term_lattice(h, T);
    dev_free_async(T.feat, h->stream);
    dev_free_async(T.compat, h->stream);
    T.feat = T.compat = nullptr;
}

// Label compatibility of a term (host values and device copy).
int set_term_compat(dcrf_crf *h, Term &T, int kind, const float *compat) {
    const int M = h->M;
    T.ckind = kind;
    T.compat_h.clear();
    if (kind == DCRF_COMPAT_POTTS) {
        T.potts_w = compat[0];
    } else if (kind == DCRF_COMPAT_DIAGONAL) {
        T.compat_h.assign(compat, compat + M);
    } else if (kind == DCRF_COMPAT_MATRIX) {
        T.compat_h.resize((size_t)M * M);
        for (int a = 0; a < M; a++)  // MatrixCompatibility symmetrises: 0.5*(m + m^T) (labelcompatibility.cpp:79)
            for (int b = 0; b < M; b++) {
                float s = compat[a * M + b] + compat[b * M + a];
                T.compat_h[(size_t)a * M + b] = 0.5f * s;
            }
    } else {
        return set_err(DCRF_ERR_INVALID_ARG, "unknown compatibility kind");
    }
    if (!T.compat_h.empty()) {
        int rc;
        if (!T.compat) {
            if ((rc = dev_alloc_async(&T.compat, (size_t)M * M, h->stream))) return rc;
        }
        CU(cudaMemcpyAsync(T.compat, T.compat_h.data(), T.compat_h.size() * sizeof(float), cudaMemcpyHostToDevice,
                           h->stream));
    }
    return DCRF_OK;
}

// (Re)builds term k's lattice from its features and kernel parameters, then
// its normalisation (DenseKernel::initLattice, pairwise.cpp:40-62) and the
// member weights with the normalisation folded in.
int build_term(dcrf_crf *h, int k) {
    Term &T = h->terms[k];
    int rc;
    free_term_lattice(h, T);
    // features the lattice is built on: p_j f_j (DIAG) or P f (FULL) once parameters were set
    const float *feat = T.feat;
    float *scaled = nullptr;
    if (T.params_set && T.ktype != DCRF_CONST_KERNEL) {
        const size_t np = T.ktype == DCRF_FULL_KERNEL ? (size_t)T.d * T.d : (size_t)T.d;
        float *dp = nullptr;
        if ((rc = dev_alloc_async(&scaled, (size_t)T.d * h->N, h->stream))) return rc;
        if ((rc = dev_alloc_async(&dp, np, h->stream))) return rc;
        CU(cudaMemcpyAsync(dp, T.params.data(), np * sizeof(float), cudaMemcpyHostToDevice, h->stream));
        CU(launch_scale_features(T.feat, scaled, dp, T.d, h->N, T.ktype == DCRF_FULL_KERNEL, h->stream));
        dev_free_async(dp, h->stream);
        feat = scaled;
    }
    Segments seg;
    seg.start = h->seg;
    seg.dev_start = h->d_seg;
    TileMapDev tm;
    tm.ntiles = h->ntiles;
    tm.slot_pt = h->slot_pt;
    tm.tile_vbase = h->tile_vbase;
    float load = h->tune.hash_load;
    for (int attempt = 0;; attempt++) {
        ProfScope ps(h, DCRF_KCLASS_LATTICE);
        rc = lattice_build(feat, T.d, h->N, seg, tm, T.variant, load, h->tune.task, h->MP, h->nslots, h->stream,
                           h->status, &T.lat);
        if (rc == DCRF_ERR_HASH_FULL && attempt < 3) {
            load *= 4.f;
            continue;
        }
        break;
    }
    dev_free_async(scaled, h->stream);
    if (rc) return set_err(rc, lattice_last_message());
    T.V[0] = T.lat.V0;
    T.V[1] = T.lat.V1;
    T.pv = T.lat.pv;
    T.pout = T.lat.pout;
    T.norm = T.lat.norm;
    T.mem_wn = T.lat.mem_wn;
    // the normalisation (K * 1, pairwise.cpp:44) is computed for all new terms
    // together before their first use (flush_norms); no synchronisation here
    T.norm_pending = true;
    CU(cudaGetLastError());
    h->version++;
    return DCRF_OK;
}

// Normalisation of every term built since the last use (DenseKernel::initLattice,
// pairwise.cpp:40-62): one value-size-1 filter of ones through all of them in
// the same launches, then each term's norm and its member weights with the
// norm folded in (the forward pre-normalisation of the splat).  Called at the
// start of every call that uses the terms.  A device status it leaves is
// reported by the next synchronising call.
int flush_norms(dcrf_crf *h) {
    std::vector<int> which;
    for (size_t k = 0; k < h->terms.size(); k++)
        if (h->terms[k].norm_pending) which.push_back((int)k);
    if (which.empty()) return DCRF_OK;
    for (int k : which) h->terms[k].norm_pending = false;
    // profiled as a class of its own
    struct ForceClass {
        dcrf_crf *h;
        ~ForceClass() { h->prof_class = -1; }
    } force{h};
    h->prof_class = DCRF_KCLASS_NORM;
    PPArgs a = pp_args(h, PP_ONES | PP_SPLAT, which, false, true);
    for (size_t q = 0; q < which.size(); q++) a.ts.t[q].pre_norm = a.ts.t[q].post_norm = 0;
    CU(pp(h, a, 1));
    int rc;
    if ((rc = filter_phase(h, which, false, true, false))) return rc;
    a = pp_args(h, PP_NORM, which, false, true);
    for (size_t q = 0; q < which.size(); q++) {
        Term &T = h->terms[which[q]];
        a.ts.t[q].V = v1_buffer(h, T, T.V[(T.d + 1) & 1]);
        // the forward (SYMMETRIC, BEFORE) or the transpose (SYMMETRIC, AFTER)
        // normalises before its splat
        a.wn_out[q] = T.ntype != DCRF_NO_NORMALIZATION ? T.mem_wn : nullptr;
    }
    CU(pp(h, a, 1));
    return DCRF_OK;
}

// check_handle, then the normalisation of terms built since the last use.
int check_ready(dcrf_crf *h) {
    int rc = check_handle(h);
    if (rc) return rc;
    return flush_norms(h);
}

int add_term(dcrf_crf *h, const float *feat_dev_owned, int d, int compat_kind, const float *compat, int ktype,
             int ntype, int *term_out) {
    // feat_dev_owned: [d][N] device buffer, ownership passes to the term
    Term T;
    T.d = d;
    T.ktype = ktype;
    T.ntype = ntype;
    T.variant = h->variant;
    T.feat = const_cast<float *>(feat_dev_owned);
    // kernel parameters start at the identity (pairwise.cpp:117-121)
    if (ktype == DCRF_DIAG_KERNEL) T.params.assign(d, 1.f);
    if (ktype == DCRF_FULL_KERNEL) {
        T.params.assign((size_t)d * d, 0.f);
        for (int j = 0; j < d; j++) T.params[(size_t)j * d + j] = 1.f;
    }
    int rc = set_term_compat(h, T, compat_kind, compat);
    if (rc) {
        free_term(h, T);
        return rc;
    }
    h->terms.push_back(T);
    h->tuned = false;  // a new configuration for the autotuner
    const int k = (int)h->terms.size() - 1;
    if ((rc = build_term(h, k))) {
        free_term(h, h->terms[k]);
        h->terms.pop_back();
        return rc;
    }
    if (term_out) *term_out = k;
    return ok();
}

int validate_compat(int kind, const float *compat) {
    if (kind < DCRF_COMPAT_POTTS || kind > DCRF_COMPAT_MATRIX)
        return set_err(DCRF_ERR_INVALID_ARG, "unknown compatibility kind");
    if (!compat) return set_err(DCRF_ERR_INVALID_ARG, "null compatibility");
    return DCRF_OK;
}

int validate_kn(int ktype, int ntype) {
    if (ktype < DCRF_CONST_KERNEL || ktype > DCRF_FULL_KERNEL) return set_err(DCRF_ERR_INVALID_ARG, "unknown kernel type");
    if (ntype < DCRF_NO_NORMALIZATION || ntype > DCRF_NORMALIZE_SYMMETRIC)
        return set_err(DCRF_ERR_INVALID_ARG, "unknown normalization type");
    return DCRF_OK;
}

// ---- more than 32 labels --------------------------------------------------------
// The labels are processed in chunks of 32 (chunk_offset layout): the splat,
// reduce and blur are linear per label and run chunk by chunk through the same
// kernels as narrower handles; the messages, compatibilities and the softmax,
// which mix labels, run in wide_kernel.
bool is_wide(const dcrf_crf *h) { return h->MP > DCRF_MAX_MP; }

int wide_unsupported(const char *what) {
    return set_err(DCRF_ERR_INVALID_ARG, std::string(what) + " supports at most " + std::to_string(DCRF_MAX_MP) +
                                             " labels");
}

WideArgs wide_args(dcrf_crf *h, int mode, const std::vector<int> &w) {
    WideArgs a{};
    a.N = h->N;
    a.M = h->M;
    a.MP = h->MP;
    a.mode = mode;
    a.ntiles = h->ntiles;
    a.nslots = h->nslots;
    a.slot_pt = h->slot_pt;
    a.U = h->has_unary ? h->U : nullptr;
    a.Qin = h->Q;
    a.Qout = h->Q;
    a.F = h->wideF;
    a.map_out = h->map;
    a.kl_part = h->kl_part;
    a.ts.n = (int)w.size();
    for (size_t k = 0; k < w.size(); k++) {
        const Term &T = h->terms[w[k]];
        a.ts.t[k] = term_dev(h, T, false, false);
        a.pv_chunk[k] = (long long)chunk_base((size_t)T.lat.P + 1, 1);
    }
    return a;
}

// The Matrix terms' message rows of wide_kernel (allocated outside any graph capture).
int ensure_wide_bufs(dcrf_crf *h) {
    if (!is_wide(h)) return DCRF_OK;
    size_t nmat = 0;
    for (const Term &T : h->terms) nmat += T.ckind == DCRF_COMPAT_MATRIX ? 1 : 0;
    const size_t need = nmat * (size_t)h->nslots * h->MP;
    if (need > h->wideF_cap) {
        dev_free_async(h->wideF, h->stream);
        h->wideF = nullptr;
        h->wideF_cap = 0;
        int rc = dev_alloc_async(&h->wideF, need, h->stream);
        if (rc) return rc;
        h->wideF_cap = need;
    }
    return DCRF_OK;
}

int wide(dcrf_crf *h, int mode, const std::vector<int> &w) {
    ProfScope ps(h, DCRF_KCLASS_POINT);
    CU(launch_wide(wide_args(h, mode, w), h->stream));
    return DCRF_OK;
}

// splat h->Q into every term's lattice and filter it, label chunk by chunk
int wide_splat_filter(dcrf_crf *h, const std::vector<int> &w) {
    const int nc = label_chunks(h->MP);
    for (int c = 0; c < nc; c++) CU(pp(h, pp_args(h, PP_LOAD_Q | PP_SPLAT, w, false, false, c), chunk_width(h->MP, c)));
    for (int c = 0; c < nc; c++) {
        int rc = filter_phase(h, w, false, false, true, nullptr, nullptr, c);
        if (rc) return rc;
    }
    return DCRF_OK;
}

int issue_inference_wide(dcrf_crf *h, int T, int final_mode) {
    std::vector<int> w = all_terms(h);
    const int fin = (final_mode & PP_MAP) ? WP_MAP : WP_WRITE_Q;
    if (T <= 0 || w.empty()) return wide(h, fin, w);
    int rc;
    if ((rc = wide(h, WP_WRITE_Q, w))) return rc;  // Q_0 = softmax(-U)
    for (int it = 1; it <= T; it++) {
        if ((rc = wide_splat_filter(h, w))) return rc;
        if ((rc = wide(h, WP_MSG | (it < T ? WP_WRITE_Q : fin), w))) return rc;
    }
    return DCRF_OK;
}

// Launch sequence of T mean-field iterations starting from softmax(-U); the
// final pass writes per final_mode (Q into h->Q, or the MAP labels).
int issue_inference(dcrf_crf *h, int T, int final_mode, float *ckpt = nullptr) {
    if (is_wide(h)) return issue_inference_wide(h, T, final_mode);
    std::vector<int> w = all_terms(h);
    const size_t qsz = (size_t)h->MP * h->nslots;
    int rc;
    if (T <= 0 || w.empty()) {
        PPArgs a = pp_args(h, final_mode | (ckpt ? PP_WRITE_Q : 0), w, false, false);
        if (ckpt) a.Qout = ckpt;
        CU(pp(h, a, h->MP));
        if (ckpt)  // every iterate equals Q_0 without pairwise terms
            for (int it = 1; it <= T; it++)
                CU(cudaMemcpyAsync(ckpt + it * qsz, ckpt, qsz * sizeof(float), cudaMemcpyDeviceToDevice, h->stream));
        return DCRF_OK;
    }
    {
        PPArgs a = pp_args(h, PP_SPLAT | (ckpt ? PP_WRITE_Q : 0), w, false, false);
        if (ckpt) a.Qout = ckpt;
        CU(pp(h, a, h->MP));
    }
    for (int it = 1; it <= T; it++) {
        if (ckpt && h->ckv) {  // keep S and B of Q_{it-1} for the adjoint
            float *S[DCRF_MAX_TERMS], *B[DCRF_MAX_TERMS];
            for (size_t k = 0; k < w.size(); k++) {
                S[k] = h->ckv + (size_t)(it - 1) * h->ckv_iter + h->ckv_off[w[k]];
                B[k] = S[k] + ((size_t)h->terms[w[k]].lat.L + 1) * h->MP;
            }
            if ((rc = filter_phase(h, w, false, false, true, S, B))) return rc;
        } else if ((rc = filter_phase(h, w, false, false, true))) {
            return rc;
        }
        int mode = PP_MSG | (it < T ? PP_SPLAT : final_mode) | (ckpt ? PP_WRITE_Q : 0);
        PPArgs a = pp_args(h, mode, w, false, false);
        if (ckpt) a.Qout = ckpt + it * qsz;
        if (ckpt && h->cky)
            for (size_t k = 0; k < w.size(); k++)
                if (h->cky_off[w[k]] >= 0) a.ckY[k] = h->cky + h->cky_off[w[k]] + (size_t)(it - 1) * qsz;
        CU(pp(h, a, h->MP));
    }
    return DCRF_OK;
}

// n mean-field iterations from Q_start (device slot rows; null: softmax(-U)).
// With ckq (n+1 rows) every iterate Q_0..Q_n of the range is written there and,
// with ckv / cky, the splats and blurred lattices / sliced values of its steps
// (the layout of dcrf_inference_checkpointed, relative to the range); without
// ckq only the last iterate, into q_last.  The arithmetic is the forward's, so
// a range recomputed from a stored iterate reproduces its iterates bit for bit.
int issue_steps(dcrf_crf *h, const float *Qstart, int n, float *ckq, float *ckv, float *cky, float *q_last) {
    std::vector<int> w = all_terms(h);
    const size_t qsz = (size_t)h->MP * h->nslots;
    int rc;
    if (n <= 0 || w.empty()) {  // every iterate equals the start
        float *dst = ckq ? ckq : q_last;
        if (Qstart) {
            CU(cudaMemcpyAsync(dst, Qstart, qsz * sizeof(float), cudaMemcpyDeviceToDevice, h->stream));
        } else {
            PPArgs a = pp_args(h, PP_WRITE_Q, w, false, false);
            a.Qout = dst;
            CU(pp(h, a, h->MP));
        }
        for (int it = 1; ckq && it <= n; it++)
            CU(cudaMemcpyAsync(ckq + it * qsz, ckq, qsz * sizeof(float), cudaMemcpyDeviceToDevice, h->stream));
        if (!ckq && n > 0 && q_last != dst)
            CU(cudaMemcpyAsync(q_last, dst, qsz * sizeof(float), cudaMemcpyDeviceToDevice, h->stream));
        return DCRF_OK;
    }
    {
        PPArgs a = pp_args(h, PP_SPLAT | (Qstart ? PP_LOAD_Q : 0) | (ckq ? PP_WRITE_Q : 0), w, false, false);
        if (Qstart) a.Qin = Qstart;
        if (ckq) a.Qout = ckq;
        CU(pp(h, a, h->MP));
    }
    for (int it = 1; it <= n; it++) {
        if (ckv) {
            float *S[DCRF_MAX_TERMS], *B[DCRF_MAX_TERMS];
            for (size_t k = 0; k < w.size(); k++) {
                S[k] = ckv + (size_t)(it - 1) * h->ckv_iter + h->ckv_off[w[k]];
                B[k] = S[k] + ((size_t)h->terms[w[k]].lat.L + 1) * h->MP;
            }
            if ((rc = filter_phase(h, w, false, false, true, S, B))) return rc;
        } else if ((rc = filter_phase(h, w, false, false, true))) {
            return rc;
        }
        PPArgs a = pp_args(h, PP_MSG | (it < n ? PP_SPLAT : 0) | (ckq || it == n ? PP_WRITE_Q : 0), w, false, false);
        a.Qout = ckq ? ckq + it * qsz : q_last;
        if (ckq && cky)
            for (size_t k = 0; k < w.size(); k++)
                if (h->cky_off[w[k]] >= 0) a.ckY[k] = cky + h->cky_off[w[k]] + (size_t)(it - 1) * qsz;
        CU(pp(h, a, h->MP));
    }
    return DCRF_OK;
}

// Runs issue_inference as one CUDA graph: captured on the handle's capture
// stream, instantiated once and afterwards updated in place (same kernels,
// new arguments), launched on the handle's stream.  Profiling launches the
// kernels directly so that the per-launch events can be recorded.
// ---- autotuner ----------------------------------------------------------------
// Picks the launch and build knobs per configuration -- labels, per-term (d,
// compatibility kind, normalisation, arithmetic variant), one image or a batch,
// and the size class log2(N) -- by timing candidates on the handle's own
// lattices, and remembers the choice for the process.  Build knobs: hash load
// factor (1.5, 2, 3) and splat task length (16, 24, 32), scored as one build
// plus ten iterations; launch knobs: threads per point (1, 2) and the point
// pass's shared-memory budget (default, or 72 KB for three CTAs per SM).
// Only the task length changes results (the grouping of the splat sums).

std::mutex g_tune_mu;
std::map<std::string, TuneCfg> g_tune_cache;

std::string tune_key(const dcrf_crf *h) {
    int lg = 0;
    while ((1ll << (lg + 1)) <= (long long)h->N) lg++;
    std::string k = "M" + std::to_string(h->M) + (h->seg.size() > 2 ? "/batch" : "/one") + "/N2^" + std::to_string(lg);
    for (const Term &T : h->terms)
        k += "/d" + std::to_string(T.d) + "c" + std::to_string(T.ckind) + "n" + std::to_string(T.ntype) + "v" +
             std::to_string(T.variant);
    return k;
}

int rebuild_terms(dcrf_crf *h) {
    for (size_t k = 0; k < h->terms.size(); k++) {
        int rc = build_term(h, (int)k);
        if (rc) return rc;
    }
    return DCRF_OK;
}

// Device time of n mean-field iterations (min of reps), launched directly.
int time_iterations(dcrf_crf *h, int n, int reps, float *ms_out) {
    int frc = flush_norms(h);
    if (!frc) frc = ensure_wide_bufs(h);
    if (frc) return frc;
    cudaEvent_t a = take_event(h), b = take_event(h);
    float best = 1e30f;
    int rc = DCRF_OK;
    for (int r = 0; r <= reps && !rc; r++) {
        CU(cudaEventRecord(a, h->stream));
        rc = issue_inference(h, n, PP_WRITE_Q);
        CU(cudaEventRecord(b, h->stream));
        CU(cudaEventSynchronize(b));
        float ms = 0.f;
        CU(cudaEventElapsedTime(&ms, a, b));
        if (r > 0) best = std::min(best, ms);  // the first run warms up
    }
    h->event_pool.push_back(a);
    h->event_pool.push_back(b);
    *ms_out = best;
    return rc;
}

int autotune_now(dcrf_crf *h) {
    if (h->terms.empty()) return DCRF_OK;
    const bool prof = h->profiling;
    h->profiling = false;
    int rc = DCRF_OK;
    // build knobs: one build plus ten iterations
    TuneCfg best = h->tune;
    double best_score = 1e30;
    const float loads[3] = {1.5f, 2.0f, 3.0f};
    // longer tasks split fewer partials, so more tiles skip the splat's combine phase
    const int tasks[4] = {16, 24, 32, 48};
    for (float ld : loads)
        for (int tk : tasks) {
            h->tune.hash_load = ld;
            h->tune.task = tk;
            auto t0 = std::chrono::steady_clock::now();
            if ((rc = rebuild_terms(h))) break;
            const double build_ms =
                std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
            float it_ms = 0.f;
            if ((rc = time_iterations(h, 2, 2, &it_ms))) break;
            const double score = build_ms + 5.0 * it_ms;
            if (score < best_score) {
                best_score = score;
                best.hash_load = ld;
                best.task = tk;
            }
        }
    if (!rc) {
        h->tune.hash_load = best.hash_load;
        h->tune.task = best.task;
        rc = rebuild_terms(h);
    }
    // launch knobs on the chosen lattices
    if (!rc) {
        float best_ms = 1e30f;
        const int splits[2] = {1, 2};
        const int smems[2] = {0, 72};
        for (int co = 0; co < 2 && !rc; co++)
            for (int sp : splits) {
                if (sp == 2 && h->MP % 8 != 0) continue;
                for (int sm : smems) {
                    h->tune.split = sp;
                    h->tune.smem_kb = sm;
                    h->tune.coop = co;
                    float ms = 0.f;
                    if ((rc = time_iterations(h, 2, 3, &ms))) break;
                    if (ms < best_ms) {
                        best_ms = ms;
                        best.split = sp;
                        best.smem_kb = sm;
                        best.coop = co;
                    }
                }
                if (rc) break;
            }
        h->tune.split = best.split;
        h->tune.smem_kb = best.smem_kb;
        h->tune.coop = best.coop;
    }
    h->profiling = prof;
    if (rc) return rc;
    h->tuned = true;
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune_cache[tune_key(h)] = h->tune;
    return DCRF_OK;
}

// Applies knobs; rebuilds the lattices when a build knob changes.
int apply_tuning(dcrf_crf *h, const TuneCfg &c) {
    const bool rebuild = c.task != h->tune.task || c.hash_load != h->tune.hash_load;
    h->tune = c;
    h->tuned = true;
    return rebuild ? rebuild_terms(h) : DCRF_OK;
}

// Automatic mode: tune (or take the remembered choice) before the first
// inference of a configuration.
int maybe_autotune(dcrf_crf *h) {
    if (!h->autotune || h->tuned || h->terms.empty()) return DCRF_OK;
    TuneCfg c;
    bool hit = false;
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        auto it = g_tune_cache.find(tune_key(h));
        if (it != g_tune_cache.end()) {
            c = it->second;
            hit = true;
        }
    }
    return hit ? apply_tuning(h, c) : autotune_now(h);
}

int run_inference(dcrf_crf *h, int T, int final_mode, float *ckpt = nullptr) {
    int trc = maybe_autotune(h);
    if (!trc) trc = flush_norms(h);  // (re)built by the tuner: normalised before any capture
    if (!trc) trc = ensure_wide_bufs(h);
    if (trc) return trc;
    if (h->profiling || !h->use_graphs || h->inference_runs++ == 0) return issue_inference(h, T, final_mode, ckpt);
    cudaStream_t user = h->stream;
    h->stream = h->capture;
    CU(cudaStreamBeginCapture(h->capture, cudaStreamCaptureModeThreadLocal));
    int rc = issue_inference(h, T, final_mode, ckpt);
    cudaGraph_t graph = nullptr;
    cudaError_t ce = cudaStreamEndCapture(h->capture, &graph);
    h->stream = user;
    if (rc) {
        if (graph) cudaGraphDestroy(graph);
        return rc;
    }
    if (ce != cudaSuccess) return set_err(DCRF_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(ce));
    bool updated = false;
    if (h->gexec) {
        cudaGraphExecUpdateResultInfo info;
        if (cudaGraphExecUpdate(h->gexec, graph, &info) == cudaSuccess)
            updated = true;
        else {
            cudaGetLastError();
            cudaGraphExecDestroy(h->gexec);
            h->gexec = nullptr;
        }
    }
    if (!updated) {
        ce = cudaGraphInstantiate(&h->gexec, graph, 0);
        if (ce != cudaSuccess) {
            cudaGraphDestroy(graph);
            h->gexec = nullptr;
            return set_err(DCRF_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(ce));
        }
    }
    cudaGraphDestroy(graph);
    CU(cudaGraphLaunch(h->gexec, h->stream));
    return DCRF_OK;
}

// ---- adjoint helpers --------------------------------------------------------

bool fwd_pre(const Term &T) { return T.ntype == DCRF_NORMALIZE_SYMMETRIC || T.ntype == DCRF_NORMALIZE_BEFORE; }
bool fwd_post(const Term &T) { return T.ntype == DCRF_NORMALIZE_SYMMETRIC || T.ntype == DCRF_NORMALIZE_AFTER; }
bool tr_pre(const Term &T) { return T.ntype == DCRF_NORMALIZE_SYMMETRIC || T.ntype == DCRF_NORMALIZE_AFTER; }
bool tr_post(const Term &T) { return T.ntype == DCRF_NORMALIZE_SYMMETRIC || T.ntype == DCRF_NORMALIZE_BEFORE; }

// Adjoint work lattices of a term, allocated on first use; row 0 of each is
// the zero sentinel the blur reads for missing neighbours.
int ensure_adjoint_bufs(dcrf_crf *h, Term &T) {
    const size_t rows = (size_t)T.lat.L + 1;
    int rc;
    for (float *&b : T.bv)
        if (!b) {
            if ((rc = dev_alloc_async(&b, rows * h->MP, h->stream))) return rc;
            CU(cudaMemsetAsync(b, 0, sizeof(float) * rows * h->MP, h->stream));
        }
    for (float *&b : T.b1)
        if (!b) {
            if ((rc = dev_alloc_async(&b, rows, h->stream))) return rc;
            CU(cudaMemsetAsync(b, 0, sizeof(float) * rows, h->stream));
        }
    return DCRF_OK;
}

// S (vertex rows) = splat of the slot rows x with the plain barycentric weights
// (the splat of Permutohedral::compute, permutohedral.cpp:545-553).
// With prenorm, the splat of norm .* x, through the member weights that carry
// the norm of their point (the term must be normalised).
int splat_into(dcrf_crf *h, int k, const float *x, float *S, bool value1, bool prenorm = false) {
    Term &T = h->terms[k];
    const int MP = value1 ? 1 : h->MP;
    std::vector<int> one{k};
    PPArgs a = pp_args(h, PP_LOAD_Q | PP_SPLAT, one, false, value1);
    a.ts.t[0].pre_norm = 0;
    a.ts.t[0].mem_w = prenorm ? T.mem_wn : T.lat.mem_w;
    a.Qin = x;
    CU(pp(h, a, MP));
    ReduceArgs ra{};
    ra.n = 1;
    ra.t[0] = {T.lat.red_beg, T.pout, S, T.lat.L, T.lat.P};
    ProfScope ps(h, DCRF_KCLASS_REDUCE);
    CU(launch_reduce(ra, MP, h->stream));
    return DCRF_OK;
}

// The splat of the same slot rows x through several terms in one point pass
// and one reduce: S[q] (vertex rows) of term ks[q], with its norm folded into
// the member weights where prenorm[q] (see splat_into).
int splat_terms_into(dcrf_crf *h, const std::vector<int> &ks, const float *x, const std::vector<float *> &S,
                     const std::vector<bool> &prenorm) {
    if (ks.empty()) return DCRF_OK;
    PPArgs a = pp_args(h, PP_LOAD_Q | PP_SPLAT, ks, false, false);
    ReduceArgs ra{};
    ra.n = (int)ks.size();
    for (size_t q = 0; q < ks.size(); q++) {
        Term &T = h->terms[ks[q]];
        a.ts.t[q].pre_norm = 0;
        a.ts.t[q].mem_w = prenorm[q] ? T.mem_wn : T.lat.mem_w;
        ra.t[q] = {T.lat.red_beg, T.pout, S[q], T.lat.L, T.lat.P};
    }
    a.Qin = x;
    CU(pp(h, a, h->MP));
    ProfScope ps(h, DCRF_KCLASS_REDUCE);
    CU(launch_reduce(ra, h->MP, h->stream));
    return DCRF_OK;
}

// Independent blur chains advanced together, one launch per axis pass: chain c
// blurs S along axes 0..d (d..0 when reverse, permutohedral.cpp:556) through
// the ping-pong pair b[0], b[1] into Out.  Chains of one launch must not share
// buffers; chains whose arithmetic flavour differs (scalar build) go in
// separate launches.
struct Chain {
    int k;
    const float *S;
    float *b[2];
    float *Out;
    bool reverse;
};

// Launch plan of a chain: launch i runs passes pass[i] (and pass[i] + 1 when
// two[i]) from in[i] into out[i].  Passes go two per launch with the
// intermediate buffers planned backwards from Out, alternating b[0] and b[1];
// a chain whose S would be overwritten by its first launch keeps one pass per
// launch (the original ping-pong).
struct ChainPlan {
    int n = 0;
    int pass[DCRF_MAX_D + 1];
    bool two[DCRF_MAX_D + 1];
    const float *in[DCRF_MAX_D + 1];
    float *out[DCRF_MAX_D + 1];
};

ChainPlan plan_chain(const Chain &c, int d) {
    ChainPlan p;
    const int n2 = (d + 2) / 2;
    float *x[DCRF_MAX_D + 2];
    x[n2] = c.Out;
    x[n2 - 1] = c.Out == c.b[0] ? c.b[1] : c.b[0];
    for (int i = n2 - 2; i >= 1; i--) x[i] = x[i + 1] == c.b[0] ? c.b[1] : c.b[0];
    const bool clash = (n2 >= 2 && x[1] == c.S) || (n2 == 1 && c.Out == c.S);
    if (!clash) {
        p.n = n2;
        for (int i = 0; i < n2; i++) {
            p.pass[i] = 2 * i;
            p.two[i] = 2 * i + 1 <= d;
            p.in[i] = i == 0 ? c.S : x[i];
            p.out[i] = x[i + 1];
        }
        return p;
    }
    p.n = d + 1;
    for (int q = 0; q <= d; q++) {
        p.pass[q] = q;
        p.two[q] = false;
        p.in[q] = q == 0 ? c.S : c.b[(q - 1) & 1];
        p.out[q] = q == d ? c.Out : c.b[q & 1];
    }
    return p;
}

int blur_chains(dcrf_crf *h, const std::vector<Chain> &chains, bool value1) {
    const int MP = value1 ? 1 : h->MP;
    const int NV = MP % 4 == 0 ? MP / 4 : MP % 2 == 0 ? MP / 2 : MP;
    for (int flavour = 0; flavour < 2; flavour++) {
        std::vector<const Chain *> cs;
        for (const Chain &c : chains) {
            const bool seq = value1 || h->M <= 2 || h->terms[c.k].variant == DCRF_VARIANT_SCALAR;
            if ((int)seq == flavour) cs.push_back(&c);
        }
        for (size_t g0 = 0; g0 < cs.size(); g0 += DCRF_MAX_TERMS) {
            const size_t g1 = std::min(cs.size(), g0 + DCRF_MAX_TERMS);
            std::vector<ChainPlan> plans;
            int steps = 0;
            for (size_t q = g0; q < g1; q++) {
                plans.push_back(plan_chain(*cs[q], h->terms[cs[q]->k].d));
                steps = std::max(steps, plans.back().n);
            }
            for (int i = 0; i < steps; i++) {
                BlurArgs ba{};
                ba.n = 0;
                ba.begin[0] = 0;
                for (size_t q = g0; q < g1; q++) {
                    const Chain &c = *cs[q];
                    const ChainPlan &pl = plans[q - g0];
                    const Term &T = h->terms[c.k];
                    if (i >= pl.n) continue;
                    const int p = pl.pass[i];
                    BlurArgs::T &bt = ba.t[ba.n];
                    bt.Vin = pl.in[i];
                    bt.Vout = pl.out[i];
                    bt.nbr = T.lat.nbr;
                    bt.L = T.lat.L;
                    bt.axis = c.reverse ? T.d - p : p;
                    bt.axis2 = !pl.two[i] ? -1 : c.reverse ? T.d - (p + 1) : p + 1;
                    bt.pv = nullptr;
                    ba.begin[ba.n + 1] = ba.begin[ba.n] + (long long)T.lat.L * NV;
                    ba.n++;
                }
                ProfScope ps(h, DCRF_KCLASS_BLUR);
                CU(launch_blur(ba, MP, flavour == 1, h->stream));
            }
        }
    }
    return DCRF_OK;
}

// Out = the d+1 blur passes of S, axes 0..d or d..0 for the transpose
// (permutohedral.cpp:556); S is kept, the term's V buffers are the ping-pong.
int blur_into(dcrf_crf *h, int k, const float *S, float *Out, bool reverse, bool value1) {
    Term &T = h->terms[k];
    const int MP = value1 ? 1 : h->MP;
    const bool seq = value1 || h->M <= 2 || T.variant == DCRF_VARIANT_SCALAR;
    if (!h->tune.coop) {
        int rc = blur_chains(h, {Chain{k, S, {T.V[1], T.V[0]}, Out, reverse}}, value1);
        if (rc) return rc;
        if (value1) return zero_sentinels(h, T);
        return DCRF_OK;
    }
    {
        BlurChainArgs ca{};
        ca.n = 1;
        ca.npass = T.d + 1;
        ca.bar = h->bar;
        ca.status = h->status;
        BlurChainArgs::C &c = ca.c[0];
        c.S = S;
        c.buf[0] = T.V[1];
        c.buf[1] = T.V[0];
        c.Out = Out;
        c.nbr = T.lat.nbr;
        c.L = T.lat.L;
        c.d = T.d;
        c.reverse = reverse ? 1 : 0;
        ProfScope ps(h, DCRF_KCLASS_BLUR);
        CU(launch_blur_chains(ca, MP, seq, h->stream));
        if (value1) return zero_sentinels(h, T);
        return DCRF_OK;
    }
}

// out (slot rows) = slice of the vertex rows V (permutohedral.cpp:574-584);
// with post, also Fpost = [norm .*] out (norm when post_norm) and
// Gacc += compat(Fpost) (either may be null).
int slice_from(dcrf_crf *h, int k, const float *V, float *out, bool value1, bool post_norm = false,
               float *Fpost = nullptr, float *Gacc = nullptr) {
    std::vector<int> one{k};
    PPArgs f = pp_args(h, PP_FILTER, one, false, value1);
    f.ts.t[0].V = V;
    f.ts.t[0].post_norm = post_norm ? 1 : 0;
    f.Qout = out;
    f.Fpost = Fpost;
    f.Gacc = Gacc;
    CU(pp(h, f, value1 ? 1 : h->MP));
    return DCRF_OK;
}

// T.df += sign * sum over labels of z . d(slice of V)/d(features): the
// per-point part of Permutohedral::gradient (permutohedral.cpp:612-695).
// z2scale (optional, [nslots]): the second pair's z is z2 .* z2scale per point.
// V3, V4 (optional, value size 1, [L+1]): two more pairs in the same pass, V3
// with z = 1 and V4 with z = z4, both with sign34.
int slice_grad_into(dcrf_crf *h, int k, const float *V, const float *z, float sign, bool value1,
                    const float *V2 = nullptr, const float *z2 = nullptr, float sign2 = 1.f,
                    const float *z2scale = nullptr, const float *V3 = nullptr, const float *V4 = nullptr,
                    const float *z4 = nullptr, float sign34 = 1.f) {
    Term &T = h->terms[k];
    SliceGradArgs g{};
    g.z2scale = z2scale;
    g.V3 = V3;
    g.V4 = V4;
    g.z4 = z4;
    g.V2 = V2;
    g.z2 = z2;
    g.N = h->N;
    g.M = value1 ? 1 : h->M;
    g.d = T.d;
    g.nslots = h->nslots;
    g.slot_pt = h->slot_pt;
    g.off = T.lat.off;
    g.rank = T.lat.rank;
    g.V = V;
    g.z = z;
    const float inv_std_dev = (float)(std::sqrt(2.0 / 3.0) * (T.d + 1));
    for (int i = 0; i < T.d; i++)
        g.sf[i] = (float)(1.0 / std::sqrt((double)((i + 2) * (i + 1))) * (double)inv_std_dev);
    g.alpha = 1.0f / (1.0f + std::pow(2.0f, (float)-T.d)) / (float)(T.d + 1) * sign;
    g.alpha2 = 1.0f / (1.0f + std::pow(2.0f, (float)-T.d)) / (float)(T.d + 1) * sign2;
    g.alpha3 = g.alpha4 = 1.0f / (1.0f + std::pow(2.0f, (float)-T.d)) / (float)(T.d + 1) * sign34;
    g.df = T.df;
    CU(launch_slice_grad(g, value1 ? 1 : h->MP, h->stream));
    return DCRF_OK;
}

int compat_count(const dcrf_crf *h, const Term &T) {
    return T.ckind == DCRF_COMPAT_POTTS ? 1 : T.ckind == DCRF_COMPAT_DIAGONAL ? h->M : h->M * h->M;
}

int kernel_count(const Term &T) {
    return T.ktype == DCRF_FULL_KERNEL ? T.d * T.d : T.ktype == DCRF_DIAG_KERNEL ? T.d : 0;
}

}  // namespace

// A wait on a flag that nothing sets, bounded like the library's other device
// waits (poll, sleep, give up): it must end in the status block, not hang.
__global__ void bounded_wait_probe_kernel(const volatile unsigned *flag, int spins, DevStatus *st) {
    if (threadIdx.x != 0) return;
    for (int it = 0; it < spins; it++) {
        if (*flag != 0u) return;
        __nanosleep(256);
    }
    dcrf_set_error(st, DCRF_ERR_TIMEOUT, -1);
}

extern "C" {

int dcrf_abi_version(void) { return DCRF_ABI_VERSION; }

int dcrf_last_error(char *buf, size_t len) {
    if (buf && len) {
        size_t n = std::min(len - 1, g_err.size());
        std::memcpy(buf, g_err.data(), n);
        buf[n] = 0;
    }
    return g_code;
}

int dcrf_create(int N, int M, dcrf_crf **out) { return create(M, {N}, {}, {}, out); }

int dcrf_create_2d(int W, int H, int M, dcrf_crf **out) {
    if (W <= 0 || H <= 0) return set_err(DCRF_ERR_INVALID_ARG, "W and H must be positive");
    if ((long long)W * H > 0x7FFFFFFF) return set_err(DCRF_ERR_INVALID_ARG, "image too large");
    return create(M, {W * H}, {W}, {H}, out);
}

int dcrf_create_batch(int n_images, const int *N, int M, dcrf_crf **out) {
    if (n_images <= 0 || !N) return set_err(DCRF_ERR_INVALID_ARG, "a batch needs at least one image");
    return create(M, std::vector<int>(N, N + n_images), {}, {}, out);
}

int dcrf_create_batch_2d(int n_images, const int *W, const int *H, int M, dcrf_crf **out) {
    if (n_images <= 0 || !W || !H) return set_err(DCRF_ERR_INVALID_ARG, "a batch needs at least one image");
    std::vector<int> Ns(n_images), Ws(W, W + n_images), Hs(H, H + n_images);
    for (int b = 0; b < n_images; b++) {
        if (W[b] <= 0 || H[b] <= 0) return set_err(DCRF_ERR_INVALID_ARG, "W and H must be positive");
        if ((long long)W[b] * H[b] > 0x7FFFFFFF) return set_err(DCRF_ERR_INVALID_ARG, "image too large");
        Ns[b] = W[b] * H[b];
    }
    return create(M, Ns, Ws, Hs, out);
}

int dcrf_batch_info(dcrf_crf *h, int *n_images, int *point_start) {
    int rc = check_handle(h);
    if (rc) return rc;
    if (n_images) *n_images = (int)h->seg.size() - 1;
    if (point_start) std::memcpy(point_start, h->seg.data(), h->seg.size() * sizeof(int));
    return ok();
}

int dcrf_destroy(dcrf_crf *h) {
    if (!h) return ok();
    cudaSetDevice(h->device);
    if (h->stream) cudaStreamSynchronize(h->stream);
    release_marks(h);
    for (cudaEvent_t e : h->event_pool) cudaEventDestroy(e);
    h->event_pool.clear();
    for (Term &T : h->terms) free_term(h, T);
    dev_free_async(h->ckpt, h->stream);
    dev_free_async(h->segq, h->stream);
    dev_free_async(h->ckv, h->stream);
    dev_free_async(h->cky, h->stream);
    for (float *&b : h->bw) dev_free_async(b, h->stream);
    for (float *&b : h->bw1) dev_free_async(b, h->stream);
    dev_free_async(h->dpart, h->stream);
    dev_free_async(h->dacc, h->stream);
    dev_free_async(h->wideF, h->stream);
    for (auto *v : {&h->adjF, &h->adjY})
        for (float *p : *v) dev_free_async(p, h->stream);
    dev_free_async(h->L_d, h->stream);
    dev_free_async(h->f_d, h->stream);
    for (void *p : {(void *)h->status, (void *)h->bar, (void *)h->U, (void *)h->Q, (void *)h->tmp,
                    (void *)h->stage, (void *)h->map, (void *)h->kl_part, (void *)h->d_seg, (void *)h->d_imgW})
        dev_free_async(p, h->stream);
    if (h->gexec) cudaGraphExecDestroy(h->gexec);
    if (h->xorder) cudaEventDestroy(h->xorder);
    if (h->capture) cudaStreamDestroy(h->capture);
    if (h->own) cudaStreamDestroy(h->own);
    delete h;
    return ok();
}

int dcrf_check_bounded_wait(dcrf_crf *h, int spins) {
    int rc = check_ready(h);
    if (rc) return rc;
    if (spins < 1 || spins > (1 << 20)) return set_err(DCRF_ERR_INVALID_ARG, "spins must be in [1, 1048576]");
    unsigned *flag = nullptr;
    if ((rc = dev_alloc_async(&flag, 1, h->stream))) return rc;
    CU(cudaMemsetAsync(flag, 0, sizeof(unsigned), h->stream));
    DCRF_LAUNCH(bounded_wait_probe_kernel<<<1, 32, 0, h->stream>>>(flag, spins, h->status));
    dev_free_async(flag, h->stream);
    rc = sync_check(h);
    if (rc == DCRF_ERR_TIMEOUT) set_err(rc, "bounded device wait gave up as expected (" + g_err + ")");
    return rc;
}

int dcrf_set_stream(dcrf_crf *h, void *s) {
    int rc = check_handle(h);
    if (rc) return rc;
    CU(cudaStreamSynchronize(h->stream));
    h->stream = s ? (cudaStream_t)s : h->own;
    return ok();
}

int dcrf_set_variant(dcrf_crf *h, int variant) {
    int rc = check_handle(h);
    if (rc) return rc;
    if (variant != DCRF_VARIANT_SSE && variant != DCRF_VARIANT_SCALAR)
        return set_err(DCRF_ERR_INVALID_ARG, "unknown variant");
    for (const Term &T : h->terms)
        if (T.variant != variant)
            return set_err(DCRF_ERR_STATE, "the lattice variant must be chosen before adding pairwise terms");
    h->variant = variant;
    return ok();
}

int dcrf_set_unary(dcrf_crf *h, const float *U, int layout, int where) {
    int rc = check_handle(h);
    if (rc) return rc;
    if (!U) return set_err(DCRF_ERR_INVALID_ARG, "null unary");
    if ((rc = load_mn(h, U, layout, where, h->U))) return rc;
    h->nfeat = 0;  // a constant unary from now on
    h->has_unary = true;
    h->version++;
    if ((rc = sync_check(h))) return rc;
    return ok();
}

// ---- logistic unary and the parameter vectors ------------------------------
static int upload_logistic_L(dcrf_crf *h) {
    CU(cudaMemcpyAsync(h->L_d, h->L_h.data(), h->L_h.size() * sizeof(float), cudaMemcpyHostToDevice, h->stream));
    CU(launch_logistic_unary(h->L_d, h->f_d, h->M, h->nfeat, h->N, h->nslots, h->slot_pt, h->U, h->stream));
    return DCRF_OK;
}

int dcrf_set_unary_logistic(dcrf_crf *h, const float *L, int nfeat, const float *f, int where) {
    int rc = check_handle(h);
    if (rc) return rc;
    if (!L || !f) return set_err(DCRF_ERR_INVALID_ARG, "null argument");
    if (nfeat < 1) return set_err(DCRF_ERR_INVALID_ARG, "the logistic unary needs at least one feature");
    const size_t nL = (size_t)h->M * nfeat, nf = (size_t)nfeat * h->N;
    h->L_h.resize(nL);
    if (where == DCRF_DEVICE)
        CU(cudaMemcpy(h->L_h.data(), L, nL * sizeof(float), cudaMemcpyDeviceToHost));
    else
        std::memcpy(h->L_h.data(), L, nL * sizeof(float));
    dev_free_async(h->L_d, h->stream);
    dev_free_async(h->f_d, h->stream);
    h->L_d = h->f_d = nullptr;
    h->nfeat = 0;
    if ((rc = dev_alloc_async(&h->L_d, nL, h->stream)) || (rc = dev_alloc_async(&h->f_d, nf, h->stream))) return rc;
    CU(cudaMemcpyAsync(h->f_d, f, nf * sizeof(float),
                       where == DCRF_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, h->stream));
    h->nfeat = nfeat;
    if ((rc = upload_logistic_L(h))) return rc;
    h->has_unary = true;
    h->version++;
    if ((rc = sync_check(h))) return rc;
    return ok();
}

// Copies n = count values to out when out is non-null and capacity >= n.
static int give_vector(const std::vector<float> &v, float *out, int capacity, int *n) {
    if (n) *n = (int)v.size();
    if (out) {
        if (capacity < (int)v.size())
            return set_err(DCRF_ERR_INVALID_ARG, "output holds " + std::to_string(capacity) + " values, " +
                                                     std::to_string(v.size()) + " needed");
        std::copy(v.begin(), v.end(), out);
    }
    return ok();
}

int dcrf_unary_parameters(dcrf_crf *h, float *out, int capacity, int *n) {
    int rc = check_handle(h);
    if (rc) return rc;
    std::vector<float> v((size_t)h->M * h->nfeat);
    for (int m = 0; m < h->M; m++)
        for (int j = 0; j < h->nfeat; j++) v[(size_t)m + (size_t)h->M * j] = h->L_h[(size_t)m * h->nfeat + j];
    return give_vector(v, out, capacity, n);
}

int dcrf_set_unary_parameters(dcrf_crf *h, const float *v, int n) {
    int rc = check_handle(h);
    if (rc) return rc;
    if (n != h->M * h->nfeat)
        return set_err(DCRF_ERR_INVALID_ARG, "the unary has " + std::to_string(h->M * h->nfeat) + " parameters, got " +
                                                 std::to_string(n));
    if (n == 0) return ok();  // a constant unary has none (UnaryEnergy::setParameters, unary.cpp:35-36)
    if (!v) return set_err(DCRF_ERR_INVALID_ARG, "null parameters");
    for (int m = 0; m < h->M; m++)
        for (int j = 0; j < h->nfeat; j++) h->L_h[(size_t)m * h->nfeat + j] = v[(size_t)m + (size_t)h->M * j];
    if ((rc = upload_logistic_L(h))) return rc;
    h->version++;
    if ((rc = sync_check(h))) return rc;
    return ok();
}

// LabelCompatibility::parameters of term k (labelcompatibility.cpp:50-54,69-71,88-94)
static std::vector<float> compat_parameters(const dcrf_crf *h, const Term &T) {
    const int M = h->M;
    if (T.ckind == DCRF_COMPAT_POTTS) return {T.potts_w};
    if (T.ckind == DCRF_COMPAT_DIAGONAL) return T.compat_h;
    std::vector<float> r;
    for (int i = 0; i < M; i++)
        for (int j = i; j < M; j++) r.push_back(T.compat_h[(size_t)i * M + j]);
    return r;
}

// DenseKernel::parameters (pairwise.cpp:129-139): DIAG the d scales, FULL the
// d x d matrix column-major, CONST none
static std::vector<float> kernel_parameters(const Term &T) {
    if (T.ktype == DCRF_DIAG_KERNEL) return T.params;
    if (T.ktype != DCRF_FULL_KERNEL) return {};
    std::vector<float> r((size_t)T.d * T.d);
    for (int a = 0; a < T.d; a++)
        for (int b = 0; b < T.d; b++) r[(size_t)a + (size_t)T.d * b] = T.params[(size_t)a * T.d + b];
    return r;
}

int dcrf_label_compatibility_parameters(dcrf_crf *h, float *out, int capacity, int *n) {
    int rc = check_handle(h);
    if (rc) return rc;
    std::vector<float> v;
    for (const Term &T : h->terms) {
        std::vector<float> p = compat_parameters(h, T);
        v.insert(v.end(), p.begin(), p.end());
    }
    return give_vector(v, out, capacity, n);
}

int dcrf_set_label_compatibility_parameters(dcrf_crf *h, const float *v, int n) {
    int rc = check_handle(h);
    if (rc) return rc;
    int total = 0;
    for (const Term &T : h->terms) total += (int)compat_parameters(h, T).size();
    if (n != total)
        return set_err(DCRF_ERR_INVALID_ARG, "the compatibilities have " + std::to_string(total) +
                                                 " parameters, got " + std::to_string(n));
    if (n > 0 && !v) return set_err(DCRF_ERR_INVALID_ARG, "null parameters");
    const int M = h->M;
    int i = 0;
    for (Term &T : h->terms) {
        if (T.ckind == DCRF_COMPAT_POTTS) {
            if ((rc = set_term_compat(h, T, DCRF_COMPAT_POTTS, v + i))) return rc;
            i += 1;
        } else if (T.ckind == DCRF_COMPAT_DIAGONAL) {
            if ((rc = set_term_compat(h, T, DCRF_COMPAT_DIAGONAL, v + i))) return rc;
            i += M;
        } else {  // the packed upper triangle of the symmetric matrix (labelcompatibility.cpp:95-100)
            std::vector<float> m((size_t)M * M);
            for (int a = 0; a < M; a++)
                for (int b = a; b < M; b++) m[(size_t)a * M + b] = m[(size_t)b * M + a] = v[i++];
            if ((rc = set_term_compat(h, T, DCRF_COMPAT_MATRIX, m.data()))) return rc;
        }
    }
    h->version++;
    if ((rc = sync_check(h))) return rc;
    return ok();
}

int dcrf_kernel_parameters(dcrf_crf *h, float *out, int capacity, int *n) {
    int rc = check_handle(h);
    if (rc) return rc;
    std::vector<float> v;
    for (const Term &T : h->terms) {
        std::vector<float> p = kernel_parameters(T);
        v.insert(v.end(), p.begin(), p.end());
    }
    return give_vector(v, out, capacity, n);
}

int dcrf_set_kernel_parameters(dcrf_crf *h, const float *v, int n) {
    int rc = check_handle(h);
    if (rc) return rc;
    int total = 0;
    for (const Term &T : h->terms) total += (int)kernel_parameters(T).size();
    if (n != total)
        return set_err(DCRF_ERR_INVALID_ARG, "the kernels have " + std::to_string(total) + " parameters, got " +
                                                 std::to_string(n));
    if (n > 0 && !v) return set_err(DCRF_ERR_INVALID_ARG, "null parameters");
    int i = 0;
    for (int k = 0; k < (int)h->terms.size(); k++) {
        Term &T = h->terms[k];
        if (T.ktype == DCRF_CONST_KERNEL) continue;
        std::vector<float> p;
        if (T.ktype == DCRF_DIAG_KERNEL) {
            p.assign(v + i, v + i + T.d);
            i += T.d;
        } else {  // column-major d x d (pairwise.cpp:146-150) -> row-major P
            p.resize((size_t)T.d * T.d);
            for (int a = 0; a < T.d; a++)
                for (int b = 0; b < T.d; b++) p[(size_t)a * T.d + b] = v[i + a + T.d * b];
            i += T.d * T.d;
        }
        if ((rc = dcrf_set_kernel_params(h, k, p.data()))) return rc;
    }
    return ok();
}

int dcrf_unary_gradient(dcrf_crf *h, double *out, int capacity, int *n) {
    int rc = check_handle(h);
    if (rc) return rc;
    const int K = h->M * h->nfeat;
    if (n) *n = K;
    if (!out || K == 0) return ok();
    if (capacity < K) return set_err(DCRF_ERR_INVALID_ARG, "output too small for the unary gradient");
    if (h->du_version != h->version || !h->bw[2])
        return set_err(DCRF_ERR_STATE, "dcrf_unary_gradient needs a dcrf_backward of the current model");
    const size_t npart = (size_t)logistic_grad_blocks(h->nslots, h->M, h->nfeat) * K;
    if (npart == 0) return set_err(DCRF_ERR_INVALID_ARG, "too many logistic features for the gradient kernel");
    if (npart > h->dpart_cap) {
        dev_free_async(h->dpart, h->stream);
        h->dpart = nullptr;
        h->dpart_cap = 0;
        if ((rc = dev_alloc_async(&h->dpart, npart, h->stream))) return rc;
        h->dpart_cap = npart;
    }
    if ((size_t)K + 1 > h->dacc_cap) {
        dev_free_async(h->dacc, h->stream);
        h->dacc = nullptr;
        h->dacc_cap = 0;
        if ((rc = dev_alloc_async(&h->dacc, (size_t)K + 1, h->stream))) return rc;
        h->dacc_cap = (size_t)K + 1;
    }
    // LogisticUnaryEnergy::gradient (unary.cpp:64-67) of the summed adjoint: (sum_t b_t) f^T = dL/dU f^T
    CU(launch_logistic_grad(h->bw[2], h->f_d, h->M, h->nfeat, h->N, h->nslots, h->slot_pt, h->dpart, h->dacc,
                            h->stream));
    CU(cudaMemcpyAsync(out, h->dacc, sizeof(double) * K, cudaMemcpyDeviceToHost, h->stream));
    if ((rc = sync_check(h))) return rc;
    return ok();
}

int dcrf_add_pairwise(dcrf_crf *h, const float *feat, int d, int where, int compat_kind, const float *compat,
                      int kernel_type, int normalization_type, int *term_out) {
    int rc = check_handle(h);
    if (rc) return rc;
    if (!feat) return set_err(DCRF_ERR_INVALID_ARG, "null features");
    if (d < 1 || d > DCRF_MAX_D) return set_err(DCRF_ERR_INVALID_ARG, "feature dimension must be in [1, 16]");
    if ((rc = validate_compat(compat_kind, compat)) || (rc = validate_kn(kernel_type, normalization_type))) return rc;
    if ((int)h->terms.size() >= DCRF_MAX_TERMS) return set_err(DCRF_ERR_INVALID_ARG, "too many pairwise terms");
    float *f = nullptr;
    if ((rc = dev_alloc_async(&f, (size_t)d * h->N, h->stream))) return rc;
    cudaError_t e = cudaMemcpyAsync(f, feat, sizeof(float) * (size_t)d * h->N,
                                    where == DCRF_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                                    h->stream);
    if (e != cudaSuccess) {
        dev_free_async(f, h->stream);
        return set_err(DCRF_ERR_CUDA, std::string("feature copy: ") + cudaGetErrorString(e));
    }
    return add_term(h, f, d, compat_kind, compat, kernel_type, normalization_type, term_out);
}

int dcrf_add_pairwise_gaussian(dcrf_crf *h, float sx, float sy, int compat_kind, const float *compat,
                               int kernel_type, int normalization_type, int *term_out) {
    int rc = check_handle(h);
    if (rc) return rc;
    if (!h->grid2d) return set_err(DCRF_ERR_STATE, "addPairwiseGaussian needs a DenseCRF2D handle");
    if ((rc = validate_compat(compat_kind, compat)) || (rc = validate_kn(kernel_type, normalization_type))) return rc;
    if ((int)h->terms.size() >= DCRF_MAX_TERMS) return set_err(DCRF_ERR_INVALID_ARG, "too many pairwise terms");
    float *f = nullptr;
    if ((rc = dev_alloc_async(&f, (size_t)2 * h->N, h->stream))) return rc;
    cudaError_t e = launch_features_2d(h->N, h->d_seg, h->d_imgW, (int)h->seg.size() - 1, sx, sy, nullptr, 1.f, 1.f, 1.f, f,
                                       h->stream);
    if (e != cudaSuccess) {
        dev_free_async(f, h->stream);
        return set_err(DCRF_ERR_CUDA, std::string("features: ") + cudaGetErrorString(e));
    }
    return add_term(h, f, 2, compat_kind, compat, kernel_type, normalization_type, term_out);
}

int dcrf_add_pairwise_bilateral(dcrf_crf *h, float sx, float sy, float sr, float sg, float sb, const uint8_t *rgb,
                                int where, int compat_kind, const float *compat, int kernel_type,
                                int normalization_type, int *term_out) {
    int rc = check_handle(h);
    if (rc) return rc;
    if (!h->grid2d) return set_err(DCRF_ERR_STATE, "addPairwiseBilateral needs a DenseCRF2D handle");
    if (!rgb) return set_err(DCRF_ERR_INVALID_ARG, "null image");
    if ((rc = validate_compat(compat_kind, compat)) || (rc = validate_kn(kernel_type, normalization_type))) return rc;
    if ((int)h->terms.size() >= DCRF_MAX_TERMS) return set_err(DCRF_ERR_INVALID_ARG, "too many pairwise terms");
    float *f = nullptr;
    uint8_t *img = nullptr;
    if ((rc = dev_alloc_async(&f, (size_t)5 * h->N, h->stream))) return rc;
    const uint8_t *src = rgb;
    if (where != DCRF_DEVICE) {
        if ((rc = dev_alloc_async(&img, (size_t)3 * h->N, h->stream))) {
            dev_free_async(f, h->stream);
            return rc;
        }
        cudaError_t e = cudaMemcpyAsync(img, rgb, (size_t)3 * h->N, cudaMemcpyHostToDevice, h->stream);
        if (e != cudaSuccess) {
            dev_free_async(f, h->stream);
            dev_free_async(img, h->stream);
            return set_err(DCRF_ERR_CUDA, std::string("image copy: ") + cudaGetErrorString(e));
        }
        src = img;
    }
    cudaError_t e = launch_features_2d(h->N, h->d_seg, h->d_imgW, (int)h->seg.size() - 1, sx, sy, src, sr, sg, sb, f,
                                       h->stream);
    if (e != cudaSuccess) {
        dev_free_async(f, h->stream);
        dev_free_async(img, h->stream);
        return set_err(DCRF_ERR_CUDA, std::string("features: ") + cudaGetErrorString(e));
    }
    rc = add_term(h, f, 5, compat_kind, compat, kernel_type, normalization_type, term_out);
    dev_free_async(img, h->stream);
    return rc;
}

int dcrf_inference(dcrf_crf *h, int n_iterations, float *Q, int layout, int where) {
    int rc = check_ready(h);
    if (rc) return rc;
    if (!Q) return set_err(DCRF_ERR_INVALID_ARG, "null output");
    if ((rc = run_inference(h, n_iterations, PP_WRITE_Q))) return rc;
    if ((rc = store_mn(h, h->Q, Q, layout, where))) return rc;
    if ((rc = sync_check(h))) return rc;
    return ok();
}

int dcrf_start_inference(dcrf_crf *h, float *Q, int layout, int where) {
    int rc = check_ready(h);
    if (rc) return rc;
    if (!Q) return set_err(DCRF_ERR_INVALID_ARG, "null output");
    if (!h->has_unary) {  // densecrf.cpp:179-184: zeros without a unary
        CU(cudaMemsetAsync(h->Q, 0, sizeof(float) * (size_t)h->nslots * h->MP, h->stream));
    } else if (is_wide(h)) {
        if ((rc = wide(h, WP_WRITE_Q, {}))) return rc;
    } else {
        CU(pp(h, pp_args(h, PP_WRITE_Q, {}, false, false), h->MP));
    }
    if ((rc = store_mn(h, h->Q, Q, layout, where))) return rc;
    if ((rc = sync_check(h))) return rc;
    return ok();
}

int dcrf_step_inference(dcrf_crf *h, float *Q, int layout, int where) {
    int rc = check_ready(h);
    if (rc) return rc;
    if (!Q) return set_err(DCRF_ERR_INVALID_ARG, "null marginals");
    if ((rc = load_mn(h, Q, layout, where, h->Q))) return rc;
    std::vector<int> w = all_terms(h);
    if (is_wide(h)) {
        if ((rc = ensure_wide_bufs(h))) return rc;
        if (!w.empty() && (rc = wide_splat_filter(h, w))) return rc;
        if ((rc = wide(h, (w.empty() ? 0 : WP_MSG) | WP_WRITE_Q, w))) return rc;
    } else {
        if (!w.empty()) {
            CU(pp(h, pp_args(h, PP_LOAD_Q | PP_SPLAT, w, false, false), h->MP));
            if ((rc = filter_phase(h, w, false, false, true))) return rc;
        }
        CU(pp(h, pp_args(h, PP_MSG | PP_WRITE_Q, w, false, false), h->MP));
    }
    if ((rc = store_mn(h, h->Q, Q, layout, where))) return rc;
    if ((rc = sync_check(h))) return rc;
    return ok();
}

int dcrf_kl_divergence(dcrf_crf *h, const float *Q, int layout, int where, double *kl_out) {
    int rc = check_ready(h);
    if (rc) return rc;
    if (!Q || !kl_out) return set_err(DCRF_ERR_INVALID_ARG, "null argument");
    if ((rc = load_mn(h, Q, layout, where, h->Q))) return rc;
    std::vector<int> w = all_terms(h);
    if (is_wide(h)) {
        if ((rc = ensure_wide_bufs(h))) return rc;
        if (!w.empty() && (rc = wide_splat_filter(h, w))) return rc;
        if ((rc = wide(h, WP_LOAD_Q | WP_KL | (w.empty() ? 0 : WP_MSG), w))) return rc;
    } else {
        if (!w.empty()) {
            CU(pp(h, pp_args(h, PP_LOAD_Q | PP_SPLAT, w, false, false), h->MP));
            if ((rc = filter_phase(h, w, false, false, true))) return rc;
        }
        CU(pp(h, pp_args(h, PP_LOAD_Q | PP_MSG | PP_KL, w, false, false), h->MP));
    }
    std::vector<double> part(h->ntiles);
    CU(cudaMemcpyAsync(part.data(), h->kl_part, sizeof(double) * h->ntiles, cudaMemcpyDeviceToHost, h->stream));
    if ((rc = sync_check(h))) return rc;
    double s = 0.0;
    for (double v : part) s += v;
    *kl_out = s;
    return ok();
}

int dcrf_map(dcrf_crf *h, int n_iterations, int16_t *labels, int where) {
    int rc = check_ready(h);
    if (rc) return rc;
    if (!labels) return set_err(DCRF_ERR_INVALID_ARG, "null output");
    if ((rc = run_inference(h, n_iterations, PP_MAP))) return rc;
    CU(cudaMemcpyAsync(labels, h->map, sizeof(int16_t) * h->N,
                       where == DCRF_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, h->stream));
    if ((rc = sync_check(h))) return rc;
    return ok();
}

// Labels from the caller into a device buffer of the handle's pool.
static int load_labels(dcrf_crf *h, const int16_t *labels, int where, int16_t **out) {
    int rc;
    if ((rc = dev_alloc_async(out, (size_t)h->N, h->stream))) return rc;
    CU(cudaMemcpyAsync(*out, labels, sizeof(int16_t) * h->N,
                       where == DCRF_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, h->stream));
    return DCRF_OK;
}

static int store_energy(dcrf_crf *h, const float *src, float *energy, int where) {
    CU(cudaMemcpyAsync(energy, src, sizeof(float) * h->N,
                       where == DCRF_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, h->stream));
    return DCRF_OK;
}

// pairwiseEnergy for more than 32 labels (densecrf.cpp:160-177): the one-hot
// labelling in the label-chunk layout goes through the chunked splat and
// filter of the selected terms like a marginal, and the wide update pass in
// energy mode adds -1/2 * each term's message at the point's own label.
static int pairwise_energy_wide(dcrf_crf *h, const int16_t *labels, int where, int term, float *energy,
                                int where_out) {
    int rc;
    std::vector<int> w;
    for (int k = 0; k < (int)h->terms.size(); k++)
        if (term < 0 || k == term) w.push_back(k);
    int16_t *lab = nullptr;
    float *e = nullptr;
    if ((rc = ensure_wide_bufs(h)) || (rc = load_labels(h, labels, where, &lab))) return rc;
    if ((rc = dev_alloc_async(&e, (size_t)h->N, h->stream))) return rc;
    CU(cudaMemsetAsync(e, 0, sizeof(float) * h->N, h->stream));  // points of no slot (none) stay 0
    // h->Q is the handle's scratch marginals (every call that reads it loads it first)
    CU(launch_onehot_chunked(lab, h->M, h->MP, h->nslots, h->slot_pt, h->Q, h->stream));
    if ((rc = wide_splat_filter(h, w))) return rc;
    WideArgs a = wide_args(h, WP_MSG | WP_LOAD_Q | WP_ENERGY, w);
    a.labels = lab;
    a.energy = e;
    CU(launch_wide(a, h->stream));
    rc = store_energy(h, e, energy, where_out);
    dev_free_async(lab, h->stream);
    dev_free_async(e, h->stream);
    if (rc) return rc;
    if ((rc = sync_check(h))) return rc;
    return ok();
}

int dcrf_unary_energy(dcrf_crf *h, const int16_t *labels, int where, float *energy, int where_out) {
    int rc = check_ready(h);
    if (rc) return rc;
    if (!labels || !energy) return set_err(DCRF_ERR_INVALID_ARG, "null argument");
    int16_t *lab = nullptr;
    float *e = nullptr;
    if ((rc = load_labels(h, labels, where, &lab))) return rc;
    if ((rc = dev_alloc_async(&e, (size_t)h->N, h->stream))) return rc;
    CU(launch_label_energy(h->has_unary ? h->U : nullptr, lab, h->M, h->nslots, h->N, h->pt_slot, 1.f, 0, e,
                           h->stream));
    rc = store_energy(h, e, energy, where_out);
    dev_free_async(lab, h->stream);
    dev_free_async(e, h->stream);
    if (rc) return rc;
    if ((rc = sync_check(h))) return rc;
    return ok();
}

int dcrf_pairwise_energy(dcrf_crf *h, const int16_t *labels, int where, int term, float *energy, int where_out) {
    int rc = check_ready(h);
    if (rc) return rc;
    if (!labels || !energy) return set_err(DCRF_ERR_INVALID_ARG, "null argument");
    if (term < -1 || term >= (int)h->terms.size()) return set_err(DCRF_ERR_INVALID_ARG, "no such term");
    if (is_wide(h)) return pairwise_energy_wide(h, labels, where, term, energy, where_out);
    const int M = h->M, ns = h->nslots;
    const size_t qsz = (size_t)h->MP * ns;
    for (float *&b : h->bw)
        if (!b && (rc = dev_alloc_async(&b, qsz, h->stream))) return rc;
    int16_t *lab = nullptr;
    float *e = nullptr;
    if ((rc = load_labels(h, labels, where, &lab))) return rc;
    if ((rc = dev_alloc_async(&e, (size_t)h->N, h->stream))) return rc;
    float *q = h->bw[0], *qn = h->bw[1], *g = h->bw[2];
    h->du_version = ~0ull;  // bw[2] no longer holds dL/dU
    CU(launch_onehot(lab, M, ns, h->slot_pt, q, h->stream));
    CU(cudaMemsetAsync(g, 0, qsz * sizeof(float), h->stream));
    // g = sum over the terms of PairwisePotential::apply(one-hot) (pairwise.cpp:173-178)
    for (int k = 0; k < (int)h->terms.size(); k++) {
        if (term >= 0 && k != term) continue;
        Term &Tk = h->terms[k];
        if ((rc = ensure_adjoint_bufs(h, Tk))) return rc;
        const float *xs = q;
        if (fwd_pre(Tk)) {
            CU(launch_scale_norm(q, qn, Tk.norm, M, ns, 1, h->stream));
            xs = qn;
        }
        if ((rc = splat_into(h, k, xs, Tk.bv[0], false))) return rc;
        if ((rc = blur_into(h, k, Tk.bv[0], Tk.bv[1], false, false))) return rc;
        if ((rc = slice_from(h, k, Tk.bv[1], nullptr, false, fwd_post(Tk), nullptr, g))) return rc;
    }
    // r = -0.5 * message at the point's own label (densecrf.cpp:169-174)
    CU(launch_label_energy(g, lab, M, ns, h->N, h->pt_slot, -0.5f, 0, e, h->stream));
    rc = store_energy(h, e, energy, where_out);
    dev_free_async(lab, h->stream);
    dev_free_async(e, h->stream);
    if (rc) return rc;
    if ((rc = sync_check(h))) return rc;
    return ok();
}

int dcrf_synchronize(dcrf_crf *h) {
    int rc = check_ready(h);
    if (rc) return rc;
    if ((rc = sync_check(h))) return rc;
    return ok();
}

int dcrf_info(dcrf_crf *h, int *N, int *M, int *n_terms) {
    if (!h) return set_err(DCRF_ERR_INVALID_ARG, "null handle");
    if (N) *N = h->N;
    if (M) *M = h->M;
    if (n_terms) *n_terms = (int)h->terms.size();
    return ok();
}

int dcrf_lattice_info(dcrf_crf *h, int term, int *d, int *L) {
    if (!h) return set_err(DCRF_ERR_INVALID_ARG, "null handle");
    if (term < 0 || term >= (int)h->terms.size()) return set_err(DCRF_ERR_INVALID_ARG, "no such term");
    if (d) *d = h->terms[term].d;
    if (L) *L = h->terms[term].lat.L;
    return ok();
}

int dcrf_lattice_dump(dcrf_crf *h, int term, int *offset, int *rank, float *bary, int *neighbors, int16_t *keys) {
    int rc = check_ready(h);
    if (rc) return rc;
    if (term < 0 || term >= (int)h->terms.size()) return set_err(DCRF_ERR_INVALID_ARG, "no such term");
    Term &T = h->terms[term];
    const int N = h->N, d1 = T.d + 1, L = T.lat.L;
    CU(cudaStreamSynchronize(h->stream));
    if (offset) {
        std::vector<int> o((size_t)d1 * N);
        CU(cudaMemcpy(o.data(), T.lat.off, o.size() * sizeof(int), cudaMemcpyDeviceToHost));
        for (int i = 0; i < N; i++)
            for (int r = 0; r < d1; r++) offset[(size_t)i * d1 + r] = o[(size_t)r * N + i];
    }
    if (rank) {
        std::vector<uint8_t> o((size_t)d1 * N);
        CU(cudaMemcpy(o.data(), T.lat.rank, o.size(), cudaMemcpyDeviceToHost));
        for (int i = 0; i < N; i++)
            for (int r = 0; r < d1; r++) rank[(size_t)i * d1 + r] = o[(size_t)r * N + i];
    }
    if (bary) {
        std::vector<float> o((size_t)d1 * N);
        CU(cudaMemcpy(o.data(), T.lat.bary, o.size() * sizeof(float), cudaMemcpyDeviceToHost));
        for (int i = 0; i < N; i++)
            for (int r = 0; r < d1; r++) bary[(size_t)i * d1 + r] = o[(size_t)r * N + i];
    }
    if (neighbors) {
        std::vector<int2> o((size_t)d1 * L);
        CU(cudaMemcpy(o.data(), T.lat.nbr, o.size() * sizeof(int2), cudaMemcpyDeviceToHost));
        for (size_t x = 0; x < o.size(); x++) {
            neighbors[2 * x] = o[x].x - 1;
            neighbors[2 * x + 1] = o[x].y - 1;
        }
    }
    if (keys) {
        std::vector<uint16_t> o((size_t)d1 * L);
        CU(cudaMemcpy(o.data(), T.lat.vkeys, o.size() * sizeof(uint16_t), cudaMemcpyDeviceToHost));
        for (int v = 0; v < L; v++)
            for (int q = 0; q < T.d; q++) keys[(size_t)v * T.d + q] = (int16_t)o[(size_t)v * d1 + q + 1];
    }
    return ok();
}

int dcrf_term_norm(dcrf_crf *h, int term, float *norm) {
    int rc = check_ready(h);
    if (rc) return rc;
    if (term < 0 || term >= (int)h->terms.size() || !norm) return set_err(DCRF_ERR_INVALID_ARG, "bad argument");
    Term &T = h->terms[term];
    if ((rc = store_mn(h, T.norm, norm, DCRF_LAYOUT_LM, DCRF_HOST, 1))) return rc;
    if ((rc = sync_check(h))) return rc;
    if (T.ntype == DCRF_NO_NORMALIZATION) {  // pairwise.cpp:46-53: every entry = N / sum(K*1), float sum
        float mean = 0.f;
        for (int i = 0; i < h->N; i++) mean += norm[i];
        mean = (float)h->N / mean;
        for (int i = 0; i < h->N; i++) norm[i] = mean;
    }
    return ok();
}

int dcrf_lattice_filter(dcrf_crf *h, int term, const float *in, int value_size, int reverse, float *out) {
    int rc = check_ready(h);
    if (rc) return rc;
    if (term < 0 || term >= (int)h->terms.size() || !in || !out) return set_err(DCRF_ERR_INVALID_ARG, "bad argument");
    if (value_size != 1 && value_size != h->M) return set_err(DCRF_ERR_INVALID_ARG, "value_size must be 1 or M");
    bool v1 = value_size == 1;
    if (!h->tmp) {  // the raw filter's slot rows, made at its first use
        const size_t rows = (size_t)h->nslots * h->MP;
        if ((rc = dev_alloc_async(&h->tmp, rows, h->stream))) return rc;
        CU(cudaMemsetAsync(h->tmp, 0, rows * sizeof(float), h->stream));
    }
    if ((rc = load_mn(h, in, DCRF_LAYOUT_LM, DCRF_HOST, h->tmp, value_size))) return rc;
    // the value-size-1 zero row (element MP) is row 1 of the full-width passes
    // that may have run since the build
    if (v1 && (rc = zero_sentinels(h, h->terms[term]))) return rc;
    std::vector<int> one{term};
    // splat, blur and slice are linear per label: more than 32 labels are
    // filtered label chunk by label chunk, each through its own lattice rows
    const int nc = v1 ? 1 : label_chunks(h->MP);
    for (int c = 0; c < nc; c++) {
        const int MPc = v1 ? 1 : chunk_width(h->MP, c);
        float *rows = h->tmp + (v1 ? 0 : chunk_base(h->nslots, c));
        PPArgs a = pp_args(h, PP_LOAD_Q | PP_SPLAT, one, reverse != 0, v1, c);
        a.ts.t[0].pre_norm = 0;
        a.ts.t[0].mem_w = h->terms[term].lat.mem_w;  // raw filter: no normalisation folded in
        a.Qin = rows;
        CU(pp(h, a, MPc));
        if ((rc = filter_phase(h, one, reverse != 0, v1, false, nullptr, nullptr, c))) return rc;
        a = pp_args(h, PP_FILTER, one, reverse != 0, v1, c);
        a.Qout = rows;
        CU(pp(h, a, MPc));
    }
    if (v1 && (rc = zero_sentinels(h, h->terms[term]))) return rc;
    if ((rc = store_mn(h, h->tmp, out, DCRF_LAYOUT_LM, DCRF_HOST, value_size))) return rc;
    if ((rc = sync_check(h))) return rc;
    return ok();
}

int dcrf_clear_pairwise(dcrf_crf *h) {
    int rc = check_handle(h);
    if (rc) return rc;
    for (Term &T : h->terms) free_term(h, T);
    h->terms.clear();
    h->tuned = false;
    h->version++;
    return ok();
}

int dcrf_launch_count(unsigned long long *count) {
    if (!count) return set_err(DCRF_ERR_INVALID_ARG, "null argument");
    *count = g_launches.load();
    return ok();
}

int dcrf_set_autotune(dcrf_crf *h, int on) {
    int rc = check_handle(h);
    if (rc) return rc;
    h->autotune = on != 0;
    return ok();
}

int dcrf_autotune(dcrf_crf *h) {
    int rc = check_ready(h);
    if (rc) return rc;
    if (h->terms.empty()) return set_err(DCRF_ERR_STATE, "autotune needs at least one pairwise term");
    if ((rc = autotune_now(h))) return rc;
    if ((rc = sync_check(h))) return rc;
    return ok();
}

int dcrf_get_tuning(dcrf_crf *h, int *split, int *smem_kb, int *task_len, float *hash_load, int *coop_blur) {
    int rc = check_handle(h);
    if (rc) return rc;
    if (coop_blur) *coop_blur = h->tune.coop;
    if (split) *split = pick_split(h, false, chunk_width(h->MP, 0));
    if (smem_kb) *smem_kb = h->tune.smem_kb > 0 ? h->tune.smem_kb : pointpass_smem_budget(h->MP) / 1024;
    if (task_len) *task_len = h->tune.task;
    if (hash_load) *hash_load = h->tune.hash_load;
    return ok();
}

int dcrf_set_tuning(dcrf_crf *h, int split, int smem_kb, int task_len, float hash_load, int coop_blur) {
    int rc = check_ready(h);
    if (rc) return rc;
    if (split < 0 || split > 2 || smem_kb < 0 || smem_kb > 224 || task_len < 1 || task_len > 63 ||
        !(hash_load >= 1.f) || coop_blur < 0 || coop_blur > 1)
        return set_err(DCRF_ERR_INVALID_ARG, "tuning values out of range");
    TuneCfg c;
    c.coop = coop_blur;
    c.split = split;
    c.smem_kb = smem_kb;
    c.task = task_len;
    c.hash_load = hash_load;
    if ((rc = apply_tuning(h, c))) return rc;
    if ((rc = sync_check(h))) return rc;
    return ok();
}

int dcrf_set_profiling(dcrf_crf *h, int on) {
    int rc = check_handle(h);
    if (rc) return rc;
    CU(cudaStreamSynchronize(h->stream));
    release_marks(h);
    h->profiling = on != 0;
    return ok();
}

int dcrf_profile(dcrf_crf *h, int kernel_class, double *total_ms, long long *launches) {
    int rc = check_ready(h);
    if (rc) return rc;
    if (kernel_class < 0 || kernel_class >= DCRF_NUM_KCLASSES) return set_err(DCRF_ERR_INVALID_ARG, "bad class");
    CU(cudaStreamSynchronize(h->stream));
    double ms = 0.0;
    long long n = 0;
    for (auto &m : h->marks)
        if (m.cls == kernel_class) {
            float t = 0.f;
            CU(cudaEventElapsedTime(&t, m.a, m.b));
            ms += t;
            n++;
        }
    if (total_ms) *total_ms = ms;
    if (launches) *launches = n;
    return ok();
}

int dcrf_term_stats(dcrf_crf *h, int term, int *L, int *P, int *ntiles) {
    if (!h) return set_err(DCRF_ERR_INVALID_ARG, "null handle");
    if (term < 0 || term >= (int)h->terms.size()) return set_err(DCRF_ERR_INVALID_ARG, "no such term");
    if (L) *L = h->terms[term].lat.L;
    if (P) *P = h->terms[term].lat.P;
    if (ntiles) *ntiles = h->terms[term].lat.ntiles;
    return ok();
}

int dcrf_term_buffer(dcrf_crf *h, int term, int which, float *out, size_t count) {
    int rc = check_ready(h);
    if (rc) return rc;
    if (term < 0 || term >= (int)h->terms.size() || !out || which < 0 || which > 2)
        return set_err(DCRF_ERR_INVALID_ARG, "bad argument");
    Term &T = h->terms[term];
    size_t avail = which < 2 ? ((size_t)T.lat.L + 1) * h->MP : (size_t)std::max(T.lat.P, 1) * h->MP;
    if (count > avail) return set_err(DCRF_ERR_INVALID_ARG, "count exceeds the buffer");
    const float *src = which == 0 ? T.V[0] : which == 1 ? T.V[1] : T.pv;
    CU(cudaStreamSynchronize(h->stream));
    CU(cudaMemcpy(out, src, count * sizeof(float), cudaMemcpyDeviceToHost));
    return ok();
}

int dcrf_set_compat(dcrf_crf *h, int term, int compat_kind, const float *compat) {
    int rc = check_handle(h);
    if (rc) return rc;
    if (term < 0 || term >= (int)h->terms.size()) return set_err(DCRF_ERR_INVALID_ARG, "no such term");
    if ((rc = validate_compat(compat_kind, compat))) return rc;
    if (compat_kind != h->terms[term].ckind) h->tuned = false;
    if ((rc = set_term_compat(h, h->terms[term], compat_kind, compat))) return rc;
    h->version++;
    if ((rc = sync_check(h))) return rc;
    return ok();
}

int dcrf_set_kernel_params(dcrf_crf *h, int term, const float *params) {
    int rc = check_ready(h);
    if (rc) return rc;
    if (term < 0 || term >= (int)h->terms.size() || !params) return set_err(DCRF_ERR_INVALID_ARG, "bad argument");
    Term &T = h->terms[term];
    if (T.ktype == DCRF_CONST_KERNEL) return ok();  // no parameters (pairwise.cpp:140-151)
    T.params.assign(params, params + kernel_count(T));
    T.params_set = true;
    if ((rc = build_term(h, term))) return rc;
    return ok();
}

int dcrf_param_counts(dcrf_crf *h, int term, int *n_compat, int *n_kernel) {
    if (!h) return set_err(DCRF_ERR_INVALID_ARG, "null handle");
    if (term < 0 || term >= (int)h->terms.size()) return set_err(DCRF_ERR_INVALID_ARG, "no such term");
    if (n_compat) *n_compat = compat_count(h, h->terms[term]);
    if (n_kernel) *n_kernel = kernel_count(h->terms[term]);
    return ok();
}

int dcrf_set_checkpoint_interval(dcrf_crf *h, int every) {
    int rc = check_handle(h);
    if (rc) return rc;
    if (every < 1) return set_err(DCRF_ERR_INVALID_ARG, "the checkpoint interval must be at least 1");
    h->ckpt_every = every;
    return ok();
}

int dcrf_inference_checkpointed(dcrf_crf *h, int n_iterations, float *Q, int layout, int where) {
    int rc = check_ready(h);
    if (rc) return rc;
    if (is_wide(h)) return wide_unsupported("the adjoint (dcrf_inference_checkpointed / dcrf_backward)");
    if (!Q || n_iterations < 0) return set_err(DCRF_ERR_INVALID_ARG, "bad argument");
    const int every = std::max(1, std::min(h->ckpt_every, std::max(1, n_iterations)));
    const size_t qsz = (size_t)h->MP * h->nslots;
    // stored iterates: all of them, or Q_0, Q_k, ... and Q_T; the steps kept
    // (splats, blurred lattices, sliced values): all, or one segment's
    const size_t nstore = every > 1 ? (size_t)n_iterations / every + 2 : (size_t)n_iterations + 1;
    const size_t kept = every > 1 ? (size_t)every : (size_t)n_iterations;
    const size_t need = qsz * nstore;
    if (every > 1 && qsz * (kept + 1) > h->segq_cap) {
        dev_free_async(h->segq, h->stream);
        h->segq = nullptr;
        h->segq_cap = 0;
        if ((rc = dev_alloc_async(&h->segq, qsz * (kept + 1), h->stream))) return rc;
        h->segq_cap = qsz * (kept + 1);
    }
    if (need > h->ckpt_cap) {
        dev_free_async(h->ckpt, h->stream);
        h->ckpt = nullptr;
        h->ckpt_cap = 0;
        if ((rc = dev_alloc_async(&h->ckpt, need, h->stream))) return rc;
        h->ckpt_cap = need;
    }
    // the forward's splat S and blurred lattice B of every iterate, per term
    h->ckv_off.assign(h->terms.size(), 0);
    size_t per_it = 0;
    for (size_t k = 0; k < h->terms.size(); k++) {
        h->ckv_off[k] = per_it;
        per_it += 2 * ((size_t)h->terms[k].lat.L + 1) * h->MP;
    }
    const size_t vneed = std::max<size_t>(per_it * kept, 1);
    bool fresh = per_it != h->ckv_iter;
    h->ckv_iter = per_it;
    if (vneed > h->ckv_cap) {
        dev_free_async(h->ckv, h->stream);
        h->ckv = nullptr;
        h->ckv_cap = 0;
        if ((rc = dev_alloc_async(&h->ckv, vneed, h->stream))) return rc;
        h->ckv_cap = vneed;
        fresh = true;
    }
    // row 0 of every S and B is the zero sentinel and is never written afterwards
    // y checkpoints of the terms whose kernel gradient needs them
    h->cky_off.assign(h->terms.size(), -1);
    size_t ny = 0;
    for (size_t k = 0; k < h->terms.size(); k++) {
        const Term &Tk = h->terms[k];
        if (Tk.ktype != DCRF_CONST_KERNEL &&
            (Tk.ntype == DCRF_NORMALIZE_SYMMETRIC || Tk.ntype == DCRF_NORMALIZE_AFTER)) {
            h->cky_off[k] = (long long)ny;
            ny += qsz * kept;
        }
    }
    if (ny > h->cky_cap) {
        dev_free_async(h->cky, h->stream);
        h->cky = nullptr;
        h->cky_cap = 0;
        if ((rc = dev_alloc_async(&h->cky, ny, h->stream))) return rc;
        h->cky_cap = ny;
    }
    if (ny == 0) h->cky_off.assign(h->terms.size(), -1);
    std::vector<size_t> sig = h->ckv_off;
    for (const Term &Tk : h->terms) sig.push_back((size_t)Tk.lat.L);
    if (fresh || h->ckv_layout != sig) CU(cudaMemsetAsync(h->ckv, 0, sizeof(float) * vneed, h->stream));
    h->ckv_layout = sig;
    const float *qT;
    if (every == 1) {
        if ((rc = run_inference(h, n_iterations, 0, h->ckpt))) return rc;
        qT = h->ckpt + (size_t)n_iterations * qsz;
    } else {  // segments of `every` iterations, each stored iterate the start of the next
        if ((rc = maybe_autotune(h)) || (rc = flush_norms(h))) return rc;
        float *last = h->ckpt + (nstore - 1) * qsz;
        if ((rc = issue_steps(h, nullptr, 0, nullptr, nullptr, nullptr, h->ckpt))) return rc;
        for (int j = 0, t0 = 0; t0 < n_iterations; j++, t0 += every) {
            const int n = std::min(every, n_iterations - t0);
            float *dst = t0 + n == n_iterations ? last : h->ckpt + (size_t)(j + 1) * qsz;
            if ((rc = issue_steps(h, h->ckpt + (size_t)j * qsz, n, nullptr, nullptr, nullptr, dst))) return rc;
        }
        if (n_iterations == 0)
            CU(cudaMemcpyAsync(last, h->ckpt, qsz * sizeof(float), cudaMemcpyDeviceToDevice, h->stream));
        qT = last;
    }
    if ((rc = store_mn(h, qT, Q, layout, where))) return rc;
    if ((rc = sync_check(h))) return rc;
    h->ckpt_T = n_iterations;
    h->ckpt_every_used = every;
    h->ckpt_version = h->version;
    return ok();
}

int dcrf_backward(dcrf_crf *h, const float *dQ, int layout, int where, float *dU, double *dcompat, double *dkernel) {
    int rc = check_ready(h);
    if (rc) return rc;
    if (is_wide(h)) return wide_unsupported("the adjoint (dcrf_inference_checkpointed / dcrf_backward)");
    if (!dQ) return set_err(DCRF_ERR_INVALID_ARG, "null gradient");
    if (h->ckpt_T < 0 || h->ckpt_version != h->version)
        return set_err(DCRF_ERR_STATE, "dcrf_backward needs a dcrf_inference_checkpointed of the current model");
    const int M = h->M, ns = h->nslots, T = h->ckpt_T, nt = (int)h->terms.size();
    const size_t qsz = (size_t)h->MP * ns;
    const bool want_compat = dcompat != nullptr, want_kernel = dkernel != nullptr;
    for (float *&b : h->bw)
        if (!b && (rc = dev_alloc_async(&b, qsz, h->stream))) return rc;
    for (float *&b : h->bw1)
        if (!b && (rc = dev_alloc_async(&b, (size_t)ns, h->stream))) return rc;
    if (!h->ckv || h->ckv_off.size() != h->terms.size())
        return set_err(DCRF_ERR_STATE, "dcrf_backward needs a dcrf_inference_checkpointed of the current model");
    // reduction space: per term compat (M or M*M) and kernel (d*d) accumulators
    std::vector<size_t> coff(nt), koff(nt);
    size_t nacc = 0;
    int maxd = 1;
    for (int k = 0; k < nt; k++) {
        const Term &Tk = h->terms[k];
        coff[k] = nacc;
        nacc += Tk.ckind == DCRF_COMPAT_MATRIX ? (size_t)M * M : (size_t)M;
        koff[k] = nacc;
        nacc += (size_t)Tk.d * Tk.d;
        maxd = std::max(maxd, Tk.d);
    }
    // label products: one partial block per term, added up over the iterations
    // and reduced once at the end
    const size_t lpb = std::max((size_t)label_products_blocks(ns), (size_t)h->ntiles);
    std::vector<size_t> lpoff(nt);
    size_t nlp = 0;
    for (int k = 0; k < nt; k++) {
        lpoff[k] = nlp;
        nlp += lpb * (h->terms[k].ckind == DCRF_COMPAT_MATRIX ? (size_t)M * M : (size_t)M);
    }
    const size_t npart = std::max(want_compat ? nlp : 0, (size_t)kernel_param_blocks(h->N) * maxd * maxd);
    if (npart > h->dpart_cap) {
        dev_free_async(h->dpart, h->stream);
        h->dpart = nullptr;
        if ((rc = dev_alloc_async(&h->dpart, npart, h->stream))) return rc;
        h->dpart_cap = npart;
    }
    if (nacc + 1 > h->dacc_cap) {
        dev_free_async(h->dacc, h->stream);
        h->dacc = nullptr;
        if ((rc = dev_alloc_async(&h->dacc, nacc + 1, h->stream))) return rc;
        h->dacc_cap = nacc + 1;
    }
    CU(cudaMemsetAsync(h->dacc, 0, sizeof(double) * (nacc + 1), h->stream));
    if (want_kernel)
        for (Term &Tk : h->terms)
            if (Tk.ktype != DCRF_CONST_KERNEL) {
                if (!Tk.df && (rc = dev_alloc_async(&Tk.df, (size_t)h->N * Tk.d, h->stream))) return rc;
                CU(cudaMemsetAsync(Tk.df, 0, sizeof(float) * (size_t)h->N * Tk.d, h->stream));
            }
    // slot-row work buffers
    float *b = h->bw[0], *g = h->bw[1], *du = h->bw[2], *xn = h->bw[3], *Fn = h->bw[5],
          *y = h->bw[6], *cq = h->bw[8], *yn = h->bw[9], *fb = h->bw[10], *c1 = h->bw[11];
    float *x1 = h->bw1[0], *ones1 = h->bw1[1];
    CU(launch_fill(ones1, 1.f, 1, ns, h->slot_pt, h->stream));
    for (int k = 0; k < nt; k++) {
        Term &Tk = h->terms[k];
        if ((rc = ensure_adjoint_bufs(h, Tk))) return rc;
        // R1: the reverse-blurred splat of ones (fixed per lattice), for the
        // normalisation's dependence on the features
        if (want_kernel && Tk.ktype != DCRF_CONST_KERNEL && Tk.ntype != DCRF_NO_NORMALIZATION && !Tk.r1_valid) {
            if ((rc = splat_into(h, k, ones1, Tk.b1[0], true))) return rc;
            if ((rc = blur_into(h, k, Tk.b1[0], Tk.b1[2], true, true))) return rc;
            Tk.r1_valid = true;
        }
    }
    // seed: b = -dL/dA_T from dL/dQ_T (densecrf.cpp:256-258)
    if ((rc = load_mn(h, dQ, layout, where, g))) return rc;
    const int every = h->ckpt_every_used;
    const float *qT = every > 1 ? h->ckpt + ((size_t)T / every + 1) * qsz : h->ckpt + (size_t)T * qsz;
    CU(launch_softmax_adjoint(qT, g, b, nullptr, M, ns, h->slot_pt, h->stream));
    CU(cudaMemcpyAsync(du, b, qsz * sizeof(float), cudaMemcpyDeviceToDevice, h->stream));
    // rows of 4k labels: the per-point work of an iteration in one tile pass
    // (launch_adjoint_tile), the next b into a second buffer
    const bool fused = h->MP % 4 == 0;
    float *bnext = h->bw[12];
    if (fused) {
        for (auto *v : {&h->adjF, &h->adjY})
            if (v->size() < (size_t)nt) v->resize(nt, nullptr);
        for (int k = 0; k < nt; k++) {
            if (!want_kernel || h->terms[k].ktype == DCRF_CONST_KERNEL) continue;
            if (!h->adjF[k] && (rc = dev_alloc_async(&h->adjF[k], qsz, h->stream))) return rc;
            if (!h->adjY[k] && !(h->cky && h->cky_off[k] >= 0) && (rc = dev_alloc_async(&h->adjY[k], qsz, h->stream)))
                return rc;
        }
    }
    // iterations in segments: all at once, or (interval k) the k-step segments
    // from the last, each recomputed from its stored first iterate
    int t0 = T, seg_end = T;
    const float *segQ = h->ckpt;
    for (int it = T - 1; it >= 0; it--) {
        if (it < t0) {
            seg_end = it + 1;
            t0 = every > 1 ? (it / every) * every : 0;
            if (every > 1) {
                if ((rc = issue_steps(h, h->ckpt + (size_t)(t0 / every) * qsz, seg_end - t0, h->segq, h->ckv, h->cky,
                                      nullptr)))
                    return rc;
                segQ = h->segq;
            }
        }
        const int rel = it - t0;  // the step within the segment's stored data
        const float *Qt = segQ + (size_t)rel * qsz;
        if (!fused) CU(cudaMemsetAsync(g, 0, qsz * sizeof(float), h->stream));
        // x~ = b with the transpose's first normalisation (per term)
        auto xtilde = [&](Term &Tk) -> const float * {
            if (!tr_pre(Tk)) return b;
            if (launch_scale_norm(b, xn, Tk.norm, M, ns, 1, h->stream) != cudaSuccess) return nullptr;
            return xn;
        };
        // phase 1, per term: S_b = splat of x~; for kernel gradients also C S_t.
        // Then all blur chains of all terms advance together: A = K_raw^T
        // (reverse) of S_b, B = forward blur of S_b, C = reverse blur of C S_t.
        std::vector<Chain> chains;
        {  // S_b = splat of x~ = norm .* b when the transpose starts normalised (the
           // norm in the weights), all terms in one pass
            std::vector<int> ks(nt);
            std::vector<float *> Ss(nt);
            std::vector<bool> pre(nt);
            for (int k = 0; k < nt; k++) {
                ks[k] = k;
                Ss[k] = h->terms[k].bv[0];
                pre[k] = tr_pre(h->terms[k]);
            }
            if ((rc = splat_terms_into(h, ks, b, Ss, pre))) return rc;
        }
        for (int k = 0; k < nt; k++) {
            Term &Tk = h->terms[k];
            const size_t rows = (size_t)Tk.lat.L + 1;
            const float *St = h->ckv + (size_t)rel * h->ckv_iter + h->ckv_off[k];  // forward splat of Q_t
            const bool kgrad = want_kernel && Tk.ktype != DCRF_CONST_KERNEL;
            chains.push_back(Chain{k, Tk.bv[0], {Tk.V[1], Tk.V[0]}, Tk.bv[1], true});
            if (kgrad) {
                CU(launch_compat(St, Tk.bv[2], M, (int)rows, Tk.ckind, Tk.potts_w, Tk.compat, 0, 0, h->stream));
                chains.push_back(Chain{k, Tk.bv[0], {Tk.bv[3], Tk.bv[4]}, Tk.bv[5], false});
                chains.push_back(Chain{k, Tk.bv[2], {Tk.bv[6], Tk.bv[7]}, Tk.bv[8], true});
            }
        }
        if ((rc = blur_chains(h, chains, false))) return rc;
        // phase 2: per term F = K_raw^T x~ and Fp = K^T b = [norm .*] F, g += C^T Fp
        // (applyTranspose, pairwise.cpp:179-183; the compatibilities are
        // symmetric), the compatibility gradients sum b (K Q_t)^T = sum (K^T b)
        // Q_t^T (PairwisePotential::gradient, pairwise.cpp:190-195), then the
        // next b from g; then the kernel gradients of the terms that have them
        auto need_F_of = [&](const Term &Tk) {
            return want_kernel && Tk.ktype != DCRF_CONST_KERNEL &&
                   (Tk.ntype == DCRF_NORMALIZE_SYMMETRIC || Tk.ntype == DCRF_NORMALIZE_BEFORE);
        };
        // y = K_raw [norm] Q_t of each term with kernel gradients (SYMMETRIC,
        // AFTER): kept by the forward, else sliced from its blurred lattice
        std::vector<const float *> yk(nt, nullptr);
        for (int k = 0; k < nt; k++) {
            Term &Tk = h->terms[k];
            const bool kgrad = want_kernel && Tk.ktype != DCRF_CONST_KERNEL;
            if (!kgrad || !(Tk.ntype == DCRF_NORMALIZE_SYMMETRIC || Tk.ntype == DCRF_NORMALIZE_AFTER)) continue;
            if (h->cky && h->cky_off[k] >= 0) {
                yk[k] = h->cky + h->cky_off[k] + (size_t)rel * qsz;
            } else {
                float *yb = fused ? h->adjY[k] : h->bw[6];
                const float *Bt = h->ckv + (size_t)rel * h->ckv_iter + h->ckv_off[k] + ((size_t)Tk.lat.L + 1) * h->MP;
                if ((rc = slice_from(h, k, Bt, yb, false))) return rc;
                yk[k] = yb;
            }
        }
        if (fused) {
            AdjArgs aa{};
            aa.N = h->N;
            aa.M = M;
            aa.nslots = ns;
            aa.ntiles = h->ntiles;
            aa.slot_pt = h->slot_pt;
            aa.Qt = Qt;
            aa.b_next = bnext;
            aa.du = du;
            aa.lp_accum = it < T - 1 ? 1 : 0;
            aa.n = nt;
            aa.ts.n = nt;
            for (int k = 0; k < nt; k++) {
                Term &Tk = h->terms[k];
                aa.ts.t[k] = term_dev(h, Tk, true, false);
                aa.a[k].A = Tk.bv[1];
                aa.a[k].post = tr_post(Tk) ? 1 : 0;
                aa.a[k].Fraw = need_F_of(Tk) ? h->adjF[k] : nullptr;
                aa.a[k].lp = want_compat ? h->dpart + lpoff[k] : nullptr;
                aa.a[k].lp_mode = Tk.ckind == DCRF_COMPAT_MATRIX ? 1 : 0;
            }
            ProfScope ps(h, DCRF_KCLASS_OTHER);
            CU(launch_adjoint_tile(aa, h->MP, h->stream));
        }
        for (int k = 0; k < nt; k++) {
            Term &Tk = h->terms[k];
            const size_t rows = (size_t)Tk.lat.L + 1;
            const float *St = h->ckv + (size_t)rel * h->ckv_iter + h->ckv_off[k];
            const float *Bt = St + rows * h->MP;  // the forward's blurred lattice of Q_t
            const bool kgrad = want_kernel && Tk.ktype != DCRF_CONST_KERNEL;
            const bool need_F = need_F_of(Tk);
            float *F = fused && need_F ? h->adjF[k] : h->bw[4];
            if (!fused) {
                if ((rc = slice_from(h, k, Tk.bv[1], need_F ? F : nullptr, false, tr_post(Tk),
                                     want_compat ? Fn : nullptr, g)))
                    return rc;
                if (want_compat)
                    CU(launch_label_products_part(Fn, Qt, M, ns, h->slot_pt, Tk.ckind == DCRF_COMPAT_MATRIX ? 1 : 0,
                                                  h->dpart + lpoff[k], it < T - 1 ? 1 : 0, h->stream));
            }
            if (!kgrad) continue;
            // kernelGradient (pairwise.cpp:202-207) through featureGradient (87-114)
            // y = K_raw [norm] Q_t: kept by the forward, else sliced from its blurred lattice
            const float *yt = yk[k] ? yk[k] : y;
            if (fused) {
                // y~ = [norm] C Q_t and the normalisation's coefficients in one pass
                CU(launch_norm_terms(b, yt, F, Qt, Tk.norm, M, ns, Tk.ntype, Tk.ckind, Tk.potts_w, Tk.compat, yn, x1,
                                     h->stream));
                // d/df x~^T K_raw y~: the forward-blurred S_b against y~ plus the
                // reverse-blurred splat of y~ (= C S_t) against x~, in one pass
                // the normalisation's terms first: - d/df c1^T K_raw 1, the forward-
                // blurred splat of c1 (one value per point) against ones and the
                // reverse-blurred splat of ones against c1
                const bool nrm = Tk.ntype != DCRF_NO_NORMALIZATION;
                if (nrm) {
                    if ((rc = splat_into(h, k, x1, Tk.b1[0], true))) return rc;
                    if ((rc = blur_into(h, k, Tk.b1[0], Tk.b1[1], false, true))) return rc;
                }
                // then all four slice-gradient pairs in one pass (x~ = norm .* b when the
                // transpose starts normalised: the norm is applied to b as the pass reads it)
                if ((rc = slice_grad_into(h, k, Tk.bv[5], yn, 1.f, false, Tk.bv[8], b, 1.f,
                                          tr_pre(Tk) ? Tk.norm : nullptr, nrm ? Tk.b1[1] : nullptr,
                                          nrm ? Tk.b1[2] : nullptr, x1, -1.f)))
                    return rc;
                continue;
            }
            const float *xs = xtilde(Tk);
            if (!xs) return set_err(DCRF_ERR_CUDA, "scale launch failed");
            const float *y_ = yt;
            CU(launch_compat(Qt, cq, M, ns, Tk.ckind, Tk.potts_w, Tk.compat, 0, 0, h->stream));
            const float *ys = cq;  // y~ = C Q_t with the forward's first normalisation
            if (fwd_pre(Tk)) {
                CU(launch_scale_norm(cq, yn, Tk.norm, M, ns, 1, h->stream));
                ys = yn;
            }
            if ((rc = slice_grad_into(h, k, Tk.bv[5], ys, 1.f, false, Tk.bv[8], xs, 1.f))) return rc;
            if (Tk.ntype != DCRF_NO_NORMALIZATION) {
                // - d/df c1^T K_raw 1 with c1 the normalisation's coefficients; the
                // contraction with ones reduces to one value per point
                if (Tk.ntype == DCRF_NORMALIZE_SYMMETRIC) {
                    CU(launch_compat(y_, fb, M, ns, Tk.ckind, Tk.potts_w, Tk.compat, 0, 0, h->stream));
                    CU(launch_prod(b, fb, F, cq, 0.5f, Tk.norm, 3, c1, M, ns, h->stream));
                } else if (Tk.ntype == DCRF_NORMALIZE_AFTER) {
                    CU(launch_compat(y_, fb, M, ns, Tk.ckind, Tk.potts_w, Tk.compat, 0, 0, h->stream));
                    CU(launch_prod(b, fb, nullptr, nullptr, 1.f, Tk.norm, 2, c1, M, ns, h->stream));
                } else {
                    CU(launch_prod(F, cq, nullptr, nullptr, 1.f, Tk.norm, 2, c1, M, ns, h->stream));
                }
                CU(launch_row_sum(c1, x1, M, ns, h->stream));
                if ((rc = splat_into(h, k, x1, Tk.b1[0], true))) return rc;
                if ((rc = blur_into(h, k, Tk.b1[0], Tk.b1[1], false, true))) return rc;
                if ((rc = slice_grad_into(h, k, Tk.b1[1], ones1, -1.f, true, Tk.b1[2], x1, -1.f))) return rc;
            }
        }
        // b = -dL/dA_t (densecrf.cpp:290)
        if (fused)
            std::swap(b, bnext);
        else
            CU(launch_softmax_adjoint(Qt, g, b, du, M, ns, h->slot_pt, h->stream));
    }
    if (want_compat && T > 0)
        for (int k = 0; k < nt; k++) {
            const int K = h->terms[k].ckind == DCRF_COMPAT_MATRIX ? M * M : M;
            // the fused pass leaves one partial per tile, the separate products one per LP block
            CU(launch_sum_parts_bm(h->dpart + lpoff[k], fused ? h->ntiles : (int)lpb, K, h->dacc + coff[k], 0,
                                   h->stream));
        }
    if (dU && (rc = store_mn(h, du, dU, layout, where))) return rc;
    h->du_version = h->version;
    if (want_kernel)
        for (int k = 0; k < nt; k++) {
            Term &Tk = h->terms[k];
            if (Tk.ktype == DCRF_CONST_KERNEL) continue;
            CU(launch_kernel_param_grad(Tk.feat, Tk.df, Tk.d, h->N, Tk.ktype == DCRF_FULL_KERNEL, h->dpart,
                                        h->dacc + koff[k], 0, h->stream));
        }
    std::vector<double> acc(nacc + 1);
    CU(cudaMemcpyAsync(acc.data(), h->dacc, sizeof(double) * (nacc + 1), cudaMemcpyDeviceToHost, h->stream));
    if ((rc = sync_check(h))) return rc;
    size_t oc = 0, ok_ = 0;
    for (int k = 0; k < nt; k++) {
        const Term &Tk = h->terms[k];
        if (dcompat) {
            if (Tk.ckind == DCRF_COMPAT_POTTS) {  // m = -w KQ: dL/dw = -sum b.*KQ (labelcompatibility.cpp:57-61)
                double sacc = 0.0;
                for (int m = 0; m < M; m++) sacc += acc[coff[k] + m];
                dcompat[oc] = -sacc;
            } else {
                const int n = compat_count(h, Tk);
                for (int x = 0; x < n; x++) dcompat[oc + x] = acc[coff[k] + x];
            }
        }
        oc += compat_count(h, Tk);
        if (dkernel) {
            const int n = kernel_count(Tk);
            for (int x = 0; x < n; x++) dkernel[ok_ + x] = acc[koff[k] + x];
        }
        ok_ += kernel_count(Tk);
    }
    return ok();
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Allocation-free raw filter: scratch in one static device array per GPU.
// ---------------------------------------------------------------------------
namespace {

// Scratch of dcrf_lattice_filter_noalloc.  Every GPU that loads the library
// holds these DCRF_NOALLOC_MAX_FLOATS floats until the process exits.
static __device__ __align__(256) float g_noalloc_scratch[DCRF_NOALLOC_MAX_FLOATS];

std::mutex g_noalloc_mu;
float *g_noalloc_ptr[256] = {};

// Device address of the scratch array on `device`, resolved once with that
// device current.  (In host code the array's name is only a host-side stand-in,
// never a device address.)
int noalloc_scratch(int device, float **out) {
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (device < 0 || device >= 256) return set_err(DCRF_ERR_INVALID_ARG, "device ordinal out of range");
    if (!g_noalloc_ptr[device]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p)
            return set_err(DCRF_ERR_CUDA, std::string("cudaGetSymbolAddress of the scratch array: ") +
                                              cudaGetErrorString(e));
        g_noalloc_ptr[device] = static_cast<float *>(p);
    }
    *out = g_noalloc_ptr[device];
    return DCRF_OK;
}

size_t pad64(size_t n) { return (n + 63) & ~(size_t)63; }

}  // namespace

extern "C" int dcrf_lattice_filter_noalloc(dcrf_crf *h, int term, const float *in, int value_size, int reverse,
                                           float *out, void *stream) {
    int rc = check_ready(h);
    if (rc) return rc;
    if (term < 0 || term >= (int)h->terms.size() || !in || !out) return set_err(DCRF_ERR_INVALID_ARG, "bad argument");
    if (value_size != 1 && value_size != h->M) return set_err(DCRF_ERR_INVALID_ARG, "value_size must be 1 or M");
    const bool v1 = value_size == 1;
    // the scratch holds one label chunk (at most 32 labels) at a time; more
    // labels are filtered chunk by chunk through the same scratch
    const int MPv = v1 ? 1 : chunk_width(h->MP, 0);
    Term &T = h->terms[term];
    const size_t n_in = pad64((size_t)MPv * h->nslots);
    const size_t n_pv = pad64(((size_t)T.lat.P + 1) * MPv);
    const size_t n_v = pad64(((size_t)T.lat.L + 1) * MPv);
    const size_t need = n_in + n_pv + 2 * n_v;
    if (need > (size_t)DCRF_NOALLOC_MAX_FLOATS)
        return set_err(DCRF_ERR_INVALID_ARG, "this filter needs " + std::to_string(need) +
                                                 " floats of scratch; the allocation-free entry point has " +
                                                 std::to_string((size_t)DCRF_NOALLOC_MAX_FLOATS));
    float *scr = nullptr;
    if ((rc = noalloc_scratch(h->device, &scr))) return rc;
    float *in_s = scr, *pv = in_s + n_in, *V0 = pv + n_pv, *V1 = V0 + n_v;
    float *Vb[2] = {V0, V1};
    cudaStream_t s = (cudaStream_t)stream;
    // The term's tables may still be in flight on the handle's stream (a build
    // returns before its last kernels finish): `s` starts after them.  On the
    // way out the handle's stream waits for this call's kernels, so that a later
    // rebuild, clear or destroy does not free tables they still read.
    CU(cudaEventRecord(h->xorder, h->stream));
    CU(cudaStreamWaitEvent(s, h->xorder, 0));
    // the array keeps the previous call's contents: the zero sentinel rows are restored
    CU(cudaMemsetAsync(V0, 0, sizeof(float) * MPv, s));
    CU(cudaMemsetAsync(V1, 0, sizeof(float) * MPv, s));
    std::vector<int> one{term};
    const bool seq = v1 || h->M <= 2 || T.variant == DCRF_VARIANT_SCALAR;
    const int nseg = (int)h->seg.size() - 1, nc = v1 ? 1 : label_chunks(h->MP);
    for (int c = 0; c < nc; c++) {
        // labels [m0, m0 + mc) of the caller's rows, in slot rows of w floats
        const int w = v1 ? 1 : chunk_width(h->MP, c), m0 = DCRF_LCHUNK * c, mc = std::min(w, value_size - m0);
        CU(launch_to_slots(in, 0, mc, value_size, m0, w, h->N, h->d_seg, nseg, h->slot_pt, h->nslots, in_s, s));
        PPArgs a = pp_args(h, PP_LOAD_Q | PP_SPLAT, one, reverse != 0, v1, c);
        a.ts.t[0].pre_norm = 0;
        a.ts.t[0].mem_w = T.lat.mem_w;
        a.ts.t[0].pv = pv;
        a.ts.t[0].pout = pv;  // splat-only pass: the scratch takes the vertex-grouped partials
        a.Qin = in_s;
        CU(launch_pointpass(a, w, s));
        ReduceArgs ra{};
        ra.n = 1;
        ra.t[0] = {T.lat.red_beg, pv, V0, T.lat.L, T.lat.P};
        CU(launch_reduce(ra, w, s));
        const int NV = w % 4 == 0 ? w / 4 : w % 2 == 0 ? w / 2 : w;
        for (int pass = 0; pass <= T.d; pass++) {
            BlurArgs ba{};
            ba.n = 1;
            ba.begin[0] = 0;
            ba.begin[1] = (long long)T.lat.L * NV;
            ba.t[0].Vin = Vb[pass & 1];
            ba.t[0].Vout = Vb[(pass + 1) & 1];
            ba.t[0].nbr = T.lat.nbr;
            ba.t[0].L = T.lat.L;
            ba.t[0].axis = reverse ? T.d - pass : pass;
            ba.t[0].axis2 = -1;
            ba.t[0].pv = nullptr;
            CU(launch_blur(ba, w, seq, s));
        }
        PPArgs f = pp_args(h, PP_FILTER, one, reverse != 0, v1, c);
        f.ts.t[0].V = Vb[(T.d + 1) & 1];
        f.Qout = in_s;
        CU(launch_pointpass(f, w, s));
        CU(launch_from_slots(in_s, mc, value_size, m0, w, h->N, h->d_seg, nseg, h->slot_pt, h->nslots, h->pt_slot, 0, out,
                             s));
    }
    CU(cudaEventRecord(h->xorder, s));
    CU(cudaStreamWaitEvent(h->stream, h->xorder, 0));
    return ok();
}
