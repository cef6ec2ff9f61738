// lattice.cuh -- device permutohedral lattice of one pairwise term (or of one
// term over a batch of images: every table below is then the concatenation of
// the images' tables, and vertex ids are global).
#pragma once
#include <vector>

#include "dcrf_common.cuh"

namespace dcrf {

constexpr int SPLAT_TILE = 256;  // points per tile of the in-kernel splat
// default members per splat task (load balance of the in-kernel splat against
// per-task overhead: 24 measured best with 32, 2-4 us ahead of 8-16 per point
// pass at 640x480 with 21 labels)
constexpr int SPLAT_TASK = 24;

struct LatticeDev {
    int d = 0, N = 0, L = 0, P = 0, ntiles = 0, variant = 0;
    float alpha = 0.f;
    int *off = nullptr;          // [d+1][N]
    float *bary = nullptr;       // [d+1][N]
    float *wslice = nullptr;     // [d+1][N]
    uint8_t *rank = nullptr;     // [d+1][N]
    int2 *nbr = nullptr;         // [d+1][L]
    uint16_t *vkeys = nullptr;   // [L][d+1]: field 0 = image, 1..d = coordinates
    int max_np = 0;              // largest number of partials of one tile
    int *part_v = nullptr;       // [P] vertex of partial p
    int *part_mend = nullptr;    // [P+8] end of partial p's members, relative to its tile's member block
    int *tile_pbeg = nullptr;    // [ntiles+1] partial range of tile t
    uint16_t *mem_pt = nullptr;  // [ntiles][SPLAT_TILE*(d+1)] tile-local point of each member
    float *mem_w = nullptr;      // [ntiles][SPLAT_TILE*(d+1)] splat weight of each member
    // splat tasks: runs of at most SPLAT_TASK members of one partial, in partial order;
    // task = (local partial << 19) | (first member << 6) | length
    int max_nt = 0;               // largest number of tasks of one tile
    uint32_t *task = nullptr;     // [T+8]
    uint32_t *tsched = nullptr;   // [T+8] per tile, its task indices by descending length (the
                                  // order the point pass deals tasks to its lane groups)
    int *tile_tbeg = nullptr;     // [ntiles+1] task range of tile t
    int *red_beg = nullptr;      // [L+1]
    int *red_list = nullptr;     // [P] partials grouped by vertex (each vertex's in tile order)
    int *ppos = nullptr;         // [P+1] position of partial p in red_list (its inverse): the row
                                 // of p in the vertex-grouped splat output that the reduce reads
    // tile-ordered slice tables: corner r of slot li of tile t at (t*(d+1)+r)*SPLAT_TILE+li
    uint16_t *tl_loc = nullptr;  // index of the corner's vertex among the tile's partials
    float *tl_w = nullptr;       // the corner's barycentric weight
    // value buffers of the mean-field passes, carved from the lattice's memory
    // (sizes from the build's MP and slot count): V0, V1 [L+1][MP] in label
    // chunks (sentinel rows zeroed, see launch_lattice_zero_rows), pv and pout
    // [P+1][MP], norm [nslots], mem_wn [ntiles][SPLAT_TILE*(d+1)]
    float *V0 = nullptr, *V1 = nullptr, *pv = nullptr, *pout = nullptr, *norm = nullptr, *mem_wn = nullptr;
    size_t bytes = 0;
    std::vector<void *> blocks;  // the pool blocks the tables above are carved from
};

// Image segmentation of the point set (a single image: nseg = 1).
struct Segments {
    std::vector<int> start;       // nseg+1 prefix offsets of the images' points
    const int *dev_start = nullptr;  // the same on the device
};

// Assignment of points to splat tiles: tile t owns slots [t*SPLAT_TILE,
// (t+1)*SPLAT_TILE); slot_pt[slot] is a point index or -1.  tile_vbase[t] is
// the number of valid slots in tiles before t (tile_vbase[ntiles] = N).
struct TileMapDev {
    int ntiles = 0;
    const int *slot_pt = nullptr;     // device [ntiles*SPLAT_TILE]
    const int *tile_vbase = nullptr;  // device [ntiles+1]
};

// Builds the lattice of `feat` ([d][N], device) on `s`, with its value
// buffers for MP-float rows and `nslots` slots.  `variant` selects the x86
// (SSE) or scalar arithmetic of the reference; SSE also inserts the
// zero-feature padding points of each image (N_img % 4 != 0).  `load` is the
// hash-table capacity factor (capacity = pow2 >= load * corners); `task_len`
// the most members of one splat task (1..63).  Returns a DCRF status; on
// DCRF_ERR_HASH_FULL the caller may retry with a larger load.  The host waits
// once, for the vertex and partial counts (a failed insert or an overflowing key
// is reported then); the kernels after it may still be in flight on return,
// and a status they leave is reported at the caller's next synchronisation.
int lattice_build(const float *feat, int d, int N, const Segments &seg, const TileMapDev &tm, int variant, float load,
                  int task_len, int MP, int nslots, cudaStream_t s, DevStatus *status, LatticeDev *out);

void lattice_free(LatticeDev *lat, cudaStream_t s);

// The value-size-1 passes of a lattice with MP-label rows (MP > 1) use the
// last L+1 floats of its value buffers, whose row 0 is their zero sentinel:
// that region holds no label chunk's row 0.
inline size_t lattice_v1_offset(size_t L, int MP) { return MP > 1 ? (L + 1) * (size_t)(MP - 1) : 0; }

// Zeroes the sentinel rows of both value buffers: row 0 of every label chunk
// and the value-size-1 row 0 (one launch).
cudaError_t launch_lattice_zero_rows(float *V0, float *V1, size_t L, int MP, cudaStream_t s);

// Host-side error text of the last failing build.
const char *lattice_last_message();

}  // namespace dcrf
