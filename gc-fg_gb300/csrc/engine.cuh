// engine.cuh -- the tile-space max-flow engine (batched, device-driven).
//
// Every image of a batch is cut into 32x32 tiles.  All tiles of all images
// live in one tile-major arena: tile t owns pixel slots [t*1024, t*1024+1024)
// in row-major order inside the tile, so a tile is 16 KB of capacities plus
// 4 KB of excess plus 4 KB of heights, contiguous in HBM.  Tiles of one image
// are consecutive and row-major, so a tile's neighbours are t-1, t+1,
// t-tiles_x, t+tiles_x.  A batch is one big graph whose components are the
// images; one image is a batch of one.
//
// The whole solve (global relabels, checkerboard push rounds, termination,
// source-side reachability) runs in ONE persistent cooperative kernel that
// takes its work from device queues of tiles and synchronises with a bounded
// grid barrier, so the host never waits inside a solve.
#pragma once

#include "gcfg_internal.cuh"

namespace gcfg {

constexpr int TPX = TILE_W * TILE_H;  // pixels per tile

// Immutable description of one image of a batch (uploaded by the host).
struct ImgDesc {
    int W, H, tiles_x, tiles_y;
    int tile0, n_tiles;
    long long pix0;   // offset of the image in packed row-major inputs/outputs
    double lambda;
    long long out0;   // offset of the image in the packed output label arrays
};

// Per-image state written by the device.
struct ImgState {
    unsigned long long interior_dp;  // sum of dp over interior pixels
    unsigned long long ref_init;     // reference's initial energy (int32 wrap)
    unsigned long long pos_excess;   // sum of positive excess (last count)
    unsigned long long active;       // active nodes (last count)
    unsigned long long sigma_sum;    // sum of ||dI||^2 over neighbour pairs
    double s2;                       // sigma^2 = sigma_sum / pairs (0: constant image)
    float ex2_scale;                 // (float)(log2(e) / (2 sigma^2)); 0: constant image
    float lambda_f;                  // (float)lambda
    int const_w;                     // round(lambda): every weight of a constant image
    int done;
    float nl_margin;                 // n-link fast-path margin (see nlink_quant)
    int pad_;
};

enum { L_PUSH0 = 0, L_PUSH1, L_PUSH2, L_GR0, L_GR1, L_NLISTS };

// Control block of one solve (zeroed before every launch).
constexpr int GR_TIMELINE = 32;

struct Ctl {
    unsigned bar_count;
    unsigned bar_gen;
    int err;          // nonzero: a barrier timed out or an iteration cap was hit
    int err_code;
    int size[L_NLISTS];
    int take[L_NLISTS];
    unsigned long long total_active;
    unsigned long long push_tiles, gr_tiles, reach_tiles;
    int gr_rounds, push_phases, reach_rounds, outer_iters;
    int global_relabels;
    int open_images;     // images left open by the last termination check
    int closure_checks;  // termination checks by sink-side closure
    int closure_ends;    // solves that the closure check ended (no final global relabel)
    // device time per phase (ns, %globaltimer read by block 0 at barriers)
    unsigned long long t_init, t_gr, t_count, t_push, t_reach;
    unsigned long long push_sweeps, push_bfs;
    // SM cycles per section of the push visits, summed over visits
    unsigned long long cyc_load, cyc_bfs, cyc_sweep, cyc_wb, cyc_take;
    // tile-BFS loop iterations (levels and halo jumps) of push and global-
    // relabel visits, and SM cycles summed over global-relabel visits
    unsigned long long bfs_it_push, bfs_it_gr, cyc_gr;
    // push phases' tail: per phase (by parity) the earliest time a block ran
    // out of work, stored bit-inverted so that 0 means none and atomicMax
    // keeps the earliest; t_push_tail sums (phase end - earliest idle)
    unsigned long long push_idle[2], t_push_tail;
    // timeline of the global relabel of a phase-1 launch (the phase-split
    // diagnostic; %globaltimer ns, block 0 after each grid barrier):
    // gr_time[0] its start, [1] after round 0, [2]
    // after the pull check, [3 + k] after frontier round k (k < GR_TIMELINE);
    // gr_front[k] the tiles of frontier round k
    unsigned long long gr_time[3 + GR_TIMELINE];
    int gr_front[GR_TIMELINE];
    // per frontier round of that relabel: the latest end of a tile visit
    // (%globaltimer ns) and the longest visit (SM cycles); other launches
    // leave these alone (their global atomics would serialise on one address)
    unsigned long long gr_front_end[GR_TIMELINE], gr_front_maxcyc[GR_TIMELINE];
};

struct Batch {
    int n_img, n_tiles;
    // Optional subset of the arena to solve: tiles tlist[0..n_tlist) (images
    // outside the subset must be marked done).  NULL: every tile 0..n_tiles.
    const int *tlist;
    int n_tlist;
    // Optional list of the images being solved (per-image loops visit only
    // these); NULL: every image 0..n_img.
    const int *ilist;
    int n_ilist;
    const ImgDesc *img;
    ImgState *ist;
    const int *tile_img;
    int4 *cap;
    int *exc;
    int *h;
    int *hb;                 // per tile, its border heights [4][32]: top row, bottom row, left, right column
    int4 *tile_nb;           // per tile: left, right, upper, lower neighbour tile (-1: image edge); set by the builds
    unsigned *hfin;          // per tile, 32 row masks: finite height after its last global-relabel visit
    unsigned *reach;         // 32 row masks per tile (source-side reachability)
    // Per-tile row bitmask planes, kept exact by every writer of cap/exc:
    // tmask[(t*6 + k)*32 + row], k = 0..3 residual capacity toward left,
    // right, up, down; 4: e < 0 (sink-connected); 5: e > 0 (excess).
    unsigned *tmask;
    int *tile_act;                  // active pixels of the tile at its last relabel visit
    unsigned long long *tile_pos;   // sum of positive excess of the tile
    int *lists;              // L_NLISTS work queues of tile indices, list_cap each
    int list_cap;
    int *mark_push, *mark_gr;
    Ctl *ctl;
};

struct SolveParams {
    int max_outer;     // outer iterations (global relabel + push rounds)
    int push_rounds;   // checkerboard rounds between global relabels
    int max_sweeps;    // push/relabel sweeps per tile visit
    int bfs_every;     // exact local relabel at least every this many sweeps
    int bfs_first;     // exact local relabel at the start of every tile visit
    int max_rounds;    // cap on BFS rounds of one global relabel / reach pass
    int push_only;     // 1: sweeps only push; heights change only by exact local relabels
    // Diagnostic split of one solve into two launches, so that a profiler
    // sees the two main phases as separate kernels.  0: the whole solve.
    // 1: initialisation, the first exact global relabel and its count pass,
    // then return (the work queues of the first push round stay in the
    // control block).  2: continue from the state a phase-1 launch left (the
    // control block not cleared in between): the push rounds of the first
    // outer iteration, then return.  A split leaves the solve unfinished.
    int phase;
    int warps;         // warps per block of the solver kernel (block shape 32 x warps over a 32x32 tile):
                       // 4, 8, 16 or 32; 0: by the solve's size (solve_warps)
};

// Default solver settings of every entry point (before any tuning): 2 push
// rounds per global relabel, 24 sweeps per tile visit, an exact local relabel
// every 4 sweeps.  Measured on single images from 256x256 to 4096x4096 and on
// the 256-image batch, these are at or near the fastest of the settings tried
// for every case (4 rounds with 64 sweeps and a local relabel every 16 sweeps
// took up to 2.9x longer on the 1920x1080 image with lambda 200).  The block
// shape goes by the solve's size (solve_warps).
constexpr SolveParams kDefaultSolveParams{64, 2, 24, 4, 0, 1 << 20, 0, 0, 0};

// The block shape of a solve of n_tiles tiles: the shape asked for, or for 0
// 32 x 16 up to 2048 tiles (a 1920x1080 image has 2040) and 32 x 8 above.
// A small solve keeps few tiles busy at once, so its time is the latency of
// single tile visits, which 16 warps (2 rows each) shorten; a large one keeps
// every SM busy, where 8 warps at 4 blocks per SM do more per cycle.
constexpr int kSmallSolveTiles = 2048;
inline int solve_warps(int warps, int n_tiles) {
    if (warps == 4 || warps == 8 || warps == 16 || warps == 32) return warps;
    return n_tiles <= kSmallSolveTiles ? 16 : 8;
}

__host__ __device__ __forceinline__ int batch_ntiles(const Batch &b) { return b.tlist ? b.n_tlist : b.n_tiles; }
__device__ __forceinline__ int batch_tile(const Batch &b, int k) { return b.tlist ? __ldg(b.tlist + k) : k; }
__host__ __device__ __forceinline__ int batch_nimg(const Batch &b) { return b.ilist ? b.n_ilist : b.n_img; }
__device__ __forceinline__ int batch_img(const Batch &b, int k) { return b.ilist ? __ldg(b.ilist + k) : k; }

// Error codes in Ctl::err_code.
enum {
    ERRC_BARRIER = 1,
    ERRC_GR_ROUNDS = 2,
    ERRC_OUTER = 3,
    ERRC_REACH_ROUNDS = 4,
    ERRC_HEIGHT_DECREASE = 5,
    ERRC_QUEUE = 6
};

}  // namespace gcfg

namespace gcfg {

// Host launchers (engine.cu).
// Co-resident blocks of the persistent kernel of a block shape (warps per
// block), capped by max_grid when > 0 and by half the tiles.
int solve_grid_blocks(int n_tiles, int max_grid = 0, int warps = 8);
gcfg_status launch_solve(const Batch &b, const SolveParams &prm, int n_tiles, cudaStream_t st,
                         int max_grid = 0);
gcfg_status launch_build_arrays(const Batch &b, const int *dp, const int *dn, int penalty, const int *up,
                                const int *down, const int *left, const int *right, cudaStream_t st);
gcfg_status launch_extract(const Batch &b, uint8_t *smin, uint8_t *smax, int *label, cudaStream_t st);
// The cuts of the images of a chunk map (the data-term pass's blocks: CHUNK_PX
// consecutive pixels of one image each), written by aligned 16-byte windows.
gcfg_status launch_extract_rows(const Batch &b, const int2 *chunk_map, long long n_chunks, uint8_t *smin,
                               uint8_t *smax, cudaStream_t st);

}  // namespace gcfg

namespace gcfg {

// ---- device helpers shared by the build kernels and the solver ----

// Mask planes and positive-excess sum of one tile from per-pixel values held
// by a block (warp w owns rows w, w+8, w+16, w+24; lane = column).
__device__ __forceinline__ void write_tile_masks(const Batch &b, int t, int r, int4 c, int e) {
    const unsigned ml = __ballot_sync(0xffffffffu, c.x > 0);
    const unsigned mr = __ballot_sync(0xffffffffu, c.y > 0);
    const unsigned mu = __ballot_sync(0xffffffffu, c.z > 0);
    const unsigned md = __ballot_sync(0xffffffffu, c.w > 0);
    const unsigned mn = __ballot_sync(0xffffffffu, e < 0);
    const unsigned mp = __ballot_sync(0xffffffffu, e > 0);
    const int lane = threadIdx.x & 31;
    if (lane < 6) {
        const unsigned v = lane == 0 ? ml : lane == 1 ? mr : lane == 2 ? mu : lane == 3 ? md : lane == 4 ? mn : mp;
        b.tmask[((size_t)t * 6 + lane) * 32 + r] = v;
    }
}

// Sum of v over the block, stored by thread 0 (blocks of TILE_THREADS).
__device__ __forceinline__ void block_store_sum(unsigned long long *dst, unsigned long long v) {
    __shared__ unsigned long long part[TILE_THREADS / 32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long tot = 0;
        for (int w = 0; w < TILE_THREADS / 32; ++w) tot += part[w];
        *dst = tot;
    }
}

}  // namespace gcfg
