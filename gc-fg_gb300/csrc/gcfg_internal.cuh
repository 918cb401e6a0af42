// gcfg_internal.cuh -- shared definitions of the GB300 graph-cut library.
//
// Residual graph layout in HBM (one image, padded to whole tiles):
//   cap  : int4  per pixel {left, right, up, down} residual capacity (16 B)
//   exc  : int32 per pixel, reduced excess  e = dp - dn + inflow - outflow
//          (e > 0: excess to route; e < 0: remaining capacity to the sink)
//   h    : int32 per pixel, height / BFS distance to the sink (INF = none)
//   tile_active : int32 per 32x32 tile, "has active nodes"
// Pixels outside the image and on its 1-pixel border carry zero caps and zero
// excess, which reproduces the reference's interior-only graph
// (GraphCutKernels.cu:122-146).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>

#include "../../include/gcfg.h"

namespace gcfg {

constexpr int TILE_W = 32;
constexpr int TILE_H = 32;
constexpr int TILE_THREADS = 256;              // 8 warps; each thread owns 4 pixels of a column
constexpr int ROWS_PER_WARP = TILE_H / (TILE_THREADS / 32);
constexpr int INF_H = 1 << 30;                 // "cannot reach the sink"

// Bounds on every loop of the solver (none of them is unbounded).
constexpr int MAX_GR_LAUNCHES = 1 << 20;
constexpr int MAX_OUTER = 1 << 16;
constexpr int MAX_TILE_ITERS = TILE_W * TILE_H + 2;

struct GraphDev {
    int W, H, Wp, Hp, tiles_x, tiles_y;
    int4 *cap;
    int *exc;
    int *h;
    int *tile_active;
    uint8_t *mark;
};

// Device-side counters of one solve (kept in one small device buffer).
struct Counters {
    unsigned long long interior_dp;   // sum of dp over interior pixels
    unsigned long long ref_init;      // reference's "Initial energy level" (wraps like int32)
    unsigned long long pos_excess;    // sum of positive excess
    unsigned long long active;        // active nodes (e > 0, h < INF)
    unsigned long long push_tiles;    // tiles processed by push launches
    int changed;                      // a tile sweep changed something
    int error;                        // input validation failure
    int pad[2];
};

extern std::atomic<long long> g_launches;

constexpr int PK_COUNT_KINDS = GCFG_PK_NKINDS;
bool prof_on();
bool prof_on();
void prof_begin(cudaStream_t st);
void prof_end(int kind, cudaStream_t st);

// Launch a kernel, counting it and (when profiling) timing it with events.
#define GCFG_LAUNCH(kind, st, ...)                      \
    do {                                                \
        ::gcfg::prof_begin(st);                         \
        __VA_ARGS__;                                    \
        ::gcfg::prof_end(kind, st);                     \
        ::gcfg::g_launches.fetch_add(1, std::memory_order_relaxed); \
    } while (0)

inline int div_up(int a, int b) { return (a + b - 1) / b; }

#define GCFG_CK(call)                                  \
    do {                                               \
        cudaError_t e_ = (call);                       \
        if (e_ != cudaSuccess) return GCFG_ERR_CUDA;   \
    } while (0)

#define GCFG_TRY(call)                                 \
    do {                                               \
        gcfg_status s_ = (call);                       \
        if (s_ != GCFG_OK) return s_;                  \
    } while (0)

#define GCFG_LAUNCHED() (::gcfg::g_launches.fetch_add(1, std::memory_order_relaxed))

// Warp-level sum then one atomic per warp.
__device__ __forceinline__ void warp_atomic_add_u64(unsigned long long *dst, unsigned long long v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0 && v) atomicAdd(dst, v);
}

}  // namespace gcfg
