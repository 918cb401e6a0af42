// solver.cu -- exact push-relabel max-flow on a 4-connected grid, GB300.
//
// Replaces the reference's GraphCut.cu host driver and GraphCutKernels.cu
// kernels.  The algorithm keeps the reference's model (reduced t-link
// excess, heights = residual distance to the sink, global relabel as a BFS
// from the sink, cut = pixels that cannot reach the sink) but reorganises
// the work for the GPU:
//
//  * 32x32 tiles staged in shared memory with a one-pixel halo.  A tile
//    runs many push/relabel sweeps per launch (flow moves many pixels per
//    HBM pass) instead of the reference's one Relabel + one WavePush launch
//    per host iteration (GraphCut.cu:416-492).
//  * Tiles are processed in two checkerboard colours.  While a tile runs, no
//    edge-adjacent tile runs, so its halo heights are exact and frozen, the
//    labelling stays valid at every push (h(u) <= h(v) + 1 on every residual
//    edge), and flow pushed into a halo pixel is handed over with plain
//    atomics.  The reference instead freezes heights by splitting Relabel
//    and WavePush into separate launches (GraphCutKernels.cu:433-724).
//  * The global relabel is an exact Bellman-Ford BFS from the sink, iterated
//    to a fixpoint tile by tile (GraphCutKernels.cu:757-875 computes the
//    same distances 10 steps per launch with a host round trip each).
//  * Termination is exact: the solve ends when, after an exact global
//    relabel, no node with positive excess can reach the sink.  This
//    replaces the reference's activity heuristic (UpdateActivity,
//    GraphCutKernels.cu:729-743).
//  * Cut extraction: S_max = pixels with no residual path to the sink (the
//    reference's InitLabels/SpreadLabels output, GraphCutKernels.cu:228-351)
//    and S_min = pixels reachable from the source (from positive excess).
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "gcfg_internal.cuh"
#include "solver.cuh"

namespace gcfg {

std::atomic<long long> g_launches{0};

// ---------------------------------------------------------------------------
// Graph build from caller arrays (GC_SetGraph -> InitGraph / InitGraphVarEdges)
// ---------------------------------------------------------------------------

// One thread per padded pixel.  Interior pixels take their caps from the
// arrays (or the penalty); caps that point into the border ring are zeroed
// (GraphCutKernels.cu:143-146, 200-203); excess = dp - dn.
__global__ void k_build_arrays(GraphDev g, const int *__restrict__ dp, const int *__restrict__ dn,
                               int penalty, const int *__restrict__ up,
                               const int *__restrict__ down, const int *__restrict__ left,
                               const int *__restrict__ right, Counters *cnt) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    const int W = g.W, H = g.H;
    int4 c = make_int4(0, 0, 0, 0);
    int e = 0;
    unsigned long long idp = 0, rinit = 0;
    int bad = 0;
    if (x < W && y < H) {
        const int i = y * W + x;
        const int vdp = dp[i];
        // The reference sums max(dp,0) over padded positions x + y*W32 < W*H
        // (GraphCut.cu:359-376 with EnergyLevel, GraphCutKernels.cu:883-898).
        const long long w32 = (long long)((W + 31) / 32) * 32;
        if ((long long)x + (long long)y * w32 < (long long)W * H && vdp > 0) rinit = (unsigned)vdp;
        const bool inside = x > 0 && y > 0 && x < W - 1 && y < H - 1;
        if (inside) {
            const int vdn = dn[i];
            if (up) {
                c = make_int4(left[i], right[i], up[i], down[i]);
            } else {
                c = make_int4(penalty, penalty, penalty, penalty);
            }
            bad = (vdp < 0) | (vdn < 0) | (vdp > GCFG_MAX_CAP) | (vdn > GCFG_MAX_CAP) |
                  (c.x < 0) | (c.y < 0) | (c.z < 0) | (c.w < 0) | (c.x > GCFG_MAX_CAP) |
                  (c.y > GCFG_MAX_CAP) | (c.z > GCFG_MAX_CAP) | (c.w > GCFG_MAX_CAP);
            if (x == 1) c.x = 0;
            if (x == W - 2) c.y = 0;
            if (y == 1) c.z = 0;
            if (y == H - 2) c.w = 0;
            e = vdp - vdn;
            idp = (unsigned long long)(long long)vdp;
        }
    }
    if (x < g.Wp && y < g.Hp) {
        const size_t p = (size_t)y * g.Wp + x;
        g.cap[p] = c;
        g.exc[p] = e;
    }
    if (bad) cnt->error = 1;
    warp_atomic_add_u64(&cnt->interior_dp, idp);
    warp_atomic_add_u64(&cnt->ref_init, rinit);
}

// ---------------------------------------------------------------------------
// Global relabel: exact BFS distances to the sink, in place in g.h
// ---------------------------------------------------------------------------

__global__ void k_gr_init(GraphDev g) {
    const size_t n = (size_t)g.Wp * g.Hp;
    for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < n;
         p += (size_t)gridDim.x * blockDim.x) {
        g.h[p] = g.exc[p] < 0 ? 1 : INF_H;
    }
}

// Loads the heights of the tile's one-pixel halo (INF outside the padded grid).
__device__ __forceinline__ void load_halo_h(const GraphDev &g, int x0, int y0,
                                            int (*h_s)[TILE_W + 2]) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (warp == 0) {
        const int y = y0 - 1;
        h_s[0][lane + 1] = y >= 0 ? g.h[(size_t)y * g.Wp + x0 + lane] : INF_H;
    } else if (warp == 1) {
        const int y = y0 + TILE_H;
        h_s[TILE_H + 1][lane + 1] = y < g.Hp ? g.h[(size_t)y * g.Wp + x0 + lane] : INF_H;
    } else if (warp == 2) {
        const int x = x0 - 1;
        h_s[lane + 1][0] = x >= 0 ? g.h[(size_t)(y0 + lane) * g.Wp + x] : INF_H;
    } else if (warp == 3) {
        const int x = x0 + TILE_W;
        h_s[lane + 1][TILE_W + 1] = x < g.Wp ? g.h[(size_t)(y0 + lane) * g.Wp + x] : INF_H;
    }
}

// One Bellman-Ford round: every tile relaxes d(u) = min(d(u), d(v) + 1) over
// residual edges u->v until its own pixels stop changing, reading its halo
// from the last values other tiles wrote.  Values only decrease and are
// always lengths of real residual paths, so concurrent tiles are benign.
__global__ void __launch_bounds__(TILE_THREADS) k_gr_tile(GraphDev g, Counters *cnt) {
    __shared__ int d_s[TILE_H + 2][TILE_W + 2];
    __shared__ uint8_t rm[TILE_H][TILE_W];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int x0 = blockIdx.x * TILE_W, y0 = blockIdx.y * TILE_H;
    int d0[ROWS_PER_WARP];
#pragma unroll
    for (int k = 0; k < ROWS_PER_WARP; ++k) {
        const int r = warp + 8 * k;
        const size_t p = (size_t)(y0 + r) * g.Wp + x0 + lane;
        const int4 c = g.cap[p];
        rm[r][lane] = (uint8_t)((c.x > 0) | ((c.y > 0) << 1) | ((c.z > 0) << 2) | ((c.w > 0) << 3));
        d0[k] = g.h[p];
        d_s[r + 1][lane + 1] = d0[k];
    }
    load_halo_h(g, x0, y0, d_s);
    __syncthreads();
    for (int it = 0; it < MAX_TILE_ITERS; ++it) {
        int changed = 0;
#pragma unroll
        for (int k = 0; k < ROWS_PER_WARP; ++k) {
            const int r = warp + 8 * k;
            const int d = d_s[r + 1][lane + 1];
            const int bits = rm[r][lane];
            if (d > 1 && bits) {
                int m = INF_H;
                if (bits & 1) m = min(m, d_s[r + 1][lane]);
                if (bits & 2) m = min(m, d_s[r + 1][lane + 2]);
                if (bits & 4) m = min(m, d_s[r][lane + 1]);
                if (bits & 8) m = min(m, d_s[r + 2][lane + 1]);
                if (m < INF_H && m + 1 < d) {
                    d_s[r + 1][lane + 1] = m + 1;
                    changed = 1;
                }
            }
        }
        if (!__syncthreads_or(changed)) break;
    }
    int wrote = 0;
#pragma unroll
    for (int k = 0; k < ROWS_PER_WARP; ++k) {
        const int r = warp + 8 * k;
        const int d = d_s[r + 1][lane + 1];
        if (d != d0[k]) {
            g.h[(size_t)(y0 + r) * g.Wp + x0 + lane] = d;
            wrote = 1;
        }
    }
    if (__syncthreads_or(wrote) && threadIdx.x == 0) cnt->changed = 1;
}

// After a global relabel: count active nodes, mark active tiles, and sum
// the positive excess (for the flow value).
__global__ void __launch_bounds__(TILE_THREADS) k_count(GraphDev g, Counters *cnt) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int x0 = blockIdx.x * TILE_W, y0 = blockIdx.y * TILE_H;
    unsigned long long act = 0, pos = 0;
#pragma unroll
    for (int k = 0; k < ROWS_PER_WARP; ++k) {
        const int r = warp + 8 * k;
        const size_t p = (size_t)(y0 + r) * g.Wp + x0 + lane;
        const int e = g.exc[p];
        if (e > 0) {
            pos += (unsigned long long)e;
            if (g.h[p] < INF_H) act++;
        }
    }
    warp_atomic_add_u64(&cnt->active, act);
    warp_atomic_add_u64(&cnt->pos_excess, pos);
    const int any = __syncthreads_or(act != 0);
    if (threadIdx.x == 0) g.tile_active[blockIdx.y * g.tiles_x + blockIdx.x] = any;
}

// ---------------------------------------------------------------------------
// Tile push/relabel (one checkerboard colour per launch)
// ---------------------------------------------------------------------------

__global__ void __launch_bounds__(TILE_THREADS) k_push_tile(GraphDev g, int color, int max_sweeps,
                                                             Counters *cnt) {
    const int tx = blockIdx.x, ty = blockIdx.y;
    if (((tx + ty) & 1) != color) return;
    const int t = ty * g.tiles_x + tx;
    if (!g.tile_active[t]) return;
    if (threadIdx.x == 0) atomicAdd(&cnt->push_tiles, 1ULL);

    __shared__ int h_s[TILE_H + 2][TILE_W + 2];
    __shared__ int e_s[TILE_H][TILE_W];
    __shared__ int4 c_s[TILE_H][TILE_W];
    __shared__ int halo_in[4][32];  // flow into halo: 0 top, 1 bottom, 2 left, 3 right

    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int x0 = tx * TILE_W, y0 = ty * TILE_H;
#pragma unroll
    for (int k = 0; k < ROWS_PER_WARP; ++k) {
        const int r = warp + 8 * k;
        const size_t p = (size_t)(y0 + r) * g.Wp + x0 + lane;
        c_s[r][lane] = g.cap[p];
        e_s[r][lane] = g.exc[p];
        h_s[r + 1][lane + 1] = g.h[p];
    }
    load_halo_h(g, x0, y0, h_s);
    if (warp < 4) halo_in[warp][lane] = 0;
    __syncthreads();

    for (int s = 0; s < max_sweeps; ++s) {
        // ---- push phase: heights are fixed inside this phase ----
#pragma unroll
        for (int k = 0; k < ROWS_PER_WARP; ++k) {
            const int r = warp + 8 * k;
            int e = e_s[r][lane];
            const int hh = h_s[r + 1][lane + 1];
            if (e > 0 && hh < INF_H) {
                const int4 c = c_s[r][lane];
                const int e0 = e;
                if (c.x > 0 && hh == h_s[r + 1][lane] + 1) {  // left
                    const int f = min(e, c.x);
                    e -= f;
                    c_s[r][lane].x = c.x - f;
                    if (lane > 0) {
                        c_s[r][lane - 1].y += f;
                        atomicAdd(&e_s[r][lane - 1], f);
                    } else {
                        atomicAdd(&halo_in[2][r], f);
                    }
                }
                if (e > 0 && c.y > 0 && hh == h_s[r + 1][lane + 2] + 1) {  // right
                    const int f = min(e, c.y);
                    e -= f;
                    c_s[r][lane].y = c.y - f;
                    if (lane < TILE_W - 1) {
                        c_s[r][lane + 1].x += f;
                        atomicAdd(&e_s[r][lane + 1], f);
                    } else {
                        atomicAdd(&halo_in[3][r], f);
                    }
                }
                if (e > 0 && c.z > 0 && hh == h_s[r][lane + 1] + 1) {  // up
                    const int f = min(e, c.z);
                    e -= f;
                    c_s[r][lane].z = c.z - f;
                    if (r > 0) {
                        c_s[r - 1][lane].w += f;
                        atomicAdd(&e_s[r - 1][lane], f);
                    } else {
                        atomicAdd(&halo_in[0][lane], f);
                    }
                }
                if (e > 0 && c.w > 0 && hh == h_s[r + 2][lane + 1] + 1) {  // down
                    const int f = min(e, c.w);
                    e -= f;
                    c_s[r][lane].w = c.w - f;
                    if (r < TILE_H - 1) {
                        c_s[r + 1][lane].z += f;
                        atomicAdd(&e_s[r + 1][lane], f);
                    } else {
                        atomicAdd(&halo_in[1][lane], f);
                    }
                }
                if (e != e0) atomicSub(&e_s[r][lane], e0 - e);
            }
        }
        __syncthreads();
        // ---- relabel phase: caps and excess are fixed inside this phase ----
        int any = 0;
#pragma unroll
        for (int k = 0; k < ROWS_PER_WARP; ++k) {
            const int r = warp + 8 * k;
            const int e = e_s[r][lane];
            int hh = h_s[r + 1][lane + 1];
            if (e > 0 && hh < INF_H) {
                const int4 c = c_s[r][lane];
                int m = INF_H;
                if (c.x > 0) m = min(m, h_s[r + 1][lane]);
                if (c.y > 0) m = min(m, h_s[r + 1][lane + 2]);
                if (c.z > 0) m = min(m, h_s[r][lane + 1]);
                if (c.w > 0) m = min(m, h_s[r + 2][lane + 1]);
                if (m >= hh) {  // no admissible edge left
                    hh = m >= INF_H - 1 ? INF_H : m + 1;
                    h_s[r + 1][lane + 1] = hh;
                }
                any |= hh < INF_H;
            }
        }
        if (!__syncthreads_or(any)) break;
    }

    int my_active = 0;
#pragma unroll
    for (int k = 0; k < ROWS_PER_WARP; ++k) {
        const int r = warp + 8 * k;
        const size_t p = (size_t)(y0 + r) * g.Wp + x0 + lane;
        const int e = e_s[r][lane], hh = h_s[r + 1][lane + 1];
        g.cap[p] = c_s[r][lane];
        g.exc[p] = e;
        g.h[p] = hh;
        my_active |= e > 0 && hh < INF_H;
    }
    // Hand flow pushed into halo pixels to their (idle) owner tiles.
    if (warp < 4) {
        const int f = halo_in[warp][lane];
        if (f) {
            size_t q;
            int comp, tn;
            if (warp == 0) {          // pixel above -> its DOWN edge gets the reverse capacity
                q = (size_t)(y0 - 1) * g.Wp + x0 + lane; comp = 3; tn = t - g.tiles_x;
            } else if (warp == 1) {   // pixel below -> its UP edge
                q = (size_t)(y0 + TILE_H) * g.Wp + x0 + lane; comp = 2; tn = t + g.tiles_x;
            } else if (warp == 2) {   // pixel left -> its RIGHT edge
                q = (size_t)(y0 + lane) * g.Wp + x0 - 1; comp = 1; tn = t - 1;
            } else {                  // pixel right -> its LEFT edge
                q = (size_t)(y0 + lane) * g.Wp + x0 + TILE_W; comp = 0; tn = t + 1;
            }
            atomicAdd(&g.exc[q], f);
            atomicAdd(reinterpret_cast<int *>(&g.cap[q]) + comp, f);
            g.tile_active[tn] = 1;
        }
    }
    const int any = __syncthreads_or(my_active);
    if (threadIdx.x == 0) g.tile_active[t] = any;
}

// ---------------------------------------------------------------------------
// Source-side reachability (S_min) and label extraction
// ---------------------------------------------------------------------------

__global__ void k_reach_init(GraphDev g) {
    const size_t n = (size_t)g.Wp * g.Hp;
    for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < n;
         p += (size_t)gridDim.x * blockDim.x)
        g.mark[p] = g.exc[p] > 0;
}

// v becomes reachable if a reachable neighbour u has residual capacity u->v.
__global__ void __launch_bounds__(TILE_THREADS) k_reach_tile(GraphDev g, Counters *cnt) {
    __shared__ uint8_t m_s[TILE_H + 2][TILE_W + 2];
    __shared__ uint8_t in_s[TILE_H][TILE_W];  // bit d: the neighbour in direction d can push into me
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int x0 = blockIdx.x * TILE_W, y0 = blockIdx.y * TILE_H;
    uint8_t m0[ROWS_PER_WARP];
#pragma unroll
    for (int k = 0; k < ROWS_PER_WARP; ++k) {
        const int r = warp + 8 * k;
        const size_t p = (size_t)(y0 + r) * g.Wp + x0 + lane;
        m0[k] = g.mark[p];
        m_s[r + 1][lane + 1] = m0[k];
        in_s[r][lane] = 0;
    }
    // halo marks and the halo pixels' capacities toward the tile
    if (warp == 0) {
        const int y = y0 - 1;
        m_s[0][lane + 1] = y >= 0 && g.mark[(size_t)y * g.Wp + x0 + lane] &&
                           g.cap[(size_t)y * g.Wp + x0 + lane].w > 0;
    } else if (warp == 1) {
        const int y = y0 + TILE_H;
        m_s[TILE_H + 1][lane + 1] = y < g.Hp && g.mark[(size_t)y * g.Wp + x0 + lane] &&
                                    g.cap[(size_t)y * g.Wp + x0 + lane].z > 0;
    } else if (warp == 2) {
        const int x = x0 - 1;
        m_s[lane + 1][0] = x >= 0 && g.mark[(size_t)(y0 + lane) * g.Wp + x] &&
                           g.cap[(size_t)(y0 + lane) * g.Wp + x].y > 0;
    } else if (warp == 3) {
        const int x = x0 + TILE_W;
        m_s[lane + 1][TILE_W + 1] = x < g.Wp && g.mark[(size_t)(y0 + lane) * g.Wp + x] &&
                                    g.cap[(size_t)(y0 + lane) * g.Wp + x].x > 0;
    }
    __syncthreads();
    // in-tile incoming residual bits: neighbour u at direction d pushes into me
    // if u's capacity toward me is positive.  Halo bits were folded into m_s.
#pragma unroll
    for (int k = 0; k < ROWS_PER_WARP; ++k) {
        const int r = warp + 8 * k;
        const size_t p = (size_t)(y0 + r) * g.Wp + x0 + lane;
        (void)p;
        uint8_t b = 0;
        if (lane > 0 && g.cap[(size_t)(y0 + r) * g.Wp + x0 + lane - 1].y > 0) b |= 1;
        if (lane < TILE_W - 1 && g.cap[(size_t)(y0 + r) * g.Wp + x0 + lane + 1].x > 0) b |= 2;
        if (r > 0 && g.cap[(size_t)(y0 + r - 1) * g.Wp + x0 + lane].w > 0) b |= 4;
        if (r < TILE_H - 1 && g.cap[(size_t)(y0 + r + 1) * g.Wp + x0 + lane].z > 0) b |= 8;
        if (lane == 0) b |= 1;            // halo bits already include the capacity test
        if (lane == TILE_W - 1) b |= 2;
        if (r == 0) b |= 4;
        if (r == TILE_H - 1) b |= 8;
        in_s[r][lane] = b;
    }
    __syncthreads();
    for (int it = 0; it < MAX_TILE_ITERS; ++it) {
        int changed = 0;
#pragma unroll
        for (int k = 0; k < ROWS_PER_WARP; ++k) {
            const int r = warp + 8 * k;
            if (m_s[r + 1][lane + 1]) continue;
            const int b = in_s[r][lane];
            if (((b & 1) && m_s[r + 1][lane]) || ((b & 2) && m_s[r + 1][lane + 2]) ||
                ((b & 4) && m_s[r][lane + 1]) || ((b & 8) && m_s[r + 2][lane + 1])) {
                m_s[r + 1][lane + 1] = 1;
                changed = 1;
            }
        }
        if (!__syncthreads_or(changed)) break;
    }
    int wrote = 0;
#pragma unroll
    for (int k = 0; k < ROWS_PER_WARP; ++k) {
        const int r = warp + 8 * k;
        if (m_s[r + 1][lane + 1] != m0[k]) {
            g.mark[(size_t)(y0 + r) * g.Wp + x0 + lane] = 1;
            wrote = 1;
        }
    }
    if (__syncthreads_or(wrote) && threadIdx.x == 0) cnt->changed = 1;
}

// smin = source-reachable, smax = interior and cannot reach the sink.
__global__ void k_extract(GraphDev g, uint8_t *smin, uint8_t *smax, int *label) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= g.W || y >= g.H) return;
    const size_t p = (size_t)y * g.Wp + x;
    const size_t i = (size_t)y * g.W + x;
    const bool inside = x > 0 && y > 0 && x < g.W - 1 && y < g.H - 1;
    const uint8_t sm = inside && g.h[p] >= INF_H;
    if (smin) smin[i] = g.mark[p];
    if (smax) smax[i] = sm;
    if (label) label[i] = sm;
}

// ---------------------------------------------------------------------------
// Host driver
// ---------------------------------------------------------------------------

gcfg_status solver_alloc(SolverState &s, int max_w, int max_h) {
    s.max_pixels = (size_t)div_up(max_w, TILE_W) * TILE_W * (size_t)div_up(max_h, TILE_H) * TILE_H;
    s.max_tiles = div_up(max_w, TILE_W) * div_up(max_h, TILE_H);
    if (cudaMalloc(&s.cap, s.max_pixels * sizeof(int4)) != cudaSuccess) return GCFG_ERR_OOM;
    if (cudaMalloc(&s.exc, s.max_pixels * sizeof(int)) != cudaSuccess) return GCFG_ERR_OOM;
    if (cudaMalloc(&s.h, s.max_pixels * sizeof(int)) != cudaSuccess) return GCFG_ERR_OOM;
    if (cudaMalloc(&s.mark, s.max_pixels) != cudaSuccess) return GCFG_ERR_OOM;
    if (cudaMalloc(&s.tile_active, (size_t)s.max_tiles * sizeof(int)) != cudaSuccess)
        return GCFG_ERR_OOM;
    if (cudaMalloc(&s.cnt, sizeof(Counters)) != cudaSuccess) return GCFG_ERR_OOM;
    if (cudaMallocHost(&s.h_cnt, sizeof(Counters)) != cudaSuccess) return GCFG_ERR_OOM;
    GCFG_CK(cudaEventCreate(&s.ev0));
    GCFG_CK(cudaEventCreate(&s.ev1));
    return GCFG_OK;
}

void solver_free(SolverState &s) {
    cudaFree(s.cap);
    cudaFree(s.exc);
    cudaFree(s.h);
    cudaFree(s.mark);
    cudaFree(s.tile_active);
    cudaFree(s.cnt);
    if (s.h_cnt) cudaFreeHost(s.h_cnt);
    if (s.ev0) cudaEventDestroy(s.ev0);
    if (s.ev1) cudaEventDestroy(s.ev1);
    s = SolverState();
}

GraphDev solver_view(SolverState &s, int W, int H) {
    GraphDev g;
    g.W = W;
    g.H = H;
    g.Wp = div_up(W, TILE_W) * TILE_W;
    g.Hp = div_up(H, TILE_H) * TILE_H;
    g.tiles_x = g.Wp / TILE_W;
    g.tiles_y = g.Hp / TILE_H;
    g.cap = s.cap;
    g.exc = s.exc;
    g.h = s.h;
    g.tile_active = s.tile_active;
    g.mark = s.mark;
    return g;
}

static gcfg_status read_counters(SolverState &s, cudaStream_t st) {
    GCFG_CK(cudaMemcpyAsync(s.h_cnt, s.cnt, sizeof(Counters), cudaMemcpyDeviceToHost, st));
    GCFG_CK(cudaStreamSynchronize(st));
    return GCFG_OK;
}

gcfg_status build_from_arrays(SolverState &s, const GraphDev &g, const int *dp, const int *dn,
                              int penalty, const int *up, const int *down, const int *left,
                              const int *right, cudaStream_t st) {
    GCFG_CK(cudaMemsetAsync(s.cnt, 0, sizeof(Counters), st));
    dim3 blk(32, 8);
    dim3 grd(g.Wp / 32, g.Hp / 8);
    GCFG_LAUNCH(GCFG_PK_BUILD, st, k_build_arrays<<<grd, blk, 0, st>>>(g, dp, dn, penalty, up, down, left, right, s.cnt));
    GCFG_CK(cudaGetLastError());
    GCFG_TRY(read_counters(s, st));
    if (s.h_cnt->error) return GCFG_ERR_INVALID;
    s.interior_dp = (long long)s.h_cnt->interior_dp;
    s.ref_init = (unsigned)s.h_cnt->ref_init;
    return GCFG_OK;
}

static int grid_stride_blocks(size_t n) {
    size_t b = (n + 255) / 256;
    return (int)(b > 152 * 16 ? 152 * 16 : (b ? b : 1));
}

// Exact global relabel; leaves counters (active, pos_excess) of the result.
static gcfg_status global_relabel(SolverState &s, const GraphDev &g, cudaStream_t st,
                                  gcfg_result *res) {
    const size_t n = (size_t)g.Wp * g.Hp;
    GCFG_LAUNCH(GCFG_PK_GR_INIT, st, k_gr_init<<<grid_stride_blocks(n), 256, 0, st>>>(g));
    dim3 tg(g.tiles_x, g.tiles_y);
    int launches = 0;
    for (;;) {
        GCFG_CK(cudaMemsetAsync(&s.cnt->changed, 0, sizeof(int), st));
        GCFG_LAUNCH(GCFG_PK_GR_TILE, st, k_gr_tile<<<tg, TILE_THREADS, 0, st>>>(g, s.cnt));
        launches++;
        GCFG_TRY(read_counters(s, st));
        if (!s.h_cnt->changed) break;
        if (launches >= MAX_GR_LAUNCHES) return GCFG_ERR_NOT_CONVERGED;
    }
    if (res) {
        res->global_relabels++;
        res->gr_sweeps += launches;
        res->gr_tiles += (long long)launches * g.tiles_x * g.tiles_y;
    }
    GCFG_CK(cudaMemsetAsync(&s.cnt->pos_excess, 0, 2 * sizeof(unsigned long long), st));
    GCFG_LAUNCH(GCFG_PK_COUNT, st, k_count<<<tg, TILE_THREADS, 0, st>>>(g, s.cnt));
    GCFG_TRY(read_counters(s, st));
    return GCFG_OK;
}

gcfg_status solve(SolverState &s, const GraphDev &g, cudaStream_t st, int push_rounds,
                  int max_sweeps, gcfg_result *res) {
    gcfg_result local;
    memset(&local, 0, sizeof(local));
    GCFG_CK(cudaEventRecord(s.ev0, st));
    dim3 tg(g.tiles_x, g.tiles_y);
    gcfg_status rc = GCFG_OK;
    int outer = 0;
    for (;; ++outer) {
        rc = global_relabel(s, g, st, &local);
        if (rc) break;
        if (outer == 0) local.active_after_first_gr = (long long)s.h_cnt->active;
        if (s.h_cnt->active == 0) break;
        if (outer >= MAX_OUTER) { rc = GCFG_ERR_NOT_CONVERGED; break; }
        for (int r = 0; r < push_rounds; ++r) {
            for (int color = 0; color < 2; ++color) {
                GCFG_LAUNCH(GCFG_PK_PUSH, st, k_push_tile<<<tg, TILE_THREADS, 0, st>>>(g, color, max_sweeps, s.cnt));
            }
            local.push_rounds++;
        }
        GCFG_CK(cudaGetLastError());
    }
    if (rc == GCFG_OK) {
        // interior_dp and ref_init were accumulated by the build kernel into
        // the same counter block and arrive with every counter read-back.
        const long long pos = (long long)s.h_cnt->pos_excess;
        local.flow = (long long)s.h_cnt->interior_dp - pos;
        local.push_tiles = (long long)s.h_cnt->push_tiles;
        local.ref_energy = (int32_t)((uint32_t)s.h_cnt->ref_init - (uint32_t)(unsigned long long)pos);
        // source-side reachability
        const size_t n = (size_t)g.Wp * g.Hp;
        GCFG_LAUNCH(GCFG_PK_REACH_INIT, st, k_reach_init<<<grid_stride_blocks(n), 256, 0, st>>>(g));
        for (int it = 0;; ++it) {
            GCFG_CK(cudaMemsetAsync(&s.cnt->changed, 0, sizeof(int), st));
            GCFG_LAUNCH(GCFG_PK_REACH, st, k_reach_tile<<<tg, TILE_THREADS, 0, st>>>(g, s.cnt));
            local.cut_sweeps++;
            GCFG_TRY(read_counters(s, st));
            if (!s.h_cnt->changed) break;
            if (it >= MAX_GR_LAUNCHES) { rc = GCFG_ERR_NOT_CONVERGED; break; }
        }
    }
    GCFG_CK(cudaEventRecord(s.ev1, st));
    GCFG_CK(cudaEventSynchronize(s.ev1));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, s.ev0, s.ev1);
    local.ms = ms;
    local.status = rc;
    if (res) *res = local;
    return rc;
}

gcfg_status extract(const GraphDev &g, uint8_t *smin, uint8_t *smax, int *label, cudaStream_t st) {
    dim3 blk(32, 8);
    dim3 grd(div_up(g.W, 32), div_up(g.H, 8));
    GCFG_LAUNCH(GCFG_PK_EXTRACT, st, k_extract<<<grd, blk, 0, st>>>(g, smin, smax, label));
    GCFG_CK(cudaGetLastError());
    return GCFG_OK;
}

}  // namespace gcfg

// ---------------------------------------------------------------------------
// C ABI: graph API (drop-in for GraphCut.cu's GC_* functions)
// ---------------------------------------------------------------------------

using namespace gcfg;

struct gcfg_graph {
    int W = 0, H = 0;
    SolverState s;
    const int32_t *dp = nullptr, *dn = nullptr;
    const int32_t *up = nullptr, *down = nullptr, *left = nullptr, *right = nullptr;
    int32_t penalty = 0;
    bool varying = false;
    bool built = false;
    cudaStream_t stream = nullptr;
    int push_rounds = 4;
    int max_sweeps = 64;
    int32_t *d_label = nullptr;
};

extern "C" {

gcfg_status gcfg_set_dataterms(gcfg_graph *g, const int32_t *dp, const int32_t *dn) {
    if (!g) return GCFG_ERR_INVALID;
    g->dp = dp;
    g->dn = dn;
    g->built = false;
    return GCFG_OK;
}

gcfg_status gcfg_set_edges(gcfg_graph *g, const int32_t *up, const int32_t *down,
                           const int32_t *left, const int32_t *right) {
    if (!g) return GCFG_ERR_INVALID;
    if (!up || !down || !left || !right) return GCFG_ERR_INVALID;
    g->varying = true;
    g->up = up;
    g->down = down;
    g->left = left;
    g->right = right;
    g->built = false;
    return GCFG_OK;
}

gcfg_status gcfg_set_penalty(gcfg_graph *g, int32_t penalty) {
    if (!g) return GCFG_ERR_INVALID;
    if (penalty < 0 || penalty > GCFG_MAX_CAP) return GCFG_ERR_INVALID;
    g->varying = false;
    g->penalty = penalty;
    g->built = false;
    return GCFG_OK;
}

gcfg_status gcfg_set_graph(gcfg_graph *g) {
    if (!g) return GCFG_ERR_INVALID;
    if (!g->dp || !g->dn) return GCFG_ERR_STATE;
    GraphDev v = solver_view(g->s, g->W, g->H);
    gcfg_status rc = build_from_arrays(g->s, v, g->dp, g->dn, g->penalty,
                                       g->varying ? g->up : nullptr, g->down, g->left, g->right,
                                       g->stream);
    g->built = rc == GCFG_OK;
    return rc;
}

gcfg_status gcfg_init(int w, int h, const int32_t *dp, const int32_t *dn, int32_t penalty,
                      const int32_t *up, const int32_t *down, const int32_t *left,
                      const int32_t *right, gcfg_graph **out) {
    if (!out || w <= 0 || h <= 0 || (long long)w * h > (1LL << 31) - 1) return GCFG_ERR_INVALID;
    if (penalty < 0 || penalty > GCFG_MAX_CAP) return GCFG_ERR_INVALID;
    gcfg_graph *g = new gcfg_graph();
    g->W = w;
    g->H = h;
    gcfg_status rc = solver_alloc(g->s, w, h);
    if (rc == GCFG_OK && cudaMalloc(&g->d_label, (size_t)w * h * sizeof(int32_t)) != cudaSuccess)
        rc = GCFG_ERR_OOM;
    if (rc) {
        solver_free(g->s);
        cudaFree(g->d_label);
        delete g;
        return rc;
    }
    g->penalty = penalty;
    if (dp) {
        gcfg_set_dataterms(g, dp, dn);
        if (up) gcfg_set_edges(g, up, down, left, right);
        rc = gcfg_set_graph(g);
        if (rc) {
            solver_free(g->s);
            cudaFree(g->d_label);
            delete g;
            return rc;
        }
    }
    *out = g;
    return GCFG_OK;
}

gcfg_status gcfg_set_stream(gcfg_graph *g, void *stream) {
    if (!g) return GCFG_ERR_INVALID;
    g->stream = (cudaStream_t)stream;
    return GCFG_OK;
}

gcfg_status gcfg_set_schedule(gcfg_graph *g, int push_rounds_per_gr, int max_tile_sweeps) {
    if (!g || push_rounds_per_gr < 1 || max_tile_sweeps < 1) return GCFG_ERR_INVALID;
    g->push_rounds = push_rounds_per_gr;
    g->max_sweeps = max_tile_sweeps;
    return GCFG_OK;
}

gcfg_status gcfg_optimize(gcfg_graph *g, int32_t *host_label, gcfg_result *res) {
    if (!g) return GCFG_ERR_INVALID;
    if (!g->built) return GCFG_ERR_STATE;
    GraphDev v = solver_view(g->s, g->W, g->H);
    gcfg_status rc = solve(g->s, v, g->stream, g->push_rounds, g->max_sweeps, res);
    // The graph is consumed in place, as in the reference: re-solving needs
    // gcfg_set_graph again.
    g->built = false;
    if (rc) return rc;
    if (host_label) {
        rc = extract(v, nullptr, nullptr, g->d_label, g->stream);
        if (rc) return rc;
        GCFG_CK(cudaMemcpyAsync(host_label, g->d_label, (size_t)g->W * g->H * sizeof(int32_t),
                                cudaMemcpyDeviceToHost, g->stream));
        GCFG_CK(cudaStreamSynchronize(g->stream));
    }
    return GCFG_OK;
}

gcfg_status gcfg_get_cuts(gcfg_graph *g, uint8_t *d_smin, uint8_t *d_smax) {
    if (!g) return GCFG_ERR_INVALID;
    GraphDev v = solver_view(g->s, g->W, g->H);
    gcfg_status rc = extract(v, d_smin, d_smax, nullptr, g->stream);
    if (rc) return rc;
    GCFG_CK(cudaStreamSynchronize(g->stream));
    return GCFG_OK;
}

gcfg_status gcfg_end(gcfg_graph *g) {
    if (!g) return GCFG_ERR_INVALID;
    solver_free(g->s);
    cudaFree(g->d_label);
    delete g;
    return GCFG_OK;
}

const char *gcfg_strerror(gcfg_status s) {
    switch (s) {
    case GCFG_OK: return "ok";
    case GCFG_ERR_INVALID: return "invalid argument";
    case GCFG_ERR_OOM: return "out of device memory";
    case GCFG_ERR_CUDA: return "CUDA error";
    case GCFG_ERR_NOT_CONVERGED: return "iteration cap reached";
    case GCFG_ERR_STATE: return "call out of order";
    case GCFG_ERR_CAPACITY: return "admission refused: memory cap";
    }
    return "unknown";
}

int64_t gcfg_launch_count(void) { return g_launches.load(); }

}  // extern "C"
