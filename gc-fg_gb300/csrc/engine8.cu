// engine8.cu -- graphs with the 8-neighbourhood (the reference built with
// NEIGHBORHOOD == 8: GraphCut.h:22, the #if NEIGHBORHOOD == 8 blocks of
// GraphCut.cu and GraphCutKernels.cu).
//
// A separate engine from the tiled 4-neighbour solver, so that the latter
// keeps its layout and tuning.  Pixels are row-major; the residual
// capacities are eight planes, cap[d * n + i] from pixel i toward direction
// d (0 left, 1 right, 2 up, 3 down, 4 up-left, 5 up-right, 6 down-left,
// 7 down-right).  One cooperative launch runs the whole solve:
//   * exact global relabel: the distances to the sink-connected pixels
//     (excess < 0) over the residual edges, by Bellman-Ford rounds over
//     32x32 tiles, each tile relaxed to its fixpoint in shared memory
//     (gr8_tile);
//   * count: pixels with excess that can still reach the sink; none left
//     after an exact global relabel means the preflow is maximum (an exact
//     termination test);
//   * tile rounds: every 32x8 tile once per round, each visit a few
//     block-local push/relabel sweeps in shared memory (tile8_visit), the
//     results added back as deltas;
//   * cuts: S_max = pixels at height INF after the last exact global
//     relabel, S_min = the forward closure of the pixels with excess, by
//     rounds over 32x32 tiles like the global relabel (reach8_tile).
// Every spin is bounded; a timeout or an iteration cap sets an error that
// the host reports as GCFG_ERR_NOT_CONVERGED.
#include <cstring>

#include "engine.cuh"

namespace gcfg {
namespace {

constexpr int ND = 8;
__device__ __forceinline__ int dxd(int d) { return d == 0 || d == 4 || d == 6 ? -1 : (d == 1 || d == 5 || d == 7 ? 1 : 0); }
__device__ __forceinline__ int dyd(int d) { return d == 2 || d == 4 || d == 5 ? -1 : (d == 3 || d == 6 || d == 7 ? 1 : 0); }
__device__ __forceinline__ int opp(int d) { return d < 4 ? (d ^ 1) : 11 - d; }

struct Ctl8 {
    unsigned bar_count, bar_gen;
    int err, err_code;
    int round_active[3];  // tiles that had work (or changed a height) in round p, at [p % 3]
    unsigned long long active, pos_excess, interior_dp, ref_init;
    unsigned long long tile_visits;  // push visits of tiles that had work
    int global_relabels, tile_rounds, gr_rounds, reach_rounds;
};

struct G8 {
    int W, H;
    long long n;
    int *cap;  // 8 * n
    int *e, *h, *mark;
    Ctl8 *ctl;
};

struct P8 {
    int max_outer;   // global relabels at most
    int rounds;      // tile rounds between global relabels
    int sweeps;      // push/relabel sweeps per tile visit
};

enum { E8_BARRIER = 1, E8_OUTER = 2 };

__device__ __forceinline__ void set_err8(Ctl8 *c, int code) {
    atomicExch(&c->err, 1);
    atomicCAS(&c->err_code, 0, code);
}

// Grid barrier (bounded spin).
__device__ __forceinline__ unsigned atom_add_acq_rel8(unsigned *p, unsigned v) {
    unsigned old;
    asm volatile("atom.add.acq_rel.gpu.global.u32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
    return old;
}

__device__ __forceinline__ unsigned ld_acquire8(const unsigned *p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ bool sync8(Ctl8 *c) {
    __syncthreads();
    if (threadIdx.x == 0) {
        const unsigned gen = ld_acquire8(&c->bar_gen);
        if (atom_add_acq_rel8(&c->bar_count, 1u) == gridDim.x - 1) {
            c->bar_count = 0;
            atom_add_acq_rel8(&c->bar_gen, 1u);
        } else {
            unsigned long long it = 0;
            while (ld_acquire8(&c->bar_gen) == gen) {
                if (++it > (1ull << 25)) {
                    set_err8(c, E8_BARRIER);
                    break;
                }
                __nanosleep(32);
            }
        }
    }
    // thread 0's reading of the error word decides for the whole block
    return !__syncthreads_or(threadIdx.x == 0 && *(volatile int *)&c->err != 0);
}

// Graph of the reference's InitGraph / InitGraphVarEdges with NEIGHBORHOOD
// == 8 (GraphCutKernels.cu:112-214): interior pixels only, excess dp - dn,
// caps from the arrays (or the penalty), edges toward the 1-pixel border
// zeroed, diagonals included.
struct Arr8 {
    const int *a[8];  // left, right, up, down, up-left, up-right, down-left, down-right (NULL: penalty)
};

__global__ void k8_build(G8 g, const int *__restrict__ dp, const int *__restrict__ dn, int penalty, Arr8 arr) {
    const long long w32 = (long long)((g.W + 31) / 32) * 32;
    unsigned long long idp = 0, rinit = 0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < g.n; i += (long long)gridDim.x * blockDim.x) {
        const int x = (int)(i % g.W), y = (int)(i / g.W);
        const bool inside = x > 0 && y > 0 && x < g.W - 1 && y < g.H - 1;
        const int vdp = dp[i];
        if ((long long)x + (long long)y * w32 < g.n && vdp > 0) rinit += (unsigned)vdp;
        int e = 0;
        if (inside) {
            e = vdp - dn[i];
            idp += (unsigned)vdp;
            if (vdp < 0 || dn[i] < 0 || vdp > GCFG_MAX_CAP8 || dn[i] > GCFG_MAX_CAP8) set_err8(g.ctl, 9);
        }
        for (int d = 0; d < ND; ++d) {
            int c = 0;
            if (inside) {
                c = arr.a[0] ? arr.a[d][i] : penalty;
                if (c < 0 || c > GCFG_MAX_CAP8) set_err8(g.ctl, 9);
                const int xx = x + dxd(d), yy = y + dyd(d);
                if (xx < 1 || yy < 1 || xx > g.W - 2 || yy > g.H - 2) c = 0;  // toward the border ring
            }
            g.cap[(long long)d * g.n + i] = c;
        }
        g.e[i] = e;
    }
    // one atomic per warp and counter: per-thread atomics on these two
    // addresses serialise in L2 (about 0.4 ms for a 640x480 graph)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        idp += __shfl_down_sync(0xffffffffu, idp, o);
        rinit += __shfl_down_sync(0xffffffffu, rinit, o);
    }
    if ((threadIdx.x & 31) == 0) {
        if (idp) atomicAdd(&g.ctl->interior_dp, idp);
        if (rinit) atomicAdd(&g.ctl->ref_init, rinit);
    }
}

// One push visit of a 32x8 tile (one pixel per thread): the tile's
// capacities, excess and heights and a one-pixel ring of heights (corners
// included) are staged in shared memory, up to `sweeps` push/relabel sweeps
// run with block barriers only, and the results go back as additive deltas.
// A tile without a pixel that has excess and a finite height is left after
// reading its excess and heights (returns false).
// Every tile of the image is visited concurrently in a round, so a tile's
// ring heights are a snapshot and its neighbours change its pixels meanwhile;
// that stays safe because every concurrent update is an addition: a pixel's
// own capacity toward a neighbour falls only by its own pushes (never more
// than the value it read, which others can only have raised), excess falls
// only by its owner's pushes, and flow into another tile is added with
// global atomics to the receiver's excess and reverse capacity.  Heights are
// written only by their owner.  Stale ring heights can only make labels
// inexact, never a flow invalid; the exact global relabel and its count
// decide termination.
constexpr int T8W = 32, T8H = 8;
#ifndef GCFG_N8_ROUNDS
#define GCFG_N8_ROUNDS 12   // tile rounds between global relabels
#endif
#ifndef GCFG_N8_SWEEPS
#define GCFG_N8_SWEEPS 8    // sweeps per tile visit
#endif
__device__ bool tile8_visit(const G8 &g, int t, int tiles_x, int sweeps) {
    __shared__ int sh[T8H + 2][T8W + 2];
    __shared__ int se[T8H][T8W];
    __shared__ int sc[ND][T8H][T8W];
    const int lx = threadIdx.x & 31, ly = threadIdx.x >> 5;
    const int x = (t % tiles_x) * T8W + lx, y = (t / tiles_x) * T8H + ly;
    const bool inb = x < g.W && y < g.H;
    const long long i = (long long)y * g.W + x;
    const int e0 = inb ? g.e[i] : 0;
    int hh = inb ? g.h[i] : INF_H;
    if (!__syncthreads_or(e0 > 0 && hh < INF_H)) return false;  // nothing to push here
    int c0[ND];
#pragma unroll
    for (int d = 0; d < ND; ++d) {
        c0[d] = inb ? g.cap[(long long)d * g.n + i] : 0;
        sc[d][ly][lx] = c0[d];
    }
    se[ly][lx] = e0;
    auto hat = [&](int xx, int yy) -> int {
        return xx >= 0 && yy >= 0 && xx < g.W && yy < g.H ? g.h[(long long)yy * g.W + xx] : INF_H;
    };
    sh[ly + 1][lx + 1] = hh;
    if (ly == 0) sh[0][lx + 1] = hat(x, y - 1);
    if (ly == T8H - 1) sh[T8H + 1][lx + 1] = hat(x, y + 1);
    if (lx == 0) sh[ly + 1][0] = hat(x - 1, y);
    if (lx == T8W - 1) sh[ly + 1][T8W + 1] = hat(x + 1, y);
    if (lx == 0 && ly == 0) sh[0][0] = hat(x - 1, y - 1);
    if (lx == T8W - 1 && ly == 0) sh[0][T8W + 1] = hat(x + 1, y - 1);
    if (lx == 0 && ly == T8H - 1) sh[T8H + 1][0] = hat(x - 1, y + 1);
    if (lx == T8W - 1 && ly == T8H - 1) sh[T8H + 1][T8W + 1] = hat(x + 1, y + 1);
    __syncthreads();
    for (int s = 0; s < sweeps; ++s) {
        // push half: heights fixed
        bool pushed = false;
        int e = se[ly][lx];
        if (e > 0 && hh < INF_H) {
            const int e_in = e;
#pragma unroll
            for (int d = 0; d < ND; ++d) {
                const int dx = dxd(d), dy = dyd(d);
                const int cd = sc[d][ly][lx];
                if (e <= 0 || cd <= 0 || sh[ly + 1 + dy][lx + 1 + dx] != hh - 1) continue;
                const int f = min(e, cd);
                sc[d][ly][lx] = cd - f;
                e -= f;
                const int nx = lx + dx, ny = ly + dy;
                if (nx >= 0 && ny >= 0 && nx < T8W && ny < T8H) {
                    atomicAdd(&se[ny][nx], f);
                    atomicAdd(&sc[opp(d)][ny][nx], f);
                } else {
                    const long long j = (long long)(y + dy) * g.W + (x + dx);
                    atomicAdd(&g.e[j], f);
                    atomicAdd(&g.cap[(long long)opp(d) * g.n + j], f);
                }
            }
            if (e != e_in) {
                atomicSub(&se[ly][lx], e_in - e);
                pushed = true;
            }
        }
        __syncthreads_or(pushed);
        // relabel half: capacities and excess fixed
        e = se[ly][lx];
        if (e > 0 && hh < INF_H) {
            int m = INF_H;
#pragma unroll
            for (int d = 0; d < ND; ++d)
                if (sc[d][ly][lx] > 0) m = min(m, sh[ly + 1 + dyd(d)][lx + 1 + dxd(d)]);
            if (m >= hh) {
                hh = m >= INF_H - 1 ? INF_H : m + 1;
                sh[ly + 1][lx + 1] = hh;
            }
        }
        if (!__syncthreads_or(e > 0 && hh < INF_H)) break;
    }
    if (inb) {
        g.h[i] = hh;
        const int de = se[ly][lx] - e0;
        if (de) atomicAdd(&g.e[i], de);
#pragma unroll
        for (int d = 0; d < ND; ++d) {
            const int dc = sc[d][ly][lx] - c0[d];
            if (dc) atomicAdd(&g.cap[(long long)d * g.n + i], dc);
        }
    }
    __syncthreads();  // the shared arrays are reused by the block's next tile
    return true;
}

// ---- exact global relabel: Bellman-Ford rounds over 32x32 tiles ----
// Heights are 1 on the sink-connected pixels (excess < 0) and otherwise
// 1 + the fewest residual edges to one of them (INF when there is none), as a
// frontier BFS from those pixels would give.  A round visits every tile once:
// the tile's heights and a ring of its neighbours' heights go to shared
// memory, h(u) = min(h(u), 1 + min over residual u -> v of h(v)) is swept to
// the tile's fixpoint, and the heights go back.  Every height ever written is
// the length of a real path to the sink (or INF), so a neighbour that reads a
// height mid-round reads a valid upper bound; a round in which no tile
// changed a height leaves every residual edge with h(u) <= h(v) + 1, which
// with those upper bounds makes every height exact.  A shortest path about
// as long as a tile side crosses few tiles, so a relabel takes a few rounds
// (grid barriers) where a level-synchronous BFS takes one per level.
constexpr int G8W = 32, G8H = 32;
constexpr int G8_ROWS = G8H / 8;  // rows per thread (256 threads)

// first: the stored heights are stale, so every height starts from the seed
// (1 if excess < 0, else INF) and the ring reads seeds from the excess too.
// Returns whether a height of the tile ended below its value at the start of
// the visit (the value a neighbour may have read).
__device__ bool gr8_tile(const G8 &g, int t, int tiles_x, bool first) {
    __shared__ int gh[G8H + 2][G8W + 2];
    const int lx = threadIdx.x & 31, wy = threadIdx.x >> 5;
    const int x0 = (t % tiles_x) * G8W, y0 = (t / tiles_x) * G8H;
    auto outside = [&](int xx, int yy) { return xx < 0 || yy < 0 || xx >= g.W || yy >= g.H; };
    auto height = [&](long long j) -> int {
        return first ? (g.e[j] < 0 ? 1 : INF_H) : *(volatile const int *)&g.h[j];
    };
    auto ring = [&](int xx, int yy) -> int {
        return outside(xx, yy) ? INF_H : height((long long)yy * g.W + xx);
    };
    unsigned rm[G8_ROWS];  // residual directions of this thread's pixels (bit d: cap toward d > 0)
    int h0[G8_ROWS];
#pragma unroll
    for (int k = 0; k < G8_ROWS; ++k) {
        const int ly = wy + 8 * k, x = x0 + lx, y = y0 + ly;
        int hv = INF_H;
        unsigned m = 0;
        if (!outside(x, y)) {
            const long long i = (long long)y * g.W + x;
            hv = height(i);
            if (hv != 1) {
#pragma unroll
                for (int d = 0; d < ND; ++d) m |= (g.cap[(long long)d * g.n + i] > 0 ? 1u : 0u) << d;
            }
        }
        rm[k] = m;
        h0[k] = hv;
        gh[ly + 1][lx + 1] = hv;
    }
    if (wy == 0) gh[0][lx + 1] = ring(x0 + lx, y0 - 1);
    if (wy == 1) gh[G8H + 1][lx + 1] = ring(x0 + lx, y0 + G8H);
    if (wy == 2) gh[lx + 1][0] = ring(x0 - 1, y0 + lx);
    if (wy == 3) gh[lx + 1][G8W + 1] = ring(x0 + G8W, y0 + lx);
    if (wy == 4 && lx < 4) {
        const int cx = lx & 1 ? G8W + 1 : 0, cy = lx & 2 ? G8H + 1 : 0;
        gh[cy][cx] = ring(x0 - 1 + cx, y0 - 1 + cy);
    }
    __syncthreads();
    // A tile's fixpoint takes at most one sweep per pixel of the tile (plus
    // the sweep that sees no change); a visit that stops at the bound has
    // changed heights, so another round follows.
    for (int s = 0; s <= G8W * G8H; ++s) {
        bool ch = false;
#pragma unroll
        for (int k = 0; k < G8_ROWS; ++k) {
            if (!rm[k]) continue;
            const int ly = wy + 8 * k;
            int m = INF_H;
#pragma unroll
            for (int d = 0; d < ND; ++d)
                if ((rm[k] >> d) & 1u) m = min(m, gh[ly + 1 + dyd(d)][lx + 1 + dxd(d)]);
            const int nh = m >= INF_H - 1 ? INF_H : m + 1;
            if (nh < gh[ly + 1][lx + 1]) {
                gh[ly + 1][lx + 1] = nh;
                ch = true;
            }
        }
        if (!__syncthreads_or(ch)) break;
    }
    bool changed = false;
#pragma unroll
    for (int k = 0; k < G8_ROWS; ++k) {
        const int ly = wy + 8 * k, x = x0 + lx, y = y0 + ly;
        if (outside(x, y)) continue;
        const int hv = gh[ly + 1][lx + 1];
        if (first || hv != h0[k]) g.h[(long long)y * g.W + x] = hv;
        changed |= hv != h0[k];
    }
    return __syncthreads_or(changed);  // also: gh is reused by the block's next tile
}

// ---- the source-side closure (S_min) by rounds over 32x32 tiles ----
// Marks start on the pixels with excess > 0; a visit stages the marks of the
// tile and its ring, spreads them along the residual edges of the tile's
// pixels (inside the tile and onto the ring) until nothing changes, and
// writes the new marks back, ring pixels included (their own tile spreads
// them in a later round).  Marks only ever go from 0 to 1, so a round in
// which no visit wrote a mark leaves every residual edge out of a marked
// pixel ending at a marked pixel: the marks are the closure.  Returns
// whether the visit wrote a mark.
__device__ bool reach8_tile(const G8 &g, int t, int tiles_x) {
    __shared__ int gm[G8H + 2][G8W + 2];
    const int lx = threadIdx.x & 31, wy = threadIdx.x >> 5;
    const int x0 = (t % tiles_x) * G8W, y0 = (t / tiles_x) * G8H;
    auto outside = [&](int xx, int yy) { return xx < 0 || yy < 0 || xx >= g.W || yy >= g.H; };
    // a cell outside the image counts as marked, so that nothing is written there
    auto mark_at = [&](int xx, int yy) -> int {
        return outside(xx, yy) ? 1 : *(volatile const int *)&g.mark[(long long)yy * g.W + xx];
    };
    unsigned rm[G8_ROWS];
    int m0[G8_ROWS];
#pragma unroll
    for (int k = 0; k < G8_ROWS; ++k) {
        const int ly = wy + 8 * k, x = x0 + lx, y = y0 + ly;
        const int mv = mark_at(x, y);
        unsigned m = 0;
        if (!outside(x, y)) {
            const long long i = (long long)y * g.W + x;
#pragma unroll
            for (int d = 0; d < ND; ++d) m |= (g.cap[(long long)d * g.n + i] > 0 ? 1u : 0u) << d;
        }
        rm[k] = m;
        m0[k] = mv;
        gm[ly + 1][lx + 1] = mv;
    }
    // the ring: warps 0-3 one side each, warp 4 the corners; each keeps what it read
    int rx = 0, ry = 0, r0 = 1;
    if (wy < 4 || (wy == 4 && lx < 4)) {
        if (wy == 0) { rx = lx + 1; ry = 0; }
        else if (wy == 1) { rx = lx + 1; ry = G8H + 1; }
        else if (wy == 2) { rx = 0; ry = lx + 1; }
        else if (wy == 3) { rx = G8W + 1; ry = lx + 1; }
        else { rx = lx & 1 ? G8W + 1 : 0; ry = lx & 2 ? G8H + 1 : 0; }
        r0 = mark_at(x0 - 1 + rx, y0 - 1 + ry);
        gm[ry][rx] = r0;
    }
    __syncthreads();
    // each sweep that changes something marks a new cell of the tile or ring
    for (int s = 0; s <= (G8W + 2) * (G8H + 2); ++s) {
        bool ch = false;
#pragma unroll
        for (int k = 0; k < G8_ROWS; ++k) {
            const int ly = wy + 8 * k;
            if (!rm[k] || !gm[ly + 1][lx + 1]) continue;
#pragma unroll
            for (int d = 0; d < ND; ++d) {
                if (!((rm[k] >> d) & 1u)) continue;
                int *cell = &gm[ly + 1 + dyd(d)][lx + 1 + dxd(d)];
                if (!*cell) {
                    *cell = 1;
                    ch = true;
                }
            }
        }
        if (!__syncthreads_or(ch)) break;
    }
    bool wrote = false;
#pragma unroll
    for (int k = 0; k < G8_ROWS; ++k) {
        const int ly = wy + 8 * k, x = x0 + lx, y = y0 + ly;
        if (!m0[k] && gm[ly + 1][lx + 1]) {  // m0 is 1 outside the image
            g.mark[(long long)y * g.W + x] = 1;
            wrote = true;
        }
    }
    if (!r0 && gm[ry][rx]) {  // r0 is 1 for threads without a ring cell and outside the image
        g.mark[(long long)(y0 - 1 + ry) * g.W + (x0 - 1 + rx)] = 1;
        wrote = true;
    }
    return __syncthreads_or(wrote);  // also: gm is reused by the block's next tile
}

__global__ void __launch_bounds__(256) k8_solve(G8 g, P8 prm) {
    Ctl8 *c = g.ctl;
    const long long gtid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const long long nth = (long long)gridDim.x * blockDim.x;
    bool finished = false;
    int R = 0;  // tile and relabel rounds so far in this solve (grid-uniform)
    const int gtiles_x = (g.W + G8W - 1) / G8W;
    const int gtiles = gtiles_x * ((g.H + G8H - 1) / G8H);
    for (int outer = 0; outer < prm.max_outer; ++outer) {
        // ---- exact global relabel (gr8_tile rounds) ----
        // The round counters are the tile rounds' (round_active, R), with the
        // same clearing rule.
        for (int q = 0;; ++q) {
            if (gtid == 0) {
                c->round_active[(R + 1) % 3] = 0;
                if (q == 0) c->active = 0;
            }
            int changed = 0;
            for (int t = blockIdx.x; t < gtiles; t += gridDim.x) changed += gr8_tile(g, t, gtiles_x, q == 0);
            if (threadIdx.x == 0 && changed) atomicAdd(&c->round_active[R % 3], changed);
            if (gtid == 0) c->gr_rounds++;
            if (!sync8(c)) return;
            const int more = *(volatile int *)&c->round_active[R % 3];
            ++R;
            if (!more) break;
            if (q > g.n) {  // unreachable: a round makes at least one more path segment exact
                if (gtid == 0) set_err8(c, E8_OUTER);
                return;
            }
        }
        if (gtid == 0) c->global_relabels++;
        // ---- count: excess that can still reach the sink ----
        // one atomic per warp: per-thread atomics on one address serialise in L2
        unsigned act = 0;
        for (long long i = gtid; i < g.n; i += nth) act += g.e[i] > 0 && g.h[i] < INF_H;
        act = __reduce_add_sync(0xffffffffu, act);
        if ((threadIdx.x & 31) == 0 && act) atomicAdd(&c->active, (unsigned long long)act);
        if (!sync8(c)) return;
        if (*(volatile unsigned long long *)&c->active == 0) {
            finished = true;
            break;
        }
        // ---- tile rounds: every tile once per round, block-local sweeps ----
        const int tiles_x = (g.W + T8W - 1) / T8W;
        const int ntiles = tiles_x * ((g.H + T8H - 1) / T8H);
        for (int p = 0; p < prm.rounds; ++p) {
            // round_active[R % 3] counts this round's tiles with work and is read
            // after the round's barrier; the counter of round R + 1 was last read
            // after the barrier of round R - 2, which every block has passed
            if (gtid == 0) c->round_active[(R + 1) % 3] = 0;
            int worked = 0;
            for (int t = blockIdx.x; t < ntiles; t += gridDim.x) worked += tile8_visit(g, t, tiles_x, prm.sweeps);
            if (threadIdx.x == 0 && worked) {
                atomicAdd(&c->round_active[R % 3], worked);
                atomicAdd(&c->tile_visits, (unsigned long long)worked);
            }
            if (gtid == 0) c->tile_rounds++;
            if (!sync8(c)) return;
            const int done_round = *(volatile int *)&c->round_active[R % 3] == 0;
            ++R;
            if (done_round) break;  // nothing left to push: relabel
        }
    }
    if (!finished) {
        if (gtid == 0) set_err8(c, E8_OUTER);
        return;
    }
    // ---- final positive excess and the source-side closure (S_min) ----
    unsigned long long pos = 0;
    for (long long i = gtid; i < g.n; i += nth) {
        const int e = g.e[i];
        if (e > 0) pos += (unsigned)e;
        g.mark[i] = e > 0;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) pos += __shfl_down_sync(0xffffffffu, pos, o);
    if ((threadIdx.x & 31) == 0 && pos) atomicAdd(&c->pos_excess, pos);
    if (!sync8(c)) return;
    if (*(volatile unsigned long long *)&c->pos_excess == 0) return;  // nothing marked: S_min is empty
    for (int q = 0;; ++q) {
        if (gtid == 0) c->round_active[(R + 1) % 3] = 0;
        int changed = 0;
        for (int t = blockIdx.x; t < gtiles; t += gridDim.x) changed += reach8_tile(g, t, gtiles_x);
        if (threadIdx.x == 0 && changed) atomicAdd(&c->round_active[R % 3], changed);
        if (gtid == 0) c->reach_rounds++;
        if (!sync8(c)) return;
        const int more = *(volatile int *)&c->round_active[R % 3];
        ++R;
        if (!more) break;
        if (q > g.n) {  // unreachable: every round but the last marks at least one more pixel
            if (gtid == 0) set_err8(c, E8_OUTER);
            return;
        }
    }
}

__global__ void k8_extract(G8 g, int *label, uint8_t *smin, uint8_t *smax) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < g.n; i += (long long)gridDim.x * blockDim.x) {
        const int x = (int)(i % g.W), y = (int)(i / g.W);
        const bool inside = x > 0 && y > 0 && x < g.W - 1 && y < g.H - 1;
        const int s = inside && g.h[i] >= INF_H;
        if (label) label[i] = s;
        if (smax) smax[i] = (uint8_t)s;
        if (smin) smin[i] = (uint8_t)g.mark[i];
    }
}

int grid8(long long n) {
    long long b = (n + 255) / 256;
    return (int)(b < 4096 ? (b > 0 ? b : 1) : 4096);
}

}  // namespace
}  // namespace gcfg

using namespace gcfg;

struct gcfg_graph8 {
    int W = 0, H = 0;
    long long n = 0;
    const int32_t *dp = nullptr, *dn = nullptr;
    const int32_t *arr[8] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    int32_t penalty = 0;
    bool varying = false, built = false, solved = false;
    int *cap = nullptr, *e = nullptr, *h = nullptr, *mark = nullptr;
    int32_t *d_label = nullptr;
    Ctl8 *ctl = nullptr, *h_ctl = nullptr;
    cudaStream_t st = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr, ev2 = nullptr;  // solve start, solve end, extract end
    // schedule (measured on a 640x480 graph with a constant penalty of 600,
    // 8 sweeps per visit, solve kernel time: 12 tile rounds per global
    // relabel take 0.96 ms at 3 blocks per SM and 1.03 ms at 2; 8 rounds
    // 0.99 ms, 16 rounds 1.05 ms, 32 rounds 1.17 ms, 4 rounds 1.20 ms)
    int rounds = GCFG_N8_ROUNDS, max_outer = 100000, blocks_per_sm = 3, sweeps = GCFG_N8_SWEEPS;

    G8 g() const {
        G8 x;
        x.W = W;
        x.H = H;
        x.n = n;
        x.cap = cap;
        x.e = e;
        x.h = h;
        x.mark = mark;
        x.ctl = ctl;
        return x;
    }
    void release() {
        cudaFree(cap); cudaFree(e); cudaFree(h); cudaFree(mark);
        cudaFree(d_label); cudaFree(ctl);
        if (h_ctl) cudaFreeHost(h_ctl);
        if (ev0) cudaEventDestroy(ev0);
        if (ev1) cudaEventDestroy(ev1);
        if (ev2) cudaEventDestroy(ev2);
    }
};

extern "C" {

gcfg_status gcfg_set_dataterms8(gcfg_graph8 *g, const int32_t *dp, const int32_t *dn) {
    if (!g) return GCFG_ERR_INVALID;
    g->dp = dp;
    g->dn = dn;
    g->built = false;
    return GCFG_OK;
}

gcfg_status gcfg_set_edges8(gcfg_graph8 *g, const int32_t *up, const int32_t *down, const int32_t *left,
                            const int32_t *right, const int32_t *upleft, const int32_t *upright,
                            const int32_t *downleft, const int32_t *downright) {
    if (!g || !up || !down || !left || !right || !upleft || !upright || !downleft || !downright)
        return GCFG_ERR_INVALID;
    const int32_t *a[8] = {left, right, up, down, upleft, upright, downleft, downright};
    memcpy(g->arr, a, sizeof(a));
    g->varying = true;
    g->built = false;
    return GCFG_OK;
}

gcfg_status gcfg_set_penalty8(gcfg_graph8 *g, int32_t penalty) {
    if (!g || penalty < 0 || penalty > GCFG_MAX_CAP8) return GCFG_ERR_INVALID;
    g->penalty = penalty;
    g->varying = false;
    g->built = false;
    return GCFG_OK;
}

gcfg_status gcfg_set_schedule8(gcfg_graph8 *g, int rounds_per_gr, int blocks_per_sm) {
    if (!g || rounds_per_gr < 1 || blocks_per_sm < 0) return GCFG_ERR_INVALID;
    g->rounds = rounds_per_gr;
    g->blocks_per_sm = blocks_per_sm;
    return GCFG_OK;
}

gcfg_status gcfg_set_stream8(gcfg_graph8 *g, void *stream) {
    if (!g) return GCFG_ERR_INVALID;
    g->st = (cudaStream_t)stream;
    return GCFG_OK;
}

gcfg_status gcfg_set_graph8(gcfg_graph8 *g) {
    if (!g || !g->dp || !g->dn) return GCFG_ERR_STATE;
    GCFG_CK(cudaMemsetAsync(g->ctl, 0, sizeof(Ctl8), g->st));
    Arr8 arr;
    for (int d = 0; d < 8; ++d) arr.a[d] = g->varying ? g->arr[d] : nullptr;
    k8_build<<<grid8(g->n), 256, 0, g->st>>>(g->g(), g->dp, g->dn, g->penalty, arr);
    g_launches.fetch_add(1, std::memory_order_relaxed);
    GCFG_CK(cudaGetLastError());
    GCFG_CK(cudaMemcpyAsync(g->h_ctl, g->ctl, sizeof(Ctl8), cudaMemcpyDeviceToHost, g->st));
    GCFG_CK(cudaStreamSynchronize(g->st));
    if (g->h_ctl->err) return GCFG_ERR_INVALID;  // capacities outside [0, GCFG_MAX_CAP8]
    g->built = true;
    g->solved = false;
    return GCFG_OK;
}

gcfg_status gcfg_init8(int w, int h, const int32_t *dp, const int32_t *dn, int32_t penalty, const int32_t *up,
                       const int32_t *down, const int32_t *left, const int32_t *right, const int32_t *upleft,
                       const int32_t *upright, const int32_t *downleft, const int32_t *downright,
                       gcfg_graph8 **out) {
    if (!out || w <= 0 || h <= 0 || (long long)w * h > (1LL << 31) - 1) return GCFG_ERR_INVALID;
    if (penalty < 0 || penalty > GCFG_MAX_CAP8) return GCFG_ERR_INVALID;
    gcfg_graph8 *g = new gcfg_graph8();
    g->W = w;
    g->H = h;
    g->n = (long long)w * h;
    g->penalty = penalty;
    const size_t n = (size_t)g->n;
    gcfg_status rc = GCFG_OK;
    if (cudaMalloc(&g->cap, 8 * n * sizeof(int)) != cudaSuccess || cudaMalloc(&g->e, n * sizeof(int)) != cudaSuccess ||
        cudaMalloc(&g->h, n * sizeof(int)) != cudaSuccess || cudaMalloc(&g->mark, n * sizeof(int)) != cudaSuccess ||
        cudaMalloc(&g->d_label, n * sizeof(int)) != cudaSuccess || cudaMalloc(&g->ctl, sizeof(Ctl8)) != cudaSuccess ||
        cudaMallocHost(&g->h_ctl, sizeof(Ctl8)) != cudaSuccess)
        rc = GCFG_ERR_OOM;
    if (rc == GCFG_OK && (cudaEventCreate(&g->ev0) != cudaSuccess || cudaEventCreate(&g->ev1) != cudaSuccess ||
                          cudaEventCreate(&g->ev2) != cudaSuccess))
        rc = GCFG_ERR_CUDA;
    if (rc == GCFG_OK && dp) {
        gcfg_set_dataterms8(g, dp, dn);
        if (up) rc = gcfg_set_edges8(g, up, down, left, right, upleft, upright, downleft, downright);
        if (rc == GCFG_OK) rc = gcfg_set_graph8(g);
    }
    if (rc) {
        g->release();
        delete g;
        return rc;
    }
    *out = g;
    return GCFG_OK;
}

gcfg_status gcfg_optimize8(gcfg_graph8 *g, int32_t *host_label, gcfg_result *res) {
    if (!g) return GCFG_ERR_INVALID;
    if (!g->built) return GCFG_ERR_STATE;
    int per_sm = 0, sms = 0, dev = 0;
    GCFG_CK(cudaGetDevice(&dev));
    GCFG_CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    GCFG_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k8_solve, 256, 0));
    long long want = (g->n + 255) / 256;
    if (g->blocks_per_sm > 0 && g->blocks_per_sm < per_sm) per_sm = g->blocks_per_sm;
    long long grid = (long long)(per_sm > 0 ? per_sm : 1) * (sms > 0 ? sms : 1);
    if (want < grid) grid = want > 0 ? want : 1;
    G8 gg = g->g();
    P8 prm{g->max_outer, g->rounds, g->sweeps};
    void *args[] = {&gg, &prm};
    GCFG_CK(cudaEventRecord(g->ev0, g->st));
    GCFG_CK(cudaLaunchCooperativeKernel((const void *)k8_solve, dim3((unsigned)grid), dim3(256), args, 0, g->st));
    g_launches.fetch_add(1, std::memory_order_relaxed);
    GCFG_CK(cudaEventRecord(g->ev1, g->st));
    k8_extract<<<grid8(g->n), 256, 0, g->st>>>(gg, g->d_label, nullptr, nullptr);
    g_launches.fetch_add(1, std::memory_order_relaxed);
    GCFG_CK(cudaGetLastError());
    GCFG_CK(cudaEventRecord(g->ev2, g->st));
    if (host_label)
        GCFG_CK(cudaMemcpyAsync(host_label, g->d_label, (size_t)g->n * sizeof(int32_t), cudaMemcpyDeviceToHost, g->st));
    GCFG_CK(cudaMemcpyAsync(g->h_ctl, g->ctl, sizeof(Ctl8), cudaMemcpyDeviceToHost, g->st));
    GCFG_CK(cudaStreamSynchronize(g->st));
    g->built = false;  // the graph is consumed, as in the reference
    const Ctl8 &c = *g->h_ctl;
    const gcfg_status st = c.err ? GCFG_ERR_NOT_CONVERGED : GCFG_OK;
    g->solved = st == GCFG_OK;
    if (res) {
        memset(res, 0, sizeof(*res));
        res->flow = (long long)c.interior_dp - (long long)c.pos_excess;
        res->ref_energy = (int32_t)((uint32_t)c.ref_init - (uint32_t)c.pos_excess);
        res->status = st;
        res->global_relabels = c.global_relabels;
        res->gr_sweeps = c.gr_rounds;
        res->push_rounds = c.tile_rounds;
        res->cut_sweeps = c.reach_rounds;
        res->push_tiles = (int64_t)c.tile_visits;
        res->gr_tiles = (int64_t)c.gr_rounds * (((g->W + G8W - 1) / G8W) * (long long)((g->H + G8H - 1) / G8H));
        float ms = 0.f;
        cudaEventElapsedTime(&ms, g->ev0, g->ev1);
        res->ms = ms;
    }
    return st;
}

gcfg_status gcfg_get_cuts8(gcfg_graph8 *g, uint8_t *d_smin, uint8_t *d_smax) {
    if (!g) return GCFG_ERR_INVALID;
    if (!g->solved) return GCFG_ERR_STATE;
    k8_extract<<<grid8(g->n), 256, 0, g->st>>>(g->g(), nullptr, d_smin, d_smax);
    g_launches.fetch_add(1, std::memory_order_relaxed);
    GCFG_CK(cudaGetLastError());
    GCFG_CK(cudaStreamSynchronize(g->st));
    return GCFG_OK;
}

gcfg_status gcfg_end8(gcfg_graph8 *g) {
    if (!g) return GCFG_ERR_INVALID;
    cudaStreamSynchronize(g->st);
    g->release();
    delete g;
    return GCFG_OK;
}

}  // extern "C"
