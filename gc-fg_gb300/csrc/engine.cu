// engine.cu -- persistent tile-space push-relabel solver (GB300, sm_103a).
//
// Algorithm (exact max-flow on a 4-connected grid, the reference's model):
//   excess e = dp - dn (+ inflow - outflow); heights = residual distance to
//   the sink (sink-connected nodes, e < 0, have height 1); the solve ends
//   when, after an exact global relabel, no node with e > 0 can reach the
//   sink.  Cuts: S_max = nodes that cannot reach the sink (the reference's
//   labels, GraphCutKernels.cu:228-351), S_min = nodes reachable from the
//   source (from nodes with e > 0).
//
// GPU organisation:
//   * Tile BFS: a 32x32 tile is 32 row bitmasks per residual direction; one
//     warp (lane = row) grows the BFS frontier of the whole tile with shifts,
//     warp shuffles and ballots, seeded by sink nodes (level 1) and by the
//     halo's heights.  It gives exact distances for the tile given the halo.
//   * Global relabel (GraphCutKernels.cu:757-875 does 10 Bellman-Ford steps
//     per launch with a host round trip each): tiles recompute with the tile
//     BFS until no tile border changes; a tile whose border distances
//     decrease queues its neighbours (frontier of tiles, de-duplicated).
//   * Push (GraphCutKernels.cu:433-581 WavePush + :600-724 Relabel): tiles
//     of one checkerboard colour run at a time, so a running tile's halo is
//     frozen; inside the tile, shared-memory push/relabel sweeps with an
//     exact local relabel (tile BFS against the frozen halo) every few
//     sweeps; flow pushed into the halo is handed over with atomics and the
//     receiving tile is queued for the next colour phase.
//   * Everything above runs in one cooperative persistent kernel; phases are
//     separated by a grid barrier whose spin is bounded (on timeout the
//     kernel records an error and returns).
#include <atomic>
#include <cstdio>
#include <cstring>
#include <vector>

#include "dataterm.cuh"  // CHUNK_PX: the data-term pass's chunks, reused by k_extract_rows
#include "engine.cuh"

namespace gcfg {

constexpr unsigned FULL = 0xffffffffu;
constexpr int BFS_MAX_ITERS = TPX + 4 * 32 + 8;
// lines of a tile's border array (Batch::hb, 128 ints per tile)
constexpr int HB_TOP = 0, HB_BOT = 32, HB_LFT = 64, HB_RGT = 96;
constexpr unsigned long long SPIN_LIMIT = 1ull << 25;   // about a second of polling

// ---------------------------------------------------------------------------
// helpers
// ---------------------------------------------------------------------------

struct TileGeo {
    int img, tx, ty, color;
    int nb[4];  // left, right, up, down tile (-1 at the image edge)
};

__device__ __forceinline__ TileGeo tile_geo(const Batch &b, int t) {
    TileGeo g;
    g.img = __ldg(b.tile_img + t);
    const int tile0 = __ldg(&b.img[g.img].tile0);
    const int tx_n = __ldg(&b.img[g.img].tiles_x);
    const int ty_n = __ldg(&b.img[g.img].tiles_y);
    const int lt = t - tile0;
    g.tx = lt % tx_n;
    g.ty = lt / tx_n;
    g.color = (g.tx + g.ty) & 1;
    g.nb[0] = g.tx > 0 ? t - 1 : -1;
    g.nb[1] = g.tx < tx_n - 1 ? t + 1 : -1;
    g.nb[2] = g.ty > 0 ? t - tx_n : -1;
    g.nb[3] = g.ty < ty_n - 1 ? t + tx_n : -1;
    return g;
}

// Neighbours of tile t from the per-tile table the builds fill (one load).
__device__ __forceinline__ void tile_nbs(const Batch &b, int t, int nb[4]) {
    const int4 v = __ldcg(b.tile_nb + t);
    nb[0] = v.x;
    nb[1] = v.y;
    nb[2] = v.z;
    nb[3] = v.w;
}

__device__ __forceinline__ int4 nb_of(const TileGeo &g) { return make_int4(g.nb[0], g.nb[1], g.nb[2], g.nb[3]); }

__device__ __forceinline__ void set_error(const Batch &b, int code) {
    atomicExch(&b.ctl->err, 1);
    atomicCAS(&b.ctl->err_code, 0, code);
}

// Queue tile t under `tag` in list `slot` unless it is already queued for it.
// A queue never holds a tile twice, so it cannot overflow; the bound check
// records an error instead of writing out of range should that ever fail.
__device__ __forceinline__ void enqueue(const Batch &b, int *mark, int slot, int tag, int t) {
    if (atomicMax(mark + t, tag) < tag) {
        const int pos = atomicAdd(&b.ctl->size[slot], 1);
        if (pos < b.list_cap) b.lists[(size_t)slot * b.list_cap + pos] = t;
        else set_error(b, ERRC_QUEUE);
    }
}

// Warp-collective enqueue (all 32 lanes call it): each lane with `want`
// queues its tile t as enqueue() does, and the lanes that queue something
// share one atomic on the list size.
__device__ __forceinline__ void enqueue_warp(const Batch &b, int *mark, int slot, int tag, int t, bool want) {
    const int lane = threadIdx.x & 31;
    const bool won = want && atomicMax(mark + t, tag) < tag;
    const unsigned m = __ballot_sync(0xffffffffu, won);
    if (!m) return;
    const int leader = __ffs(m) - 1;
    int base = 0;
    if (lane == leader) base = atomicAdd(&b.ctl->size[slot], __popc(m));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (won) {
        const int pos = base + __popc(m & ((1u << lane) - 1u));
        if (pos < b.list_cap) b.lists[(size_t)slot * b.list_cap + pos] = t;
        else set_error(b, ERRC_QUEUE);
    }
}

// Grid-wide barrier over the co-resident blocks of the cooperative launch.
// The last block to arrive clears the queues named in reset_mask before it
// releases the others.  The spin is bounded: on timeout the error flag is
// set and every block returns false.
__device__ __forceinline__ unsigned atom_add_acq_rel(unsigned *p, unsigned v) {
    unsigned old;
    asm volatile("atom.add.acq_rel.gpu.global.u32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
    return old;
}

__device__ __forceinline__ unsigned ld_acquire(const unsigned *p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// Thread 0 of each block arrives with an acquire-release add (after the
// block barrier, so it publishes the whole block's writes and, for the last
// arriver, acquires every other block's); the last arriver clears the queues
// and releases the others by bumping the generation, on which they spin with
// acquire loads.  (Measured 2.3 us per barrier over 608 blocks, against
// 2.9 us with full fences.)
__device__ bool grid_sync(const Batch &b, unsigned reset_mask) {
    Ctl *c = b.ctl;
    __syncthreads();
    if (threadIdx.x == 0) {
        const unsigned gen = ld_acquire(&c->bar_gen);
        const unsigned arrived = atom_add_acq_rel(&c->bar_count, 1u);
        if (arrived == gridDim.x - 1) {
            for (int s = 0; s < L_NLISTS; ++s)
                if ((reset_mask >> s) & 1u) {
                    c->size[s] = 0;
                    c->take[s] = 0;
                }
            c->bar_count = 0;
            atom_add_acq_rel(&c->bar_gen, 1u);
        } else {
            unsigned long long it = 0;
            while (ld_acquire(&c->bar_gen) == gen) {
                if (++it > SPIN_LIMIT) {
                    set_error(b, ERRC_BARRIER);
                    break;
                }
                __nanosleep(32);
            }
        }
    }
    // thread 0's reading of the error word decides for the whole block, so
    // that every thread of a block leaves (or continues) together
    return !__syncthreads_or(threadIdx.x == 0 && *(volatile int *)&c->err != 0);
}

__device__ __forceinline__ int vload(const int *p) { return *(volatile const int *)p; }

__device__ __forceinline__ unsigned long long gtimer() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Phase clock: block 0 / thread 0 charges the time since the last mark to
// one phase counter (all blocks leave a grid barrier together).
struct PhaseClock {
    unsigned long long t;
    __device__ void start() {
        if (blockIdx.x == 0 && threadIdx.x == 0) t = gtimer();
    }
    __device__ void charge(unsigned long long *slot) {
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            const unsigned long long now = gtimer();
            *slot += now - t;
            t = now;
        }
    }
};

// ---------------------------------------------------------------------------
// Bit-parallel tile BFS (one warp, lane = row)
// ---------------------------------------------------------------------------
// Rl/Rr/Ru/Rd: row masks of residual capacity toward left/right/up/down.
// sink: nodes of this row at level 1 (e < 0).
// hl/hr: level of this row's left/right halo node; ht/hb: level of the halo
// node above/below column `lane`.

// One BFS expansion: the nodes outside S that have a residual edge into S or
// into a halo node of level <= lvl (they get level lvl + 1).
__device__ __forceinline__ unsigned bfs_expand(unsigned S, int lvl, unsigned Rl, unsigned Rr, unsigned Ru,
                                               unsigned Rd, int hl, int hr, int ht, int hb, int lane) {
    const unsigned T = __ballot_sync(FULL, ht <= lvl);
    const unsigned B = __ballot_sync(FULL, hb <= lvl);
    unsigned up = __shfl_up_sync(FULL, S, 1);
    unsigned dn = __shfl_down_sync(FULL, S, 1);
    if (lane == 0) up = T;
    if (lane == 31) dn = B;
    const unsigned lin = (S << 1) | (hl <= lvl ? 1u : 0u);
    const unsigned rin = (S >> 1) | (hr <= lvl ? 0x80000000u : 0u);
    return ((Rl & lin) | (Rr & rin) | (Ru & up) | (Rd & dn)) & ~S;
}

// Smallest halo level above lvl (warp-uniform), INF when there is none.
__device__ __forceinline__ int bfs_next_halo(int lvl, int hl, int hr, int ht, int hb) {
    int cand = INF_H;
    if (hl > lvl) cand = min(cand, hl);
    if (hr > lvl) cand = min(cand, hr);
    if (ht > lvl) cand = min(cand, ht);
    if (hb > lvl) cand = min(cand, hb);
    return __reduce_min_sync(FULL, cand);
}

// The tile BFS loops below take several levels per round (lvl -> lvl + 1 ->
// ..., each expansion from the previous one's result) and decide once, so
// the loop-carried path holds one vote and one branch per round: four levels
// in tile_bfs_gr and tile_bfs_rec, two in tile_bfs_direct.  When no level of
// a round grows the frontier, the level jumps to the next halo level above
// the round's last; when only the first ones grow, the next round's
// expansions find what a jump would (the halo levels up to the round's last
// have already been used).

// Scratch of one warp's global-relabel tile BFS: the index of the expansion
// that reached each pixel, as GR_NPL bit planes per row (lane = row, bit =
// column), and the level of each index.
constexpr int GR_NPL = 7;
constexpr int GR_NIDX = 1 << GR_NPL;  // expansions per segment (the seeds are index 0)
struct GrScratch {
    unsigned pl[GR_NPL][32];  // plane b of row r: pixels whose index has bit b set
    unsigned reached[32], base[32];
    int lv[GR_NIDX];
};

// The global relabel's tile BFS with each new pixel's level stored into
// hs[row * stride + col] as it is reached (unreachable pixels get INF);
// returns this lane's row of the reached set.  Two levels per vote.  Its instruction count is small when the
// BFS is short, as in round 0 of a relabel, where most tiles hold many sinks:
// there, with every SM busy and several tiles per warp, issue bounds the round
// and this loop is the faster one (batch256 round 0: 76 us against 115 us with
// tile_bfs_gr); the divergent stores make it the slower one wherever a visit's
// latency bounds the round.
__device__ unsigned tile_bfs_direct(unsigned Rl, unsigned Rr, unsigned Ru, unsigned Rd, unsigned sink, int hl,
                         int hr, int ht, int hb, int *hs, int stride, int *iters) {
    const int lane = threadIdx.x & 31;
    int *row = hs + lane * stride;
    // INF, and level 1 on the seeds, in one uniform pass (a loop over the
    // seed bits would run as long as the row with the most seeds)
#pragma unroll 8
    for (int x = 0; x < 32; ++x) row[x] = (sink >> x) & 1u ? 1 : INF_H;
    unsigned S = sink;
    int lvl = 1;
    int it = 0;
    for (; it < BFS_MAX_ITERS; ++it) {
        unsigned nw1 = bfs_expand(S, lvl, Rl, Rr, Ru, Rd, hl, hr, ht, hb, lane);
        const unsigned S1 = S | nw1;
        unsigned nw2 = bfs_expand(S1, lvl + 1, Rl, Rr, Ru, Rd, hl, hr, ht, hb, lane);
        if (__any_sync(FULL, (nw1 | nw2) != 0)) {
            S = S1 | nw2;
            for (; nw1; nw1 &= nw1 - 1) row[__ffs(nw1) - 1] = lvl + 1;
            for (; nw2; nw2 &= nw2 - 1) row[__ffs(nw2) - 1] = lvl + 2;
            lvl += 2;
        } else {
            const int nxt = bfs_next_halo(lvl + 1, hl, hr, ht, hb);
            if (nxt >= INF_H) break;
            lvl = nxt;
        }
    }
    *iters = it;
    return S;
}

// The global relabel's tile BFS: writes the level of every pixel of the tile
// to h (the tile's 32x32 heights, row-major; INF where unreachable) and
// returns this lane's row of the reached set; vt / vb get this lane's column's
// top and bottom heights, vl / vr its row's first and last.
//
// Each expansion only ORs its new pixels into the bit planes of its index
// (the same few uniform instructions for every lane); the heights are written
// afterwards with lane = column, row by row: the planes of the row give each
// pixel's index, the index its level, and the stores are coalesced.  (Storing
// each new pixel's level as it is reached takes a loop over the new bits of
// the lane's row, which diverges: a frontier that enters the tile along a
// side reaches a whole row per level, 32 stores in a row for one lane, and a
// one-warp micro-benchmark measured 61K cycles for such a tile against 5.3K
// this way, and 4.1–6.0K against 7.4–11.1K on random tiles.)  After GR_NIDX
// expansions the levels found so far are written out and the planes start a
// new segment.
__device__ unsigned tile_bfs_gr(unsigned Rl, unsigned Rr, unsigned Ru, unsigned Rd, unsigned sink, int hl, int hr,
                                int ht, int hb, int *h, GrScratch &sc, int *iters, int &vt, int &vb, int &vl,
                                int &vr) {
    const int lane = threadIdx.x & 31;
    unsigned S = sink, base = 0u;
    unsigned P[GR_NPL];
#pragma unroll
    for (int k = 0; k < GR_NPL; ++k) P[k] = 0u;
    if (lane == 0) sc.lv[0] = 1;  // index 0: the seeds
    int nidx = 1, lvl = 1, it = 0;
    vt = vb = vl = vr = INF_H;
    // write the levels of the pixels reached in this segment (and, at the end,
    // INF for the pixels never reached)
    auto flush = [&](bool final) {
#pragma unroll
        for (int k = 0; k < GR_NPL; ++k) sc.pl[k][lane] = P[k];
        sc.reached[lane] = S;
        sc.base[lane] = base;
        {
            // this lane's row: its first and last pixel, from its own planes
            const unsigned fresh = S & ~base;
            int i0 = 0, i31 = 0;
#pragma unroll
            for (int k = 0; k < GR_NPL; ++k) {
                i0 |= (int)(P[k] & 1u) << k;
                i31 |= (int)(P[k] >> 31) << k;
            }
            const int a0 = sc.lv[i0], a31 = sc.lv[i31];
            if (fresh & 1u) vl = a0;
            if (fresh >> 31) vr = a31;
        }
        __syncwarp();
        const unsigned bit = 1u << lane;
#pragma unroll 8
        for (int r = 0; r < 32; ++r) {
            const unsigned sr = sc.reached[r], br = sc.base[r];
            int idx = 0;
#pragma unroll
            for (int k = 0; k < GR_NPL; ++k) idx |= (int)((sc.pl[k][r] >> lane) & 1u) << k;
            const bool fresh = ((sr & ~br) & bit) != 0;
            const bool wr = fresh || (final && !(sr & bit));
            const int v = fresh ? sc.lv[idx] : INF_H;
            if (wr) h[r * 32 + lane] = v;
            if (r == 0) vt = wr ? v : vt;
            if (r == 31) vb = wr ? v : vb;
        }
        __syncwarp();
#pragma unroll
        for (int k = 0; k < GR_NPL; ++k) P[k] = 0u;
        base = S;
        nidx = 0;
    };
    for (; it < BFS_MAX_ITERS; ++it) {
        const unsigned nw1 = bfs_expand(S, lvl, Rl, Rr, Ru, Rd, hl, hr, ht, hb, lane);
        const unsigned S1 = S | nw1;
        const unsigned nw2 = bfs_expand(S1, lvl + 1, Rl, Rr, Ru, Rd, hl, hr, ht, hb, lane);
        const unsigned S2 = S1 | nw2;
        const unsigned nw3 = bfs_expand(S2, lvl + 2, Rl, Rr, Ru, Rd, hl, hr, ht, hb, lane);
        const unsigned S3 = S2 | nw3;
        const unsigned nw4 = bfs_expand(S3, lvl + 3, Rl, Rr, Ru, Rd, hl, hr, ht, hb, lane);
        if (__any_sync(FULL, (nw1 | nw2 | nw3 | nw4) != 0)) {
            if (nidx + 4 > GR_NIDX) flush(false);
            const unsigned nw[4] = {nw1, nw2, nw3, nw4};
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int idx = nidx + j;  // warp-uniform
#pragma unroll
                for (int k = 0; k < GR_NPL; ++k)
                    if ((idx >> k) & 1) P[k] |= nw[j];
            }
            if (lane < 4) sc.lv[nidx + lane] = lvl + 1 + lane;
            S = S3 | nw4;
            nidx += 4;
            lvl += 4;
        } else {
            const int nxt = bfs_next_halo(lvl + 3, hl, hr, ht, hb);
            if (nxt >= INF_H) break;
            lvl = nxt;
        }
    }
    flush(true);
    *iters = it;
    return S;
}

// The push visits' exact local relabel: the same levels as tile_bfs_gr, but
// instead of storing each new pixel's level on the spot (a divergent loop on
// the loop-carried path of a single warp) every expansion records the reached
// rows, srec[row * NRS + k], and its level lv[k], while four more records
// fit (k + 4 <= NREC); later expansions store their pixels' levels directly
// in the level array hs.  sfin gets the final reached rows.  Four expansions
// (levels lvl + 1 .. lvl + 4, each from the previous one's result) share one
// vote and one branch, so the loop-carried path holds one vote per four
// levels; a level that adds nothing is recorded all the same (its record
// repeats the previous set, which the records' search tolerates).  When none
// of the four grows the frontier, the level jumps to the next halo level
// above lvl + 3.  Returns the number of records (warp-uniform); the whole
// block then fills in the heights (height_from_records).
constexpr int NREC = 64;
constexpr int NRS = NREC + 1;  // odd row stride: a warp's record stores and searches spread over the banks
__device__ int tile_bfs_rec(unsigned Rl, unsigned Rr, unsigned Ru, unsigned Rd, unsigned sink, int hl, int hr,
                            int ht, int hb, int *hs, int stride, unsigned *srec, int *lv, unsigned *sfin,
                            int *iters) {
    const int lane = threadIdx.x & 31;
    int *row = hs + lane * stride;
    unsigned *rec = srec + lane * NRS;
    unsigned S = sink;
    int lvl = 1, nrec = 0, it = 0;
    for (; it < BFS_MAX_ITERS; ++it) {
        const unsigned nw1 = bfs_expand(S, lvl, Rl, Rr, Ru, Rd, hl, hr, ht, hb, lane);
        const unsigned S1 = S | nw1;
        const unsigned nw2 = bfs_expand(S1, lvl + 1, Rl, Rr, Ru, Rd, hl, hr, ht, hb, lane);
        const unsigned S2 = S1 | nw2;
        const unsigned nw3 = bfs_expand(S2, lvl + 2, Rl, Rr, Ru, Rd, hl, hr, ht, hb, lane);
        const unsigned S3 = S2 | nw3;
        const unsigned nw4 = bfs_expand(S3, lvl + 3, Rl, Rr, Ru, Rd, hl, hr, ht, hb, lane);
        if (__any_sync(FULL, (nw1 | nw2 | nw3 | nw4) != 0)) {
            S = S3 | nw4;
            if (nrec + 4 <= NREC) {  // the usual case: the four levels recorded
                rec[nrec] = S1;
                rec[nrec + 1] = S2;
                rec[nrec + 2] = S3;
                rec[nrec + 3] = S;
                if (lane < 4) lv[nrec + lane] = lvl + 1 + lane;
                nrec += 4;
            } else {
                for (unsigned m = nw1; m; m &= m - 1) row[__ffs(m) - 1] = lvl + 1;
                for (unsigned m = nw2; m; m &= m - 1) row[__ffs(m) - 1] = lvl + 2;
                for (unsigned m = nw3; m; m &= m - 1) row[__ffs(m) - 1] = lvl + 3;
                for (unsigned m = nw4; m; m &= m - 1) row[__ffs(m) - 1] = lvl + 4;
            }
            lvl += 4;
        } else {
            const int nxt = bfs_next_halo(lvl + 3, hl, hr, ht, hb);
            if (nxt >= INF_H) break;
            lvl = nxt;
        }
    }
    sfin[lane] = S;
    *iters = it;
    return nrec;
}

// Height of pixel x of row r after tile_bfs_rec: INF outside the final
// reached set, 1 on the seeds, else the level of the first record that holds
// it, else the level stored directly by an expansion past the records.  The
// records are cumulative (a set bit stays set), so the first record holding
// the bit is found by a fixed six-step search with no loop or branch: the
// four rows a thread fills run their searches side by side.
__device__ __forceinline__ int height_from_records(int r, int x, unsigned seed, const unsigned *srec,
                                                   const int *lv, const unsigned *sfin, int nrec, int stored) {
    const unsigned *rec = srec + r * NRS;
    const bool fin = (sfin[r] >> x) & 1u;
    const bool in_rec = nrec > 0 && ((rec[nrec > 0 ? nrec - 1 : 0] >> x) & 1u);
    int pos = -1;  // the last record without the bit (-1: none)
#pragma unroll
    for (int step = NREC / 2; step >= 1; step >>= 1) {
        const int q = pos + step;
        if (q < nrec - 1 && !((rec[q] >> x) & 1u)) pos = q;
    }
    const int level = lv[pos + 1];
    return !fin ? INF_H : ((seed >> x) & 1u) ? 1 : !in_rec ? stored : level;
}

// ---------------------------------------------------------------------------
// Shared memory of the persistent kernel (phases reuse the same bytes)
// ---------------------------------------------------------------------------

// Per-block solver statistics, accumulated in shared memory with shared
// atomics and added to the Ctl counters once when the kernel ends, so that
// no tile visit issues a global atomic on a shared counter address.
enum {
    ST_PUSH_TILES, ST_GR_TILES, ST_REACH_TILES, ST_PUSH_SWEEPS, ST_PUSH_BFS,
    ST_CYC_LOAD, ST_CYC_BFS, ST_CYC_SWEEP, ST_CYC_WB, ST_CYC_TAKE,
    ST_BFS_IT_PUSH, ST_BFS_IT_GR, ST_CYC_GR, ST_N
};

__device__ __forceinline__ void stat_add(unsigned long long *st, int k, unsigned long long v) {
    atomicAdd(st + k, v);
}

__device__ __forceinline__ unsigned long long *ctl_stat(Ctl *c, int k) {
    switch (k) {
        case ST_PUSH_TILES: return &c->push_tiles;
        case ST_GR_TILES: return &c->gr_tiles;
        case ST_REACH_TILES: return &c->reach_tiles;
        case ST_PUSH_SWEEPS: return &c->push_sweeps;
        case ST_PUSH_BFS: return &c->push_bfs;
        case ST_CYC_LOAD: return &c->cyc_load;
        case ST_CYC_BFS: return &c->cyc_bfs;
        case ST_CYC_SWEEP: return &c->cyc_sweep;
        case ST_CYC_WB: return &c->cyc_wb;
        case ST_CYC_TAKE: return &c->cyc_take;
        case ST_BFS_IT_PUSH: return &c->bfs_it_push;
        case ST_BFS_IT_GR: return &c->bfs_it_gr;
        default: return &c->cyc_gr;
    }
}

template <int NW>  // warps per block
struct SmemPush {
    int4 c[TILE_H][TILE_W];
    int e[TILE_H][TILE_W];
    int h[TILE_H + 2][TILE_W + 2];
    int halo_in[4][32];
    unsigned m[5][32];  // left, right, up, down, sink row masks
    unsigned srec[32 * NRS];  // local relabel: reached rows after each recorded expansion, [row * NRS + k]
    int lv[NREC];             // and its level
    unsigned sfin[32];        // final reached rows
    int nrec;
    unsigned long long part[NW];
    int idx;
};
template <int NW>
struct SmemWarp {  // one of each per warp: the global relabel's tile BFS
    GrScratch g[NW];
    int hs[NW][32 * 33];
};
template <int NW>
union Smem {
    SmemPush<NW> p;
    SmemWarp<NW> w;
};

// ---------------------------------------------------------------------------
// Global relabel / reach (warp per tile)
// ---------------------------------------------------------------------------

// This lane's row of the six mask planes of tile t (lane = row).
__device__ __forceinline__ void load_tile_masks(const Batch &b, int t, unsigned m[6]) {
    const unsigned *base = b.tmask + (size_t)t * 6 * 32 + (threadIdx.x & 31);
#pragma unroll
    for (int k = 0; k < 6; ++k) m[k] = __ldcg(base + k * 32);
}

__device__ __forceinline__ unsigned mask_word(const Batch &b, int t, int k, int row) {
    return __ldcg(b.tmask + ((size_t)t * 6 + k) * 32 + row);
}

// Where a global-relabel tile visit starts: the tile's neighbours and whether
// its image is finished.  Loaded one visit ahead, so that the dependent loads
// tile -> image -> descriptor overlap the previous visit's BFS; the masks and
// halo words then load in one level at the start of the visit.
struct GrGeo {
    int nb[4];
    bool skip;
};

__device__ __forceinline__ void gr_prefetch(const Batch &b, int t, GrGeo &gg, bool check_done) {
    tile_nbs(b, t, gg.nb);
    // only the first round can meet a finished image: a later round visits
    // tiles queued by neighbours of the same image, which was visited
    gg.skip = check_done && vload(&b.ist[__ldg(b.tile_img + t)].done) != 0;
}

// Exact distances of tile t given its halo.  round0: the heights of every
// tile are stale, so the halo comes from the neighbours' sink-connected
// pixels and no neighbour is queued (gr_pull_check decides the first
// frontier round once every tile has its round-0 distances).  Later rounds
// queue a neighbour only when this tile's new border gives one of the
// neighbour's facing pixels, through its residual edge into this tile, a
// shorter path than its current height; the heights read for that are at
// least current (distances only fall during a relabel), so no needed visit is
// missed.
__device__ void gr_run(const Batch &b, int t, const GrGeo &g, bool round0, bool direct, int tag_next, int slot_next,
                       GrScratch &sc, int *hs, unsigned long long *st) {
    const int lane = threadIdx.x & 31;
    const size_t base = (size_t)t * TPX;
    unsigned m[6];
    load_tile_masks(b, t, m);
    int ht, hb, hl, hr;
    // the neighbours' facing pixels with a residual edge into this tile: upper
    // row 31 downward, lower row 0 upward (bit = column); left column 31
    // rightward, right column 0 leftward (this lane's row)
    unsigned fu = 0, fd = 0, fl = 0, fr = 0;
    if (round0) {
        ht = g.nb[2] >= 0 && ((mask_word(b, g.nb[2], 4, 31) >> lane) & 1u) ? 1 : INF_H;
        hb = g.nb[3] >= 0 && ((mask_word(b, g.nb[3], 4, 0) >> lane) & 1u) ? 1 : INF_H;
        hl = g.nb[0] >= 0 && (mask_word(b, g.nb[0], 4, lane) >> 31) ? 1 : INF_H;
        hr = g.nb[1] >= 0 && (mask_word(b, g.nb[1], 4, lane) & 1u) ? 1 : INF_H;
    } else {
        // the neighbours' facing border lines (coalesced, from the border array)
        ht = g.nb[2] >= 0 ? __ldcg(b.hb + (size_t)g.nb[2] * 128 + HB_BOT + lane) : INF_H;
        hb = g.nb[3] >= 0 ? __ldcg(b.hb + (size_t)g.nb[3] * 128 + HB_TOP + lane) : INF_H;
        hl = g.nb[0] >= 0 ? __ldcg(b.hb + (size_t)g.nb[0] * 128 + HB_RGT + lane) : INF_H;
        hr = g.nb[1] >= 0 ? __ldcg(b.hb + (size_t)g.nb[1] * 128 + HB_LFT + lane) : INF_H;
        fu = g.nb[2] >= 0 ? mask_word(b, g.nb[2], 3, 31) : 0u;
        fd = g.nb[3] >= 0 ? mask_word(b, g.nb[3], 2, 0) : 0u;
        fl = g.nb[0] >= 0 ? mask_word(b, g.nb[0], 1, lane) >> 31 : 0u;
        fr = g.nb[1] >= 0 ? mask_word(b, g.nb[1], 0, lane) & 1u : 0u;
    }
    int its = 0;
    int vt, vb, vl, vr;  // the tile's border heights (this lane's column / row)
    unsigned reached;
    if (direct) {  // warp-uniform
        reached = tile_bfs_direct(m[0], m[1], m[2], m[3], m[4], hl, hr, ht, hb, hs, 33, &its);
        __syncwarp();
#pragma unroll 4
        for (int r = 0; r < 32; ++r) b.h[base + r * 32 + lane] = hs[r * 33 + lane];
        vt = hs[lane];
        vb = hs[31 * 33 + lane];
        vl = hs[lane * 33];
        vr = hs[lane * 33 + 31];
    } else {
        reached = tile_bfs_gr(m[0], m[1], m[2], m[3], m[4], hl, hr, ht, hb, b.h + base, sc, &its, vt, vb, vl, vr);
    }
    if (lane == 0) stat_add(st, ST_BFS_IT_GR, (unsigned long long)its);
    b.hfin[(size_t)t * 32 + lane] = reached;  // finite heights of this row (the extraction's S_max)
    int act = __popc(m[5] & reached);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) act += __shfl_down_sync(FULL, act, o);
    if (lane == 0) b.tile_act[t] = act;
    {
        int *own = b.hb + (size_t)t * 128;
        own[HB_TOP + lane] = vt;
        own[HB_BOT + lane] = vb;
        own[HB_LFT + lane] = vl;
        own[HB_RGT + lane] = vr;
    }
    if (!round0) {
        const bool up_t = __any_sync(FULL, ((fu >> lane) & 1u) && vt < INF_H && vt + 1 < ht);
        const bool up_b = __any_sync(FULL, ((fd >> lane) & 1u) && vb < INF_H && vb + 1 < hb);
        const bool up_l = __any_sync(FULL, fl && vl < INF_H && vl + 1 < hl);
        const bool up_r = __any_sync(FULL, fr && vr < INF_H && vr + 1 < hr);
        // lanes 0..3 queue the left, right, upper and lower neighbour
        const int nbt = lane == 0 ? g.nb[0] : lane == 1 ? g.nb[1] : lane == 2 ? g.nb[2] : g.nb[3];
        const bool up = lane == 0 ? up_l : lane == 1 ? up_r : lane == 2 ? up_t : up_b;
        enqueue_warp(b, b.mark_gr, slot_next, tag_next, nbt, lane < 4 && up && nbt >= 0);
    }
    __syncwarp();
}

// After round 0 of a global relabel: tile t joins the first frontier round
// when a neighbour's border, as round 0 left it, gives one of t's border
// pixels (through its residual edge out of the tile) a shorter path than its
// own round-0 distance.
// Two tiles per call (t1 < 0: one), every load that depends only on the
// tile issued first for both (image, neighbour table, own border lines and
// masks), then the image's finished flag and the neighbours' border lines:
// two memory round trips for the pair where one tile alone took four.  A
// tile of a finished image is not checked.
__device__ void gr_pull_check(const Batch &b, int t0, int t1, int tag_next, int slot_next) {
    const int lane = threadIdx.x & 31;
    const int tt[2] = {t0, t1 >= 0 ? t1 : t0};
    int img[2], ot[2], ob[2], ol[2], orr[2];
    int4 nb[2];
    unsigned ru[2], rd[2], rl[2], rr[2];
#pragma unroll
    for (int q = 0; q < 2; ++q) {
        const int t = tt[q];
        img[q] = __ldg(b.tile_img + t);
        nb[q] = __ldcg(b.tile_nb + t);
        const int *own = b.hb + (size_t)t * 128;
        ot[q] = __ldcg(own + HB_TOP + lane);
        ob[q] = __ldcg(own + HB_BOT + lane);
        ol[q] = __ldcg(own + HB_LFT + lane);
        orr[q] = __ldcg(own + HB_RGT + lane);
        ru[q] = mask_word(b, t, 2, 0);  // bit = column
        rd[q] = mask_word(b, t, 3, 31);
        rl[q] = mask_word(b, t, 0, lane) & 1u;
        rr[q] = mask_word(b, t, 1, lane) >> 31;
    }
    bool want[2];
#pragma unroll
    for (int q = 0; q < 2; ++q) {
        const int done = __ldcg(&b.ist[img[q]].done);
        const int ht = nb[q].z >= 0 ? __ldcg(b.hb + (size_t)nb[q].z * 128 + HB_BOT + lane) : INF_H;
        const int hb = nb[q].w >= 0 ? __ldcg(b.hb + (size_t)nb[q].w * 128 + HB_TOP + lane) : INF_H;
        const int hl = nb[q].x >= 0 ? __ldcg(b.hb + (size_t)nb[q].x * 128 + HB_RGT + lane) : INF_H;
        const int hr = nb[q].y >= 0 ? __ldcg(b.hb + (size_t)nb[q].y * 128 + HB_LFT + lane) : INF_H;
        const bool imp = (((ru[q] >> lane) & 1u) && ht < INF_H && ht + 1 < ot[q]) ||
                         (((rd[q] >> lane) & 1u) && hb < INF_H && hb + 1 < ob[q]) ||
                         (rl[q] && hl < INF_H && hl + 1 < ol[q]) || (rr[q] && hr < INF_H && hr + 1 < orr[q]);
        want[q] = !done && __any_sync(FULL, imp);  // done is warp-uniform
    }
    enqueue_warp(b, b.mark_gr, slot_next, tag_next, t0, lane == 0 && want[0]);
    if (t1 >= 0) enqueue_warp(b, b.mark_gr, slot_next, tag_next, t1, lane == 0 && want[1]);
}
// Source-side reachability closure of tile t given the halo's reach bits.
__device__ void reach_tile(const Batch &b, int t, bool round0, int tag_next, int slot_next) {
    const int lane = threadIdx.x & 31;
    GrGeo g;  // only the neighbours are used
    tile_nbs(b, t, g.nb);
    unsigned m[6];
    load_tile_masks(b, t, m);
    const unsigned old = round0 ? 0u : __ldcg(b.reach + (size_t)t * 32 + lane);
    // halo pixels that are reached and have residual capacity into the tile
    const unsigned Tin = g.nb[2] >= 0 ? __ldcg(b.reach + (size_t)g.nb[2] * 32 + 31) & mask_word(b, g.nb[2], 3, 31) : 0u;
    const unsigned Bin = g.nb[3] >= 0 ? __ldcg(b.reach + (size_t)g.nb[3] * 32) & mask_word(b, g.nb[3], 2, 0) : 0u;
    const unsigned lbit =
        g.nb[0] >= 0 ? ((__ldcg(b.reach + (size_t)g.nb[0] * 32 + lane) & mask_word(b, g.nb[0], 1, lane)) >> 31) : 0u;
    const unsigned rbit =
        g.nb[1] >= 0 ? ((__ldcg(b.reach + (size_t)g.nb[1] * 32 + lane) & mask_word(b, g.nb[1], 0, lane) & 1u) << 31) : 0u;
    const unsigned Rl = m[0], Rr = m[1], Ru = m[2], Rd = m[3];
    unsigned S = m[5] | old;
    for (int it = 0; it < BFS_MAX_ITERS; ++it) {
        unsigned up = __shfl_up_sync(FULL, S & Rd, 1);
        unsigned dn = __shfl_down_sync(FULL, S & Ru, 1);
        if (lane == 0) up = Tin;
        if (lane == 31) dn = Bin;
        const unsigned nw = ((((S & Rr) << 1) | lbit) | (((S & Rl) >> 1) | rbit) | up | dn) & ~S;
        if (!__any_sync(FULL, nw != 0)) break;
        S |= nw;
    }
    b.reach[(size_t)t * 32 + lane] = S;
    const unsigned fresh = S & ~old;
    const bool out_l = __any_sync(FULL, (fresh & Rl & 1u) != 0);
    const bool out_r = __any_sync(FULL, (fresh & Rr & 0x80000000u) != 0);
    const bool out_u = __any_sync(FULL, lane == 0 && (fresh & Ru) != 0);
    const bool out_d = __any_sync(FULL, lane == 31 && (fresh & Rd) != 0);
    const int nbt = lane == 0 ? g.nb[0] : lane == 1 ? g.nb[1] : lane == 2 ? g.nb[2] : g.nb[3];
    const bool out = lane == 0 ? out_l : lane == 1 ? out_r : lane == 2 ? out_u : out_d;
    enqueue_warp(b, b.mark_gr, slot_next, tag_next, nbt, lane < 4 && out && nbt >= 0);
}

// Sink-side reachability closure of tile t: the pixels that can reach a
// sink-connected pixel (e < 0) along residual edges, written to hfin (the
// complement of S_max inside the image).  The expansion of tile_bfs without
// levels.  round0: the neighbours' sets are not known yet, so the halo starts
// from their sink-connected pixels; later rounds read their hfin rows, all
// written by this pass (the sets only grow, so the rounds converge).
__device__ void sink_reach_tile(const Batch &b, int t, bool round0, int tag_next, int slot_next) {
    const int lane = threadIdx.x & 31;
    int nb[4];
    tile_nbs(b, t, nb);
    unsigned m[6];
    load_tile_masks(b, t, m);
    const unsigned old = round0 ? 0u : __ldcg(b.hfin + (size_t)t * 32 + lane);
    auto halo_row = [&](int nt, int row) -> unsigned {
        if (nt < 0) return 0u;
        return round0 ? mask_word(b, nt, 4, row) : __ldcg(b.hfin + (size_t)nt * 32 + row);
    };
    const unsigned T = halo_row(nb[2], 31), B = halo_row(nb[3], 0);
    const unsigned lbit = halo_row(nb[0], lane) >> 31;         // left tile, column 31
    const unsigned rbit = (halo_row(nb[1], lane) & 1u) << 31;  // right tile, column 0
    const unsigned Rl = m[0], Rr = m[1], Ru = m[2], Rd = m[3];
    unsigned S = m[4] | old;
    for (int it = 0; it < BFS_MAX_ITERS; ++it) {
        unsigned up = __shfl_up_sync(FULL, S, 1);
        unsigned dn = __shfl_down_sync(FULL, S, 1);
        if (lane == 0) up = T;
        if (lane == 31) dn = B;
        const unsigned nw = ((Rl & ((S << 1) | lbit)) | (Rr & ((S >> 1) | rbit)) | (Ru & up) | (Rd & dn)) & ~S;
        if (!__any_sync(FULL, nw != 0)) break;
        S |= nw;
    }
    b.hfin[(size_t)t * 32 + lane] = S;
    // a neighbour is queued when a pixel new in this tile's set has a facing
    // pixel with a residual edge into it that the neighbour's set (as read
    // above, never ahead of the truth) does not hold yet
    const unsigned fresh = S & ~old;
    const unsigned in_u = nb[2] >= 0 ? mask_word(b, nb[2], 3, 31) & ~T : 0u;         // bit = column
    const unsigned in_d = nb[3] >= 0 ? mask_word(b, nb[3], 2, 0) & ~B : 0u;
    const unsigned in_l = nb[0] >= 0 ? (mask_word(b, nb[0], 1, lane) >> 31) & ~lbit : 0u;  // this row
    const unsigned in_r = nb[1] >= 0 ? (mask_word(b, nb[1], 0, lane) & 1u) & ~(rbit >> 31) : 0u;
    const bool out_l = __any_sync(FULL, (fresh & 1u) && in_l);
    const bool out_r = __any_sync(FULL, (fresh >> 31) && in_r);
    const bool out_u = __any_sync(FULL, lane == 0 && (fresh & in_u) != 0);
    const bool out_d = __any_sync(FULL, lane == 31 && (fresh & in_d) != 0);
    const int nbt = lane == 0 ? nb[0] : lane == 1 ? nb[1] : lane == 2 ? nb[2] : nb[3];
    const bool out = lane == 0 ? out_l : lane == 1 ? out_r : lane == 2 ? out_u : out_d;
    enqueue_warp(b, b.mark_gr, slot_next, tag_next, nbt, lane < 4 && out && nbt >= 0);
}

// ---------------------------------------------------------------------------
// Push/relabel on one tile (whole block)
// ---------------------------------------------------------------------------

// The block's next queue entry is taken (thread 0, from take_ctr) when the
// sweeps end, so that the atomic overlaps the write-back; it is left in s.idx
// for the caller.
template <int NW>
__device__ void push_tile(const Batch &b, int t, const SolveParams &prm, int phase, SmemPush<NW> &s,
                          unsigned long long *st, int *take_ctr) {
    constexpr int RPW = TILE_H / NW;  // rows per warp: thread (warp, lane) owns rows warp + NW k, column lane
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    long long c0 = clock64(), c1, cb = 0, cs = 0;
    GrGeo g;  // only the neighbours are used
    tile_nbs(b, t, g.nb);
    const size_t base = (size_t)t * TPX;
#pragma unroll
    for (int k = 0; k < RPW; ++k) {
        const int r = warp + NW * k;
        s.c[r][lane] = __ldcg(b.cap + base + r * 32 + lane);
        s.e[r][lane] = __ldcg(b.exc + base + r * 32 + lane);
        s.h[r + 1][lane + 1] = __ldcg(b.h + base + r * 32 + lane);
    }
    if (warp == 0) s.h[0][lane + 1] = g.nb[2] >= 0 ? __ldcg(b.hb + (size_t)g.nb[2] * 128 + HB_BOT + lane) : INF_H;
    if (warp == 1) s.h[TILE_H + 1][lane + 1] = g.nb[3] >= 0 ? __ldcg(b.hb + (size_t)g.nb[3] * 128 + HB_TOP + lane) : INF_H;
    if (warp == 2) s.h[lane + 1][0] = g.nb[0] >= 0 ? __ldcg(b.hb + (size_t)g.nb[0] * 128 + HB_RGT + lane) : INF_H;
    if (warp == 3) s.h[lane + 1][TILE_W + 1] = g.nb[1] >= 0 ? __ldcg(b.hb + (size_t)g.nb[1] * 128 + HB_LFT + lane) : INF_H;
    if (warp < 4) s.halo_in[warp][lane] = 0;
    __syncthreads();
    c1 = clock64();
    const long long c_load = c1 - c0;

    int any = 1;
    int sweeps = 0, bfs = 0;
    int since_bfs = 0;
    // Exact local relabel: tile BFS against the frozen halo (warp 0), the
    // residual masks of the current capacities first.
    auto local_relabel = [&]() {
        ++bfs;
        since_bfs = 0;
#pragma unroll
        for (int k = 0; k < RPW; ++k) {
            const int r = warp + NW * k;
            const int4 c = s.c[r][lane];
            const int e = s.e[r][lane];
            const unsigned ml = __ballot_sync(FULL, c.x > 0);
            const unsigned mr = __ballot_sync(FULL, c.y > 0);
            const unsigned mu = __ballot_sync(FULL, c.z > 0);
            const unsigned md = __ballot_sync(FULL, c.w > 0);
            const unsigned mn = __ballot_sync(FULL, e < 0);
            if (lane == 0) {
                s.m[0][r] = ml; s.m[1][r] = mr; s.m[2][r] = mu; s.m[3][r] = md; s.m[4][r] = mn;
            }
        }
        __syncthreads();
        const long long cb0 = clock64();
        if (warp == 0) {
            int its = 0;
            const int nrec = tile_bfs_rec(s.m[0][lane], s.m[1][lane], s.m[2][lane], s.m[3][lane], s.m[4][lane],
                                          s.h[lane + 1][0], s.h[lane + 1][TILE_W + 1], s.h[0][lane + 1],
                                          s.h[TILE_H + 1][lane + 1], &s.h[1][1], TILE_W + 2, s.srec, s.lv, s.sfin,
                                          &its);
            if (lane == 0) {
                s.nrec = nrec;
                stat_add(st, ST_BFS_IT_PUSH, (unsigned long long)its);
            }
        }
        __syncthreads();
        {
            const int nrec = s.nrec;
#pragma unroll
            for (int k = 0; k < RPW; ++k) {
                const int r = warp + NW * k;
                s.h[r + 1][lane + 1] =
                    height_from_records(r, lane, s.m[4][r], s.srec, s.lv, s.sfin, nrec, s.h[r + 1][lane + 1]);
            }
        }
        __syncthreads();
        cb += clock64() - cb0;
    };
    // The exact local relabel (tile BFS) runs at the first sweep when
    // prm.bfs_first is set, after a sweep that pushed nothing while active
    // pixels remain, and at least every prm.bfs_every sweeps.
    bool need_bfs = prm.bfs_first != 0;
    for (int sw = 0; sw < prm.max_sweeps; ++sw) {
        ++sweeps;
        if (need_bfs || since_bfs >= prm.bfs_every) local_relabel();
        ++since_bfs;
        // ---- push phase: heights fixed.  All loads first, flows in
        // registers, then fire-and-forget shared atomics. ----
        int ev[RPW], hv[RPW];
#pragma unroll
        for (int k = 0; k < RPW; ++k) {
            const int r = warp + NW * k;
            ev[k] = s.e[r][lane];
            hv[k] = s.h[r + 1][lane + 1];
        }
        bool pushed = false;
#pragma unroll
        for (int k = 0; k < RPW; ++k) {
            const int r = warp + NW * k;
            const int hh = hv[k];
            if (ev[k] > 0 && hh < INF_H) {
                const int4 c = s.c[r][lane];
                const int hl = s.h[r + 1][lane], hr = s.h[r + 1][lane + 2];
                const int hu = s.h[r][lane + 1], hd = s.h[r + 2][lane + 1];
                int e = ev[k];
                const int fl = (c.x > 0 && hh == hl + 1) ? min(e, c.x) : 0;
                e -= fl;
                const int fr = (c.y > 0 && hh == hr + 1) ? min(e, c.y) : 0;
                e -= fr;
                const int fu = (c.z > 0 && hh == hu + 1) ? min(e, c.z) : 0;
                e -= fu;
                const int fd = (c.w > 0 && hh == hd + 1) ? min(e, c.w) : 0;
                e -= fd;
                if (fl) {
                    s.c[r][lane].x = c.x - fl;
                    if (lane > 0) {
                        atomicAdd(reinterpret_cast<int *>(&s.c[r][lane - 1]) + 1, fl);
                        atomicAdd(&s.e[r][lane - 1], fl);
                    } else {
                        atomicAdd(&s.halo_in[0][r], fl);
                    }
                }
                if (fr) {
                    s.c[r][lane].y = c.y - fr;
                    if (lane < TILE_W - 1) {
                        atomicAdd(reinterpret_cast<int *>(&s.c[r][lane + 1]) + 0, fr);
                        atomicAdd(&s.e[r][lane + 1], fr);
                    } else {
                        atomicAdd(&s.halo_in[1][r], fr);
                    }
                }
                if (fu) {
                    s.c[r][lane].z = c.z - fu;
                    if (r > 0) {
                        atomicAdd(reinterpret_cast<int *>(&s.c[r - 1][lane]) + 3, fu);
                        atomicAdd(&s.e[r - 1][lane], fu);
                    } else {
                        atomicAdd(&s.halo_in[2][lane], fu);
                    }
                }
                if (fd) {
                    s.c[r][lane].w = c.w - fd;
                    if (r < TILE_H - 1) {
                        atomicAdd(reinterpret_cast<int *>(&s.c[r + 1][lane]) + 2, fd);
                        atomicAdd(&s.e[r + 1][lane], fd);
                    } else {
                        atomicAdd(&s.halo_in[3][lane], fd);
                    }
                }
                if (e != ev[k]) {
                    atomicSub(&s.e[r][lane], ev[k] - e);
                    pushed = true;
                }
            }
        }
        // block-uniform "anything pushed in this sweep" (every warp takes the
        // same branch below; a shared flag could be overwritten by a warp
        // already in the next sweep)
        const int pushed_any = __syncthreads_or(pushed);
        if (prm.push_only) {
            // heights change only here: a sweep that moved nothing gets an
            // exact local relabel, after which the visit ends if no pixel
            // with excess can reach the sink or the halo
            if (!pushed_any) {
                local_relabel();
                int act = 0;
#pragma unroll
                for (int k = 0; k < RPW; ++k) {
                    const int r = warp + NW * k;
                    act |= s.e[r][lane] > 0 && s.h[r + 1][lane + 1] < INF_H;
                }
                any = __syncthreads_or(act);
                if (!any) break;
            }
            need_bfs = false;
            continue;
        }
        // ---- relabel phase: capacities and excess fixed (own heights as
        // loaded for the push phase: only their owner writes them) ----
        int act = 0;
#pragma unroll
        for (int k = 0; k < RPW; ++k) {
            const int r = warp + NW * k;
            ev[k] = s.e[r][lane];
        }
#pragma unroll
        for (int k = 0; k < RPW; ++k) {
            const int r = warp + NW * k;
            int hh = hv[k];
            if (ev[k] > 0 && hh < INF_H) {
                const int4 c = s.c[r][lane];
                const int hl = s.h[r + 1][lane], hr = s.h[r + 1][lane + 2];
                const int hu = s.h[r][lane + 1], hd = s.h[r + 2][lane + 1];
                int m = INF_H;
                if (c.x > 0) m = min(m, hl);
                if (c.y > 0) m = min(m, hr);
                if (c.z > 0) m = min(m, hu);
                if (c.w > 0) m = min(m, hd);
                if (m >= hh) {
                    hh = m >= INF_H - 1 ? INF_H : m + 1;
                    s.h[r + 1][lane + 1] = hh;
                }
                act |= hh < INF_H;
            }
        }
        any = __syncthreads_or(act);
        if (!any) break;
        need_bfs = !pushed_any;  // stalled: nothing was pushed in this sweep
    }
    const long long c2 = clock64();
    int next_idx = 0;
    if (threadIdx.x == 0) next_idx = atomicAdd(take_ctr, 1);
    // A tile still active queues itself for its colour's next phase.  The
    // queue append is two dependent atomics; with 8 or more warps, warp 4 (no
    // hand-over duty) issues it here, so that its round trips overlap the
    // write-back and the hand-over of warps 0..3 instead of following them
    // (the slot of phase + 2 was emptied at the last barrier and is not read
    // in this phase)
    if (NW >= 8 && any && threadIdx.x == 4 * 32) enqueue(b, b.mark_push, (phase + 2) % 3, phase + 2, t);
    cs = c2 - c1 - cb;
    // ---- write back (and refresh the tile's mask planes and excess sum) ----
    unsigned long long pos = 0;
#pragma unroll
    for (int k = 0; k < RPW; ++k) {
        const int r = warp + NW * k;
        const int4 c = s.c[r][lane];
        const int e = s.e[r][lane];
        b.cap[base + r * 32 + lane] = c;
        b.exc[base + r * 32 + lane] = e;
        b.h[base + r * 32 + lane] = s.h[r + 1][lane + 1];
        write_tile_masks(b, t, r, c, e);
        if (e > 0) pos += (unsigned)e;
    }
    if (warp < 4) {  // the border lines, for the neighbours' halos
        int *own = b.hb + (size_t)t * 128;
        const int v = warp == 0 ? s.h[1][lane + 1] : warp == 1 ? s.h[TILE_H][lane + 1]
                    : warp == 2 ? s.h[lane + 1][1] : s.h[lane + 1][TILE_W];
        own[warp * 32 + lane] = v;  // HB_TOP, HB_BOT, HB_LFT, HB_RGT
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) pos += __shfl_down_sync(FULL, pos, o);
    if (lane == 0) s.part[warp] = pos;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long tot = 0;
        for (int w = 0; w < NW; ++w) tot += s.part[w];
        b.tile_pos[t] = tot;
    }
    // ---- hand halo flow to the (idle) neighbour tiles ----
    if (warp < 4) {
        const int f = s.halo_in[warp][lane];
        const int nt = warp == 0 ? g.nb[0] : warp == 1 ? g.nb[1] : warp == 2 ? g.nb[2] : g.nb[3];
        bool activated = false;  // a pixel of nt now has excess: nt needs a visit
        if (f && nt >= 0) {
            int px, comp;
            if (warp == 0) { px = lane * 32 + 31; comp = 1; }       // left tile, its RIGHT edge
            else if (warp == 1) { px = lane * 32; comp = 0; }       // right tile, its LEFT edge
            else if (warp == 2) { px = 31 * 32 + lane; comp = 3; }  // upper tile, its DOWN edge
            else { px = lane; comp = 2; }                           // lower tile, its UP edge
            const size_t q = (size_t)nt * TPX + px;
            const int old_e = atomicAdd(b.exc + q, f);
            const int new_e = old_e + f;
            const int old_c = atomicAdd(reinterpret_cast<int *>(b.cap + q) + comp, f);
            // keep the receiving tile's mask planes and excess sum exact
            unsigned *mt = b.tmask + (size_t)nt * 6 * 32;
            const int row = px >> 5;
            const unsigned bit = 1u << (px & 31);
            if (old_c == 0) atomicOr(mt + comp * 32 + row, bit);
            if (old_e < 0 && new_e >= 0) atomicAnd(mt + 4 * 32 + row, ~bit);
            if (old_e <= 0 && new_e > 0) atomicOr(mt + 5 * 32 + row, bit);
            const int dpos = max(new_e, 0) - max(old_e, 0);
            if (dpos) atomicAdd(b.tile_pos + nt, (unsigned long long)dpos);
            // flow that only fills sink capacity (the excess stays <= 0) leaves
            // nothing to push there
            activated = new_e > 0;
        }
        if (__any_sync(FULL, activated) && lane == 0)
            enqueue(b, b.mark_push, (phase + 1) % 3, phase + 1, nt);
    }
    if (NW < 8 && any && threadIdx.x == 0) enqueue(b, b.mark_push, (phase + 2) % 3, phase + 2, t);
    if (threadIdx.x == 0) s.idx = next_idx;
    __syncthreads();
    if (threadIdx.x == 0) {
        stat_add(st, ST_PUSH_TILES, 1ull);
        stat_add(st, ST_PUSH_SWEEPS, (unsigned long long)sweeps);
        stat_add(st, ST_PUSH_BFS, (unsigned long long)bfs);
        stat_add(st, ST_CYC_LOAD, (unsigned long long)c_load);
        stat_add(st, ST_CYC_BFS, (unsigned long long)cb);
        stat_add(st, ST_CYC_SWEEP, (unsigned long long)cs);
        stat_add(st, ST_CYC_WB, (unsigned long long)(clock64() - c2));
    }
}

// ---------------------------------------------------------------------------
// The persistent solve kernel
// ---------------------------------------------------------------------------

// Termination check without distances, run after push rounds.  An image
// whose pixels with excess can none of them reach the sink is finished: its
// preflow is maximum.  A sink-side reachability closure (bit-parallel, no
// heights) decides that and gives S_max, far more cheaply than the exact
// global relabel that would otherwise find it; images that fail the check go
// on to that relabel.  Also leaves each checked image's exact sum of positive
// excess.  Returns 1 when every image is finished, 0 when some are not, -1
// on an error (recorded in the control block).  Called by every thread of the
// grid; kept out of line so that its registers do not add to the solver's.
template <int NW>
__device__ __noinline__ int closure_check(const Batch &b, const SolveParams &prm, int &G) {
    Ctl *ctl = b.ctl;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int gwarp = blockIdx.x * NW + warp, nwarps = gridDim.x * NW;
    const int swarp = warp * gridDim.x + blockIdx.x;
    const int gtid = blockIdx.x * blockDim.x + threadIdx.x, nthreads = gridDim.x * blockDim.x;
    const int nt = batch_ntiles(b);
    for (int k = gtid; k < batch_nimg(b); k += nthreads) {
        const int i = batch_img(b, k);
        if (!b.ist[i].done) {
            b.ist[i].pos_excess = 0;
            b.ist[i].active = 0;
        }
    }
    if (gtid == 0) ctl->open_images = 0;
    for (int k = gwarp; k < nt; k += nwarps) {
        const int t = batch_tile(b, k);
        if (vload(&b.ist[__ldg(b.tile_img + t)].done)) continue;  // warp-uniform
        sink_reach_tile(b, t, true, G + 1, L_GR0 + ((G + 1) & 1));
    }
    if (!grid_sync(b, 0)) return -1;
    ++G;
    for (int k = 1;; ++k) {
        const int slot = L_GR0 + (G & 1);
        const int n = vload(&ctl->size[slot]);
        if (n == 0) break;
        if (k > prm.max_rounds) {
            if (gtid == 0) set_error(b, ERRC_GR_ROUNDS);
            return -1;
        }
        for (int idx = swarp; idx < n; idx += nwarps)
            sink_reach_tile(b, b.lists[(size_t)slot * b.list_cap + idx], false, G + 1, L_GR0 + ((G + 1) & 1));
        if (!grid_sync(b, 1u << slot)) return -1;
        ++G;
    }
    // per image: any pixel with excess inside the closure (warp per tile), and
    // the exact sum of positive excess (lane per tile)
    for (int k = gwarp; k < nt; k += nwarps) {
        const int t = batch_tile(b, k);
        const int img = __ldg(b.tile_img + t);
        if (vload(&b.ist[img].done)) continue;  // warp-uniform
        const unsigned live = __ldcg(b.hfin + (size_t)t * 32 + lane) & mask_word(b, t, 5, lane);
        if (__any_sync(FULL, live != 0) && lane == 0) b.ist[img].active = 1;
    }
    for (int kb = gtid - lane; kb < nt; kb += nthreads) {  // warp-uniform
        const int k = kb + lane;
        int img = -1;
        unsigned long long pos = 0;
        if (k < nt) {
            const int t = batch_tile(b, k);
            img = __ldg(b.tile_img + t);
            if (vload(&b.ist[img].done)) img = -1;
            else pos = __ldcg(b.tile_pos + t);
        }
        unsigned todo = __ballot_sync(FULL, img >= 0 && pos != 0);
        while (todo) {
            const int leader = __ffs(todo) - 1;
            const int limg = __shfl_sync(FULL, img, leader);
            const bool mine = ((todo >> lane) & 1u) && img == limg;
            unsigned long long vp = mine ? pos : 0ull;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) vp += __shfl_xor_sync(FULL, vp, o);
            if (lane == leader) atomicAdd(&b.ist[limg].pos_excess, vp);
            todo &= ~__ballot_sync(FULL, mine);
        }
    }
    if (!grid_sync(b, 0)) return -1;
    for (int k = gtid; k < batch_nimg(b); k += nthreads) {
        const int i = batch_img(b, k);
        if (b.ist[i].done) continue;
        if (*(volatile unsigned long long *)&b.ist[i].active == 0) b.ist[i].done = 1;
        else atomicAdd(&ctl->open_images, 1);
    }
    if (gtid == 0) ctl->closure_checks++;
    if (!grid_sync(b, 0)) return -1;
    if (vload(&ctl->open_images) != 0) return 0;
    if (gtid == 0) ctl->closure_ends++;
    return 1;
}

// The block is NW warps over one 32x32 tile (thread block 32 x NW, the
// reference's THREADS_X x THREADS_Y, GraphCut.h:39-53).  Blocks per SM the
// register budget is set for: 8 warps 4, 16 warps 2 and 32 warps 1 (64
// registers per thread); 4 warps 6, the most its shared memory allows (80
// registers, the 8 rows per thread need them).  The phases' shared memory
// (union Smem<NW>) is dynamic: above 48 KB for 16 and 32 warps (132 KB for
// 32, the global relabel's per-warp level arrays).
template <int NW>
constexpr int solve_min_blocks() { return NW == 4 ? 6 : 32 / NW; }

template <int NW>
__global__ void __launch_bounds__(NW * 32, solve_min_blocks<NW>()) k_solve(Batch b, SolveParams prm) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    Smem<NW> &sm = *reinterpret_cast<Smem<NW> *>(smem_raw);
    __shared__ unsigned long long st[ST_N];
    Ctl *ctl = b.ctl;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int gwarp = blockIdx.x * NW + warp, nwarps = gridDim.x * NW;
    const int swarp = warp * gridDim.x + blockIdx.x;  // block-interleaved warp rank
    const int gtid = blockIdx.x * blockDim.x + threadIdx.x, nthreads = gridDim.x * blockDim.x;

    if (threadIdx.x < ST_N) st[threadIdx.x] = 0;
    __syncthreads();
    // the block's statistics reach the control block once, when it leaves
    auto flush_stats = [&]() {
        __syncthreads();
        if (threadIdx.x < ST_N && st[threadIdx.x]) atomicAdd(ctl_stat(ctl, threadIdx.x), st[threadIdx.x]);
    };
    PhaseClock clk;
    clk.start();
    const int nt = batch_ntiles(b);
    if (prm.phase != 2) {
        // fresh de-duplication marks and reach bits for this solve
        for (int k = gtid; k < nt; k += nthreads) {
            const int t = batch_tile(b, k);
            b.mark_push[t] = -1;
            b.mark_gr[t] = -1;
        }
        for (size_t i = gtid; i < (size_t)nt * 32; i += nthreads)
            b.reach[(size_t)batch_tile(b, (int)(i >> 5)) * 32 + (i & 31)] = 0;
        if (!grid_sync(b, 0)) return;
        clk.charge(&ctl->t_init);
    }

    int P = 0;  // push phase counter (even at the start of every outer iteration)
    int G = 0;  // global relabel round counter (tags of the tile frontier)
    bool finished = false;
    bool timeline = false;  // block 0, thread 0 during the first global relabel: records its timeline
    for (int outer = 0; outer < prm.max_outer; ++outer) {
        if (prm.phase == 2) goto push_rounds;  // the phase-1 launch did the relabel and the count
        if (outer > 0) {
            const int rc = closure_check<NW>(b, prm, G);
            if (rc < 0) return;
            clk.charge(&ctl->t_gr);
            if (rc > 0) {
                finished = true;
                break;
            }
        }
        // ------------------------ exact global relabel ------------------------
        timeline = prm.phase == 1 && blockIdx.x == 0 && threadIdx.x == 0;  // the phase-split diagnostic
        if (timeline) ctl->gr_time[0] = gtimer();
        for (int k = gtid; k < batch_nimg(b); k += nthreads) {
            const int i = batch_img(b, k);
            if (!b.ist[i].done) {
                b.ist[i].pos_excess = 0;
                b.ist[i].active = 0;
            }
        }
        if (gtid == 0) ctl->total_active = 0;
        // round 0 visits every tile: with two or more per warp it is bound by
        // issue, and the short BFS with direct level stores is the cheaper one
        // (nt >= 2 * nwarps below)
        for (int k = gwarp; k < nt; k += nwarps) {
            const int t = batch_tile(b, k);
            GrGeo g;
            gr_prefetch(b, t, g, true);
            if (g.skip) continue;
            const long long c0 = clock64();
            gr_run(b, t, g, true, nt >= 2 * nwarps, G + 1, L_GR0 + ((G + 1) & 1), sm.w.g[warp], sm.w.hs[warp], st);
            if (lane == 0) {
                stat_add(st, ST_CYC_GR, (unsigned long long)(clock64() - c0));
                stat_add(st, ST_GR_TILES, 1ull);
            }
        }
        if (!grid_sync(b, (1u << L_PUSH0) | (1u << L_PUSH1) | (1u << L_PUSH2))) return;
        if (timeline) ctl->gr_time[1] = gtimer();
        for (int k = gwarp; k < nt; k += 2 * nwarps) {
            const int t0 = batch_tile(b, k);
            const int t1 = k + nwarps < nt ? batch_tile(b, k + nwarps) : -1;
            gr_pull_check(b, t0, t1, G + 1, L_GR0 + ((G + 1) & 1));
        }
        if (!grid_sync(b, 0)) return;
        if (timeline) ctl->gr_time[2] = gtimer();
        ++G;
        for (int k = 1;; ++k) {
            const int slot = L_GR0 + (G & 1);
            const int n = vload(&ctl->size[slot]);
            if (n == 0) break;
            if (k > prm.max_rounds) {
                if (gtid == 0) set_error(b, ERRC_GR_ROUNDS);
                return;
            }
            // static assignment, interleaved over the blocks so that a small
            // frontier spreads over every SM (no queue-take atomics)
            for (int idx = swarp; idx < n; idx += nwarps) {
                const int t = b.lists[(size_t)slot * b.list_cap + idx];
                const long long c0 = clock64();
                GrGeo g;
                gr_prefetch(b, t, g, false);
                gr_run(b, t, g, false, false, G + 1, L_GR0 + ((G + 1) & 1), sm.w.g[warp], sm.w.hs[warp], st);
                if (lane == 0) {
                    const unsigned long long cyc = (unsigned long long)(clock64() - c0);
                    stat_add(st, ST_CYC_GR, cyc);
                    stat_add(st, ST_GR_TILES, 1ull);
                    if (prm.phase == 1 && k <= GR_TIMELINE) {  // the phase-split diagnostic only
                        atomicMax(&ctl->gr_front_end[k - 1], gtimer());
                        atomicMax(&ctl->gr_front_maxcyc[k - 1], cyc);
                    }
                }
            }
            if (!grid_sync(b, 1u << slot)) return;
            if (timeline && k <= GR_TIMELINE) {
                ctl->gr_time[2 + k] = gtimer();
                ctl->gr_front[k - 1] = n;
            }
            ++G;
            if (gtid == 0) ctl->gr_rounds++;
        }
        clk.charge(&ctl->t_gr);
        // ------------------------ count active nodes ------------------------
        // warp-uniform loop: the sums of a warp's tiles go out with one
        // atomic per image (a warp's tiles belong to one or two images) and
        // one for the batch total; the queue appends share one per colour
        for (int kb = gtid - lane; kb < nt; kb += nthreads) {
            const int k = kb + lane;
            int t = 0, img = -1, nact = 0, color = 0;
            unsigned long long pos = 0;
            if (k < nt) {
                t = batch_tile(b, k);
                img = __ldg(b.tile_img + t);
                if (vload(&b.ist[img].done)) {
                    img = -1;
                } else {
                    nact = vload(b.tile_act + t);
                    pos = __ldcg(b.tile_pos + t);
                    if (nact) color = tile_geo(b, t).color;
                }
            }
            unsigned todo = __ballot_sync(FULL, img >= 0 && (nact || pos));
            while (todo) {
                const int leader = __ffs(todo) - 1;
                const int limg = __shfl_sync(FULL, img, leader);
                const bool mine = ((todo >> lane) & 1u) && img == limg;
                unsigned long long vp = mine ? pos : 0ull;
                unsigned va = mine ? (unsigned)nact : 0u;
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) {
                    vp += __shfl_xor_sync(FULL, vp, o);
                    va += __shfl_xor_sync(FULL, va, o);
                }
                if (lane == leader) {
                    if (vp) atomicAdd(&b.ist[limg].pos_excess, vp);
                    if (va) atomicAdd(&b.ist[limg].active, (unsigned long long)va);
                }
                todo &= ~__ballot_sync(FULL, mine);
            }
            const unsigned wact = __reduce_add_sync(FULL, (unsigned)nact);
            if (lane == 0 && wact) atomicAdd(&ctl->total_active, (unsigned long long)wact);
            enqueue_warp(b, b.mark_push, P % 3, P, t, nact && color == 0);
            enqueue_warp(b, b.mark_push, (P + 1) % 3, P + 1, t, nact && color == 1);
        }
        if (!grid_sync(b, 0)) return;
        clk.charge(&ctl->t_count);
        if (gtid == 0) {
            ctl->global_relabels++;
            ctl->outer_iters = outer + 1;
        }
        if (prm.phase == 1) {
            flush_stats();
            return;
        }
        {
            const unsigned long long total = *(volatile unsigned long long *)&ctl->total_active;
            for (int k = gtid; k < batch_nimg(b); k += nthreads) {
                const int i = batch_img(b, k);
                if (!b.ist[i].done && *(volatile unsigned long long *)&b.ist[i].active == 0) b.ist[i].done = 1;
            }
            if (total == 0) {
                finished = true;
                break;
            }
        }
        // ------------------------ checkerboard push rounds ------------------------
    push_rounds:
        int last = P;
        for (int r = 0; r < prm.push_rounds; ++r) {
            bool more = true;
            for (int c = 0; c < 2; ++c) {
                const int p = P + 2 * r + c;
                const int slot = p % 3;
                last = p;
                const int n = vload(&ctl->size[slot]);
                {
                    const long long ct = clock64();
                    if (threadIdx.x == 0) sm.p.idx = atomicAdd(&ctl->take[slot], 1);
                    __syncthreads();
                    if (threadIdx.x == 0) stat_add(st, ST_CYC_TAKE, (unsigned long long)(clock64() - ct));
                }
                for (;;) {
                    // the entry taken before (the first one above, later ones by
                    // the previous visit); no thread writes s.idx again before
                    // every thread has read it (push_tile's barriers come first)
                    const int idx = sm.p.idx;
                    if (idx >= n) break;
                    push_tile(b, b.lists[(size_t)slot * b.list_cap + idx], prm, p, sm.p, st, &ctl->take[slot]);
                }
                // the phase's tail: from the first block out of work to the barrier
                if (threadIdx.x == 0) atomicMax(&ctl->push_idle[p & 1], ~gtimer());
                if (gtid == 0) ctl->push_idle[(p + 1) & 1] = 0;  // last read after the previous phase
                __syncthreads();
                if (!grid_sync(b, 1u << slot)) return;
                if (gtid == 0) {
                    ctl->push_phases++;
                    const unsigned long long idle = *(volatile unsigned long long *)&ctl->push_idle[p & 1];
                    if (idle) ctl->t_push_tail += gtimer() - ~idle;
                }
                if (vload(&ctl->size[(p + 1) % 3]) == 0 && vload(&ctl->size[(p + 2) % 3]) == 0) {
                    more = false;
                    break;
                }
            }
            if (!more) break;
        }
        P = (last + 3) & ~1;
        clk.charge(&ctl->t_push);
        if (prm.phase == 2) {
            flush_stats();
            return;
        }
    }
    if (!finished) {
        if (gtid == 0) set_error(b, ERRC_OUTER);
        return;
    }
    // ------------------------ source-side reachability ------------------------
    for (int k = gwarp; k < nt; k += nwarps) reach_tile(b, batch_tile(b, k), true, G + 1, L_GR0 + ((G + 1) & 1));
    if (!grid_sync(b, 0)) return;
    ++G;
    for (int k = 1;; ++k) {
        const int slot = L_GR0 + (G & 1);
        const int n = vload(&ctl->size[slot]);
        if (n == 0) break;
        if (k > prm.max_rounds) {
            if (gtid == 0) set_error(b, ERRC_REACH_ROUNDS);
            return;
        }
        for (int idx = swarp; idx < n; idx += nwarps) {
            reach_tile(b, b.lists[(size_t)slot * b.list_cap + idx], false, G + 1, L_GR0 + ((G + 1) & 1));
            if (lane == 0) stat_add(st, ST_REACH_TILES, 1ull);
        }
        if (!grid_sync(b, 1u << slot)) return;
        ++G;
        if (gtid == 0) ctl->reach_rounds++;
    }
    clk.charge(&ctl->t_reach);
    flush_stats();
}

// ---------------------------------------------------------------------------
// Build and extraction kernels (one block per tile)
// ---------------------------------------------------------------------------

// Residual graph of image 0 from caller arrays (GC_SetGraph).  Follows
// InitGraph / InitGraphVarEdges (GraphCutKernels.cu:112-214): interior nodes
// only, caps that point into the 1-pixel border zeroed, excess = dp - dn.
__global__ void __launch_bounds__(TILE_THREADS) k_build_arrays(Batch b, const int *__restrict__ dp,
                                                                const int *__restrict__ dn, int penalty,
                                                                const int *__restrict__ up,
                                                                const int *__restrict__ down,
                                                                const int *__restrict__ left,
                                                                const int *__restrict__ right) {
    const int t = batch_tile(b, blockIdx.x);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const TileGeo g = tile_geo(b, t);
    if (threadIdx.x == 0) b.tile_nb[t] = nb_of(g);
    const int W = b.img[g.img].W, H = b.img[g.img].H;
    unsigned long long idp = 0, rinit = 0, pos = 0;
    int bad = 0;
    const long long w32 = (long long)((W + 31) / 32) * 32;
#pragma unroll
    for (int k = 0; k < ROWS_PER_WARP; ++k) {
        const int r = warp + 8 * k;
        const int x = g.tx * TILE_W + lane, y = g.ty * TILE_H + r;
        int4 c = make_int4(0, 0, 0, 0);
        int e = 0;
        if (x < W && y < H) {
            const size_t i = (size_t)y * W + x;
            const int vdp = dp[i];
            // the reference sums max(dp,0) over padded positions x + y*W32 < W*H
            // (GraphCut.cu:359-376, GraphCutKernels.cu:883-898)
            if ((long long)x + (long long)y * w32 < (long long)W * H && vdp > 0) rinit += (unsigned)vdp;
            if (x > 0 && y > 0 && x < W - 1 && y < H - 1) {
                const int vdn = dn[i];
                c = up ? make_int4(left[i], right[i], up[i], down[i])
                       : make_int4(penalty, penalty, penalty, penalty);
                bad |= (vdp < 0) | (vdn < 0) | (vdp > GCFG_MAX_CAP) | (vdn > GCFG_MAX_CAP) | (c.x < 0) |
                       (c.y < 0) | (c.z < 0) | (c.w < 0) | (c.x > GCFG_MAX_CAP) | (c.y > GCFG_MAX_CAP) |
                       (c.z > GCFG_MAX_CAP) | (c.w > GCFG_MAX_CAP);
                if (x == 1) c.x = 0;
                if (x == W - 2) c.y = 0;
                if (y == 1) c.z = 0;
                if (y == H - 2) c.w = 0;
                e = vdp - vdn;
                idp += (unsigned long long)(long long)vdp;
            }
        }
        const size_t p = (size_t)t * TPX + r * 32 + lane;
        b.cap[p] = c;
        b.exc[p] = e;
        write_tile_masks(b, t, r, c, e);
        if (e > 0) pos += (unsigned)e;
    }
    block_store_sum(b.tile_pos + t, pos);
    if (bad) set_error(b, 100);
    warp_atomic_add_u64(&b.ist[g.img].interior_dp, idp);
    warp_atomic_add_u64(&b.ist[g.img].ref_init, rinit);
}

// Labels of every image, row-major, at each image's out0 offset:
// smin = source-reachable, smax = interior and cannot reach the sink,
// label = smax as int32 (the reference's GC_Optimize output).
__global__ void __launch_bounds__(TILE_THREADS) k_extract(Batch b, uint8_t *smin, uint8_t *smax,
                                                           int *label) {
    const int t = batch_tile(b, blockIdx.x);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const TileGeo g = tile_geo(b, t);
    const int W = b.img[g.img].W, H = b.img[g.img].H;
    const long long out0 = b.img[g.img].out0;
#pragma unroll
    for (int k = 0; k < ROWS_PER_WARP; ++k) {
        const int r = warp + 8 * k;
        const int x = g.tx * TILE_W + lane, y = g.ty * TILE_H + r;
        if (x >= W || y >= H) continue;
        const size_t i = (size_t)out0 + (size_t)y * W + x;
        const bool inside = x > 0 && y > 0 && x < W - 1 && y < H - 1;
        // h == INF: not reached by the last global relabel of this tile
        const uint8_t sm = inside && !((b.hfin[(size_t)t * 32 + r] >> lane) & 1u);
        if (smin) smin[i] = (uint8_t)((b.reach[(size_t)t * 32 + r] >> lane) & 1u);
        if (smax) smax[i] = sm;
        if (label) label[i] = sm;
    }
}

// The same cuts written row-major by output windows: block = one chunk of
// an image (CHUNK_PX consecutive pixels, the data-term pass's chunk map),
// thread = one 16-byte window of the output arrays, aligned on the arrays'
// addresses (smin and smax share their alignment mod 16).  A window takes
// its bits from the row mask words of the tiles it covers, one row segment
// at a time (one or two segments when W >= 16), spreads them to 16 bytes
// and writes each cut with one 16-byte store; a window that reaches past
// the chunk writes only the chunk's bytes, one at a time.
__device__ __forceinline__ uint32_t spread4(uint32_t nib) { return (nib * 0x00204081u) & 0x01010101u; }
__device__ __forceinline__ uint4 spread16(uint32_t bits) {
    return make_uint4(spread4(bits & 15u), spread4((bits >> 4) & 15u), spread4((bits >> 8) & 15u),
                      spread4((bits >> 12) & 15u));
}

__global__ void __launch_bounds__(256) k_extract_rows(Batch b, const int2 *__restrict__ chunk_map, uint8_t *smin,
                                                      uint8_t *smax) {
    __shared__ long long s_row0;
    const int2 cm = __ldg(chunk_map + blockIdx.x);
    const int W = __ldg(&b.img[cm.x].W), H = __ldg(&b.img[cm.x].H);
    const int tile0 = __ldg(&b.img[cm.x].tile0), tiles_x = __ldg(&b.img[cm.x].tiles_x);
    const long long out0 = __ldg(&b.img[cm.x].out0);
    const long long npx = (long long)W * H;
    const long long lo = (long long)cm.y * CHUNK_PX, hi = min(npx, lo + CHUNK_PX);  // the chunk's pixels
    if (threadIdx.x == 0) s_row0 = lo / W;  // the chunk's first row
    __syncthreads();
    const long long row0 = s_row0;
    const int xlo = (int)(lo - row0 * W);
    uint8_t *ref = smax ? smax : smin;
    const uintptr_t abase = (uintptr_t)(ref + out0);  // address of the image's pixel 0
    const uintptr_t a0 = (abase + (uintptr_t)lo) & ~(uintptr_t)15;
    const int lead = (int)(abase + (uintptr_t)lo - a0);  // pixels of window 0 before the chunk
    const int nwin = (lead + (int)(hi - lo) + 15) >> 4;
    for (int w = threadIdx.x; w < nwin; w += blockDim.x) {
        const int q0 = 16 * w - lead;  // the window's first pixel, relative to lo
        const int s = max(q0, 0), e = min(q0 + 16, (int)(hi - lo));
        // row and column of pixel lo + s
        const unsigned xr = (unsigned)(xlo + s);
        int y = (int)(row0 + xr / (unsigned)W), x = (int)(xr % (unsigned)W);
        unsigned rb = 0, mb = 0;  // reach bits, smax bits; bit j = pixel q0 + j
        for (int pos = s, it = 0; pos < e && it < 16; ++it) {
            const int len = min(e - pos, W - x);
            const int sh = x & 31, r = y & 31;
            const size_t t = (size_t)tile0 + (size_t)(y >> 5) * tiles_x + (x >> 5);
            const unsigned f0 = __ldg(b.hfin + t * 32 + r), r0 = __ldg(b.reach + t * 32 + r);
            unsigned f1 = 0, r1 = 0;
            if (sh + len > 32) {  // the segment reaches into the next tile of the row
                f1 = __ldg(b.hfin + (t + 1) * 32 + r);
                r1 = __ldg(b.reach + (t + 1) * 32 + r);
            }
            const unsigned keep = len >= 32 ? 0xFFFFFFFFu : (1u << len) - 1u;
            // interior pixels: not on row 0 or H - 1, not at x = 0 or W - 1
            unsigned in = (y > 0 && y < H - 1) ? keep : 0u;
            if (x == 0) in &= ~1u;
            if (x + len == W) in &= ~(1u << (len - 1));
            const int at = pos - q0;
            rb |= (__funnelshift_r(r0, r1, sh) & keep) << at;
            mb |= (~__funnelshift_r(f0, f1, sh) & in) << at;
            pos += len;
            x = 0;
            ++y;
        }
        const size_t o = (size_t)(out0 + lo + q0);
        if (s == q0 && e == q0 + 16) {
            if (smin) *reinterpret_cast<uint4 *>(smin + o) = spread16(rb);
            if (smax) *reinterpret_cast<uint4 *>(smax + o) = spread16(mb);
        } else {
            for (int j = s - q0; j < e - q0; ++j) {
                if (smin) smin[o + j] = (uint8_t)((rb >> j) & 1u);
                if (smax) smax[o + j] = (uint8_t)((mb >> j) & 1u);
            }
        }
    }
}

}  // namespace gcfg

namespace gcfg {

namespace {

// The solver kernel of a block shape (warps per block: 4, 8, 16 or 32) and its
// dynamic shared memory.
struct SolveKernel {
    const void *fn;
    size_t smem;
};

SolveKernel solve_kernel(int warps) {
    switch (warps) {
        case 4: return {(const void *)k_solve<4>, sizeof(Smem<4>)};
        case 16: return {(const void *)k_solve<16>, sizeof(Smem<16>)};
        case 32: return {(const void *)k_solve<32>, sizeof(Smem<32>)};
        default: return {(const void *)k_solve<8>, sizeof(Smem<8>)};
    }
}

int shape_index(int warps) { return warps == 4 ? 0 : warps == 16 ? 2 : warps == 32 ? 3 : 1; }

// Co-resident blocks of the solver kernel of a shape on the current device,
// computed once per device ordinal and shape (the kernel's dynamic
// shared-memory limit is raised first where the shape needs it); several
// host threads (the server's lanes) may race to fill an entry, and they all
// store the same value.
int resident_blocks(int warps) {
    constexpr int MAX_DEV = 64;
    static std::atomic<int> cached[MAX_DEV][4];
    int dev = 0;
    cudaGetDevice(&dev);
    const bool slot = dev >= 0 && dev < MAX_DEV;
    const int si = shape_index(warps);
    int full = slot ? cached[dev][si].load(std::memory_order_relaxed) : 0;
    if (!full) {
        const SolveKernel k = solve_kernel(warps);
        cudaFuncSetAttribute(k.fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)k.smem);
        int sms = 0, per_sm = 0;
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k.fn, warps * 32, k.smem);
        full = (per_sm > 0 ? per_sm : 1) * (sms > 0 ? sms : 1);
        if (slot) cached[dev][si].store(full, std::memory_order_relaxed);
    }
    return full;
}

}  // namespace

int solve_grid_blocks(int n_tiles, int max_grid, int warps) {
    // half the tiles run in a push phase; more blocks than that only make
    // the grid barrier slower
    int cap = resident_blocks(warps);
    if (max_grid > 0 && max_grid < cap) cap = max_grid;
    const int want = (n_tiles + 1) / 2;
    return want < 1 ? 1 : (want < cap ? want : cap);
}

gcfg_status launch_solve(const Batch &b, const SolveParams &prm, int n_tiles, cudaStream_t st, int max_grid) {
    const int warps = solve_warps(prm.warps, n_tiles);
    const int grid = solve_grid_blocks(n_tiles, max_grid, warps);
    const SolveKernel k = solve_kernel(warps);
    Batch bb = b;
    SolveParams pp = prm;
    void *args[] = {&bb, &pp};
    prof_begin(st);
    const cudaError_t e = cudaLaunchCooperativeKernel(k.fn, dim3(grid), dim3(warps * 32), args, k.smem, st);
    prof_end(GCFG_PK_SOLVE, st);
    g_launches.fetch_add(1, std::memory_order_relaxed);
    return e == cudaSuccess ? GCFG_OK : GCFG_ERR_CUDA;
}

gcfg_status launch_build_arrays(const Batch &b, const int *dp, const int *dn, int penalty, const int *up,
                                const int *down, const int *left, const int *right, cudaStream_t st) {
    GCFG_LAUNCH(GCFG_PK_BUILD, st,
                k_build_arrays<<<batch_ntiles(b), TILE_THREADS, 0, st>>>(b, dp, dn, penalty, up, down, left, right));
    GCFG_CK(cudaGetLastError());
    return GCFG_OK;
}

gcfg_status launch_extract_rows(const Batch &b, const int2 *chunk_map, long long n_chunks, uint8_t *smin,
                               uint8_t *smax, cudaStream_t st) {
    if ((!smin && !smax) || n_chunks <= 0) return GCFG_OK;
    if (smin && smax && (((uintptr_t)smin ^ (uintptr_t)smax) & 15)) {
        // the windows need one alignment for both arrays: the tile-major kernel instead
        return launch_extract(b, smin, smax, nullptr, st);
    }
    GCFG_LAUNCH(GCFG_PK_EXTRACT, st, k_extract_rows<<<(unsigned)n_chunks, 256, 0, st>>>(b, chunk_map, smin, smax));
    GCFG_CK(cudaGetLastError());
    return GCFG_OK;
}

gcfg_status launch_extract(const Batch &b, uint8_t *smin, uint8_t *smax, int *label, cudaStream_t st) {
    GCFG_LAUNCH(GCFG_PK_EXTRACT, st, k_extract<<<batch_ntiles(b), TILE_THREADS, 0, st>>>(b, smin, smax, label));
    GCFG_CK(cudaGetLastError());
    return GCFG_OK;
}

}  // namespace gcfg
