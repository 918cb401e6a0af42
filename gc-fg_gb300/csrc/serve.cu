// serve.cu -- serving: continuous batching of segmentation requests with
// resident graphs and exact warm-started scribble edits.
//
// A server owns one device arena sized by its memory cap.  Every admitted
// image becomes a resident session: its pixels, scribbles, label maps, tile
// arena (residual graph), colour histograms and t-link tables stay on the
// device after it is solved.  Worker lanes (one host thread + one stream
// each) take every runnable request that is waiting when they become free,
// solve them as one batch (one data-term pass, one build, one persistent
// solver launch over the tiles of all of them) and complete them; requests
// that arrive meanwhile wait for the next free lane, so with two lanes the
// device works on two batches at once (each persistent grid is capped at half
// the GPU so that both fit).
//
// New image: admitted when its tiles fit under the memory cap (idle sessions
// are evicted least-recently-used first); cold data term + build + solve.
// Scribble edit of a resident image: the square is written into the stored
// scribbles, the histograms and t-link tables are recomputed, and every
// pixel's excess is shifted by (dp_new - dp_old) - (dn_new - dn_old); the
// stored n-link residuals and flow are kept, and the solve restarts from an
// exact global relabel.  For any state with non-negative residuals r,
// E(S) = sum(dp) - sum_{i in S} e_i + sum_{u in S, v not in S} r(u,v), so
// the warm solve ends at the same exact minimum cut and flow value as a cold
// solve of the edited image.
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "dataterm.cuh"
#include "engine.cuh"

namespace gcfg {
namespace {

// Device bytes per tile of a resident image: tile arena (cap, exc, h, border
// heights, neighbours, finite-height masks, reach, mask planes, counters, marks, owner) + its 1024 pixel slots
// of RGB, scribble and two label maps.
constexpr size_t ARENA_TILE_BYTES = sizeof(int4) * TPX + 2 * sizeof(int) * TPX + 4 * 32 * sizeof(int) + sizeof(int4) + 32 * 4 + 32 * 4 +
                                    6 * 32 * 4 + sizeof(int) + sizeof(unsigned long long) + 3 * sizeof(int);
constexpr size_t PX_BYTES = 3 + 1 + 2;
constexpr size_t TILE_BYTES = ARENA_TILE_BYTES + TPX * PX_BYTES;
// per session slot: histograms, current and previous t-link tables
constexpr size_t SLOT_BYTES = 2 * NBINS * sizeof(int) * 3 + sizeof(ImgDesc) + sizeof(ImgState);

double now_s() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// First-fit allocator of ranges in [0, cap).
struct RangeAlloc {
    std::map<long long, long long> free_;
    long long cap = 0, used = 0;
    void init(long long c) {
        cap = c;
        used = 0;
        free_.clear();
        if (c > 0) free_[0] = c;
    }
    long long alloc(long long n) {
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second < n) continue;
            const long long s = it->first, len = it->second;
            free_.erase(it);
            if (len > n) free_[s + n] = len - n;
            used += n;
            return s;
        }
        return -1;
    }
    void release(long long s, long long n) {
        used -= n;
        auto it = free_.emplace(s, n).first;
        auto nx = std::next(it);
        if (nx != free_.end() && it->first + it->second == nx->first) {
            it->second += nx->second;
            free_.erase(nx);
        }
        if (it != free_.begin()) {
            auto pv = std::prev(it);
            if (pv->first + pv->second == it->first) {
                pv->second += it->second;
                free_.erase(it);
            }
        }
    }
};

struct Session {
    bool admitted = false;  // device storage allocated
    int slot = -1;
    int W = 0, H = 0;
    double lambda = 0;
    long long tile0 = 0, n_tiles = 0, pix0 = 0;
    double last_use = 0;
    bool busy = false;   // in a lane's batch
    bool ready = false;  // solved at least once
    int pending = 0;     // queued edits that refer to it
};

struct Req {
    int64_t ticket = 0;
    gcfg_serve_request r;
    double t_submit = 0;
};

struct TicketState {
    bool done = false;
    gcfg_serve_result res;
};

// ---------------------------------------------------------------------------
// kernels of the serving path
// ---------------------------------------------------------------------------

__global__ void k_fill_tile_owner(int *tile_img, long long tile0, int n, int slot) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x)
        tile_img[tile0 + k] = slot;
}

// Zero the per-image counters of the batch's images and mark them unsolved.
__global__ void k_slot_reset(const int *ilist, int n, ImgState *ist) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    ImgState &s = ist[ilist[k]];
    s.interior_dp = 0;
    s.ref_init = 0;
    s.pos_excess = 0;
    s.active = 0;
    s.sigma_sum = 0;
    s.done = 0;
}

// Write a scribble square (class cls) into an image's stored scribbles.
__global__ void k_edit_square(uint8_t *scrib, int W, int H, int x0, int y0, int size, int cls) {
    const int dx = blockIdx.x * blockDim.x + threadIdx.x, dy = blockIdx.y * blockDim.y + threadIdx.y;
    if (dx >= size || dy >= size) return;
    const int x = x0 + dx, y = y0 + dy;
    if (x < 0 || y < 0 || x >= W || y >= H) return;
    scrib[(long long)y * W + x] = (uint8_t)cls;
}

// Warm start: shift every interior pixel's excess by the change of its
// t-links, keep capacities, refresh the mask planes and the image sums.
__global__ void __launch_bounds__(TILE_THREADS) k_reparam(Batch b, const uint8_t *__restrict__ rgb,
                                                           const int *__restrict__ dpl, const int *__restrict__ dnl,
                                                           const int *__restrict__ odpl,
                                                           const int *__restrict__ odnl) {
    const int t = batch_tile(b, blockIdx.x);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int im = b.tile_img[t];
    const ImgDesc d = b.img[im];
    const int lt = t - d.tile0;
    const int tx = lt % d.tiles_x, ty = lt / d.tiles_x;
    const int W = d.W, H = d.H;
    const long long w32 = (long long)((W + 31) / 32) * 32;
    const uint8_t *base = rgb + 3 * d.pix0;
    const size_t lo = (size_t)im * NBINS;
    unsigned long long idp = 0, rinit = 0, pos = 0;
#pragma unroll
    for (int k = 0; k < ROWS_PER_WARP; ++k) {
        const int r = warp + 8 * k;
        const int x = tx * TILE_W + lane, y = ty * TILE_H + r;
        const size_t q = (size_t)t * TPX + r * 32 + lane;
        const int4 c = b.cap[q];
        int e = b.exc[q];
        if (x < W && y < H) {
            const uint8_t *p = base + 3 * ((long long)y * W + x);
            const int bin = ((p[0] >> 4) << 8) | ((p[1] >> 4) << 4) | (p[2] >> 4);
            const int vdp = dpl[lo + bin];
            if ((long long)x + (long long)y * w32 < (long long)W * H && vdp > 0) rinit += (unsigned)vdp;
            if (x > 0 && y > 0 && x < W - 1 && y < H - 1) {
                e += (vdp - odpl[lo + bin]) - (dnl[lo + bin] - odnl[lo + bin]);
                b.exc[q] = e;
                idp += (unsigned)vdp;
            }
        }
        write_tile_masks(b, t, r, c, e);
        if (e > 0) pos += (unsigned)e;
    }
    block_store_sum(b.tile_pos + t, pos);
    warp_atomic_add_u64(&b.ist[im].interior_dp, idp);
    warp_atomic_add_u64(&b.ist[im].ref_init, rinit);
}

// ---------------------------------------------------------------------------

struct Lane;

struct Server {
    gcfg_serve_config cfg;
    int device = 0;
    long long tiles_cap = 0, px_cap = 0;
    // arena
    int4 *cap = nullptr;
    int *exc = nullptr, *h = nullptr, *hb = nullptr;
    int4 *tnb = nullptr;
    unsigned *hfin = nullptr;
    unsigned *reach = nullptr, *tmask = nullptr;
    int *tact = nullptr;
    unsigned long long *tpos = nullptr;
    int *mpush = nullptr, *mgr = nullptr, *tile_img = nullptr;
    uint8_t *rgb = nullptr, *scrib = nullptr, *smin = nullptr, *smax = nullptr;
    // slots
    ImgDesc *img = nullptr;
    ImgState *ist = nullptr;
    int *hist = nullptr, *dpl = nullptr, *dnl = nullptr, *odpl = nullptr, *odnl = nullptr;
    // host state
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<Req> queue;
    std::unordered_map<int64_t, TicketState> tickets;
    std::unordered_map<int64_t, Session> sessions;
    std::vector<int> free_slots;
    RangeAlloc tiles, pixels;
    int64_t next_ticket = 1, next_session = 1;
    long long gen = 0;  // bumped by every submission and completion
    bool stop = false;
    gcfg_serve_stats stats;
    std::vector<Lane *> lanes;

    long long bytes_in_use() const { return tiles.used * (long long)TILE_BYTES; }
};

struct Lane {
    Server *sv = nullptr;
    int id = 0;
    cudaStream_t st = nullptr;
    Ctl *ctl = nullptr, *h_ctl = nullptr;
    int *lists = nullptr;
    int list_cap = 0;
    int *d_tl = nullptr, *h_tl = nullptr;      // all tiles of the batch
    int *d_tnew = nullptr, *h_tnew = nullptr;  // tiles of new images
    int *d_tedit = nullptr, *h_tedit = nullptr;  // tiles of edited images
    int *d_il = nullptr, *h_il = nullptr;      // slots of the batch
    int2 *d_cmap = nullptr, *h_cmap = nullptr;  // per chunk: (slot, chunk within the image)
    ImgDesc *h_desc = nullptr;
    ImgState *h_ist = nullptr;
    std::thread th;
};

template <typename T>
gcfg_status dalloc(T *&p, size_t n) {
    if (cudaMalloc(&p, (n ? n : 1) * sizeof(T)) != cudaSuccess) return GCFG_ERR_OOM;
    return GCFG_OK;
}
template <typename T>
gcfg_status halloc(T *&p, size_t n) {
    if (cudaMallocHost(&p, (n ? n : 1) * sizeof(T)) != cudaSuccess) return GCFG_ERR_OOM;
    return GCFG_OK;
}

Batch arena_batch(Server &s) {
    Batch b;
    memset(&b, 0, sizeof(b));
    b.n_img = s.cfg.max_sessions;
    b.n_tiles = (int)s.tiles_cap;
    b.img = s.img;
    b.ist = s.ist;
    b.tile_img = s.tile_img;
    b.cap = s.cap;
    b.exc = s.exc;
    b.h = s.h;
    b.hb = s.hb;
    b.tile_nb = s.tnb;
    b.hfin = s.hfin;
    b.reach = s.reach;
    b.tmask = s.tmask;
    b.tile_act = s.tact;
    b.tile_pos = s.tpos;
    b.mark_push = s.mpush;
    b.mark_gr = s.mgr;
    return b;
}

int tiles_of(int W, int H) { return div_up(W, TILE_W) * div_up(H, TILE_H); }

// Evict the least recently used idle session.  Caller holds the lock.
bool evict_one(Server &s) {
    int64_t best = -1;
    double t = 1e300;
    for (auto &kv : s.sessions) {
        const Session &x = kv.second;
        if (!x.admitted || x.busy || x.pending > 0 || !x.ready) continue;
        if (x.last_use < t) {
            t = x.last_use;
            best = kv.first;
        }
    }
    if (best < 0) return false;
    Session &x = s.sessions[best];
    s.tiles.release(x.tile0, x.n_tiles);
    s.pixels.release(x.pix0, (long long)x.n_tiles * TPX);
    s.free_slots.push_back(x.slot);
    s.sessions.erase(best);
    s.stats.evicted++;
    return true;
}

void complete(Server &s, const Req &q, const gcfg_serve_result &res) {
    TicketState &ts = s.tickets[q.ticket];
    ts.done = true;
    ts.res = res;
}

gcfg_serve_result error_result(const Req &q, gcfg_status st) {
    gcfg_serve_result r;
    memset(&r, 0, sizeof(r));
    r.status = st;
    r.session = q.r.session;
    r.t_submit = q.t_submit;
    r.t_start = r.t_done = now_s();
    return r;
}

// Run one batch on a lane.  Sessions of the batch are marked busy, so no
// other thread touches their device state; no lock is held here.
gcfg_status run_batch(Lane &L, std::vector<Req> &batch, const std::vector<Session> &snap,
                      std::vector<char> &is_new) {
    Server &s = *L.sv;
    cudaStream_t st = L.st;
    const int n = (int)batch.size();
    int nt = 0, nnew = 0, nedit = 0;
    long long ch = 0;
    for (int k = 0; k < n; ++k) {
        const Session &x = snap[k];
        L.h_il[k] = x.slot;
        const long long nc = image_chunks(x.W, x.H);
        for (long long c = 0; c < nc; ++c) L.h_cmap[ch + c] = make_int2(x.slot, (int)c);
        ch += nc;
        for (long long i = 0; i < x.n_tiles; ++i) {
            const int t = (int)(x.tile0 + i);
            L.h_tl[nt++] = t;
            if (is_new[k]) L.h_tnew[nnew++] = t;
            else L.h_tedit[nedit++] = t;
        }
        if (is_new[k]) {
            // descriptor of the new session
            ImgDesc &d = L.h_desc[k];
            d.W = x.W;
            d.H = x.H;
            d.tiles_x = div_up(x.W, TILE_W);
            d.tiles_y = div_up(x.H, TILE_H);
            d.tile0 = (int)x.tile0;
            d.n_tiles = (int)x.n_tiles;
            d.pix0 = x.pix0;
            d.lambda = x.lambda;
            d.out0 = x.pix0;
            GCFG_CK(cudaMemcpyAsync(s.img + x.slot, &d, sizeof(ImgDesc), cudaMemcpyHostToDevice, st));
            k_fill_tile_owner<<<div_up((int)x.n_tiles, 256), 256, 0, st>>>(s.tile_img, x.tile0, (int)x.n_tiles, x.slot);
            g_launches.fetch_add(1, std::memory_order_relaxed);
            const size_t npx = (size_t)x.W * x.H;
            GCFG_CK(cudaMemcpyAsync(s.rgb + 3 * x.pix0, batch[k].r.h_rgb, 3 * npx, cudaMemcpyHostToDevice, st));
            GCFG_CK(cudaMemcpyAsync(s.scrib + x.pix0, batch[k].r.h_scrib, npx, cudaMemcpyHostToDevice, st));
        } else {
            // keep the current tables as the "previous" ones, then edit the scribbles
            GCFG_CK(cudaMemcpyAsync(s.odpl + (size_t)x.slot * NBINS, s.dpl + (size_t)x.slot * NBINS,
                                    NBINS * sizeof(int), cudaMemcpyDeviceToDevice, st));
            GCFG_CK(cudaMemcpyAsync(s.odnl + (size_t)x.slot * NBINS, s.dnl + (size_t)x.slot * NBINS,
                                    NBINS * sizeof(int), cudaMemcpyDeviceToDevice, st));
            const int sz = batch[k].r.edit_size;
            dim3 blk(16, 16), grd(div_up(sz, 16), div_up(sz, 16));
            k_edit_square<<<grd, blk, 0, st>>>(s.scrib + x.pix0, x.W, x.H, batch[k].r.edit_x, batch[k].r.edit_y, sz,
                                               batch[k].r.edit_class);
            g_launches.fetch_add(1, std::memory_order_relaxed);
        }
    }
    GCFG_CK(cudaMemcpyAsync(L.d_il, L.h_il, n * sizeof(int), cudaMemcpyHostToDevice, st));
    GCFG_CK(cudaMemcpyAsync(L.d_cmap, L.h_cmap, ch * sizeof(int2), cudaMemcpyHostToDevice, st));
    GCFG_CK(cudaMemcpyAsync(L.d_tl, L.h_tl, nt * sizeof(int), cudaMemcpyHostToDevice, st));
    if (nnew) GCFG_CK(cudaMemcpyAsync(L.d_tnew, L.h_tnew, nnew * sizeof(int), cudaMemcpyHostToDevice, st));
    if (nedit) GCFG_CK(cudaMemcpyAsync(L.d_tedit, L.h_tedit, nedit * sizeof(int), cudaMemcpyHostToDevice, st));
    k_slot_reset<<<div_up(n, 128), 128, 0, st>>>(L.d_il, n, s.ist);
    g_launches.fetch_add(1, std::memory_order_relaxed);

    // data term of every image of the batch (edits recompute their tables)
    DtArgs a;
    memset(&a, 0, sizeof(a));
    a.n_img = n;
    a.ilist = L.d_il;
    a.total_chunks = ch;
    a.rgb = s.rgb;
    a.scrib = s.scrib;
    a.img = s.img;
    a.ist = s.ist;
    a.chunk_map = L.d_cmap;
    a.hist = s.hist;
    a.dp_lut = s.dpl;
    a.dn_lut = s.dnl;
    for (int k = 0; k < n; ++k)
        GCFG_CK(cudaMemsetAsync(s.hist + (size_t)L.h_il[k] * 2 * NBINS, 0, 2 * NBINS * sizeof(int), st));
    GCFG_TRY(dt_tables(a, st));

    Batch b = arena_batch(s);
    b.lists = L.lists;
    b.list_cap = L.list_cap;
    b.ctl = L.ctl;
    if (nnew) {
        Batch bn = b;
        bn.tlist = L.d_tnew;
        bn.n_tlist = nnew;
        GCFG_TRY(dt_build(bn, a, st));
    }
    if (nedit) {
        Batch be = b;
        be.tlist = L.d_tedit;
        be.n_tlist = nedit;
        k_reparam<<<nedit, TILE_THREADS, 0, st>>>(be, s.rgb, s.dpl, s.dnl, s.odpl, s.odnl);
        g_launches.fetch_add(1, std::memory_order_relaxed);
        GCFG_CK(cudaGetLastError());
    }
    b.tlist = L.d_tl;
    b.n_tlist = nt;
    b.ilist = L.d_il;
    b.n_ilist = n;
    GCFG_CK(cudaMemsetAsync(L.ctl, 0, sizeof(Ctl), st));
    SolveParams prm = kDefaultSolveParams;
    prm.warps = solve_warps(prm.warps, nt);  // the lanes share the GPU in blocks of this shape
    GCFG_TRY(launch_solve(b, prm, nt, st,
                          s.cfg.lanes > 1 ? solve_grid_blocks(1 << 30, 0, prm.warps) / s.cfg.lanes : 0));
    GCFG_TRY(launch_extract_rows(b, L.d_cmap, ch, s.smin, s.smax, st));
    for (int k = 0; k < n; ++k) {
        const Session &x = snap[k];
        const size_t npx = (size_t)x.W * x.H;
        if (batch[k].r.h_smin)
            GCFG_CK(cudaMemcpyAsync(batch[k].r.h_smin, s.smin + x.pix0, npx, cudaMemcpyDeviceToHost, st));
        if (batch[k].r.h_smax)
            GCFG_CK(cudaMemcpyAsync(batch[k].r.h_smax, s.smax + x.pix0, npx, cudaMemcpyDeviceToHost, st));
        GCFG_CK(cudaMemcpyAsync(L.h_ist + k, s.ist + x.slot, sizeof(ImgState), cudaMemcpyDeviceToHost, st));
    }
    GCFG_CK(cudaMemcpyAsync(L.h_ctl, L.ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, st));
    GCFG_CK(cudaStreamSynchronize(st));
    return L.h_ctl->err ? GCFG_ERR_NOT_CONVERGED : GCFG_OK;
}

// Take runnable requests from the queue (caller holds the lock).
void take_batch(Server &s, std::vector<Req> &batch, std::vector<int64_t> &sids, std::vector<char> &is_new,
                std::vector<Session> &snap, long long max_tiles) {
    long long tiles = 0;
    for (auto it = s.queue.begin(); it != s.queue.end() && (int)batch.size() < s.cfg.max_batch_images;) {
        Req &q = *it;
        if (q.r.kind == GCFG_REQ_EDIT) {
            auto f = s.sessions.find(q.r.session);
            if (f == s.sessions.end()) {
                complete(s, q, error_result(q, GCFG_ERR_STATE));  // evicted or unknown
                it = s.queue.erase(it);
                continue;
            }
            Session &x = f->second;
            if (!x.admitted || x.busy || !x.ready || tiles + x.n_tiles > max_tiles) {
                ++it;
                continue;
            }
            x.busy = true;
            x.pending--;
            tiles += x.n_tiles;
            batch.push_back(q);
            sids.push_back(q.r.session);
            is_new.push_back(0);
            snap.push_back(x);
            it = s.queue.erase(it);
            continue;
        }
        const long long need = tiles_of(q.r.w, q.r.h);
        if (tiles + need > max_tiles) {
            ++it;
            continue;
        }
        // admission by device footprint: evict idle sessions (least recently
        // used first) until the image fits under the cap and in the arena
        long long t0 = -1, p0 = -1;
        for (;;) {
            if ((s.tiles.used + need) * (long long)TILE_BYTES <= s.cfg.mem_cap_bytes && !s.free_slots.empty()) {
                t0 = s.tiles.alloc(need);
                if (t0 >= 0) {
                    p0 = s.pixels.alloc(need * TPX);
                    if (p0 >= 0) break;
                    s.tiles.release(t0, need);
                    t0 = -1;
                }
            }
            if (!evict_one(s)) break;
        }
        if (t0 < 0) {
            ++it;  // waits until memory frees up
            continue;
        }
        Session &x = s.sessions[q.r.session];
        x.admitted = true;
        x.slot = s.free_slots.back();
        s.free_slots.pop_back();
        x.tile0 = t0;
        x.n_tiles = need;
        x.pix0 = p0;
        x.busy = true;
        const int64_t sid = q.r.session;
        s.stats.admitted++;
        tiles += need;
        batch.push_back(q);
        sids.push_back(sid);
        is_new.push_back(1);
        snap.push_back(x);
        it = s.queue.erase(it);
    }
}

void lane_main(Lane *L) {
    Server &s = *L->sv;
    cudaSetDevice(s.device);
    long long seen = -1;
    for (;;) {
        std::vector<Req> batch;
        std::vector<int64_t> sids;
        std::vector<char> is_new;
        std::vector<Session> snap;
        {
            std::unique_lock<std::mutex> lk(s.mu);
            for (;;) {
                if (s.stop) return;
                if (!s.queue.empty() && seen != s.gen) {
                    seen = s.gen;
                    take_batch(s, batch, sids, is_new, snap, L->list_cap);
                    if (!batch.empty()) break;
                    // nothing runnable now: wait for a completion or a new request
                }
                s.cv_work.wait(lk);
            }
        }
        const double t_start = now_s();
        const gcfg_status rc = run_batch(*L, batch, snap, is_new);
        const double t_done = now_s();
        {
            std::lock_guard<std::mutex> lk(s.mu);
            for (size_t k = 0; k < batch.size(); ++k) {
                Session &x = s.sessions[sids[k]];
                gcfg_serve_result r;
                memset(&r, 0, sizeof(r));
                r.status = rc;
                r.warm = is_new[k] ? 0 : 1;
                r.session = sids[k];
                r.flow = (long long)L->h_ist[k].interior_dp - (long long)L->h_ist[k].pos_excess;
                r.batch_images = (int)batch.size();
                r.lane = L->id;
                r.t_submit = batch[k].t_submit;
                r.t_start = t_start;
                r.t_done = t_done;
                complete(s, batch[k], r);
                x.busy = false;
                x.ready = rc == GCFG_OK;
                x.last_use = t_done;
            }
            s.stats.batches++;
            s.stats.completed += (long long)batch.size();
            s.gen++;
        }
        s.cv_done.notify_all();
        s.cv_work.notify_all();
    }
}

void shutdown_server(Server *s) {
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
    }
    s->cv_work.notify_all();
    for (Lane *L : s->lanes) {
        if (L->th.joinable()) L->th.join();
        cudaStreamDestroy(L->st);
        cudaFree(L->ctl); cudaFree(L->lists); cudaFree(L->d_tl); cudaFree(L->d_tnew); cudaFree(L->d_tedit);
        cudaFree(L->d_il); cudaFree(L->d_cmap);
        cudaFreeHost(L->h_ctl); cudaFreeHost(L->h_tl); cudaFreeHost(L->h_tnew); cudaFreeHost(L->h_tedit);
        cudaFreeHost(L->h_il); cudaFreeHost(L->h_cmap); cudaFreeHost(L->h_desc); cudaFreeHost(L->h_ist);
        delete L;
    }
    cudaFree(s->cap); cudaFree(s->exc); cudaFree(s->h); cudaFree(s->hb); cudaFree(s->tnb); cudaFree(s->hfin); cudaFree(s->reach); cudaFree(s->tmask); cudaFree(s->tact);
    cudaFree(s->tpos); cudaFree(s->mpush); cudaFree(s->mgr); cudaFree(s->tile_img);
    cudaFree(s->rgb); cudaFree(s->scrib); cudaFree(s->smin); cudaFree(s->smax);
    cudaFree(s->img); cudaFree(s->ist); cudaFree(s->hist); cudaFree(s->dpl); cudaFree(s->dnl);
    cudaFree(s->odpl); cudaFree(s->odnl);
}

}  // namespace
}  // namespace gcfg

using namespace gcfg;

struct gcfg_server {
    Server s;
};

extern "C" {

gcfg_status gcfg_serve_create(const gcfg_serve_config *cfg, gcfg_server **out) {
    if (!cfg || !out || cfg->mem_cap_bytes < (long long)TILE_BYTES || cfg->lanes < 1 || cfg->lanes > 8 ||
        cfg->max_batch_images < 1 || cfg->max_batch_tiles < 1 || cfg->max_sessions < 1)
        return GCFG_ERR_INVALID;
    gcfg_server *srv = new gcfg_server();
    Server *s = &srv->s;
    s->cfg = *cfg;
    memset(&s->stats, 0, sizeof(s->stats));
    cudaGetDevice(&s->device);
    s->tiles_cap = cfg->mem_cap_bytes / (long long)TILE_BYTES;
    s->px_cap = s->tiles_cap * TPX;
    s->tiles.init(s->tiles_cap);
    s->pixels.init(s->px_cap);
    const size_t T = (size_t)s->tiles_cap, NS = (size_t)cfg->max_sessions;
    gcfg_status rc = GCFG_OK;
    auto chk = [&](gcfg_status r) { if (rc == GCFG_OK) rc = r; };
    chk(dalloc(s->cap, T * TPX)); chk(dalloc(s->exc, T * TPX)); chk(dalloc(s->h, T * TPX)); chk(dalloc(s->hb, T * 4 * 32)); chk(dalloc(s->tnb, T)); chk(dalloc(s->hfin, T * 32));
    chk(dalloc(s->reach, T * 32)); chk(dalloc(s->tmask, T * 6 * 32)); chk(dalloc(s->tact, T));
    chk(dalloc(s->tpos, T)); chk(dalloc(s->mpush, T)); chk(dalloc(s->mgr, T)); chk(dalloc(s->tile_img, T));
    chk(dalloc(s->rgb, 3 * (size_t)s->px_cap)); chk(dalloc(s->scrib, (size_t)s->px_cap));
    chk(dalloc(s->smin, (size_t)s->px_cap)); chk(dalloc(s->smax, (size_t)s->px_cap));
    chk(dalloc(s->img, NS)); chk(dalloc(s->ist, NS)); chk(dalloc(s->hist, NS * 2 * NBINS));
    chk(dalloc(s->dpl, NS * NBINS)); chk(dalloc(s->dnl, NS * NBINS));
    chk(dalloc(s->odpl, NS * NBINS)); chk(dalloc(s->odnl, NS * NBINS));
    if (rc == GCFG_OK) {
        // every slot starts "solved" so that solves of other slots skip it
        std::vector<ImgState> init(NS);
        memset(init.data(), 0, NS * sizeof(ImgState));
        for (auto &x : init) x.done = 1;
        if (cudaMemcpy(s->ist, init.data(), NS * sizeof(ImgState), cudaMemcpyHostToDevice) != cudaSuccess)
            rc = GCFG_ERR_CUDA;
    }
    for (int i = cfg->max_sessions - 1; i >= 0; --i) s->free_slots.push_back(i);
    for (int l = 0; l < cfg->lanes && rc == GCFG_OK; ++l) {
        Lane *L = new Lane();
        L->sv = s;
        L->id = l;
        L->list_cap = (int)cfg->max_batch_tiles;
        const size_t LT = (size_t)cfg->max_batch_tiles, LI = (size_t)cfg->max_batch_images;
        if (cudaStreamCreateWithFlags(&L->st, cudaStreamNonBlocking) != cudaSuccess) chk(GCFG_ERR_CUDA);
        chk(dalloc(L->ctl, 1)); chk(halloc(L->h_ctl, 1));
        chk(dalloc(L->lists, (size_t)L_NLISTS * LT));
        chk(dalloc(L->d_tl, LT)); chk(halloc(L->h_tl, LT));
        chk(dalloc(L->d_tnew, LT)); chk(halloc(L->h_tnew, LT));
        chk(dalloc(L->d_tedit, LT)); chk(halloc(L->h_tedit, LT));
        chk(dalloc(L->d_il, LI)); chk(halloc(L->h_il, LI));
        // chunks of a batch: at most its pixels / CHUNK_PX + one per image
        chk(dalloc(L->d_cmap, LT * TPX / CHUNK_PX + LI + 1)); chk(halloc(L->h_cmap, LT * TPX / CHUNK_PX + LI + 1));
        chk(halloc(L->h_desc, LI)); chk(halloc(L->h_ist, LI));
        s->lanes.push_back(L);
    }
    if (rc) {
        shutdown_server(s);
        delete srv;
        return rc;
    }
    for (Lane *L : s->lanes) L->th = std::thread(lane_main, L);
    *out = srv;
    return GCFG_OK;
}

gcfg_status gcfg_serve_submit(gcfg_server *srv, const gcfg_serve_request *r, int64_t *ticket,
                              int64_t *session) {
    if (!srv || !r || !ticket) return GCFG_ERR_INVALID;
    Server *s = &srv->s;
    if (r->kind == GCFG_REQ_NEW) {
        if (r->w < 3 || r->h < 3 || !r->h_rgb || !r->h_scrib || !(r->lambda >= 0) ||
            r->lambda * 1.0000001 + 1 > (double)GCFG_MAX_CAP)
            return GCFG_ERR_INVALID;
        const long long need = tiles_of(r->w, r->h);
        if (need > s->cfg.max_batch_tiles || need * (long long)TILE_BYTES > s->cfg.mem_cap_bytes)
            return GCFG_ERR_CAPACITY;  // could never be admitted
    } else if (r->kind == GCFG_REQ_EDIT) {
        if (r->edit_size < 1 || (r->edit_class != 1 && r->edit_class != 2)) return GCFG_ERR_INVALID;
    } else {
        return GCFG_ERR_INVALID;
    }
    {
        std::lock_guard<std::mutex> lk(s->mu);
        if (r->kind == GCFG_REQ_EDIT) {
            auto f = s->sessions.find(r->session);
            if (f == s->sessions.end()) return GCFG_ERR_STATE;
            f->second.pending++;
        }
        Req q;
        q.ticket = s->next_ticket++;
        q.r = *r;
        q.t_submit = now_s();
        if (r->kind == GCFG_REQ_NEW) {
            // the resident image exists from now on; edits may refer to it
            // and wait until its first solve is done
            Session x;
            x.W = r->w;
            x.H = r->h;
            x.lambda = r->lambda;
            q.r.session = s->next_session++;
            s->sessions[q.r.session] = x;
        }
        if (session) *session = q.r.session;
        s->tickets[q.ticket] = TicketState();
        s->queue.push_back(q);
        s->stats.submitted++;
        s->gen++;
        *ticket = q.ticket;
    }
    s->cv_work.notify_one();
    return GCFG_OK;
}

gcfg_status gcfg_serve_wait(gcfg_server *srv, int64_t ticket, gcfg_serve_result *res, int timeout_ms) {
    if (!srv || !res) return GCFG_ERR_INVALID;
    Server *s = &srv->s;
    std::unique_lock<std::mutex> lk(s->mu);
    auto f = s->tickets.find(ticket);
    if (f == s->tickets.end()) return GCFG_ERR_INVALID;
    const auto until = std::chrono::steady_clock::now() + std::chrono::milliseconds(timeout_ms < 0 ? 0 : timeout_ms);
    while (!s->tickets[ticket].done) {
        if (timeout_ms < 0) s->cv_done.wait(lk);
        else if (s->cv_done.wait_until(lk, until) == std::cv_status::timeout && !s->tickets[ticket].done)
            return GCFG_ERR_NOT_CONVERGED;
    }
    *res = s->tickets[ticket].res;
    s->tickets.erase(ticket);
    return (gcfg_status)res->status;
}

gcfg_status gcfg_serve_release(gcfg_server *srv, int64_t session) {
    if (!srv) return GCFG_ERR_INVALID;
    Server *s = &srv->s;
    std::lock_guard<std::mutex> lk(s->mu);
    auto f = s->sessions.find(session);
    if (f == s->sessions.end()) return GCFG_ERR_STATE;
    Session &x = f->second;
    if (!x.admitted || x.busy || x.pending > 0) return GCFG_ERR_STATE;
    s->tiles.release(x.tile0, x.n_tiles);
    s->pixels.release(x.pix0, x.n_tiles * TPX);
    s->free_slots.push_back(x.slot);
    s->sessions.erase(f);
    return GCFG_OK;
}

gcfg_status gcfg_serve_get_stats(gcfg_server *srv, gcfg_serve_stats *out) {
    if (!srv || !out) return GCFG_ERR_INVALID;
    Server *s = &srv->s;
    std::lock_guard<std::mutex> lk(s->mu);
    *out = s->stats;
    out->bytes_in_use = s->bytes_in_use();
    out->sessions = (int64_t)s->sessions.size();
    out->queued = (int64_t)s->queue.size();
    return GCFG_OK;
}

gcfg_status gcfg_serve_destroy(gcfg_server *srv) {
    if (!srv) return GCFG_ERR_INVALID;
    shutdown_server(&srv->s);
    delete srv;
    return GCFG_OK;
}

double gcfg_serve_now(void) { return now_s(); }

}  // extern "C"
