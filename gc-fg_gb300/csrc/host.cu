// host.cu -- the engine's host side and the C ABI (include/gcfg.h).
//
// An Engine owns the device buffers of one batch (tile arena, queues,
// per-image tables) sized for a capacity that only grows, uploads the batch
// layout, and runs: data term -> build -> persistent solve -> extraction,
// all on one stream.  The reference-facing graph API, the one-image
// segmenter and the batch API are thin layers over it.
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <utility>
#include <vector>

#include "dataterm.cuh"
#include "engine.cuh"

namespace gcfg {

template <typename T>
static gcfg_status grow(T *&p, size_t &cap, size_t need) {
    if (need <= cap && p) return GCFG_OK;
    cudaFree(p);
    p = nullptr;
    cap = 0;
    size_t n = need < 1 ? 1 : need;
    if (cudaMalloc(&p, n * sizeof(T)) != cudaSuccess) return GCFG_ERR_OOM;
    cap = n;
    return GCFG_OK;
}

template <typename T>
static gcfg_status grow_host(T *&p, size_t &cap, size_t need) {
    if (need <= cap && p) return GCFG_OK;
    if (p) cudaFreeHost(p);
    p = nullptr;
    cap = 0;
    size_t n = need < 1 ? 1 : need;
    if (cudaMallocHost(&p, n * sizeof(T)) != cudaSuccess) return GCFG_ERR_OOM;
    cap = n;
    return GCFG_OK;
}

struct Engine {
    cudaStream_t st = nullptr;
    SolveParams prm = kDefaultSolveParams;

    int n_img = 0, n_tiles = 0;
    long long n_px = 0, total_chunks = 0;

    // device
    ImgDesc *d_img = nullptr; size_t c_img = 0;
    ImgState *d_ist = nullptr; size_t c_ist = 0;
    int2 *d_cmap = nullptr; size_t c_cmap = 0;  // per chunk of the data-term pass: (image, chunk in image)
    int *d_tile_img = nullptr; size_t c_timg = 0;
    int4 *d_cap = nullptr; size_t c_cap = 0;
    int *d_exc = nullptr; size_t c_exc = 0;
    int *d_h = nullptr; size_t c_h = 0;
    int *d_hb = nullptr; size_t c_hb = 0;
    int4 *d_tnb = nullptr; size_t c_tnb = 0;
    unsigned *d_hfin = nullptr; size_t c_hfin = 0;
    unsigned *d_reach = nullptr; size_t c_reach = 0;
    unsigned *d_tmask = nullptr; size_t c_tmask = 0;
    int *d_tact = nullptr; size_t c_tact = 0;
    unsigned long long *d_tpos = nullptr; size_t c_tpos = 0;
    int *d_lists = nullptr; size_t c_lists = 0; int list_cap = 0;
    int *d_mpush = nullptr; size_t c_mpush = 0;
    int *d_mgr = nullptr; size_t c_mgr = 0;
    Ctl *d_ctl = nullptr; size_t c_ctl = 0;
    int *d_hist = nullptr; size_t c_hist = 0;
    int *d_dpl = nullptr; size_t c_dpl = 0;
    int *d_dnl = nullptr; size_t c_dnl = 0;
    double *d_raw = nullptr; size_t c_raw = 0;
    // staging for host entry points
    uint8_t *d_rgb = nullptr; size_t c_rgb = 0;
    uint8_t *d_scrib = nullptr; size_t c_scrib = 0;
    uint8_t *d_smin = nullptr; size_t c_smin = 0;
    uint8_t *d_smax = nullptr; size_t c_smax = 0;
    // host (pinned)
    ImgDesc *h_img = nullptr; size_t ch_img = 0;
    ImgState *h_ist = nullptr; size_t ch_ist = 0;
    long long *h_chunk = nullptr; size_t ch_chunk = 0;  // first chunk of each image
    int2 *h_cmap = nullptr; size_t ch_cmap = 0;
    int *h_tile_img = nullptr; size_t ch_timg = 0;
    Ctl *h_ctl = nullptr; size_t ch_ctl = 0;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;

    int max_grid = 0;  // solver blocks (0: as many as fit, capped at half the tiles)

    // CUDA graphs of the device part of batch runs (opt-in, see run_batch_graph)
    struct GraphEntry {
        std::vector<int> w, h;
        std::vector<double> lam;
        const void *ptr[4];
        int kind;  // 0 device-resident run, 1 blocking host call, 2 asynchronous host call
        SolveParams prm;
        int grid;
        long long alloc_gen;
        long long kernels;
        long long last_use;
        cudaGraphExec_t exec;
    };
    static constexpr int MAX_GRAPHS = 4;
    bool graph_on = false, graph_broken = false;
    std::vector<GraphEntry> graphs;
    cudaStream_t cap_st = nullptr;
    long long graph_kernels = 0, graph_replays = 0, graph_captures = 0, graph_clock = 0;
    long long alloc_gen = 0;  // bumped whenever a buffer is reallocated

    // Host entry points of many images: groups of consecutive images are
    // uploaded on cp_st while earlier groups already compute on st.
    static constexpr int MAX_GROUPS = 4;
    struct Group {
        int i0, i1, t0, t1;
        long long p0, p1, c0, c1;
    };
    std::vector<Group> groups;
    cudaStream_t cp_st = nullptr;
    cudaEvent_t ev_in[MAX_GROUPS] = {}, ev_out[MAX_GROUPS] = {}, ev_mark = nullptr;
    int *d_iota = nullptr; size_t c_iota = 0; int iota_n = 0;   // 0, 1, 2, ... (image and tile lists)
    // sizes and lambdas of the layout currently on the device
    std::vector<int> lay_w, lay_h;
    std::vector<double> lay_lam;

    // Asynchronous host entry point: two batches in flight, each with its
    // own pinned host tables, device staging buffers and timing events.  The
    // set of the batch being queued or collected is swapped into the members
    // above for the duration of that call (slot 0 is the members' own set,
    // slot 1 is `alt`), so the rest of the engine is unchanged.  Compute of
    // the two batches stays ordered on st; their uploads (cp_st) and
    // downloads (dn_st) overlap the other batch's compute.
    struct RunSet {
        ImgDesc *h_img = nullptr; size_t ch_img = 0;
        ImgState *h_ist = nullptr; size_t ch_ist = 0;
        long long *h_chunk = nullptr; size_t ch_chunk = 0;
        int2 *h_cmap = nullptr; size_t ch_cmap = 0;
        int *h_tile_img = nullptr; size_t ch_timg = 0;
        Ctl *h_ctl = nullptr; size_t ch_ctl = 0;
        uint8_t *d_rgb = nullptr; size_t c_rgb = 0;
        uint8_t *d_scrib = nullptr; size_t c_scrib = 0;
        uint8_t *d_smin = nullptr; size_t c_smin = 0;
        uint8_t *d_smax = nullptr; size_t c_smax = 0;
        cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    };
    RunSet alt;
    struct Flight {
        bool busy = false;
        long long ticket = 0;
        int n = 0;
        cudaEvent_t ev_up = nullptr;   // inputs of the batch uploaded (cp_st)
        cudaEvent_t ev_ext = nullptr;  // labels of the batch extracted (st)
        cudaEvent_t ev_dn = nullptr;   // downloads of the batch done (dn_st)
    };
    Flight flight[2];
    cudaStream_t dn_st = nullptr;
    long long next_ticket = 1;
    int next_slot = 0;

    bool in_flight() const { return flight[0].busy || flight[1].busy; }

    void swap_set(RunSet &o) {
        std::swap(h_img, o.h_img); std::swap(ch_img, o.ch_img);
        std::swap(h_ist, o.h_ist); std::swap(ch_ist, o.ch_ist);
        std::swap(h_chunk, o.h_chunk); std::swap(ch_chunk, o.ch_chunk);
        std::swap(h_tile_img, o.h_tile_img); std::swap(ch_timg, o.ch_timg);
        std::swap(h_cmap, o.h_cmap); std::swap(ch_cmap, o.ch_cmap);
        std::swap(h_ctl, o.h_ctl); std::swap(ch_ctl, o.ch_ctl);
        std::swap(d_rgb, o.d_rgb); std::swap(c_rgb, o.c_rgb);
        std::swap(d_scrib, o.d_scrib); std::swap(c_scrib, o.c_scrib);
        std::swap(d_smin, o.d_smin); std::swap(c_smin, o.c_smin);
        std::swap(d_smax, o.d_smax); std::swap(c_smax, o.c_smax);
        std::swap(ev0, o.ev0); std::swap(ev1, o.ev1);
    }

    static void free_set(RunSet &o) {
        if (o.h_img) cudaFreeHost(o.h_img);
        if (o.h_ist) cudaFreeHost(o.h_ist);
        if (o.h_chunk) cudaFreeHost(o.h_chunk);
        if (o.h_tile_img) cudaFreeHost(o.h_tile_img);
        if (o.h_cmap) cudaFreeHost(o.h_cmap);
        if (o.h_ctl) cudaFreeHost(o.h_ctl);
        cudaFree(o.d_rgb); cudaFree(o.d_scrib); cudaFree(o.d_smin); cudaFree(o.d_smax);
        if (o.ev0) cudaEventDestroy(o.ev0);
        if (o.ev1) cudaEventDestroy(o.ev1);
        o = RunSet();
    }

    ~Engine() { release(); }

    void drop_graphs() {
        for (auto &g : graphs) cudaGraphExecDestroy(g.exec);
        graphs.clear();
    }

    bool laid_out(int n, const int *W, const int *H, const double *lam) const {
        if ((int)lay_w.size() != n) return false;
        for (int i = 0; i < n; ++i)
            if (lay_w[i] != W[i] || lay_h[i] != H[i] || lay_lam[i] != lam[i]) return false;
        return true;
    }

    void release() {
        free_set(alt);
        for (Flight &f : flight) {
            if (f.ev_up) cudaEventDestroy(f.ev_up);
            if (f.ev_ext) cudaEventDestroy(f.ev_ext);
            if (f.ev_dn) cudaEventDestroy(f.ev_dn);
            f = Flight();
        }
        if (dn_st) cudaStreamDestroy(dn_st);
        dn_st = nullptr;
        cudaFree(d_img); cudaFree(d_ist); cudaFree(d_cmap); cudaFree(d_tile_img);
        cudaFree(d_cap); cudaFree(d_exc); cudaFree(d_h); cudaFree(d_hb); cudaFree(d_tnb); cudaFree(d_hfin); cudaFree(d_reach);
        cudaFree(d_tmask); cudaFree(d_tact); cudaFree(d_tpos);
        cudaFree(d_lists);
        cudaFree(d_mpush); cudaFree(d_mgr); cudaFree(d_ctl);
        cudaFree(d_hist); cudaFree(d_dpl); cudaFree(d_dnl); cudaFree(d_raw);
        cudaFree(d_rgb); cudaFree(d_scrib); cudaFree(d_smin); cudaFree(d_smax);
        if (h_img) cudaFreeHost(h_img);
        if (h_ist) cudaFreeHost(h_ist);
        if (h_chunk) cudaFreeHost(h_chunk);
        if (h_cmap) cudaFreeHost(h_cmap);
        if (h_tile_img) cudaFreeHost(h_tile_img);
        if (h_ctl) cudaFreeHost(h_ctl);
        if (ev0) cudaEventDestroy(ev0);
        if (ev1) cudaEventDestroy(ev1);
        drop_graphs();
        if (cap_st) cudaStreamDestroy(cap_st);
        cap_st = nullptr;
        if (cp_st) cudaStreamDestroy(cp_st);
        cp_st = nullptr;
        for (int g = 0; g < MAX_GROUPS; ++g) {
            if (ev_in[g]) cudaEventDestroy(ev_in[g]);
            if (ev_out[g]) cudaEventDestroy(ev_out[g]);
            ev_in[g] = ev_out[g] = nullptr;
        }
        if (ev_mark) cudaEventDestroy(ev_mark);
        ev_mark = nullptr;
        cudaFree(d_iota);
        d_iota = nullptr;
        d_img = nullptr; d_ist = nullptr; d_cmap = nullptr; d_tile_img = nullptr;
        d_cap = nullptr; d_exc = nullptr; d_h = nullptr; d_hb = nullptr; d_tnb = nullptr; d_hfin = nullptr; d_reach = nullptr;
        d_tmask = nullptr; d_tact = nullptr; d_tpos = nullptr;
        d_lists = nullptr;
        d_mpush = d_mgr = nullptr; d_ctl = nullptr;
        d_hist = d_dpl = d_dnl = nullptr; d_raw = nullptr;
        d_rgb = d_scrib = d_smin = d_smax = nullptr;
        h_img = nullptr; h_ist = nullptr; h_chunk = nullptr; h_cmap = nullptr; h_tile_img = nullptr; h_ctl = nullptr;
        ev0 = ev1 = nullptr;
    }

    gcfg_status init() {
        GCFG_CK(cudaEventCreate(&ev0));
        GCFG_CK(cudaEventCreate(&ev1));
        GCFG_TRY(grow(d_ctl, c_ctl, 1));
        GCFG_TRY(grow_host(h_ctl, ch_ctl, 1));
        return GCFG_OK;
    }

    // Sizes of a batch -> tile count (no allocation).
    static void count(int n, const int *W, const int *H, int &tiles, long long &px) {
        tiles = 0;
        px = 0;
        for (int i = 0; i < n; ++i) {
            tiles += div_up(W[i], TILE_W) * div_up(H[i], TILE_H);
            px += (long long)W[i] * H[i];
        }
    }

    std::vector<const void *> buffers() const {
        return {d_img, d_ist, d_cmap, d_tile_img, d_cap, d_exc, d_h, d_hb, d_tnb, d_hfin, d_reach, d_tmask, d_tact, d_tpos,
                d_lists, d_mpush, d_mgr, d_ctl, d_hist, d_dpl, d_dnl, d_rgb, d_scrib, d_smin, d_smax,
                h_img, h_ist, h_chunk, h_cmap, h_tile_img, h_ctl};
    }

    // Grow the buffers; any reallocation invalidates the captured graphs.
    gcfg_status reserve(int imgs, int tiles, long long px, bool dataterm, bool staging, bool arena = true) {
        const std::vector<const void *> before = buffers();
        const gcfg_status rc = reserve_(imgs, tiles, px, dataterm, staging, arena);
        if (buffers() != before) ++alloc_gen;
        return rc;
    }

    gcfg_status reserve_(int imgs, int tiles, long long px, bool dataterm, bool staging, bool arena) {
        GCFG_TRY(grow(d_img, c_img, imgs));
        GCFG_TRY(grow(d_ist, c_ist, imgs));
        // chunks of the data-term pass: at most px / CHUNK_PX + one per image
        const size_t chunks = (size_t)(px / CHUNK_PX) + (size_t)imgs + 1;
        GCFG_TRY(grow(d_cmap, c_cmap, chunks));
        GCFG_TRY(grow_host(h_cmap, ch_cmap, chunks));
        if (arena) {
            GCFG_TRY(grow(d_tile_img, c_timg, tiles));
            GCFG_TRY(grow(d_cap, c_cap, (size_t)tiles * TPX));
            GCFG_TRY(grow(d_exc, c_exc, (size_t)tiles * TPX));
            GCFG_TRY(grow(d_h, c_h, (size_t)tiles * TPX));
            GCFG_TRY(grow(d_hb, c_hb, (size_t)tiles * 4 * 32));
            GCFG_TRY(grow(d_tnb, c_tnb, (size_t)tiles));
            GCFG_TRY(grow(d_hfin, c_hfin, (size_t)tiles * 32));
            GCFG_TRY(grow(d_reach, c_reach, (size_t)tiles * 32));
            GCFG_TRY(grow(d_tmask, c_tmask, (size_t)tiles * 6 * 32));
            GCFG_TRY(grow(d_tact, c_tact, tiles));
            GCFG_TRY(grow(d_tpos, c_tpos, tiles));
            if ((size_t)tiles > (size_t)list_cap || !d_lists) {
                GCFG_TRY(grow(d_lists, c_lists, (size_t)L_NLISTS * tiles));
                list_cap = tiles;
            }
            GCFG_TRY(grow(d_mpush, c_mpush, tiles));
            GCFG_TRY(grow(d_mgr, c_mgr, tiles));
        }
        GCFG_TRY(grow_host(h_img, ch_img, imgs));
        GCFG_TRY(grow_host(h_ist, ch_ist, imgs));
        GCFG_TRY(grow_host(h_chunk, ch_chunk, (size_t)imgs + 1));
        if (arena) GCFG_TRY(grow_host(h_tile_img, ch_timg, tiles));
        if (dataterm) {
            GCFG_TRY(grow(d_hist, c_hist, (size_t)imgs * 2 * NBINS));
            GCFG_TRY(grow(d_dpl, c_dpl, (size_t)imgs * NBINS));
            GCFG_TRY(grow(d_dnl, c_dnl, (size_t)imgs * NBINS));
        }
        if (staging) {
            GCFG_TRY(grow(d_rgb, c_rgb, (size_t)px * 3));
            GCFG_TRY(grow(d_scrib, c_scrib, (size_t)px));
            GCFG_TRY(grow(d_smin, c_smin, (size_t)px));
            GCFG_TRY(grow(d_smax, c_smax, (size_t)px));
        }
        return GCFG_OK;
    }

    // Lay out a batch: descriptors, tile -> image map, chunk offsets; upload.
    gcfg_status layout(int n, const int *W, const int *H, const double *lam, bool dataterm, bool staging,
                       bool arena = true) {
        if (n < 1) return GCFG_ERR_INVALID;
        for (int i = 0; i < n; ++i) {
            if (W[i] < 1 || H[i] < 1 || (long long)W[i] * H[i] > (1LL << 31) - 1) return GCFG_ERR_INVALID;
            if (lam && !(lam[i] >= 0.0 && lam[i] * 1.0000001 + 1 <= (double)GCFG_MAX_CAP)) return GCFG_ERR_INVALID;
        }
        int tiles;
        long long px;
        count(n, W, H, tiles, px);
        if ((long long)tiles * TPX > (1LL << 40)) return GCFG_ERR_INVALID;
        GCFG_TRY(reserve(n, tiles, px, dataterm, staging, arena));
        int t = 0;
        long long p = 0, ch = 0;
        for (int i = 0; i < n; ++i) {
            ImgDesc &d = h_img[i];
            d.W = W[i];
            d.H = H[i];
            d.tiles_x = div_up(W[i], TILE_W);
            d.tiles_y = div_up(H[i], TILE_H);
            d.tile0 = t;
            d.n_tiles = d.tiles_x * d.tiles_y;
            d.pix0 = p;
            d.lambda = lam ? lam[i] : 0.0;
            d.out0 = p;
            if (arena)
                for (int k = 0; k < d.n_tiles; ++k) h_tile_img[t + k] = i;
            h_chunk[i] = ch;
            t += d.n_tiles;
            p += (long long)W[i] * H[i];
            ch += image_chunks(W[i], H[i]);
        }
        h_chunk[n] = ch;
        for (int i = 0; i < n; ++i)
            for (long long c = h_chunk[i]; c < h_chunk[i + 1]; ++c) h_cmap[c] = make_int2(i, (int)(c - h_chunk[i]));
        n_img = n;
        n_tiles = t;
        n_px = p;
        total_chunks = ch;
        GCFG_CK(cudaMemcpyAsync(d_img, h_img, n * sizeof(ImgDesc), cudaMemcpyHostToDevice, st));
        GCFG_CK(cudaMemcpyAsync(d_cmap, h_cmap, (size_t)ch * sizeof(int2), cudaMemcpyHostToDevice, st));
        if (arena)
            GCFG_CK(cudaMemcpyAsync(d_tile_img, h_tile_img, (size_t)t * sizeof(int), cudaMemcpyHostToDevice, st));
        GCFG_CK(cudaMemsetAsync(d_ist, 0, n * sizeof(ImgState), st));
        lay_w.assign(W, W + n);
        lay_h.assign(H, H + n);
        if (lam)
            lay_lam.assign(lam, lam + n);
        else
            lay_lam.assign(n, 0.0);
        return GCFG_OK;
    }

    // Split the laid-out batch into up to MAX_GROUPS groups of consecutive
    // images of about equal pixel counts, and upload their lists.
    gcfg_status make_groups(int n, const int *W, const int *H) {
        const int G = n < MAX_GROUPS ? n : MAX_GROUPS;
        groups.clear();
        long long p = 0, c = 0;
        int t = 0, i = 0;
        for (int g = 0; g < G; ++g) {
            Group gr;
            gr.i0 = i;
            gr.p0 = p;
            gr.t0 = t;
            gr.c0 = c;
            const long long target = n_px * (g + 1) / G;
            while (i < n && (i == gr.i0 || p < target) && n - i > G - 1 - g) {
                p += (long long)W[i] * H[i];
                t += div_up(W[i], TILE_W) * div_up(H[i], TILE_H);
                ++i;
            }
            if (g == G - 1) {
                while (i < n) {
                    p += (long long)W[i] * H[i];
                    t += div_up(W[i], TILE_W) * div_up(H[i], TILE_H);
                    ++i;
                }
            }
            gr.i1 = i;
            gr.p1 = p;
            gr.t1 = t;
            gr.c1 = h_chunk[i];
            c = gr.c1;
            groups.push_back(gr);
        }
        const int need_iota = n > n_tiles ? n : n_tiles;
        if (need_iota > iota_n || !d_iota) {
            GCFG_TRY(grow(d_iota, c_iota, (size_t)need_iota));
            std::vector<int> iota((size_t)need_iota);
            for (int k = 0; k < need_iota; ++k) iota[k] = k;
            GCFG_CK(cudaMemcpy(d_iota, iota.data(), iota.size() * sizeof(int), cudaMemcpyHostToDevice));
            iota_n = need_iota;
        }
        if (!cp_st) GCFG_CK(cudaStreamCreateWithFlags(&cp_st, cudaStreamNonBlocking));
        for (int g = 0; g < MAX_GROUPS; ++g) {
            if (!ev_in[g]) GCFG_CK(cudaEventCreateWithFlags(&ev_in[g], cudaEventDisableTiming));
            if (!ev_out[g]) GCFG_CK(cudaEventCreateWithFlags(&ev_out[g], cudaEventDisableTiming));
        }
        if (!ev_mark) GCFG_CK(cudaEventCreateWithFlags(&ev_mark, cudaEventDisableTiming));
        return GCFG_OK;
    }

    Batch batch() const {
        Batch b;
        b.n_img = n_img;
        b.n_tiles = n_tiles;
        b.tlist = nullptr;
        b.n_tlist = 0;
        b.ilist = nullptr;
        b.n_ilist = 0;
        b.img = d_img;
        b.ist = d_ist;
        b.tile_img = d_tile_img;
        b.cap = d_cap;
        b.exc = d_exc;
        b.h = d_h;
        b.hb = d_hb;
        b.tile_nb = d_tnb;
        b.hfin = d_hfin;
        b.reach = d_reach;
        b.tmask = d_tmask;
        b.tile_act = d_tact;
        b.tile_pos = d_tpos;
        b.lists = d_lists;
        b.list_cap = list_cap;
        b.mark_push = d_mpush;
        b.mark_gr = d_mgr;
        b.ctl = d_ctl;
        return b;
    }

    DtArgs dt(const uint8_t *rgb, const uint8_t *scrib) const {
        DtArgs a;
        a.n_img = n_img;
        a.ilist = nullptr;
        a.total_chunks = total_chunks;
        a.rgb = rgb;
        a.scrib = scrib;
        a.img = d_img;
        a.ist = d_ist;
        a.chunk_map = d_cmap;
        a.hist = d_hist;
        a.dp_lut = d_dpl;
        a.dn_lut = d_dnl;
        a.raw_dp = nullptr;
        a.raw_dn = nullptr;
        return a;
    }

    gcfg_status build_images(const uint8_t *rgb, const uint8_t *scrib) {
        DtArgs a = dt(rgb, scrib);
        GCFG_TRY(dt_tables(a, st));
        return dt_build(batch(), a, st);
    }

    gcfg_status solve() {
        GCFG_CK(cudaMemsetAsync(d_ctl, 0, sizeof(Ctl), st));
        return launch_solve(batch(), prm, n_tiles, st, max_grid);
    }

    // Queue the read-back of the per-image states and the control block.
    gcfg_status readback() {
        GCFG_CK(cudaMemcpyAsync(h_ist, d_ist, n_img * sizeof(ImgState), cudaMemcpyDeviceToHost, st));
        GCFG_CK(cudaMemcpyAsync(h_ctl, d_ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, st));
        return GCFG_OK;
    }

    // Read the per-image states and the control block (synchronises).
    gcfg_status fetch() {
        GCFG_TRY(readback());
        GCFG_CK(cudaStreamSynchronize(st));
        return GCFG_OK;
    }

    gcfg_status status() const {
        if (h_ctl->err) return GCFG_ERR_NOT_CONVERGED;
        return GCFG_OK;
    }

    void result(int i, gcfg_result *r, float ms) const {
        memset(r, 0, sizeof(*r));
        const ImgState &s = h_ist[i];
        r->flow = (long long)s.interior_dp - (long long)s.pos_excess;
        r->ref_energy = (int32_t)((uint32_t)s.ref_init - (uint32_t)s.pos_excess);
        r->status = status();
        r->global_relabels = h_ctl->global_relabels;
        r->closure_checks = h_ctl->closure_checks;
        r->closure_ends = h_ctl->closure_ends;
        r->gr_sweeps = h_ctl->gr_rounds;
        r->push_rounds = h_ctl->push_phases;
        r->cut_sweeps = h_ctl->reach_rounds;
        r->reach_tiles = (long long)h_ctl->reach_tiles;
        r->push_tiles = (long long)h_ctl->push_tiles;
        r->gr_tiles = (long long)h_ctl->gr_tiles;
        r->push_sweeps = (long long)h_ctl->push_sweeps;
        r->push_local_relabels = (long long)h_ctl->push_bfs;
        r->t_global_relabel_ms = h_ctl->t_gr * 1e-6f;
        r->t_count_ms = h_ctl->t_count * 1e-6f;
        r->t_push_ms = h_ctl->t_push * 1e-6f;
        r->t_reach_ms = h_ctl->t_reach * 1e-6f;
        r->t_push_tail_ms = h_ctl->t_push_tail * 1e-6f;
        r->cyc_load = (long long)h_ctl->cyc_load;
        r->cyc_local_relabel = (long long)h_ctl->cyc_bfs;
        r->cyc_sweeps = (long long)h_ctl->cyc_sweep;
        r->cyc_writeback = (long long)h_ctl->cyc_wb;
        r->cyc_take = (long long)h_ctl->cyc_take;
        r->bfs_iters_push = (long long)h_ctl->bfs_it_push;
        r->bfs_iters_gr = (long long)h_ctl->bfs_it_gr;
        r->cyc_global_relabel = (long long)h_ctl->cyc_gr;
        r->ms = ms;
    }
};

std::atomic<long long> g_launches{0};

}  // namespace gcfg

using namespace gcfg;

// ---------------------------------------------------------------------------
// Graph API (drop-in for GraphCut.cu)
// ---------------------------------------------------------------------------

struct gcfg_graph {
    Engine e;
    int W = 0, H = 0;
    const int32_t *dp = nullptr, *dn = nullptr;
    const int32_t *up = nullptr, *down = nullptr, *left = nullptr, *right = nullptr;
    int32_t penalty = 0;
    bool varying = false;
    bool built = false;
    bool solved = false;
    int32_t *d_label = nullptr;
};

struct gcfg_segmenter {
    Engine e;
    int max_w = 0, max_h = 0;
};

struct gcfg_batch {
    Engine e;
};

extern "C" {

gcfg_status gcfg_set_dataterms(gcfg_graph *g, const int32_t *dp, const int32_t *dn) {
    if (!g) return GCFG_ERR_INVALID;
    g->dp = dp;
    g->dn = dn;
    g->built = false;
    return GCFG_OK;
}

gcfg_status gcfg_set_edges(gcfg_graph *g, const int32_t *up, const int32_t *down, const int32_t *left,
                           const int32_t *right) {
    if (!g || !up || !down || !left || !right) return GCFG_ERR_INVALID;
    g->varying = true;
    g->up = up;
    g->down = down;
    g->left = left;
    g->right = right;
    g->built = false;
    return GCFG_OK;
}

gcfg_status gcfg_set_penalty(gcfg_graph *g, int32_t penalty) {
    if (!g || penalty < 0 || penalty > GCFG_MAX_CAP) return GCFG_ERR_INVALID;
    g->varying = false;
    g->penalty = penalty;
    g->built = false;
    return GCFG_OK;
}

gcfg_status gcfg_set_graph(gcfg_graph *g) {
    if (!g) return GCFG_ERR_INVALID;
    if (!g->dp || !g->dn) return GCFG_ERR_STATE;
    Engine &e = g->e;
    GCFG_CK(cudaMemsetAsync(e.d_ist, 0, sizeof(ImgState), e.st));
    GCFG_CK(cudaMemsetAsync(e.d_ctl, 0, sizeof(Ctl), e.st));
    GCFG_TRY(launch_build_arrays(e.batch(), g->dp, g->dn, g->penalty, g->varying ? g->up : nullptr, g->down,
                                 g->left, g->right, e.st));
    GCFG_TRY(e.fetch());
    if (e.h_ctl->err) return GCFG_ERR_INVALID;  // capacities out of range
    g->built = true;
    g->solved = false;
    return GCFG_OK;
}

gcfg_status gcfg_init(int w, int h, const int32_t *dp, const int32_t *dn, int32_t penalty, const int32_t *up,
                      const int32_t *down, const int32_t *left, const int32_t *right, gcfg_graph **out) {
    if (!out || w <= 0 || h <= 0 || (long long)w * h > (1LL << 31) - 1) return GCFG_ERR_INVALID;
    if (penalty < 0 || penalty > GCFG_MAX_CAP) return GCFG_ERR_INVALID;
    gcfg_graph *g = new gcfg_graph();
    g->W = w;
    g->H = h;
    g->penalty = penalty;
    gcfg_status rc = g->e.init();
    if (rc == GCFG_OK) rc = g->e.layout(1, &w, &h, nullptr, false, false);
    if (rc == GCFG_OK && cudaMalloc(&g->d_label, (size_t)w * h * sizeof(int32_t)) != cudaSuccess)
        rc = GCFG_ERR_OOM;
    if (rc == GCFG_OK && dp) {
        gcfg_set_dataterms(g, dp, dn);
        if (up) rc = gcfg_set_edges(g, up, down, left, right);
        if (rc == GCFG_OK) rc = gcfg_set_graph(g);
    }
    if (rc) {
        cudaFree(g->d_label);
        delete g;
        return rc;
    }
    *out = g;
    return GCFG_OK;
}

gcfg_status gcfg_set_stream(gcfg_graph *g, void *stream) {
    if (!g) return GCFG_ERR_INVALID;
    g->e.st = (cudaStream_t)stream;
    return GCFG_OK;
}

gcfg_status gcfg_set_schedule(gcfg_graph *g, int push_rounds_per_gr, int max_tile_sweeps) {
    if (!g || push_rounds_per_gr < 1 || max_tile_sweeps < 1) return GCFG_ERR_INVALID;
    g->e.prm.push_rounds = push_rounds_per_gr;
    g->e.prm.max_sweeps = max_tile_sweeps;
    return GCFG_OK;
}

gcfg_status gcfg_optimize(gcfg_graph *g, int32_t *host_label, gcfg_result *res) {
    if (!g) return GCFG_ERR_INVALID;
    if (!g->built) return GCFG_ERR_STATE;
    Engine &e = g->e;
    GCFG_CK(cudaEventRecord(e.ev0, e.st));
    GCFG_TRY(e.solve());
    GCFG_CK(cudaEventRecord(e.ev1, e.st));
    if (host_label) GCFG_TRY(launch_extract(e.batch(), nullptr, nullptr, g->d_label, e.st));
    GCFG_TRY(e.fetch());
    // the graph is consumed in place, as in the reference: re-solving needs
    // gcfg_set_graph again (GraphCut.cu:385-534 leaves the residual graph)
    g->built = false;
    g->solved = true;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e.ev0, e.ev1);
    if (res) e.result(0, res, ms);
    GCFG_TRY(e.status());
    if (host_label) {
        GCFG_CK(cudaMemcpyAsync(host_label, g->d_label, (size_t)g->W * g->H * sizeof(int32_t),
                                cudaMemcpyDeviceToHost, e.st));
        GCFG_CK(cudaStreamSynchronize(e.st));
    }
    return GCFG_OK;
}

gcfg_status gcfg_get_cuts(gcfg_graph *g, uint8_t *d_smin, uint8_t *d_smax) {
    if (!g) return GCFG_ERR_INVALID;
    if (!g->solved) return GCFG_ERR_STATE;
    GCFG_TRY(launch_extract(g->e.batch(), d_smin, d_smax, nullptr, g->e.st));
    GCFG_CK(cudaStreamSynchronize(g->e.st));
    return GCFG_OK;
}

gcfg_status gcfg_end(gcfg_graph *g) {
    if (!g) return GCFG_ERR_INVALID;
    cudaFree(g->d_label);
    delete g;
    return GCFG_OK;
}

// ---------------------------------------------------------------------------
// Stand-alone data term and n-links (one image)
// ---------------------------------------------------------------------------

static gcfg_status one_image_tables(Engine &e, const uint8_t *rgb, const uint8_t *scrib, int w, int h,
                                    double lambda, double *raw_dp, double *raw_dn, DtArgs &a) {
    GCFG_TRY(e.init());
    GCFG_TRY(e.layout(1, &w, &h, &lambda, true, false, false));
    a = e.dt(rgb, scrib);
    if (raw_dp || raw_dn) {
        GCFG_TRY(grow(e.d_raw, e.c_raw, 2 * NBINS));
        a.raw_dp = e.d_raw;
        a.raw_dn = e.d_raw + NBINS;
    }
    return dt_tables(a, e.st);
}

gcfg_status gcfg_tlinks(const uint8_t *d_rgb, const uint8_t *d_scrib, int n, int32_t *d_dp, int32_t *d_dn,
                        double *h_raw_dp, double *h_raw_dn, void *stream) {
    if (!d_rgb || !d_scrib || !d_dp || !d_dn || n <= 0) return GCFG_ERR_INVALID;
    Engine e;
    e.st = (cudaStream_t)stream;
    DtArgs a;
    // the image is treated as n x 1: histograms and tables need no geometry
    GCFG_TRY(one_image_tables(e, d_rgb, d_scrib, n, 1, 0.0, h_raw_dp, h_raw_dn, a));
    GCFG_TRY(dt_apply_tlinks(a, n, d_dp, d_dn, e.st));
    if (h_raw_dp)
        GCFG_CK(cudaMemcpyAsync(h_raw_dp, a.raw_dp, NBINS * sizeof(double), cudaMemcpyDeviceToHost, e.st));
    if (h_raw_dn)
        GCFG_CK(cudaMemcpyAsync(h_raw_dn, a.raw_dn, NBINS * sizeof(double), cudaMemcpyDeviceToHost, e.st));
    GCFG_CK(cudaStreamSynchronize(e.st));
    return GCFG_OK;
}

gcfg_status gcfg_nlinks(const uint8_t *d_rgb, int w, int h, double lambda, int32_t *d_up, int32_t *d_down,
                        int32_t *d_left, int32_t *d_right, void *stream) {
    if (!d_rgb || !d_up || !d_down || !d_left || !d_right || w <= 0 || h <= 0) return GCFG_ERR_INVALID;
    if (!(lambda >= 0) || lambda * 1.0000001 + 1 > (double)GCFG_MAX_CAP) return GCFG_ERR_INVALID;
    Engine e;
    e.st = (cudaStream_t)stream;
    DtArgs a;
    // no scribbles: the colour tables are skipped, only the n-link table is made
    GCFG_TRY(one_image_tables(e, d_rgb, nullptr, w, h, lambda, nullptr, nullptr, a));
    GCFG_TRY(dt_apply_nlinks(a, w, h, d_up, d_down, d_left, d_right, e.st));
    GCFG_CK(cudaStreamSynchronize(e.st));
    return GCFG_OK;
}

// ---------------------------------------------------------------------------
// Segmenter (one image) and batch
// ---------------------------------------------------------------------------

static gcfg_status run_batch_eager(Engine &e, int n, const int *W, const int *H, const double *lam,
                                   const uint8_t *rgb, const uint8_t *scrib, uint8_t *smin, uint8_t *smax,
                                   int64_t *flows, gcfg_result *res, bool staging) {
    GCFG_CK(cudaEventRecord(e.ev0, e.st));
    GCFG_TRY(e.layout(n, W, H, lam, true, staging));
    if (staging) {
        const uint8_t *h_rgb = rgb, *h_scrib = scrib;
        GCFG_CK(cudaMemcpyAsync(e.d_rgb, h_rgb, (size_t)e.n_px * 3, cudaMemcpyHostToDevice, e.st));
        GCFG_CK(cudaMemcpyAsync(e.d_scrib, h_scrib, (size_t)e.n_px, cudaMemcpyHostToDevice, e.st));
        rgb = e.d_rgb;
        scrib = e.d_scrib;
    }
    GCFG_TRY(e.build_images(rgb, scrib));
    GCFG_TRY(e.solve());
    uint8_t *dmin = staging ? (smin ? e.d_smin : nullptr) : smin;
    uint8_t *dmax = staging ? (smax ? e.d_smax : nullptr) : smax;
    if (dmin || dmax) GCFG_TRY(launch_extract_rows(e.batch(), e.d_cmap, e.total_chunks, dmin, dmax, e.st));
    if (staging) {
        if (smin) GCFG_CK(cudaMemcpyAsync(smin, e.d_smin, (size_t)e.n_px, cudaMemcpyDeviceToHost, e.st));
        if (smax) GCFG_CK(cudaMemcpyAsync(smax, e.d_smax, (size_t)e.n_px, cudaMemcpyDeviceToHost, e.st));
    }
    GCFG_CK(cudaEventRecord(e.ev1, e.st));
    GCFG_TRY(e.fetch());
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e.ev0, e.ev1);
    for (int i = 0; i < n; ++i) {
        gcfg_result r;
        e.result(i, &r, ms);
        if (flows) flows[i] = r.flow;
        if (res) res[i] = r;
    }
    return e.status();
}

// The cached graph of a batch signature (sizes, lambdas, the buffers `ptr`,
// the kind of run, solver settings), laying the batch out and capturing the
// device part (per-image counter reset, data term, build, solve, read-back
// of the per-image states, extraction) first when needed.  *out is null when
// the device cannot capture; runs then continue without graphs.
static gcfg_status graph_for(Engine &e, int n, const int *W, const int *H, const double *lam,
                             const void *const ptr[4], int kind, bool staging, Engine::GraphEntry **out) {
    *out = nullptr;
    auto same = [&](const Engine::GraphEntry &g) {
        if ((int)g.w.size() != n || g.kind != kind || g.grid != e.max_grid || g.alloc_gen != e.alloc_gen)
            return false;
        if (memcmp(&g.prm, &e.prm, sizeof(SolveParams)) != 0) return false;
        for (int k = 0; k < 4; ++k)
            if (g.ptr[k] != ptr[k]) return false;
        for (int i = 0; i < n; ++i)
            if (g.w[i] != W[i] || g.h[i] != H[i] || g.lam[i] != lam[i]) return false;
        return true;
    };
    Engine::GraphEntry *hit = nullptr;
    for (auto &g : e.graphs)
        if (same(g)) hit = &g;
    if (!e.laid_out(n, W, H, lam) || !hit) {
        const long long gen = e.alloc_gen;
        GCFG_TRY(e.layout(n, W, H, lam, true, staging));
        if (e.alloc_gen != gen) {  // buffers moved: every captured graph is stale
            e.drop_graphs();
            hit = nullptr;
        }
    }
    if (!hit) {
        // the device buffers the graph bakes in
        const uint8_t *drgb = staging ? e.d_rgb : (const uint8_t *)ptr[0];
        const uint8_t *dscrib = staging ? e.d_scrib : (const uint8_t *)ptr[1];
        uint8_t *dmin = staging ? (ptr[2] ? e.d_smin : nullptr) : (uint8_t *)ptr[2];
        uint8_t *dmax = staging ? (ptr[3] ? e.d_smax : nullptr) : (uint8_t *)ptr[3];
        if (!e.cap_st) GCFG_CK(cudaStreamCreateWithFlags(&e.cap_st, cudaStreamNonBlocking));
        // the layout uploads were queued on the caller's stream; the graph is
        // launched there too, after them
        cudaStream_t user = e.st;
        e.st = e.cap_st;
        const long long l0 = g_launches.load();
        gcfg_status rc = GCFG_OK;
        cudaGraph_t g = nullptr;
        if (cudaStreamBeginCapture(e.cap_st, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
            rc = GCFG_ERR_CUDA;
        } else {
            if (cudaMemsetAsync(e.d_ist, 0, (size_t)n * sizeof(ImgState), e.st) != cudaSuccess) rc = GCFG_ERR_CUDA;
            if (rc == GCFG_OK) rc = e.build_images(drgb, dscrib);
            if (rc == GCFG_OK) rc = e.solve();
            // the state read-back first: a label download queued after the
            // graph must not hold it up on the copy engine
            if (rc == GCFG_OK) rc = e.readback();
            if (rc == GCFG_OK && (dmin || dmax))
                rc = launch_extract_rows(e.batch(), e.d_cmap, e.total_chunks, dmin, dmax, e.st);
            if (cudaStreamEndCapture(e.cap_st, &g) != cudaSuccess && rc == GCFG_OK) rc = GCFG_ERR_CUDA;
        }
        e.st = user;
        const long long kernels = g_launches.load() - l0;
        g_launches.fetch_sub(kernels);  // counted when the graph runs
        cudaGraphExec_t exec = nullptr;
        if (rc == GCFG_OK && g && cudaGraphInstantiate(&exec, g, 0) != cudaSuccess) {
            exec = nullptr;
            rc = GCFG_ERR_CUDA;
        }
        if (g) cudaGraphDestroy(g);
        if (rc != GCFG_OK) {
            cudaGetLastError();
            e.graph_broken = true;
            e.drop_graphs();
            return GCFG_OK;
        }
        if ((int)e.graphs.size() >= Engine::MAX_GRAPHS) {  // drop the least recently used
            size_t old = 0;
            for (size_t k = 1; k < e.graphs.size(); ++k)
                if (e.graphs[k].last_use < e.graphs[old].last_use) old = k;
            cudaGraphExecDestroy(e.graphs[old].exec);
            e.graphs.erase(e.graphs.begin() + old);
        }
        Engine::GraphEntry ge;
        ge.w.assign(W, W + n);
        ge.h.assign(H, H + n);
        ge.lam.assign(lam, lam + n);
        for (int k = 0; k < 4; ++k) ge.ptr[k] = ptr[k];
        ge.kind = kind;
        ge.prm = e.prm;
        ge.grid = e.max_grid;
        ge.alloc_gen = e.alloc_gen;
        ge.kernels = kernels;
        ge.last_use = 0;
        ge.exec = exec;
        e.graphs.push_back(ge);
        hit = &e.graphs.back();
        e.graph_captures++;
    }
    hit->last_use = ++e.graph_clock;
    e.graph_kernels = hit->kernels;
    *out = hit;
    return GCFG_OK;
}

// The device part of a run (per-image counters reset, data term, build,
// persistent solve, read-back of the per-image states, extraction) captured
// once into a CUDA graph and replayed while the batch is the same: same
// sizes, lambdas, buffers and solver settings.  The persistent solver already
// runs the whole push / local relabel / global relabel loop without host round
// trips; the graph removes the remaining per-kernel launch work.  Host
// copies of the host entry points stay outside the graph.
static gcfg_status run_batch_graph(Engine &e, int n, const int *W, const int *H, const double *lam,
                                   const uint8_t *rgb, const uint8_t *scrib, uint8_t *smin, uint8_t *smax,
                                   int64_t *flows, gcfg_result *res, bool staging) {
    // host inputs are copied in outside the graph; only device buffers are baked in
    const void *ptr[4] = {staging ? nullptr : rgb, staging ? nullptr : scrib, smin, smax};
    Engine::GraphEntry *hit = nullptr;
    GCFG_TRY(graph_for(e, n, W, H, lam, ptr, staging ? 1 : 0, staging, &hit));
    if (!hit) return run_batch_eager(e, n, W, H, lam, rgb, scrib, smin, smax, flows, res, staging);
    if (staging) {
        GCFG_CK(cudaMemcpyAsync(e.d_rgb, rgb, (size_t)e.n_px * 3, cudaMemcpyHostToDevice, e.st));
        GCFG_CK(cudaMemcpyAsync(e.d_scrib, scrib, (size_t)e.n_px, cudaMemcpyHostToDevice, e.st));
    }
    GCFG_CK(cudaEventRecord(e.ev0, e.st));
    GCFG_CK(cudaGraphLaunch(hit->exec, e.st));
    GCFG_CK(cudaEventRecord(e.ev1, e.st));
    g_launches.fetch_add(hit->kernels, std::memory_order_relaxed);
    e.graph_replays++;
    if (staging) {
        if (smin) GCFG_CK(cudaMemcpyAsync(smin, e.d_smin, (size_t)e.n_px, cudaMemcpyDeviceToHost, e.st));
        if (smax) GCFG_CK(cudaMemcpyAsync(smax, e.d_smax, (size_t)e.n_px, cudaMemcpyDeviceToHost, e.st));
    }
    GCFG_CK(cudaStreamSynchronize(e.st));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e.ev0, e.ev1);
    for (int i = 0; i < n; ++i) {
        gcfg_result r;
        e.result(i, &r, ms);
        if (flows) flows[i] = r.flow;
        if (res) res[i] = r;
    }
    return e.status();
}

// Pieces of the host entry points for many images (the layout and groups
// are in place): uploads of the groups' inputs on cp_st, each group's data
// term and build on st as soon as its inputs are in, and per group the
// extraction on st and the download of its labels on `out_st`.
static gcfg_status stage_uploads(Engine &e, const uint8_t *h_rgb, const uint8_t *h_scrib) {
    for (int g = 0; g < (int)e.groups.size(); ++g) {
        const Engine::Group &gr = e.groups[g];
        const size_t np = (size_t)(gr.p1 - gr.p0);
        GCFG_CK(cudaMemcpyAsync(e.d_rgb + 3 * gr.p0, h_rgb + 3 * gr.p0, 3 * np, cudaMemcpyHostToDevice, e.cp_st));
        GCFG_CK(cudaMemcpyAsync(e.d_scrib + gr.p0, h_scrib + gr.p0, np, cudaMemcpyHostToDevice, e.cp_st));
        GCFG_CK(cudaEventRecord(e.ev_in[g], e.cp_st));
    }
    return GCFG_OK;
}

static gcfg_status stage_build(Engine &e) {
    for (int g = 0; g < (int)e.groups.size(); ++g) {
        const Engine::Group &gr = e.groups[g];
        GCFG_CK(cudaStreamWaitEvent(e.st, e.ev_in[g], 0));
        DtArgs a = e.dt(e.d_rgb, e.d_scrib);
        a.n_img = gr.i1 - gr.i0;
        a.ilist = e.d_iota + gr.i0;
        a.total_chunks = gr.c1 - gr.c0;
        a.chunk_map = e.d_cmap + gr.c0;
        GCFG_CK(cudaMemsetAsync(e.d_hist + (size_t)gr.i0 * 2 * NBINS, 0,
                                (size_t)(gr.i1 - gr.i0) * 2 * NBINS * sizeof(int), e.st));
        GCFG_TRY(dt_tables(a, e.st));
        Batch b = e.batch();
        b.tlist = e.d_iota + gr.t0;
        b.n_tlist = gr.t1 - gr.t0;
        GCFG_TRY(dt_build(b, a, e.st));
    }
    return GCFG_OK;
}

static gcfg_status stage_extract(Engine &e, uint8_t *h_smin, uint8_t *h_smax, cudaStream_t out_st) {
    for (int g = 0; g < (int)e.groups.size(); ++g) {
        const Engine::Group &gr = e.groups[g];
        if (h_smin || h_smax)
            GCFG_TRY(launch_extract_rows(e.batch(), e.d_cmap + gr.c0, gr.c1 - gr.c0, h_smin ? e.d_smin : nullptr,
                                         h_smax ? e.d_smax : nullptr, e.st));
        GCFG_CK(cudaEventRecord(e.ev_out[g], e.st));
        GCFG_CK(cudaStreamWaitEvent(out_st, e.ev_out[g], 0));
        const size_t np = (size_t)(gr.p1 - gr.p0);
        if (h_smin) GCFG_CK(cudaMemcpyAsync(h_smin + gr.p0, e.d_smin + gr.p0, np, cudaMemcpyDeviceToHost, out_st));
        if (h_smax) GCFG_CK(cudaMemcpyAsync(h_smax + gr.p0, e.d_smax + gr.p0, np, cudaMemcpyDeviceToHost, out_st));
    }
    return GCFG_OK;
}

static void fill_results(const Engine &e, int n, float ms, int64_t *flows, gcfg_result *res) {
    for (int i = 0; i < n; ++i) {
        gcfg_result r;
        e.result(i, &r, ms);
        if (flows) flows[i] = r.flow;
        if (res) res[i] = r;
    }
}

static gcfg_status run_batch_staged(Engine &e, int n, const int *W, const int *H, const double *lam,
                                    const uint8_t *h_rgb, const uint8_t *h_scrib, uint8_t *h_smin,
                                    uint8_t *h_smax, int64_t *flows, gcfg_result *res) {
    GCFG_CK(cudaEventRecord(e.ev0, e.st));
    GCFG_TRY(e.layout(n, W, H, lam, true, true));
    GCFG_TRY(e.make_groups(n, W, H));
    // the uploads overwrite buffers that earlier work on st may read
    GCFG_CK(cudaEventRecord(e.ev_mark, e.st));
    GCFG_CK(cudaStreamWaitEvent(e.cp_st, e.ev_mark, 0));
    GCFG_TRY(stage_uploads(e, h_rgb, h_scrib));
    GCFG_TRY(stage_build(e));
    GCFG_TRY(e.solve());
    GCFG_TRY(stage_extract(e, h_smin, h_smax, e.cp_st));
    GCFG_TRY(e.readback());
    GCFG_CK(cudaEventRecord(e.ev_mark, e.cp_st));
    GCFG_CK(cudaStreamWaitEvent(e.st, e.ev_mark, 0));
    GCFG_CK(cudaEventRecord(e.ev1, e.st));
    GCFG_CK(cudaStreamSynchronize(e.st));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e.ev0, e.ev1);
    fill_results(e, n, ms, flows, res);
    return e.status();
}

// Queue one batch of the asynchronous host entry point into the run set that
// is swapped in.  That set's previous batch has been collected, so nothing in
// flight reads its staging buffers or host tables.  The whole upload goes
// first on cp_st, where it overlaps the compute of the batch before; the
// batch then computes in one pass on st (data term, build, solve, extraction
// over all its images, as the device-resident path does), and its labels are
// downloaded on dn_st while the next batch computes.
static gcfg_status submit_staged(Engine &e, Engine::Flight &f, int slot, int n, const int *W, const int *H,
                                 const double *lam, const uint8_t *h_rgb, const uint8_t *h_scrib, uint8_t *h_smin,
                                 uint8_t *h_smax) {
    GCFG_TRY(grow_host(e.h_ctl, e.ch_ctl, 1));
    if (!e.ev0) GCFG_CK(cudaEventCreate(&e.ev0));
    if (!e.ev1) GCFG_CK(cudaEventCreate(&e.ev1));
    if (!e.cp_st) GCFG_CK(cudaStreamCreateWithFlags(&e.cp_st, cudaStreamNonBlocking));
    if (!e.dn_st) GCFG_CK(cudaStreamCreateWithFlags(&e.dn_st, cudaStreamNonBlocking));
    for (cudaEvent_t *ev : {&f.ev_up, &f.ev_ext, &f.ev_dn})
        if (!*ev) GCFG_CK(cudaEventCreateWithFlags(ev, cudaEventDisableTiming));
    if (e.graph_on && !e.graph_broken && !prof_on()) {
        // keyed by the run set and the outputs wanted (the set's buffers may
        // not exist before its first layout; any reallocation drops every
        // graph, so the buffers a graph bakes in stay the set's own)
        const void *ptr[4] = {reinterpret_cast<const void *>((uintptr_t)slot + 1), nullptr,
                              h_smin ? reinterpret_cast<const void *>(1) : nullptr,
                              h_smax ? reinterpret_cast<const void *>(1) : nullptr};
        Engine::GraphEntry *hit = nullptr;
        GCFG_TRY(graph_for(e, n, W, H, lam, ptr, 2, true, &hit));
        if (hit) {
            GCFG_CK(cudaMemcpyAsync(e.d_rgb, h_rgb, (size_t)e.n_px * 3, cudaMemcpyHostToDevice, e.cp_st));
            GCFG_CK(cudaMemcpyAsync(e.d_scrib, h_scrib, (size_t)e.n_px, cudaMemcpyHostToDevice, e.cp_st));
            GCFG_CK(cudaEventRecord(f.ev_up, e.cp_st));
            GCFG_CK(cudaStreamWaitEvent(e.st, f.ev_up, 0));
            GCFG_CK(cudaEventRecord(e.ev0, e.st));
            GCFG_CK(cudaGraphLaunch(hit->exec, e.st));
            g_launches.fetch_add(hit->kernels, std::memory_order_relaxed);
            e.graph_replays++;
            GCFG_CK(cudaEventRecord(f.ev_ext, e.st));
            GCFG_CK(cudaStreamWaitEvent(e.dn_st, f.ev_ext, 0));
            if (h_smin) GCFG_CK(cudaMemcpyAsync(h_smin, e.d_smin, (size_t)e.n_px, cudaMemcpyDeviceToHost, e.dn_st));
            if (h_smax) GCFG_CK(cudaMemcpyAsync(h_smax, e.d_smax, (size_t)e.n_px, cudaMemcpyDeviceToHost, e.dn_st));
            GCFG_CK(cudaEventRecord(e.ev1, e.st));
            GCFG_CK(cudaEventRecord(f.ev_dn, e.dn_st));
            return GCFG_OK;
        }
    }
    GCFG_CK(cudaEventRecord(e.ev0, e.st));
    GCFG_TRY(e.layout(n, W, H, lam, true, true));
    GCFG_CK(cudaMemcpyAsync(e.d_rgb, h_rgb, (size_t)e.n_px * 3, cudaMemcpyHostToDevice, e.cp_st));
    GCFG_CK(cudaMemcpyAsync(e.d_scrib, h_scrib, (size_t)e.n_px, cudaMemcpyHostToDevice, e.cp_st));
    GCFG_CK(cudaEventRecord(f.ev_up, e.cp_st));
    GCFG_CK(cudaStreamWaitEvent(e.st, f.ev_up, 0));
    GCFG_TRY(e.build_images(e.d_rgb, e.d_scrib));
    GCFG_TRY(e.solve());
    // the small read-back of the per-image states goes before the label
    // download is queued: behind it on the copy engine it would stall st
    GCFG_TRY(e.readback());
    if (h_smin || h_smax)
        GCFG_TRY(launch_extract_rows(e.batch(), e.d_cmap, e.total_chunks, h_smin ? e.d_smin : nullptr,
                                     h_smax ? e.d_smax : nullptr, e.st));
    GCFG_CK(cudaEventRecord(f.ev_ext, e.st));
    GCFG_CK(cudaStreamWaitEvent(e.dn_st, f.ev_ext, 0));
    if (h_smin) GCFG_CK(cudaMemcpyAsync(h_smin, e.d_smin, (size_t)e.n_px, cudaMemcpyDeviceToHost, e.dn_st));
    if (h_smax) GCFG_CK(cudaMemcpyAsync(h_smax, e.d_smax, (size_t)e.n_px, cudaMemcpyDeviceToHost, e.dn_st));
    GCFG_CK(cudaEventRecord(e.ev1, e.st));
    GCFG_CK(cudaEventRecord(f.ev_dn, e.dn_st));
    return GCFG_OK;
}

static gcfg_status batch_submit(Engine &e, int n, const int *W, const int *H, const double *lam,
                                const uint8_t *h_rgb, const uint8_t *h_scrib, uint8_t *h_smin, uint8_t *h_smax,
                                int64_t *ticket) {
    const int slot = e.next_slot;
    Engine::Flight &f = e.flight[slot];
    if (f.busy) return GCFG_ERR_STATE;  // two batches in flight already
    if (slot == 1) e.swap_set(e.alt);
    const gcfg_status rc = submit_staged(e, f, slot, n, W, H, lam, h_rgb, h_scrib, h_smin, h_smax);
    if (slot == 1) e.swap_set(e.alt);
    if (rc != GCFG_OK) return rc;
    f.busy = true;
    f.n = n;
    f.ticket = e.next_ticket++;
    e.next_slot ^= 1;
    *ticket = f.ticket;
    return GCFG_OK;
}

static gcfg_status batch_wait(Engine &e, int64_t ticket, int64_t *flows, gcfg_result *res) {
    int slot = -1;
    for (int k = 0; k < 2; ++k)
        if (e.flight[k].busy && e.flight[k].ticket == ticket) slot = k;
    if (slot < 0) return GCFG_ERR_INVALID;
    Engine::Flight &f = e.flight[slot];
    f.busy = false;
    if (slot == 1) e.swap_set(e.alt);
    gcfg_status rc = GCFG_OK;
    if (cudaEventSynchronize(f.ev_dn) != cudaSuccess || cudaEventSynchronize(e.ev1) != cudaSuccess) {
        rc = GCFG_ERR_CUDA;
    } else {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e.ev0, e.ev1);
        fill_results(e, f.n, ms, flows, res);
        rc = e.status();
    }
    if (slot == 1) e.swap_set(e.alt);
    return rc;
}

static gcfg_status run_batch(Engine &e, int n, const int *W, const int *H, const double *lam,
                             const uint8_t *rgb, const uint8_t *scrib, uint8_t *smin, uint8_t *smax,
                             int64_t *flows, gcfg_result *res, bool staging) {
    if (e.in_flight()) return GCFG_ERR_STATE;  // collect the asynchronous batches first
    if (staging && n > 1) return run_batch_staged(e, n, W, H, lam, rgb, scrib, smin, smax, flows, res);
    if (e.graph_on && !e.graph_broken && !prof_on())
        return run_batch_graph(e, n, W, H, lam, rgb, scrib, smin, smax, flows, res, staging);
    return run_batch_eager(e, n, W, H, lam, rgb, scrib, smin, smax, flows, res, staging);
}

gcfg_status gcfg_seg_create(int max_w, int max_h, gcfg_segmenter **out) {
    if (!out || max_w < 1 || max_h < 1 || (long long)max_w * max_h > (1LL << 31) - 1) return GCFG_ERR_INVALID;
    gcfg_segmenter *s = new gcfg_segmenter();
    s->max_w = max_w;
    s->max_h = max_h;
    const double lam = 1.0;
    gcfg_status rc = s->e.init();
    if (rc == GCFG_OK) rc = s->e.layout(1, &max_w, &max_h, &lam, true, true);
    if (rc == GCFG_OK && cudaStreamSynchronize(s->e.st) != cudaSuccess) rc = GCFG_ERR_CUDA;
    if (rc) {
        delete s;
        return rc;
    }
    *out = s;
    return GCFG_OK;
}

gcfg_status gcfg_seg_set_stream(gcfg_segmenter *s, void *stream) {
    if (!s) return GCFG_ERR_INVALID;
    s->e.st = (cudaStream_t)stream;
    return GCFG_OK;
}

gcfg_status gcfg_seg_run(gcfg_segmenter *s, const uint8_t *d_rgb, const uint8_t *d_scrib, int w, int h,
                         double lambda, uint8_t *d_smin, uint8_t *d_smax, gcfg_result *res) {
    if (!s || !d_rgb || !d_scrib || w < 1 || h < 1 || w > s->max_w || h > s->max_h) return GCFG_ERR_INVALID;
    return run_batch(s->e, 1, &w, &h, &lambda, d_rgb, d_scrib, d_smin, d_smax, nullptr, res, false);
}

gcfg_status gcfg_seg_run_host(gcfg_segmenter *s, const uint8_t *h_rgb, const uint8_t *h_scrib, int w, int h,
                              double lambda, uint8_t *h_smin, uint8_t *h_smax, gcfg_result *res) {
    if (!s || !h_rgb || !h_scrib || w < 1 || h < 1 || w > s->max_w || h > s->max_h) return GCFG_ERR_INVALID;
    return run_batch(s->e, 1, &w, &h, &lambda, h_rgb, h_scrib, h_smin, h_smax, nullptr, res, true);
}

gcfg_status gcfg_seg_destroy(gcfg_segmenter *s) {
    if (!s) return GCFG_ERR_INVALID;
    delete s;
    return GCFG_OK;
}

gcfg_status gcfg_batch_create(int max_images, int64_t max_pixels, gcfg_batch **out) {
    if (!out || max_images < 1 || max_pixels < 1) return GCFG_ERR_INVALID;
    gcfg_batch *b = new gcfg_batch();
    gcfg_status rc = b->e.init();
    // pre-size for max_images images of average size (tiles grow on demand)
    const long long tiles = (max_pixels + TPX - 1) / TPX + 2LL * max_images;
    if (rc == GCFG_OK) rc = b->e.reserve(max_images, (int)(tiles > (1LL << 30) ? (1LL << 30) : tiles),
                                         max_pixels, true, false);
    if (rc) {
        delete b;
        return rc;
    }
    *out = b;
    return GCFG_OK;
}

gcfg_status gcfg_batch_set_stream(gcfg_batch *b, void *stream) {
    if (!b) return GCFG_ERR_INVALID;
    if (b->e.in_flight()) return GCFG_ERR_STATE;
    b->e.st = (cudaStream_t)stream;
    return GCFG_OK;
}

gcfg_status gcfg_batch_set_params(gcfg_batch *b, int push_rounds_per_gr, int max_tile_sweeps,
                                  int sweeps_per_local_relabel) {
    if (!b || push_rounds_per_gr < 1 || max_tile_sweeps < 1 || sweeps_per_local_relabel < 1)
        return GCFG_ERR_INVALID;
    b->e.prm.push_rounds = push_rounds_per_gr;
    b->e.prm.max_sweeps = max_tile_sweeps;
    b->e.prm.bfs_every = sweeps_per_local_relabel;
    return GCFG_OK;
}

gcfg_status gcfg_batch_set_solver(gcfg_batch *b, const gcfg_tuning *t) {
    if (!b || !t || t->push_rounds_per_gr < 1 || t->max_tile_sweeps < 1 || t->sweeps_per_local_relabel < 1 ||
        t->blocks_per_sm < 0 || (t->local_relabel_first != 0 && t->local_relabel_first != 1) ||
        (t->push_only != 0 && t->push_only != 1) ||
        (t->threads_y != 0 && t->threads_y != 4 && t->threads_y != 8 && t->threads_y != 16 &&
         t->threads_y != 32))
        return GCFG_ERR_INVALID;
    int dev = 0, sms = 1;
    GCFG_CK(cudaGetDevice(&dev));
    GCFG_CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    b->e.prm.push_rounds = t->push_rounds_per_gr;
    b->e.prm.max_sweeps = t->max_tile_sweeps;
    b->e.prm.bfs_every = t->sweeps_per_local_relabel;
    b->e.prm.bfs_first = t->local_relabel_first;
    b->e.prm.push_only = t->push_only;
    b->e.prm.warps = t->threads_y;  // 0: by the solve's size
    b->e.max_grid = t->blocks_per_sm * sms;  // 0: as many as fit
    return GCFG_OK;
}

gcfg_status gcfg_batch_set_graph(gcfg_batch *b, int enable) {
    if (!b) return GCFG_ERR_INVALID;
    b->e.graph_on = enable != 0;
    if (!enable) b->e.drop_graphs();
    return GCFG_OK;
}

gcfg_status gcfg_batch_graph_info(gcfg_batch *b, int *active, int64_t *captures, int64_t *replays,
                                  int64_t *kernels_per_replay) {
    if (!b) return GCFG_ERR_INVALID;
    if (active) *active = b->e.graph_on && !b->e.graph_broken;
    if (captures) *captures = b->e.graph_captures;
    if (replays) *replays = b->e.graph_replays;
    if (kernels_per_replay) *kernels_per_replay = b->e.graph_kernels;
    return GCFG_OK;
}

gcfg_status gcfg_batch_autotune(gcfg_batch *b, int n, const int *widths, const int *heights, const double *lambdas,
                                const uint8_t *d_rgb, const uint8_t *d_scrib, int reps, gcfg_tuning *out) {
    if (!b || n < 1 || !widths || !heights || !lambdas || !d_rgb || !d_scrib || reps < 1) return GCFG_ERR_INVALID;
    Engine &e = b->e;
    if (e.in_flight()) return GCFG_ERR_STATE;
    const bool graph = e.graph_on;
    e.graph_on = false;  // time the eager runs; the graph is recaptured afterwards
    e.drop_graphs();
    int dev = 0, sms = 1;
    GCFG_CK(cudaGetDevice(&dev));
    GCFG_CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    // co-resident blocks per SM of each block shape
    auto per_sm_of = [&](int warps) {
        const int f = solve_grid_blocks(1 << 30, 0, warps) / (sms > 0 ? sms : 1);
        return f < 1 ? 1 : f;
    };

    std::vector<int64_t> ref(n), got(n);
    std::vector<gcfg_result> rr(n);
    int tried = 0;
    gcfg_status rc = GCFG_OK;
    // time of one configuration: fastest of `reps` runs; every run must give
    // the flows of the first
    auto time_cfg = [&](const SolveParams &p, int bps, float *ms) -> gcfg_status {
        e.prm = p;
        e.max_grid = bps * sms;
        float best = 1e30f;
        for (int k = 0; k < reps; ++k) {
            GCFG_TRY(run_batch_eager(e, n, widths, heights, lambdas, d_rgb, d_scrib, nullptr, nullptr, got.data(),
                                     rr.data(), false));
            if (tried == 0 && k == 0) ref = got;
            if (got != ref) return GCFG_ERR_NOT_CONVERGED;
            if (rr[0].ms < best) best = rr[0].ms;
        }
        ++tried;
        *ms = best;
        return GCFG_OK;
    };
    SolveParams cur = e.prm;
    {
        long long tiles = 0;  // the batch's tiles, for the size-chosen block shape
        for (int i = 0; i < n; ++i) tiles += (long long)((widths[i] + 31) / 32) * ((heights[i] + 31) / 32);
        cur.warps = solve_warps(cur.warps, (int)(tiles < (1 << 30) ? tiles : (1 << 30)));
    }
    int cur_bps = e.max_grid > 0 ? (e.max_grid + sms - 1) / sms : per_sm_of(cur.warps);
    if (cur_bps > per_sm_of(cur.warps)) cur_bps = per_sm_of(cur.warps);
    float ms_default = 0.f;
    rc = time_cfg(cur, cur_bps, &ms_default);  // warms up, then the default
    if (rc == GCFG_OK) rc = time_cfg(cur, cur_bps, &ms_default);
    float best = ms_default;
    // Coordinate search: the block shape (warps per block, at the shape's
    // full occupancy), push rounds per global relabel, sweeps per visit,
    // sweeps between local relabels, blocks per SM, relabel-first, push-only.
    static const int c_warps[] = {4, 8, 16, 32};
    static const int c_push[] = {2, 4, 8, 16};
    static const int c_sweeps[] = {16, 24, 32, 64, 128};
    static const int c_bfs[] = {2, 4, 8, 16, 32};
    for (int pass = 0; pass < 2 && rc == GCFG_OK; ++pass) {
        for (int which = 0; which < 7 && rc == GCFG_OK; ++which) {
            const int nc = which == 0 ? 4 : which == 1 ? 4 : which == 2 || which == 3 ? 5
                         : which == 4 ? per_sm_of(cur.warps) : 2;
            for (int c = 0; c < nc && rc == GCFG_OK; ++c) {
                SolveParams p = cur;
                int bps = cur_bps;
                if (which == 0) {
                    p.warps = c_warps[c];
                    bps = per_sm_of(p.warps);
                }
                if (which == 1) p.push_rounds = c_push[c];
                if (which == 2) p.max_sweeps = c_sweeps[c];
                if (which == 3) p.bfs_every = c_bfs[c];
                if (which == 4) bps = c + 1;
                if (which == 5) p.bfs_first = c;
                if (which == 6) p.push_only = c;
                if (memcmp(&p, &cur, sizeof(p)) == 0 && bps == cur_bps) continue;
                float ms = 0.f;
                rc = time_cfg(p, bps, &ms);
                if (rc == GCFG_OK && ms < best * 0.98f) {  // keep a change only for a clear gain
                    best = ms;
                    cur = p;
                    cur_bps = bps;
                }
            }
        }
    }
    e.prm = cur;
    e.max_grid = cur_bps * sms;
    e.graph_on = graph;
    if (rc != GCFG_OK) return rc;
    if (out) {
        out->push_rounds_per_gr = cur.push_rounds;
        out->max_tile_sweeps = cur.max_sweeps;
        out->sweeps_per_local_relabel = cur.bfs_every;
        out->local_relabel_first = cur.bfs_first;
        out->push_only = cur.push_only;
        out->blocks_per_sm = cur_bps;
        out->ms_default = ms_default;
        out->ms_best = best;
        out->configs_tried = tried;
        out->tile_w = TILE_W;
        out->tile_h = TILE_H;
        out->threads_y = cur.warps;
    }
    return GCFG_OK;
}

gcfg_status gcfg_batch_run(gcfg_batch *b, int n, const int *widths, const int *heights, const double *lambdas,
                           const uint8_t *d_rgb, const uint8_t *d_scrib, uint8_t *d_smin, uint8_t *d_smax,
                           int64_t *h_flows, gcfg_result *h_res) {
    if (!b || n < 1 || !widths || !heights || !lambdas || !d_rgb || !d_scrib) return GCFG_ERR_INVALID;
    return run_batch(b->e, n, widths, heights, lambdas, d_rgb, d_scrib, d_smin, d_smax, h_flows, h_res, false);
}

gcfg_status gcfg_batch_run_host(gcfg_batch *b, int n, const int *widths, const int *heights,
                                const double *lambdas, const uint8_t *h_rgb, const uint8_t *h_scrib,
                                uint8_t *h_smin, uint8_t *h_smax, int64_t *h_flows, gcfg_result *h_res) {
    if (!b || n < 1 || !widths || !heights || !lambdas || !h_rgb || !h_scrib) return GCFG_ERR_INVALID;
    return run_batch(b->e, n, widths, heights, lambdas, h_rgb, h_scrib, h_smin, h_smax, h_flows, h_res, true);
}

gcfg_status gcfg_batch_submit_host(gcfg_batch *b, int n, const int *widths, const int *heights,
                                   const double *lambdas, const uint8_t *h_rgb, const uint8_t *h_scrib,
                                   uint8_t *h_smin, uint8_t *h_smax, int64_t *ticket) {
    if (!b || n < 1 || !widths || !heights || !lambdas || !h_rgb || !h_scrib || !ticket) return GCFG_ERR_INVALID;
    return batch_submit(b->e, n, widths, heights, lambdas, h_rgb, h_scrib, h_smin, h_smax, ticket);
}

gcfg_status gcfg_batch_wait(gcfg_batch *b, int64_t ticket, int64_t *h_flows, gcfg_result *h_res) {
    if (!b) return GCFG_ERR_INVALID;
    return batch_wait(b->e, ticket, h_flows, h_res);
}

gcfg_status gcfg_batch_phase_split(gcfg_batch *b, int n, const int *widths, const int *heights,
                                   const double *lambdas, const uint8_t *d_rgb, const uint8_t *d_scrib,
                                   gcfg_phase_split *out) {
    if (!b || n < 1 || !widths || !heights || !lambdas || !d_rgb || !d_scrib || !out) return GCFG_ERR_INVALID;
    Engine &e = b->e;
    if (e.in_flight()) return GCFG_ERR_STATE;
    memset(out, 0, sizeof(*out));
    GCFG_TRY(e.layout(n, widths, heights, lambdas, true, false));
    GCFG_TRY(e.build_images(d_rgb, d_scrib));
    cudaEvent_t ev[4] = {};
    for (auto &x : ev) GCFG_CK(cudaEventCreate(&x));
    gcfg_status rc = GCFG_OK;
    Ctl c1;
    SolveParams p = e.prm;
    do {
        if (cudaMemsetAsync(e.d_ctl, 0, sizeof(Ctl), e.st) != cudaSuccess) { rc = GCFG_ERR_CUDA; break; }
        p.phase = 1;
        cudaEventRecord(ev[0], e.st);
        if ((rc = launch_solve(e.batch(), p, e.n_tiles, e.st, e.max_grid)) != GCFG_OK) break;
        cudaEventRecord(ev[1], e.st);
        if ((rc = e.fetch()) != GCFG_OK) break;
        c1 = *e.h_ctl;
        if (c1.err) { rc = GCFG_ERR_NOT_CONVERGED; break; }
        out->grid_blocks = solve_grid_blocks(e.n_tiles, e.max_grid, solve_warps(p.warps, e.n_tiles));
        out->relabel_tiles = (int64_t)c1.gr_tiles;
        out->relabel_rounds = c1.gr_rounds;
        out->active_pixels = (int64_t)c1.total_active;
        out->push_queue = c1.size[L_PUSH0] + c1.size[L_PUSH1];
        out->relabel_round0_us = (float)((double)(c1.gr_time[1] - c1.gr_time[0]) * 1e-3);
        out->relabel_pull_us = (float)((double)(c1.gr_time[2] - c1.gr_time[1]) * 1e-3);
        for (int k = 0; k < GR_TIMELINE && k < c1.gr_rounds; ++k) {
            out->relabel_front_us[k] = (float)((double)(c1.gr_time[3 + k] - c1.gr_time[2 + k]) * 1e-3);
            out->relabel_front_tiles[k] = c1.gr_front[k];
            if (c1.gr_front_end[k] > c1.gr_time[2 + k])
                out->relabel_front_work_us[k] = (float)((double)(c1.gr_front_end[k] - c1.gr_time[2 + k]) * 1e-3);
            out->relabel_front_maxvisit_kcyc[k] = (float)((double)c1.gr_front_maxcyc[k] * 1e-3);
        }
        cudaEventElapsedTime(&out->ms_relabel, ev[0], ev[1]);
        if (c1.total_active == 0) break;  // nothing to push: the solve is over after the relabel
        p.phase = 2;  // the control block keeps the first push round's queues
        cudaEventRecord(ev[2], e.st);
        if ((rc = launch_solve(e.batch(), p, e.n_tiles, e.st, e.max_grid)) != GCFG_OK) break;
        cudaEventRecord(ev[3], e.st);
        if ((rc = e.fetch()) != GCFG_OK) break;
        const Ctl &c2 = *e.h_ctl;
        if (c2.err) { rc = GCFG_ERR_NOT_CONVERGED; break; }
        out->push_tiles = (int64_t)(c2.push_tiles - c1.push_tiles);
        out->push_sweeps = (int64_t)(c2.push_sweeps - c1.push_sweeps);
        out->push_local_relabels = (int64_t)(c2.push_bfs - c1.push_bfs);
        out->push_phases = c2.push_phases - c1.push_phases;
        cudaEventElapsedTime(&out->ms_push, ev[2], ev[3]);
    } while (false);
    for (auto &x : ev) cudaEventDestroy(x);
    return rc;
}

gcfg_status gcfg_batch_destroy(gcfg_batch *b) {
    if (!b) return GCFG_ERR_INVALID;
    delete b;
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
    case GCFG_ERR_TOO_LARGE: return "image larger than the fixed working memory of the allocation-free solve";
    }
    return "unknown";
}

int64_t gcfg_launch_count(void) { return g_launches.load(); }

}  // extern "C"
