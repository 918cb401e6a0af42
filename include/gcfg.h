/*
 * gcfg.h -- C ABI of the GB300-native gc-fg graph-cut path (libgcfg.so).
 *
 * Plain pointers and sizes only.  Device-pointer arguments are CUDA device
 * addresses; host-pointer arguments are ordinary host memory.  Every entry
 * point returns a gcfg_status (0 = success) instead of aborting the process,
 * and every loop inside the solver is bounded.  Streams are passed as
 * `void *` holding a cudaStream_t (NULL = legacy default stream).
 *
 * The graph entry points replace the reference's C++ host API
 * (GraphCut.cu, compiled into each application via #include):
 *   gcfg_init          <- GC_Init          GraphCut.cu:187-263
 *   gcfg_set_dataterms <- GC_SetDataterms  GraphCut.cu:265-269
 *   gcfg_set_edges     <- GC_SetEdges      GraphCut.cu:271-289
 *   gcfg_set_penalty   <- GC_SetPenalty    GraphCut.cu:296-299
 *   gcfg_set_graph     <- GC_SetGraph      GraphCut.cu:301-319
 *   gcfg_optimize      <- GC_Optimize      GraphCut.cu:385-534
 *   gcfg_end           <- GC_End           GraphCut.cu:542-568
 * The data-term entry points replace the DataTerm:: namespace
 * (DataTerm.h:9-19, DataTerm.cpp:52-205).
 */
#ifndef GCFG_H
#define GCFG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    GCFG_OK = 0,
    GCFG_ERR_INVALID = 1,         /* bad sizes, NULL handle, or out-of-range capacities */
    GCFG_ERR_OOM = 2,             /* device allocation failed */
    GCFG_ERR_CUDA = 3,            /* a CUDA call failed */
    GCFG_ERR_NOT_CONVERGED = 4,   /* an iteration cap was reached */
    GCFG_ERR_STATE = 5,           /* call out of order (e.g. optimize before set_graph) */
    GCFG_ERR_CAPACITY = 6,        /* admission refused: over the memory cap */
    GCFG_ERR_TOO_LARGE = 7        /* larger than the fixed working memory of gcfg_solve_noalloc */
} gcfg_status;

/* Largest accepted capacity (t-links and n-links).  Keeps every excess and
 * residual value inside int32 during the solve. */
#define GCFG_MAX_CAP ((1 << 28) - 1)

typedef struct gcfg_graph gcfg_graph;

typedef struct {
    int64_t flow;            /* exact max-flow value = energy of the min cut */
    int32_t ref_energy;      /* the value GC_Optimize prints as "Final energy level"
                                (GraphCut.cu:456-457): int32, border dp included */
    int32_t status;          /* gcfg_status of the solve */
    int32_t global_relabels; /* exact global relabels run */
    int32_t gr_sweeps;       /* tile-frontier rounds inside global relabels */
    int32_t push_rounds;     /* checkerboard push phases (one colour each) */
    int32_t cut_sweeps;      /* tile-frontier rounds of the source-side reachability */
    int64_t reach_tiles;     /* 32x32 tile visits by the source-side reachability */
    int64_t push_tiles;      /* 32x32 tile visits by push/relabel */
    int64_t gr_tiles;        /* 32x32 tile visits by global relabels */
    int64_t push_sweeps;     /* push/relabel sweeps summed over tile visits */
    int64_t push_local_relabels; /* exact local (tile BFS) relabels in push visits */
    float t_global_relabel_ms, t_count_ms, t_push_ms, t_reach_ms; /* device time per phase */
    /* SM cycles summed over push tile visits, per section (load, local
     * relabel, sweeps, write-back + hand-over, queue take) */
    int64_t cyc_load, cyc_local_relabel, cyc_sweeps, cyc_writeback, cyc_take;
    float ms;                /* device time of the solve (CUDA events) */
    float t_push_tail_ms;    /* push phases' tails: from the first solver block out of work to the phase's end */
    /* tile-BFS loop iterations summed over push visits' local relabels and
     * over global-relabel visits; SM cycles summed over global-relabel visits */
    int64_t bfs_iters_push, bfs_iters_gr, cyc_global_relabel;
    /* termination checks by a sink-side reachability closure (run after push
     * rounds instead of a global relabel when no pixel with excess can reach
     * the sink any more), and 1 when such a check ended the solve */
    int32_t closure_checks, closure_ends;
} gcfg_result;

/* ---------------- graph API (drop-in for GraphCut.cu) ---------------- */

/* GC_Init: allocate the residual graph for a w x h grid.  dp/dn are the
 * source (positive) and sink (negative) t-link capacities, W*H int32,
 * row-major, device memory, caller-owned.  If up != NULL the four arrays give
 * per-direction n-link capacities (cap from pixel p to its upper/lower/left/
 * right neighbour), else every n-link is `penalty`.  When dp != NULL the graph
 * is built immediately (GC_Init calls GC_SetGraph, GraphCut.cu:250-260). */
gcfg_status gcfg_init(int w, int h, const int32_t *dp, const int32_t *dn, int32_t penalty,
                      const int32_t *up, const int32_t *down, const int32_t *left,
                      const int32_t *right, gcfg_graph **out);
gcfg_status gcfg_set_dataterms(gcfg_graph *g, const int32_t *dp, const int32_t *dn);
gcfg_status gcfg_set_edges(gcfg_graph *g, const int32_t *up, const int32_t *down,
                           const int32_t *left, const int32_t *right);
gcfg_status gcfg_set_penalty(gcfg_graph *g, int32_t penalty);
/* GC_SetGraph: (re)build the residual graph from the stored inputs. */
gcfg_status gcfg_set_graph(gcfg_graph *g);
/* GC_Optimize: solve to the exact max flow.  If host_label != NULL it
 * receives W*H int32 labels: 1 = source side of the maximal source set
 * (pixels that cannot reach the sink), 0 = sink side and the 1-pixel border,
 * exactly like the reference's output (GraphCut.cu:507-529).  res may be
 * NULL. */
gcfg_status gcfg_optimize(gcfg_graph *g, int32_t *host_label, gcfg_result *res);
/* After gcfg_optimize: both canonical cuts into device buffers (W*H bytes
 * each, either may be NULL): smin = pixels reachable from the source in the
 * final residual graph, smax = pixels that cannot reach the sink. */
gcfg_status gcfg_get_cuts(gcfg_graph *g, uint8_t *d_smin, uint8_t *d_smax);
/* GC_End: free everything the graph owns (caller arrays are not freed). */
gcfg_status gcfg_end(gcfg_graph *g);
/* Stream used by every later call on this graph (void* = cudaStream_t). */
gcfg_status gcfg_set_stream(gcfg_graph *g, void *stream);
/* Checkerboard push rounds between global relabels, and push/relabel sweeps
 * per tile visit (solver schedule; does not change the result). */
gcfg_status gcfg_set_schedule(gcfg_graph *g, int push_rounds_per_gr, int max_tile_sweeps);

/* ---------------- graph API with the 8-neighbourhood ---------------- */

/* The reference built with NEIGHBORHOOD == 8 (GraphCut.h:22; GC_Init's extra
 * upleft/upright/downleft/downright arrays, GraphCut.cu:187-194): the same
 * calls and meanings as above with four more per-direction capacity arrays
 * (device int32 W*H each; upleft[p] is the capacity from p to the pixel above
 * and to its left, and so on).  The diagonals of the interior pixels next to
 * the border are zeroed like the straight edges (GraphCutKernels.cu:147-151,
 * 204-208).  Capacities are limited to GCFG_MAX_CAP8 so that an excess over
 * nine edges stays inside int32.  A separate engine solves these graphs
 * (32x8 tile rounds of push/relabel, exact global relabels by tile
 * relaxation, and the exact termination test, as for 4). */
typedef struct gcfg_graph8 gcfg_graph8;
#define GCFG_MAX_CAP8 ((1 << 27) - 1)

gcfg_status gcfg_init8(int w, int h, const int32_t *dp, const int32_t *dn, int32_t penalty,
                       const int32_t *up, const int32_t *down, const int32_t *left,
                       const int32_t *right, const int32_t *upleft, const int32_t *upright,
                       const int32_t *downleft, const int32_t *downright, gcfg_graph8 **out);
gcfg_status gcfg_set_dataterms8(gcfg_graph8 *g, const int32_t *dp, const int32_t *dn);
gcfg_status gcfg_set_edges8(gcfg_graph8 *g, const int32_t *up, const int32_t *down,
                            const int32_t *left, const int32_t *right, const int32_t *upleft,
                            const int32_t *upright, const int32_t *downleft,
                            const int32_t *downright);
gcfg_status gcfg_set_penalty8(gcfg_graph8 *g, int32_t penalty);
gcfg_status gcfg_set_graph8(gcfg_graph8 *g);
/* gcfg_optimize8 fills flow, ref_energy, status, global_relabels, ms (the
 * solve kernel), gr_sweeps (tile-relaxation rounds of the global relabels),
 * gr_tiles (their 32x32 tile visits), push_rounds (tile rounds), push_tiles
 * (32x8 tile visits that had work) and cut_sweeps (tile rounds of the
 * source-side closure); the other fields are 0. */
gcfg_status gcfg_optimize8(gcfg_graph8 *g, int32_t *host_label, gcfg_result *res);
gcfg_status gcfg_get_cuts8(gcfg_graph8 *g, uint8_t *d_smin, uint8_t *d_smax);
gcfg_status gcfg_end8(gcfg_graph8 *g);
gcfg_status gcfg_set_stream8(gcfg_graph8 *g, void *stream);
/* Tile rounds between exact global relabels (default 12; every 32x8 tile is
 * visited once per round, with up to 8 block-local push/relabel sweeps) and
 * blocks of the cooperative launch per SM (default 3; 0 = as many as fit);
 * the solver schedule only, results do not depend on it. */
gcfg_status gcfg_set_schedule8(gcfg_graph8 *g, int rounds_per_gr, int blocks_per_sm);

/* ---------------- data term + n-links ---------------- */

/* Colour-histogram t-links for one image: 16^3 bins of (r>>4, g>>4, b>>4)
 * over fg (scrib == 1) and bg (scrib == 2) pixels, +1 Laplace smoothing;
 * dp = round(10 * -log p_bg), dn = round(10 * -log p_fg) (int32).
 * d_rgb: 3*n bytes interleaved, d_scrib: n bytes, d_dp/d_dn: n int32 (device).
 * h_raw_dp/h_raw_dn: optional host double[4096] receiving the pre-rounding
 * per-bin values. */
gcfg_status gcfg_tlinks(const uint8_t *d_rgb, const uint8_t *d_scrib, int n, int32_t *d_dp,
                        int32_t *d_dn, double *h_raw_dp, double *h_raw_dn, void *stream);
/* Contrast-sensitive 4-connected n-links for a w x h image:
 * w = round(lambda * exp(-||dI||^2 / (2 sigma^2))), sigma^2 = mean ||dI||^2
 * over all horizontally and vertically adjacent pixel pairs.
 * Outputs W*H int32 per direction (device); edges leaving the image are 0. */
gcfg_status gcfg_nlinks(const uint8_t *d_rgb, int w, int h, double lambda, int32_t *d_up,
                        int32_t *d_down, int32_t *d_left, int32_t *d_right, void *stream);

/* ---------------- DataTerm state (drop-in for DataTerm.h:9-19) ---------------- */

/* The reference's data-term state (an image, a selection map, a colour model
 * and the two t-link arrays; DataTerm.cpp:28-165) as a handle.  The colour
 * model is the 16^3 histogram pair of gcfg_tlinks, rebuilt from the current
 * image and selection map by gcfg_dt_compute: selection class 1 = foreground
 * (the reference's only class), 2 = background (scribbles of the second class).
 * The t-links are dp = round(10 * -log p_bg) (source, "positive") and
 * dn = round(10 * -log p_fg) (sink, "negative"), W*H int32 on the device,
 * owned by the handle, ready for gcfg_init.  All host copies are blocking. */
typedef struct gcfg_dataterm gcfg_dataterm;

/* Side of the square that gcfg_dt_select_on_map marks (DataTerm.cpp:113). */
#define GCFG_DT_SELECT_SIZE 5

/* Colour models of a DataTerm handle. */
enum {
    GCFG_DT_HISTOGRAM = 0, /* default: 16^3 histogram pair of the selected pixels (see above) */
    GCFG_DT_KDE = 1        /* the reference's kernel density (DataTerm.cpp:97-137) */
};

/* init_data_term (DataTerm.cpp:28): allocate for a w x h image; empty selection. */
gcfg_status gcfg_dt_create(int w, int h, gcfg_dataterm **out);
/* free_data_term (DataTerm.cpp:67); unlike the reference the t-link arrays
 * are freed too (they belong to the handle). */
gcfg_status gcfg_dt_destroy(gcfg_dataterm *dt);
gcfg_status gcfg_dt_set_stream(gcfg_dataterm *dt, void *stream);
/* setImage (DataTerm.cpp:80): host image, 3*w*h bytes interleaved (any
 * channel order: the histogram bins and colour distances do not depend on it). */
gcfg_status gcfg_dt_set_image(gcfg_dataterm *dt, const uint8_t *h_img);
/* The same from device memory (no counterpart). */
gcfg_status gcfg_dt_set_image_device(gcfg_dataterm *dt, const uint8_t *d_img);
/* setSelection (DataTerm.cpp:139): host int32 map of w*h, each value stored
 * as one byte (0 none, 1 foreground, 2 background). */
gcfg_status gcfg_dt_set_selection(gcfg_dataterm *dt, const int32_t *h_select);
/* The selection as a device byte map of w*h (no counterpart). */
gcfg_status gcfg_dt_set_scribbles_device(gcfg_dataterm *dt, const uint8_t *d_scrib);
/* reset (DataTerm.cpp:88): clear the selection. */
gcfg_status gcfg_dt_reset(gcfg_dataterm *dt);
/* selectOnMap (DataTerm.cpp:105): mark the GCFG_DT_SELECT_SIZE square with
 * corner (x, y) as class cls (1 or 2), clipped to the image. */
gcfg_status gcfg_dt_select_on_map(gcfg_dataterm *dt, int x, int y, int cls);
/* setSigmaGaussian (DataTerm.cpp:97): stored; the histogram model has no
 * kernel width, so it does not change the t-links. */
gcfg_status gcfg_dt_set_sigma(gcfg_dataterm *dt, int sigma);
/* getDataTermsMixture (DataTerm.cpp:129): compute the t-links into the
 * handle's arrays (returns when they are written). */
gcfg_status gcfg_dt_compute(gcfg_dataterm *dt);
/* getPos / getNeg (DataTerm.cpp:12,20): the device t-link arrays. */
int32_t *gcfg_dt_pos(gcfg_dataterm *dt);
int32_t *gcfg_dt_neg(gcfg_dataterm *dt);
/* The handle's device image (3*w*h) and selection map (w*h) (no counterpart). */
uint8_t *gcfg_dt_image(gcfg_dataterm *dt);
uint8_t *gcfg_dt_selection(gcfg_dataterm *dt);
/* drawSelection (DataTerm.cpp:155): h_in becomes the current image; h_out
 * receives it with the pixels whose selection-map entry is 1 set to
 * (0, 0, 255), every other pixel unchanged, as K_DrawMap does
 * (DataTermKernels.cu:96-113). */
gcfg_status gcfg_dt_draw_selection(gcfg_dataterm *dt, const uint8_t *h_in, uint8_t *h_out);
/* Choose the colour model.  GCFG_DT_KDE is the reference's own data term: a
 * kernel density over the 256^3 colour cube (64 MB, allocated on first use)
 * to which every class-1 gcfg_dt_select_on_map adds, for each pixel of its
 * 5x5 square, gauss[floor(|c - colour|)] at every cube point c within
 * distance 101 (DataTermKernels.cu:116-150), where gauss is the 101-entry
 * table of gcfg_dt_set_sigma (default sigma 5, DataTerm.cpp:6,63); then
 * gcfg_dt_compute gives pos = (int)(300000 p), neg = (int)(300000 (1 - p))
 * with p the density at the pixel's colour (DataTermKernels.cu:61-83).  In
 * this model gcfg_dt_set_selection only sets the map and gcfg_dt_reset also
 * clears the density, as in the reference.  Unlike the reference, the square
 * is clipped to the image and every pixel gets t-links (the reference skips
 * the pixels outside whole 16x16 blocks). */
gcfg_status gcfg_dt_set_model(gcfg_dataterm *dt, int model);
/* The kernel density's 101-entry table (host float[101]); GCFG_ERR_STATE
 * before the model was first chosen. */
gcfg_status gcfg_dt_kde_table(gcfg_dataterm *dt, float *h_gauss);
/* gcfg_nlinks of the handle's current image (no counterpart). */
gcfg_status gcfg_dt_nlinks(gcfg_dataterm *dt, double lambda, int32_t *d_up, int32_t *d_down,
                           int32_t *d_left, int32_t *d_right);

/* ---------------- one-image segmentation pipeline ---------------- */

typedef struct gcfg_segmenter gcfg_segmenter;

/* A reusable solver for images up to max_w x max_h (buffers allocated once). */
gcfg_status gcfg_seg_create(int max_w, int max_h, gcfg_segmenter **out);
/* Data term + n-links + graph build + exact solve + both cuts for one image
 * already on the device.  d_smin/d_smax: W*H bytes (device, may be NULL). */
gcfg_status gcfg_seg_run(gcfg_segmenter *s, const uint8_t *d_rgb, const uint8_t *d_scrib, int w,
                         int h, double lambda, uint8_t *d_smin, uint8_t *d_smax,
                         gcfg_result *res);
/* The same, end to end from host memory: copies the image and scribbles in,
 * solves, copies the labels out (h_smin/h_smax W*H bytes, may be NULL). */
gcfg_status gcfg_seg_run_host(gcfg_segmenter *s, const uint8_t *h_rgb, const uint8_t *h_scrib,
                              int w, int h, double lambda, uint8_t *h_smin, uint8_t *h_smax,
                              gcfg_result *res);
gcfg_status gcfg_seg_set_stream(gcfg_segmenter *s, void *stream);
gcfg_status gcfg_seg_destroy(gcfg_segmenter *s);

/* ---------------- batched segmentation (many images, one solve) ---------------- */

/* The images of a batch are solved together: one data-term pass, one build,
 * one persistent solver launch over the tiles of all images, one extraction.
 * Images are packed back to back in row-major order (image i starts at pixel
 * offset sum_{j<i} w_j*h_j; RGB at 3x that byte offset). */
typedef struct gcfg_batch gcfg_batch;

/* Pre-size for max_images images totalling max_pixels pixels (buffers grow
 * on demand if a later batch is larger). */
gcfg_status gcfg_batch_create(int max_images, int64_t max_pixels, gcfg_batch **out);
gcfg_status gcfg_batch_set_stream(gcfg_batch *b, void *stream);
/* Solver schedule: push rounds between global relabels, sweeps per tile
 * visit, sweeps between exact local relabels (does not change results). */
gcfg_status gcfg_batch_set_params(gcfg_batch *b, int push_rounds_per_gr, int max_tile_sweeps,
                                  int sweeps_per_local_relabel);
/* Device-resident batch.  d_smin/d_smax (packed, may be NULL) receive the
 * two canonical cuts; h_flows (n, may be NULL) the exact flow values;
 * h_res (n, may be NULL) per-image result records. */
gcfg_status gcfg_batch_run(gcfg_batch *b, int n, const int *widths, const int *heights,
                           const double *lambdas, const uint8_t *d_rgb, const uint8_t *d_scrib,
                           uint8_t *d_smin, uint8_t *d_smax, int64_t *h_flows, gcfg_result *h_res);
/* The same from host memory: inputs copied in and labels copied out. */
gcfg_status gcfg_batch_run_host(gcfg_batch *b, int n, const int *widths, const int *heights,
                                const double *lambdas, const uint8_t *h_rgb, const uint8_t *h_scrib,
                                uint8_t *h_smin, uint8_t *h_smax, int64_t *h_flows,
                                gcfg_result *h_res);
/* Asynchronous form of gcfg_batch_run_host for a stream of batches: queue a
 * batch and return at once with a ticket; gcfg_batch_wait(ticket) blocks
 * until its labels are in h_smin/h_smax and fills h_flows/h_res as
 * gcfg_batch_run_host does.  Up to two batches are in flight per handle:
 * while one computes, the next one's inputs are uploaded and the previous
 * one's labels are downloaded.  The host buffers of a batch (pinned memory
 * for the copies to overlap) must stay valid and unchanged until its wait
 * returns.  A third submit before a wait, and any other run, autotune or
 * set_stream call while batches are in flight, return GCFG_ERR_STATE; an
 * unknown ticket GCFG_ERR_INVALID.  Tickets may be collected in any order. */
gcfg_status gcfg_batch_submit_host(gcfg_batch *b, int n, const int *widths, const int *heights,
                                   const double *lambdas, const uint8_t *h_rgb, const uint8_t *h_scrib,
                                   uint8_t *h_smin, uint8_t *h_smax, int64_t *ticket);
gcfg_status gcfg_batch_wait(gcfg_batch *b, int64_t ticket, int64_t *h_flows, gcfg_result *h_res);
gcfg_status gcfg_batch_destroy(gcfg_batch *b);

/* CUDA graph replay (off by default).  When on, the device part of a run
 * (data term, graph build, the persistent solver launch that runs the whole
 * push / local relabel / global relabel loop, extraction, read-back of the
 * results) is captured into a CUDA graph the first time a batch is run and
 * replayed while the next runs have the same sizes, lambdas, device buffers
 * and solver settings; anything else recaptures.  If the device cannot
 * capture, runs continue without the graph (gcfg_batch_graph_info: active 0).
 * Results are identical either way.  No counterpart in the reference. */
gcfg_status gcfg_batch_set_graph(gcfg_batch *b, int enable);
gcfg_status gcfg_batch_graph_info(gcfg_batch *b, int *active, int64_t *captures, int64_t *replays,
                                  int64_t *kernels_per_replay);

/* Autotuner result: the solver settings chosen for a batch.  The tile shape
 * is the thread block over each 32x32 tile of the residual graph: 32 x
 * threads_y threads, the counterpart of the reference's THREADS_X x
 * THREADS_Y (GraphCut.h:39-53, 32 x 8); the data tile itself stays 32x32,
 * the width of the bit-plane tile BFS (one 32-bit mask per row). */
typedef struct {
    int32_t push_rounds_per_gr;       /* checkerboard push rounds between global relabels */
    int32_t max_tile_sweeps;          /* push/relabel sweeps per tile visit */
    int32_t sweeps_per_local_relabel; /* sweeps between exact local (tile BFS) relabels */
    int32_t blocks_per_sm;            /* persistent solver blocks per SM (for one image: blocks per image / SMs) */
    float ms_default, ms_best;        /* device time of one run before / after tuning */
    int32_t configs_tried;
    int32_t tile_w, tile_h;           /* data tile of the residual graph (32 x 32, fixed) */
    int32_t local_relabel_first;      /* 1: exact local relabel at the start of every tile visit */
    int32_t push_only;                /* 1: sweeps only push; heights change by exact local relabels */
    int32_t threads_y;                /* solver block 32 x threads_y: 4, 8, 16 or 32; 0 in gcfg_batch_set_solver:
                                         by the solve's size, 16 up to 2048 tiles, else 8 (the default) */
} gcfg_tuning;

/* Use these solver settings for the following runs (for example the record
 * an earlier gcfg_batch_autotune returned; blocks_per_sm 0 = as many as fit;
 * ms_*, configs_tried and the tile shape are ignored).  Results do not depend
 * on them.  No counterpart in the reference. */
gcfg_status gcfg_batch_set_solver(gcfg_batch *b, const gcfg_tuning *t);

/* Time the batch (device-resident, as gcfg_batch_run) under candidate solver
 * settings (the fields above) by coordinate search, keep the fastest, and use it for the
 * following runs of this handle.  Each setting is timed as the fastest of
 * `reps` runs; every run must reproduce the flows of the first (else
 * GCFG_ERR_NOT_CONVERGED).  No counterpart in the reference. */
gcfg_status gcfg_batch_autotune(gcfg_batch *b, int n, const int *widths, const int *heights,
                                const double *lambdas, const uint8_t *d_rgb, const uint8_t *d_scrib,
                                int reps, gcfg_tuning *out);

/* Diagnostic: the batch's data term and build, then the solver's two main
 * phases as two separate launches of the persistent solver kernel, so that a
 * profiler (or the events below) sees each on its own: launch 1 = the first
 * exact global relabel with its count pass (the reference's InitGlobalRelabel
 * + GlobalRelabel, GraphCutKernels.cu:757-875), launch 2 = the push rounds
 * that follow it (WavePush + Relabel, GraphCutKernels.cu:433-724).  The solve
 * is left unfinished (no cut); run the batch again for results.  Current
 * solver settings of the handle apply. */
typedef struct {
    float ms_relabel;             /* device time of launch 1 */
    float ms_push;                /* device time of launch 2 (0 when nothing was active) */
    int64_t relabel_tiles;        /* global-relabel tile visits of launch 1 */
    int64_t active_pixels;        /* pixels with excess and finite height after the relabel */
    int64_t push_tiles;           /* push tile visits of launch 2 */
    int64_t push_sweeps;          /* push/relabel sweeps of those visits */
    int64_t push_local_relabels;  /* exact local relabels of those visits */
    int32_t relabel_rounds;       /* tile-frontier rounds of the relabel after its first */
    int32_t push_phases;          /* checkerboard colour phases of launch 2 */
    int32_t push_queue;           /* tiles queued for the first two colour phases */
    int32_t grid_blocks;          /* blocks of each launch */
    /* timeline of launch 1's global relabel (device clock, microseconds):
     * round 0 (every tile, halos from the neighbours' sink pixels), the pull
     * check that picks the first frontier, then frontier round k with
     * relabel_front_tiles[k] tiles, for k < min(relabel_rounds, 32) */
    float relabel_round0_us, relabel_pull_us;
    float relabel_front_us[32];
    int32_t relabel_front_tiles[32];
    /* per frontier round: from its start to the end of its last tile visit
     * (the rest of the round is the grid barrier), and its longest visit */
    float relabel_front_work_us[32];
    float relabel_front_maxvisit_kcyc[32];
} gcfg_phase_split;

gcfg_status gcfg_batch_phase_split(gcfg_batch *b, int n, const int *widths, const int *heights,
                                   const double *lambdas, const uint8_t *d_rgb, const uint8_t *d_scrib,
                                   gcfg_phase_split *out);

/* ---------------- serving (continuous batching, resident images) ---------------- */

/* A server keeps every admitted image resident on the device (pixels,
 * scribbles, residual graph, histograms, t-link tables) and solves waiting
 * requests in batches on `lanes` worker lanes (host thread + stream each);
 * requests that arrive while lanes are busy join the next free lane's batch,
 * and with two lanes two batches run on the device at once.  New images are
 * admitted while their device footprint fits under mem_cap_bytes (idle
 * resident images are evicted least-recently-used first).  A scribble edit of
 * a resident image is re-solved warm from its stored flow with the t-links
 * reparametrised; its result equals a cold solve of the edited image. */
typedef struct gcfg_server gcfg_server;

typedef struct {
    int64_t mem_cap_bytes;    /* device footprint cap of resident images */
    int32_t lanes;            /* worker lanes (1..8) */
    int32_t max_batch_images; /* images per batch */
    int64_t max_batch_tiles;  /* 32x32 tiles per batch (also the largest image) */
    int32_t max_sessions;     /* resident images */
    int32_t pad;
} gcfg_serve_config;

enum { GCFG_REQ_NEW = 0, GCFG_REQ_EDIT = 1 };

typedef struct {
    int32_t kind;             /* GCFG_REQ_NEW or GCFG_REQ_EDIT */
    int32_t pad0;
    int64_t session;          /* GCFG_REQ_EDIT: the resident image to edit */
    int32_t w, h;             /* GCFG_REQ_NEW: image size */
    double lambda;            /* GCFG_REQ_NEW: n-link weight */
    const uint8_t *h_rgb;     /* GCFG_REQ_NEW: host RGB (3*w*h), valid until completion */
    const uint8_t *h_scrib;   /* GCFG_REQ_NEW: host scribbles (w*h: 0/1 fg/2 bg) */
    int32_t edit_x, edit_y;   /* GCFG_REQ_EDIT: top-left corner of the scribble square */
    int32_t edit_size;        /* GCFG_REQ_EDIT: side of the square */
    int32_t edit_class;       /* GCFG_REQ_EDIT: 1 = foreground, 2 = background */
    uint8_t *h_smin, *h_smax; /* host outputs (w*h each) or NULL */
} gcfg_serve_request;

typedef struct {
    int32_t status;           /* gcfg_status of the request */
    int32_t warm;             /* 1: solved warm (scribble edit) */
    int64_t session;          /* resident image id (new for GCFG_REQ_NEW) */
    int64_t flow;             /* exact flow value */
    int32_t batch_images;     /* images in the batch that solved it */
    int32_t lane;
    double t_submit, t_start, t_done; /* host clock (gcfg_serve_now), seconds */
} gcfg_serve_result;

typedef struct {
    int64_t submitted, admitted, completed, evicted, batches;
    int64_t bytes_in_use, sessions, queued;
} gcfg_serve_stats;

gcfg_status gcfg_serve_create(const gcfg_serve_config *cfg, gcfg_server **out);
/* Non-blocking; returns a ticket for gcfg_serve_wait and the id of the
 * resident image (a new one for GCFG_REQ_NEW; edits may be submitted for it
 * at once and run after its first solve).  A new image larger than
 * max_batch_tiles or than the whole cap is refused (GCFG_ERR_CAPACITY). */
gcfg_status gcfg_serve_submit(gcfg_server *s, const gcfg_serve_request *req, int64_t *ticket,
                              int64_t *session);
/* Wait for a ticket (timeout_ms < 0: no limit).  Returns the request's status. */
gcfg_status gcfg_serve_wait(gcfg_server *s, int64_t ticket, gcfg_serve_result *res, int timeout_ms);
/* Drop a resident image (not while a request uses it). */
gcfg_status gcfg_serve_release(gcfg_server *s, int64_t session);
gcfg_status gcfg_serve_get_stats(gcfg_server *s, gcfg_serve_stats *out);
gcfg_status gcfg_serve_destroy(gcfg_server *s);
/* The host clock of the result timestamps (seconds). */
double gcfg_serve_now(void);

/* ---------------- allocation-free solve ---------------- */

/* Largest image of gcfg_solve_noalloc, in 32x32 tiles, and the size of the
 * fixed device array that holds its working memory. */
#define GCFG_NOALLOC_MAX_TILES 640
#define GCFG_NOALLOC_SCRATCH_BYTES (16u << 20)

/* Solves one graph like gcfg_init + gcfg_optimize, but allocates nothing:
 * no cudaMalloc, cudaFree or other allocating call.  It has no counterpart in
 * the reference.  It is for callers that cannot allocate device memory at
 * solve time: a host framework that owns all of the GPU's memory and forbids
 * plug-ins to allocate, a process already at its device-memory limit, or a
 * latency-bound loop that cannot afford the device-wide synchronisation that
 * cudaMalloc/cudaFree can cause.  Its working memory is one fixed file-scope
 * device array of GCFG_NOALLOC_SCRATCH_BYTES (16 MiB) that every GPU loading
 * this library holds until the process exits.
 *
 * Inputs as in gcfg_init (device arrays, caller-owned; up == NULL selects the
 * constant penalty).  Outputs: d_label (device, W*H int32) receives the
 * labels gcfg_optimize returns; *h_flow (host, may be NULL) the exact flow.
 * Limits: ceil(w/32) * ceil(h/32) <= GCFG_NOALLOC_MAX_TILES (e.g. 1024x640 or
 * 800x800 pixels), else GCFG_ERR_TOO_LARGE before any GPU work.
 * All calls share the array and it keeps the last call's contents (each call
 * clears what must start at zero); calls whose GPU work overlaps, e.g. on two
 * streams, race on it and must be serialised.  Every call looks up the
 * array's device address on the current device (cudaGetSymbolAddress, which
 * allocates nothing).
 * stream: cudaStream_t as void* (NULL = legacy default stream).  The call
 * synchronises that stream twice (after the build, to read the capacity
 * check, and after the solve, to read the flow) and returns after the solve
 * has finished. */
gcfg_status gcfg_solve_noalloc(int w, int h, const int32_t *d_dp, const int32_t *d_dn, int32_t penalty,
                               const int32_t *d_up, const int32_t *d_down, const int32_t *d_left,
                               const int32_t *d_right, int32_t *d_label, int64_t *h_flow,
                               void *stream);

/* ---------------- profiling (off by default) ---------------- */

/* Kernel kinds reported by gcfg_profile_read (index = kind). */
typedef enum {
    GCFG_PK_HIST = 0,   /* scribble colour histograms */
    GCFG_PK_TLUT,       /* per-bin t-link tables */
    GCFG_PK_SIGMA,      /* sum of ||dI||^2 */
    GCFG_PK_WLUT,       /* n-link weight tables */
    GCFG_PK_BUILD,      /* residual graph build */
    GCFG_PK_SOLVE,      /* persistent max-flow kernel (relabel, push, cuts) */
    GCFG_PK_EXTRACT,    /* label extraction */
    GCFG_PK_OTHER,
    GCFG_PK_NKINDS
} gcfg_prof_kind;

typedef struct {
    int32_t kind;
    int32_t launches;
    double ms;               /* summed device duration (CUDA events) */
} gcfg_prof_entry;

/* Bracket every kernel launch with CUDA events (adds host overhead). */
gcfg_status gcfg_profile_enable(int on);
/* Per-kind totals since the last read; out must hold GCFG_PK_NKINDS entries. */
gcfg_status gcfg_profile_read(gcfg_prof_entry *out, int max_entries, int *n_out);

/* ---------------- misc ---------------- */
const char *gcfg_strerror(gcfg_status s);
/* Number of kernel launches issued by this library in this process. */
int64_t gcfg_launch_count(void);
/* Largest relative error of the device's approximate base-2 exponential
 * (the n-link fast path) over `samples` evenly spaced points of [-64, 0];
 * the fast path's error bound assumes <= 2^-21 (no counterpart). */
gcfg_status gcfg_selftest_ex2(int64_t samples, float *max_rel_err);

#ifdef __cplusplus
}
#endif
#endif
