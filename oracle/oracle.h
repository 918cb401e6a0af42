/*
 * oracle.h -- CPU oracle for the gc-fg binary-MRF graph-cut path.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product library links, loads or
 * calls this code; only the test suite, the smoke check and the CPU-baseline
 * leg of bench.py use it, and only to check and time against.
 *
 * It restates, in plain C:
 *   - the colour-histogram data term and the contrast-sensitive n-links;
 *   - the reference's graph construction conventions
 *     (GraphCutKernels.cu:112-214: interior-only nodes, edges into the 1-pixel
 *     border zeroed, reduced t-link excess = dp - dn);
 *   - two exact max-flow solvers: a sequential push-relabel that follows the
 *     reference's algorithm (GraphCut.cu:385-534, GraphCutKernels.cu:600-875)
 *     and a Boykov-Kolmogorov augmenting-path solver (the CPU solver the
 *     reference's published comparison used), written from the 2004 paper;
 *   - cut extraction: S_max (the reference's SpreadLabels output,
 *     GraphCutKernels.cu:228-351) and S_min (source-reachable set).
 *
 * Parity of this oracle is pinned by running the reference's own CUDA
 * solver under a CPU thread emulator (oracle/refemu) on the same inputs.
 */
#ifndef GCFG_ORACLE_H
#define GCFG_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- data term: 16^3 histograms, +1 Laplace smoothing, round(10*-log p) ---- */
void or_histograms(const uint8_t *rgb, const uint8_t *scrib, int n,
                   int32_t *hist_fg, int32_t *hist_bg);
void or_tlink_lut(const int32_t *hist_fg, const int32_t *hist_bg,
                  double *raw_dp, double *raw_dn,
                  int32_t *dp_lut, int32_t *dn_lut);
void or_tlinks(const uint8_t *rgb, int n, const int32_t *dp_lut,
               const int32_t *dn_lut, int32_t *dp, int32_t *dn);

/* ---- n-links: sigma^2 = mean ||dI||^2 over all 4-neighbour pairs ---- */
void or_sigma_sum(const uint8_t *rgb, int W, int H, int64_t *sum, int64_t *count);
double or_nlink_weight_raw(int d2, double lambda, int64_t sum, int64_t count);
void or_nlinks(const uint8_t *rgb, int W, int H, double lambda,
               int32_t *up, int32_t *down, int32_t *left, int32_t *right);

/* ---- graph in the reference's conventions ----
 * caps: 4*W*H ints, per pixel {left, right, up, down} residual capacity.
 * excess: W*H ints, dp - dn on interior pixels, 0 elsewhere.
 * up/down/left/right may be NULL, in which case `penalty` is used
 * (GraphCutKernels.cu:112-157 vs 165-214). */
void or_build(int W, int H, const int32_t *dp, const int32_t *dn, int penalty,
              const int32_t *up, const int32_t *down, const int32_t *left,
              const int32_t *right, int32_t *caps, int32_t *excess);

/* ---- solvers: operate in place on caps/excess from or_build ---- */
typedef struct {
    int64_t flow;          /* exact max-flow value (int64) */
    int64_t pushes, relabels, global_relabels, augments;
} or_stats;

int or_maxflow_pr(int W, int H, int32_t *caps, int32_t *excess, or_stats *st);
int or_maxflow_bk(int W, int H, int32_t *caps, int32_t *excess, or_stats *st);

/* ---- cut extraction from a final residual graph ----
 * smax[i] = 1 iff interior and cannot reach the sink (reference labels);
 * smin[i] = 1 iff reachable from the source (from positive-excess nodes). */
void or_cuts(int W, int H, const int32_t *caps, const int32_t *excess,
             uint8_t *smin, uint8_t *smax);

/* Energy of a labelling under the original capacities (interior only). */
int64_t or_cut_energy(int W, int H, const int32_t *dp, const int32_t *dn,
                      int penalty, const int32_t *up, const int32_t *down,
                      const int32_t *left, const int32_t *right,
                      const uint8_t *label);

/* Sum over interior of dp (int64). */
int64_t or_interior_dp(int W, int H, const int32_t *dp);

/* The number the reference prints as "Final energy level", reproduced with
 * its int32 arithmetic and its padded-layout reduction (GraphCut.cu:359-376,
 * 399-401, 456-457; GraphCutKernels.cu:883-898). */
int32_t or_reference_energy(int W, int H, const int32_t *dp, const int32_t *excess_final);

/* One-call solve: build + solve + cuts. solver 0 = push-relabel, 1 = BK.
 * Returns 0 on success. */
int or_solve(int W, int H, const int32_t *dp, const int32_t *dn, int penalty,
             const int32_t *up, const int32_t *down, const int32_t *left,
             const int32_t *right, int solver, uint8_t *smin, uint8_t *smax,
             int64_t *flow, int32_t *excess_out, or_stats *st);

/* Full segmentation pipeline on one image: data term, n-links, solve. */
int or_segment(const uint8_t *rgb, const uint8_t *scrib, int W, int H,
               double lambda, int solver, int32_t *dp, int32_t *dn,
               int32_t *up, int32_t *down, int32_t *left, int32_t *right,
               uint8_t *smin, uint8_t *smax, int64_t *flow);

/* 8-connected graphs (the reference built with NEIGHBORHOOD == 8,
 * GraphCutKernels.cu:112-214 and the #if NEIGHBORHOOD == 8 blocks).
 * Directions 0 left, 1 right, 2 up, 3 down, 4 up-left, 5 up-right,
 * 6 down-left, 7 down-right.  arrays: NULL (constant penalty) or 8 W*H
 * arrays in that order (the reference's up/down/left/right/upleft/upright/
 * downleft/downright arguments). */
int or8_solve(int W, int H, const int32_t *dp, const int32_t *dn, int penalty, const int32_t *const *arrays,
              uint8_t *smin, uint8_t *smax, int64_t *flow, int32_t *excess_out);

/* The reference's kernel-density data term (DataTerm.cpp:97-137,
 * DataTermKernels.cu:19-31, 61-83, 116-161).  The class density at colour c
 * is, summed in float in selection order (one selectOnMap launch after the
 * other, each adding one term per colour-cube point),
 *   p(c) = sum_k gauss[floor(sqrt(|c - s_k|^2))]  over |c - s_k|^2 < 101^2,
 * where s_k are the colours of the selected pixels; t-links are
 *   pos = (int)(300000.0 * p),  neg = (int)(300000.0 * (1.0f - p)).
 * gauss: the 101-entry table (input); sel: n_sel colours (3 bytes each, in
 * order); img: n pixels (3 bytes each); pos/neg: n int32 outputs. */
void or_kde_terms(const float *gauss, const uint8_t *sel, int n_sel, const uint8_t *img, int n,
                  int32_t *pos, int32_t *neg);
/* The reference's Gaussian table for a sigma (K_InitGaussian), in double
 * precision rounded to float (the reference's expf may differ by an ulp). */
void or_kde_gauss(int sigma, float *gauss);
/* The colours selectOnMap(x, y) adds, in the reference's order (x offset
 * outer, y offset inner, DataTerm.cpp:111-123), clipped to the image.
 * Returns the number written (<= 25) to sel (3 bytes each). */
int or_kde_select(const uint8_t *img, int W, int H, int x, int y, uint8_t *sel);

/* Batch of independent solves over `nthreads` host threads (one image per
 * task), for the CPU baseline. Arrays are concatenated; offs[i] is the pixel
 * offset of image i.  Returns 0 on success. */
int or_segment_batch(int n_img, const int *Ws, const int *Hs, const int64_t *offs,
                     const uint8_t *rgb, const uint8_t *scrib, const double *lambdas,
                     int solver, int nthreads, uint8_t *smin, uint8_t *smax,
                     int64_t *flows);

#ifdef __cplusplus
}
#endif
#endif
