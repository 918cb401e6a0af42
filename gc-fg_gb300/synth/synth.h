/* synth.h -- deterministic synthetic inputs for the graph-cut workloads. */
#ifndef GCFG_SYNTH_H
#define GCFG_SYNTH_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

uint64_t gs_splitmix64(uint64_t *state);
double gs_uniform(uint64_t *state);
double gs_normal(uint64_t *state);
double gs_det_log(double x);
double gs_det_cos(double x);

/* family 0: "ellipse" (central ellipse + n_extra random ellipses);
 * family 1: "blobs" (n_blobs discs on a striped, noisy background). */
typedef struct {
    int family;
    int W, H;
    uint64_t seed;
    double ax, ay;
    int n_extra;
    double extra_lo, extra_hi;
    int n_blobs;
    double r_lo, r_hi;
    double sd_fg, sd_bg;
    double stripe_amp;
    double stripe_period;
} gs_params;

void gs_gen_defaults(int cfg, int W, int H, uint64_t seed, gs_params *p);
/* rgb: 3*W*H bytes interleaved; scrib: W*H bytes (0 none, 1 fg, 2 bg). */
int gs_generate(const gs_params *p, uint8_t *rgb, uint8_t *scrib);
/* n images packed back to back (pixel offsets offs[i]) over host threads. */
int gs_generate_batch(int n, const gs_params *params, const int64_t *offs, uint8_t *rgb,
                      uint8_t *scrib, int nthreads);
uint64_t gs_fnv1a(const void *data, int64_t n);

#ifdef __cplusplus
}
#endif
#endif
