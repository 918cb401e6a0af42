/*
 * synth.c -- deterministic synthetic segmentation inputs (images + scribbles)
 * for the benchmark and the tests.
 *
 * Everything here uses only IEEE +, -, *, /, sqrt, floor and frexp (the log
 * and cosine of the Box-Muller transform are series evaluated here), and is
 * compiled with -ffp-contract=off, so an image is byte-identical on x86-64
 * and aarch64 hosts.
 *
 * Workload families:
 *   cfg 0: 256x256, centred ellipse (semi-axes 80,60), fg ~ N((200,60,60),20^2),
 *          bg ~ N((60,120,200),25^2); 20x20 fg scribble at the centre and a
 *          10-pixel bg scribble strip along the border.
 *   cfg 1/4: the same plus 3 random ellipses (semi-axes U(40,200), scaled by
 *          min(W,H)/1080 below 1080 pixels), colour noise sd 30.
 *   cfg 2: 2000 discs of radius U(3,15) (disc 0 centred, radius 15), fg sd 20,
 *          bg ~ N(bg mean, 40^2) + 30 sin(2 pi x / 17).
 *   cfg 3: the cfg-0 generator with the ellipse scaled to the image size.
 */
#include "synth.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------------ */
/* Deterministic PRNG + math                                                 */
/* ------------------------------------------------------------------------ */

/* splitmix64 (Steele, Lea, Flood 2014). */
uint64_t gs_splitmix64(uint64_t *state) {
    uint64_t z = (*state += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

double gs_uniform(uint64_t *state) {
    return (double)(gs_splitmix64(state) >> 11) * (1.0 / 9007199254740992.0);
}

/* Natural log from the atanh series: log(m) = 2 * sum t^(2k+1)/(2k+1),
 * t = (m-1)/(m+1), after splitting x = m * 2^e with m in [sqrt(1/2), sqrt 2).
 * Only +,-,*,/ are used, so the result is identical on every IEEE platform. */
double gs_det_log(double x) {
    if (!(x > 0.0)) return -INFINITY;
    int e;
    double m = frexp(x, &e);            /* exact */
    if (m < 0.70710678118654752440) { m *= 2.0; e -= 1; }
    double t = (m - 1.0) / (m + 1.0);
    double t2 = t * t;
    double term = t, sum = 0.0;
    for (int k = 0; k < 14; ++k) {
        sum += term / (double)(2 * k + 1);
        term *= t2;
    }
    return 2.0 * sum + (double)e * 0.69314718055994530942;
}

/* Cosine from its Taylor series after reducing to [-pi, pi]. */
double gs_det_cos(double x) {
    const double two_pi = 6.28318530717958647692;
    double k = floor(x / two_pi + 0.5);
    double y = x - k * two_pi;
    double y2 = y * y;
    double term = 1.0, sum = 0.0;
    for (int i = 0; i < 22; ++i) {
        sum += term;
        term *= -y2 / (double)((2 * i + 1) * (2 * i + 2));
    }
    return sum;
}

/* Box-Muller, cosine branch only (one uniform pair per normal). */
double gs_normal(uint64_t *state) {
    double u1 = 1.0 - gs_uniform(state); /* (0,1] */
    double u2 = gs_uniform(state);
    return sqrt(-2.0 * gs_det_log(u1)) * gs_det_cos(6.28318530717958647692 * u2);
}

static inline uint8_t quant_u8(double v) {
    if (v < 0.0) v = 0.0;
    if (v > 255.0) v = 255.0;
    return (uint8_t)(int)floor(v + 0.5);
}

/* ------------------------------------------------------------------------ */
/* Synthetic images                                                          */
/* ------------------------------------------------------------------------ */

static const double FG_MEAN[3] = {200.0, 60.0, 60.0};
static const double BG_MEAN[3] = {60.0, 120.0, 200.0};

void gs_gen_defaults(int cfg, int W, int H, uint64_t seed, gs_params *p) {
    memset(p, 0, sizeof(*p));
    p->W = W;
    p->H = H;
    p->seed = seed;
    p->ax = 80.0;
    p->ay = 60.0;
    p->sd_fg = 20.0;
    p->sd_bg = 25.0;
    p->stripe_period = 17.0;
    switch (cfg) {
    case 1: /* 1920x1080 family: 3 extra ellipses, colour noise sd 30 */
    case 4: {
        double s = (double)(W < H ? W : H) / 1080.0;
        if (s > 1.0) s = 1.0;
        p->n_extra = 3;
        p->extra_lo = 40.0 * s;
        p->extra_hi = 200.0 * s;
        p->sd_fg = 30.0;
        p->sd_bg = 30.0;
        break;
    }
    case 2: /* blobs on a striped background */
        p->family = 1;
        p->n_blobs = 2000;
        p->r_lo = 3.0;
        p->r_hi = 15.0;
        p->sd_fg = 20.0;
        p->sd_bg = 40.0;
        p->stripe_amp = 30.0;
        break;
    case 3: /* config-0 generator, ellipse scaled with the image */
        p->ax = 80.0 * (double)W / 256.0;
        p->ay = 60.0 * (double)H / 256.0;
        break;
    default: /* 0 */
        break;
    }
}

static void scribbles(int W, int H, uint8_t *scrib) {
    int fx0 = W / 2 - 10, fy0 = H / 2 - 10;
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            uint8_t s = 0;
            if (x < 10 || x >= W - 10 || y < 10 || y >= H - 10) s = 2;
            if (x >= fx0 && x < fx0 + 20 && y >= fy0 && y < fy0 + 20) s = 1;
            scrib[(int64_t)y * W + x] = s;
        }
}

int gs_generate(const gs_params *p, uint8_t *rgb, uint8_t *scrib) {
    const int W = p->W, H = p->H;
    if (W <= 0 || H <= 0) return -1;
    uint64_t st = p->seed;
    const int64_t n = (int64_t)W * H;
    uint8_t *fg = (uint8_t *)calloc((size_t)n, 1);
    if (!fg) return -2;
    const double cx0 = (double)(W / 2), cy0 = (double)(H / 2);
    if (p->family == 0) {
        double ex[64][4];
        int ne = p->n_extra > 64 ? 64 : p->n_extra;
        for (int k = 0; k < ne; ++k) {
            ex[k][0] = gs_uniform(&st) * W;
            ex[k][1] = gs_uniform(&st) * H;
            ex[k][2] = p->extra_lo + gs_uniform(&st) * (p->extra_hi - p->extra_lo);
            ex[k][3] = p->extra_lo + gs_uniform(&st) * (p->extra_hi - p->extra_lo);
        }
        for (int y = 0; y < H; ++y)
            for (int x = 0; x < W; ++x) {
                double dx = ((double)x - cx0) / p->ax, dy = ((double)y - cy0) / p->ay;
                int in = dx * dx + dy * dy <= 1.0;
                for (int k = 0; k < ne && !in; ++k) {
                    double ux = ((double)x - ex[k][0]) / ex[k][2];
                    double uy = ((double)y - ex[k][1]) / ex[k][3];
                    in = ux * ux + uy * uy <= 1.0;
                }
                fg[(int64_t)y * W + x] = (uint8_t)in;
            }
    } else {
        for (int b = 0; b < p->n_blobs; ++b) {
            double bx, by, r;
            if (b == 0) {
                bx = cx0; by = cy0; r = p->r_hi;
            } else {
                bx = gs_uniform(&st) * W;
                by = gs_uniform(&st) * H;
                r = p->r_lo + gs_uniform(&st) * (p->r_hi - p->r_lo);
            }
            int x0 = (int)floor(bx - r), x1 = (int)ceil(bx + r);
            int y0 = (int)floor(by - r), y1 = (int)ceil(by + r);
            if (x0 < 0) x0 = 0;
            if (y0 < 0) y0 = 0;
            if (x1 > W - 1) x1 = W - 1;
            if (y1 > H - 1) y1 = H - 1;
            for (int y = y0; y <= y1; ++y)
                for (int x = x0; x <= x1; ++x) {
                    double dx = (double)x - bx, dy = (double)y - by;
                    if (dx * dx + dy * dy <= r * r) fg[(int64_t)y * W + x] = 1;
                }
        }
    }
    double *stripe = (double *)calloc((size_t)W, sizeof(double));
    if (!stripe) { free(fg); return -2; }
    if (p->stripe_amp != 0.0)
        for (int x = 0; x < W; ++x)
            stripe[x] = p->stripe_amp *
                        gs_det_cos(6.28318530717958647692 * (double)x / p->stripe_period -
                                   1.57079632679489661923);
    for (int64_t i = 0; i < n; ++i) {
        int x = (int)(i % W);
        const double *mean = fg[i] ? FG_MEAN : BG_MEAN;
        double sd = fg[i] ? p->sd_fg : p->sd_bg;
        double add = fg[i] ? 0.0 : stripe[x];
        for (int c = 0; c < 3; ++c) rgb[3 * i + c] = quant_u8(mean[c] + sd * gs_normal(&st) + add);
    }
    free(stripe);
    free(fg);
    if (scrib) scribbles(W, H, scrib);
    return 0;
}


/* ---- many images over host threads (one image per task) ---- */
typedef struct {
    int n;
    const gs_params *params;
    const int64_t *offs;
    uint8_t *rgb, *scrib;
    int next, err;
    pthread_mutex_t mu;
} gen_ctx;

static void *gen_worker(void *arg) {
    gen_ctx *c = (gen_ctx *)arg;
    for (;;) {
        pthread_mutex_lock(&c->mu);
        int k = c->next++;
        pthread_mutex_unlock(&c->mu);
        if (k >= c->n) break;
        int rc = gs_generate(&c->params[k], c->rgb + 3 * c->offs[k], c->scrib + c->offs[k]);
        if (rc) c->err = rc;
    }
    return NULL;
}

int gs_generate_batch(int n, const gs_params *params, const int64_t *offs, uint8_t *rgb,
                      uint8_t *scrib, int nthreads) {
    gen_ctx c;
    memset(&c, 0, sizeof(c));
    c.n = n; c.params = params; c.offs = offs; c.rgb = rgb; c.scrib = scrib;
    pthread_mutex_init(&c.mu, NULL);
    if (nthreads < 1) nthreads = 1;
    if (nthreads > 256) nthreads = 256;
    pthread_t th[256];
    for (int t = 0; t < nthreads; ++t) pthread_create(&th[t], NULL, gen_worker, &c);
    for (int t = 0; t < nthreads; ++t) pthread_join(th[t], NULL);
    pthread_mutex_destroy(&c.mu);
    return c.err;
}

uint64_t gs_fnv1a(const void *data, int64_t n) {
    const uint8_t *p = (const uint8_t *)data;
    uint64_t h = 1469598103934665603ULL;
    for (int64_t i = 0; i < n; ++i) {
        h ^= p[i];
        h *= 1099511628211ULL;
    }
    return h;
}
