/*
 * oracle.c -- CPU oracle for the gc-fg binary-MRF graph-cut path.
 *
 * TEST INFRASTRUCTURE ONLY: used by tests/, __graft_entry__.smoke() and the
 * cpu_baseline leg of bench.py to check and time against; never by the
 * product library.
 *
 * Compile with -ffp-contract=off so that the double arithmetic below is the
 * plain IEEE evaluation on every host.
 */
#include "oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------------ */
/* Data term                                                                 */
/* ------------------------------------------------------------------------ */

static inline int color_bin(const uint8_t *c) {
    return ((c[0] >> 4) << 8) | ((c[1] >> 4) << 4) | (c[2] >> 4);
}

void or_histograms(const uint8_t *rgb, const uint8_t *scrib, int n, int32_t *hf, int32_t *hb) {
    memset(hf, 0, 4096 * sizeof(int32_t));
    memset(hb, 0, 4096 * sizeof(int32_t));
    for (int i = 0; i < n; ++i) {
        if (scrib[i] == 1) hf[color_bin(rgb + 3 * (int64_t)i)]++;
        else if (scrib[i] == 2) hb[color_bin(rgb + 3 * (int64_t)i)]++;
    }
}

/* dp (source / foreground link) = round(10 * -log p_bg(bin)),
 * dn (sink / background link)   = round(10 * -log p_fg(bin)),
 * p_k(bin) = (H_k[bin] + 1) / (N_k + 4096). */
void or_tlink_lut(const int32_t *hf, const int32_t *hb, double *raw_dp, double *raw_dn,
                  int32_t *dp_lut, int32_t *dn_lut) {
    int64_t nf = 0, nb = 0;
    for (int b = 0; b < 4096; ++b) { nf += hf[b]; nb += hb[b]; }
    for (int b = 0; b < 4096; ++b) {
        double pf = (double)(hf[b] + 1) / (double)(nf + 4096);
        double pb = (double)(hb[b] + 1) / (double)(nb + 4096);
        double rdn = 10.0 * -log(pf);
        double rdp = 10.0 * -log(pb);
        if (raw_dp) raw_dp[b] = rdp;
        if (raw_dn) raw_dn[b] = rdn;
        dp_lut[b] = (int32_t)round(rdp);
        dn_lut[b] = (int32_t)round(rdn);
    }
}

void or_tlinks(const uint8_t *rgb, int n, const int32_t *dp_lut, const int32_t *dn_lut,
               int32_t *dp, int32_t *dn) {
    for (int i = 0; i < n; ++i) {
        int b = color_bin(rgb + 3 * (int64_t)i);
        dp[i] = dp_lut[b];
        dn[i] = dn_lut[b];
    }
}

/* ------------------------------------------------------------------------ */
/* N-links                                                                   */
/* ------------------------------------------------------------------------ */

static inline int diff2(const uint8_t *a, const uint8_t *b) {
    int d0 = (int)a[0] - b[0], d1 = (int)a[1] - b[1], d2 = (int)a[2] - b[2];
    return d0 * d0 + d1 * d1 + d2 * d2;
}

void or_sigma_sum(const uint8_t *rgb, int W, int H, int64_t *sum, int64_t *count) {
    int64_t s = 0;
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            const uint8_t *p = rgb + 3 * ((int64_t)y * W + x);
            if (x + 1 < W) s += diff2(p, p + 3);
            if (y + 1 < H) s += diff2(p, p + 3 * (int64_t)W);
        }
    *sum = s;
    *count = (int64_t)(W - 1) * H + (int64_t)W * (H - 1);
}

/* w(d2) = lambda * exp(-d2 / (2 sigma^2)), sigma^2 = sum / count; a constant
 * image (sum == 0) gives w = lambda. */
double or_nlink_weight_raw(int d2, double lambda, int64_t sum, int64_t count) {
    if (sum == 0 || count == 0) return lambda;
    double s2 = (double)sum / (double)count;
    double a = -(double)d2 / (2.0 * s2);
    return lambda * exp(a);
}

void or_nlinks(const uint8_t *rgb, int W, int H, double lambda, int32_t *up, int32_t *down,
               int32_t *left, int32_t *right) {
    int64_t sum, count;
    or_sigma_sum(rgb, W, H, &sum, &count);
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            int64_t i = (int64_t)y * W + x;
            const uint8_t *p = rgb + 3 * i;
            right[i] = x + 1 < W ? (int32_t)round(or_nlink_weight_raw(diff2(p, p + 3), lambda, sum, count)) : 0;
            left[i] = x > 0 ? (int32_t)round(or_nlink_weight_raw(diff2(p, p - 3), lambda, sum, count)) : 0;
            down[i] = y + 1 < H ? (int32_t)round(or_nlink_weight_raw(diff2(p, p + 3 * (int64_t)W), lambda, sum, count)) : 0;
            up[i] = y > 0 ? (int32_t)round(or_nlink_weight_raw(diff2(p, p - 3 * (int64_t)W), lambda, sum, count)) : 0;
        }
}

/* ------------------------------------------------------------------------ */
/* Graph construction in the reference's conventions                        */
/* ------------------------------------------------------------------------ */

enum { DL = 0, DR = 1, DU = 2, DD = 3 };

/* Follows InitGraph / InitGraphVarEdges (GraphCutKernels.cu:112-214):
 * only x in [1,W-2], y in [1,H-2] are nodes; their excess is dp - dn; their
 * caps come from the arrays (or the constant penalty); the cap of every edge
 * that points into the border ring is zeroed (:143-146, :200-203). */
void or_build(int W, int H, const int32_t *dp, const int32_t *dn, int penalty,
              const int32_t *up, const int32_t *down, const int32_t *left,
              const int32_t *right, int32_t *caps, int32_t *excess) {
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            int64_t i = (int64_t)y * W + x;
            int32_t *c = caps + 4 * i;
            int inside = x > 0 && y > 0 && x < W - 1 && y < H - 1;
            if (!inside) {
                c[0] = c[1] = c[2] = c[3] = 0;
                excess[i] = 0;
                continue;
            }
            if (up) {
                c[DL] = left[i]; c[DR] = right[i]; c[DU] = up[i]; c[DD] = down[i];
            } else {
                c[DL] = c[DR] = c[DU] = c[DD] = penalty;
            }
            if (x == 1) c[DL] = 0;
            if (x == W - 2) c[DR] = 0;
            if (y == 1) c[DU] = 0;
            if (y == H - 2) c[DD] = 0;
            excess[i] = dp[i] - dn[i];
        }
}

static inline int64_t nbr(int64_t i, int d, int W) {
    switch (d) {
    case DL: return i - 1;
    case DR: return i + 1;
    case DU: return i - W;
    default: return i + W;
    }
}

/* ------------------------------------------------------------------------ */
/* Push-relabel (sequential restatement of the reference's solver)           */
/* ------------------------------------------------------------------------ */

/* Global relabel as in InitGlobalRelabel/GlobalRelabel
 * (GraphCutKernels.cu:757-875): sink-connected nodes (excess < 0) get height
 * 1, every other node gets its residual BFS distance to them, unreachable
 * nodes get INF.  Done here as an exact BFS. */
static void pr_global_relabel(int W, int H, const int32_t *caps, const int32_t *excess,
                              int32_t *h, int32_t INF, int64_t *queue) {
    int64_t n = (int64_t)W * H, qh = 0, qt = 0;
    for (int64_t i = 0; i < n; ++i) {
        h[i] = INF;
        if (excess[i] < 0) { h[i] = 1; queue[qt++] = i; }
    }
    while (qh < qt) {
        int64_t v = queue[qh++];
        int x = (int)(v % W), y = (int)(v / W);
        for (int d = 0; d < 4; ++d) {
            if ((d == DL && x == 0) || (d == DR && x == W - 1) || (d == DU && y == 0) || (d == DD && y == H - 1))
                continue;
            int64_t u = nbr(v, d, W);
            /* u -> v is u's edge in direction opposite to d */
            if (h[u] == INF && caps[4 * u + (d ^ 1)] > 0) {
                h[u] = h[v] + 1;
                queue[qt++] = u;
            }
        }
    }
}

int or_maxflow_pr(int W, int H, int32_t *caps, int32_t *excess, or_stats *st) {
    int64_t n = (int64_t)W * H;
    const int32_t INF = (int32_t)(n + 1);
    int32_t *h = (int32_t *)malloc((size_t)n * sizeof(int32_t));
    int64_t *queue = (int64_t *)malloc((size_t)(n + 1) * sizeof(int64_t));
    int64_t *fifo = (int64_t *)malloc((size_t)(n + 1) * sizeof(int64_t));
    uint8_t *inq = (uint8_t *)calloc((size_t)n, 1);
    if (!h || !queue || !fifo || !inq) {
        free(h); free(queue); free(fifo); free(inq);
        return -2;
    }
    or_stats s = {0};
    int64_t work_since_gr = 0;
    int64_t fh = 0, fcount = 0, cap_q = n + 1;

#define FIFO_PUSH(v) do { fifo[(fh + fcount) % cap_q] = (v); fcount++; inq[v] = 1; } while (0)

    pr_global_relabel(W, H, caps, excess, h, INF, queue);
    s.global_relabels++;
    for (int64_t i = 0; i < n; ++i)
        if (excess[i] > 0 && h[i] < INF) FIFO_PUSH(i);

    while (fcount > 0) {
        int64_t u = fifo[fh];
        fh = (fh + 1) % cap_q;
        fcount--;
        inq[u] = 0;
        int x = (int)(u % W), y = (int)(u / W);
        while (excess[u] > 0 && h[u] < INF) {
            int pushed_any = 0;
            for (int d = 0; d < 4 && excess[u] > 0; ++d) {
                int32_t r = caps[4 * u + d];
                if (r <= 0) continue;
                int64_t v = nbr(u, d, W);
                if (h[u] != h[v] + 1) continue;
                int32_t f = excess[u] < r ? excess[u] : r;
                caps[4 * u + d] -= f;
                caps[4 * v + (d ^ 1)] += f;
                excess[u] -= f;
                int32_t ev = excess[v];
                excess[v] += f;
                s.pushes++;
                pushed_any = 1;
                if (ev <= 0 && excess[v] > 0 && !inq[v] && h[v] < INF) FIFO_PUSH(v);
            }
            if (excess[u] <= 0) break;
            (void)pushed_any;
            /* relabel (Relabel kernel, GraphCutKernels.cu:667-689) */
            int32_t m = INF;
            for (int d = 0; d < 4; ++d) {
                if (caps[4 * u + d] <= 0) continue;
                int64_t v = nbr(u, d, W);
                if (h[v] < m) m = h[v];
            }
            h[u] = m >= INF - 1 ? INF : m + 1;
            s.relabels++;
            work_since_gr += 12;
            (void)x; (void)y;
        }
        if (work_since_gr > 6 * n + 64 && fcount > 0) {
            pr_global_relabel(W, H, caps, excess, h, INF, queue);
            s.global_relabels++;
            work_since_gr = 0;
            fh = 0;
            fcount = 0;
            memset(inq, 0, (size_t)n);
            for (int64_t i = 0; i < n; ++i)
                if (excess[i] > 0 && h[i] < INF) FIFO_PUSH(i);
        }
    }
#undef FIFO_PUSH
    /* Exactness check: no positive excess may still reach the sink. */
    pr_global_relabel(W, H, caps, excess, h, INF, queue);
    int ok = 1;
    for (int64_t i = 0; i < n; ++i)
        if (excess[i] > 0 && h[i] < INF) { ok = 0; break; }
    free(h); free(queue); free(fifo); free(inq);
    if (st) *st = s;
    return ok ? 0 : -3;
}

/* ------------------------------------------------------------------------ */
/* Boykov-Kolmogorov augmenting paths (written from Boykov & Kolmogorov,     */
/* "An Experimental Comparison of Min-Cut/Max-Flow Algorithms for Energy     */
/* Minimization in Vision", PAMI 2004).                                      */
/* ------------------------------------------------------------------------ */

enum { P_NONE = -1, P_TERM = 4, P_ORPHAN = 5 };
enum { T_FREE = 0, T_S = 1, T_T = 2 };

typedef struct {
    int W, H;
    int64_t n;
    int32_t *caps, *tr;
    int8_t *tree, *par;
    int32_t *ts, *dist;
    int64_t *active; /* ring buffer */
    uint8_t *inact;
    int64_t ah, acount;
    int64_t *orph; /* FIFO of orphans */
    int64_t oh, ocount;
    int32_t time;
} bk_t;

static inline int bk_has_nbr(const bk_t *b, int64_t i, int d) {
    int x = (int)(i % b->W), y = (int)(i / b->W);
    return !((d == DL && x == 0) || (d == DR && x == b->W - 1) || (d == DU && y == 0) || (d == DD && y == b->H - 1));
}

static inline void bk_activate(bk_t *b, int64_t i) {
    if (b->inact[i]) return;
    b->inact[i] = 1;
    b->active[(b->ah + b->acount) % b->n] = i;
    b->acount++;
}

static inline void bk_orphan(bk_t *b, int64_t i) {
    b->par[i] = P_ORPHAN;
    b->orph[(b->oh + b->ocount) % b->n] = i;
    b->ocount++;
}

static void bk_augment(bk_t *b, int64_t a, int64_t t, int dab, int64_t *flow) {
    int32_t *caps = b->caps;
    int32_t delta = caps[4 * a + dab];
    int64_t x = a;
    while (b->par[x] != P_TERM) {
        int pd = b->par[x];
        int64_t y = nbr(x, pd, b->W);
        int32_t c = caps[4 * y + (pd ^ 1)];
        if (c < delta) delta = c;
        x = y;
    }
    if (b->tr[x] < delta) delta = b->tr[x];
    x = t;
    while (b->par[x] != P_TERM) {
        int pd = b->par[x];
        int32_t c = caps[4 * x + pd];
        if (c < delta) delta = c;
        x = nbr(x, pd, b->W);
    }
    if (-b->tr[x] < delta) delta = -b->tr[x];

    caps[4 * a + dab] -= delta;
    caps[4 * t + (dab ^ 1)] += delta;
    x = a;
    while (b->par[x] != P_TERM) {
        int pd = b->par[x];
        int64_t y = nbr(x, pd, b->W);
        caps[4 * y + (pd ^ 1)] -= delta;
        caps[4 * x + pd] += delta;
        if (caps[4 * y + (pd ^ 1)] == 0) bk_orphan(b, x);
        x = y;
    }
    b->tr[x] -= delta;
    if (b->tr[x] == 0) bk_orphan(b, x);
    x = t;
    while (b->par[x] != P_TERM) {
        int pd = b->par[x];
        int64_t y = nbr(x, pd, b->W);
        caps[4 * x + pd] -= delta;
        caps[4 * y + (pd ^ 1)] += delta;
        if (caps[4 * x + pd] == 0) bk_orphan(b, x);
        x = y;
    }
    b->tr[x] += delta;
    if (b->tr[x] == 0) bk_orphan(b, x);
    *flow += delta;
}

/* Distance of a tree node to its terminal, or -1 if its chain hits an
 * orphan; marks the chain with the current timestamp. */
static int32_t bk_origin_dist(bk_t *b, int64_t q) {
    int32_t d = 0;
    int64_t j = q;
    for (;;) {
        if (b->ts[j] == b->time) { d += b->dist[j]; break; }
        d++;
        if (b->par[j] == P_TERM) {
            b->ts[j] = b->time;
            b->dist[j] = 1;
            break;
        }
        if (b->par[j] == P_ORPHAN || b->par[j] == P_NONE) return -1;
        j = nbr(j, b->par[j], b->W);
    }
    int32_t dd = d;
    for (j = q; b->ts[j] != b->time; j = nbr(j, b->par[j], b->W)) {
        b->ts[j] = b->time;
        b->dist[j] = dd--;
    }
    return d;
}

static void bk_adopt(bk_t *b, int64_t p) {
    int tree = b->tree[p];
    int best = -1;
    int32_t best_d = 0x7fffffff;
    for (int d = 0; d < 4; ++d) {
        if (!bk_has_nbr(b, p, d)) continue;
        int64_t q = nbr(p, d, b->W);
        if (b->tree[q] != tree) continue;
        int32_t c = tree == T_S ? b->caps[4 * q + (d ^ 1)] : b->caps[4 * p + d];
        if (c <= 0) continue;
        int32_t od = bk_origin_dist(b, q);
        if (od >= 0 && od < best_d) { best_d = od; best = d; }
    }
    if (best >= 0) {
        b->par[p] = (int8_t)best;
        b->ts[p] = b->time;
        b->dist[p] = best_d + 1;
        return;
    }
    /* no parent: p becomes free; its tree neighbours may reclaim it */
    for (int d = 0; d < 4; ++d) {
        if (!bk_has_nbr(b, p, d)) continue;
        int64_t q = nbr(p, d, b->W);
        if (b->tree[q] != tree) continue;
        int32_t c = tree == T_S ? b->caps[4 * q + (d ^ 1)] : b->caps[4 * p + d];
        if (c > 0) bk_activate(b, q);
        if (b->par[q] >= 0 && b->par[q] < 4 && nbr(q, b->par[q], b->W) == p) bk_orphan(b, q);
    }
    b->tree[p] = T_FREE;
    b->par[p] = P_NONE;
}

int or_maxflow_bk(int W, int H, int32_t *caps, int32_t *excess, or_stats *st) {
    bk_t b;
    memset(&b, 0, sizeof(b));
    b.W = W;
    b.H = H;
    b.n = (int64_t)W * H;
    b.caps = caps;
    b.tr = excess;
    b.tree = (int8_t *)calloc((size_t)b.n, 1);
    b.par = (int8_t *)malloc((size_t)b.n);
    b.ts = (int32_t *)calloc((size_t)b.n, sizeof(int32_t));
    b.dist = (int32_t *)calloc((size_t)b.n, sizeof(int32_t));
    b.active = (int64_t *)malloc((size_t)b.n * sizeof(int64_t));
    b.inact = (uint8_t *)calloc((size_t)b.n, 1);
    b.orph = (int64_t *)malloc((size_t)b.n * sizeof(int64_t));
    if (!b.tree || !b.par || !b.ts || !b.dist || !b.active || !b.inact || !b.orph) {
        free(b.tree); free(b.par); free(b.ts); free(b.dist); free(b.active); free(b.inact); free(b.orph);
        return -2;
    }
    memset(b.par, P_NONE, (size_t)b.n);
    or_stats s = {0};
    int64_t flow = 0;
    for (int64_t i = 0; i < b.n; ++i) {
        if (excess[i] > 0) { b.tree[i] = T_S; b.par[i] = P_TERM; b.dist[i] = 1; bk_activate(&b, i); }
        else if (excess[i] < 0) { b.tree[i] = T_T; b.par[i] = P_TERM; b.dist[i] = 1; bk_activate(&b, i); }
    }
    b.time = 0;
    int64_t cur = -1;
    for (;;) {
        if (cur < 0) {
            while (b.acount > 0) {
                int64_t i = b.active[b.ah];
                b.ah = (b.ah + 1) % b.n;
                b.acount--;
                b.inact[i] = 0;
                if (b.tree[i] != T_FREE) { cur = i; break; }
            }
            if (cur < 0) break;
        }
        int64_t p = cur;
        int64_t ea = -1, et = -1;
        int edir = -1;
        for (int d = 0; d < 4; ++d) {
            if (!bk_has_nbr(&b, p, d)) continue;
            int64_t q = nbr(p, d, W);
            if (b.tree[p] == T_S) {
                if (caps[4 * p + d] <= 0) continue;
                if (b.tree[q] == T_FREE) {
                    b.tree[q] = T_S; b.par[q] = (int8_t)(d ^ 1);
                    b.ts[q] = b.ts[p]; b.dist[q] = b.dist[p] + 1;
                    bk_activate(&b, q);
                } else if (b.tree[q] == T_T) {
                    ea = p; et = q; edir = d;
                    break;
                } else if (b.ts[q] <= b.ts[p] && b.dist[q] > b.dist[p]) {
                    b.par[q] = (int8_t)(d ^ 1);
                    b.ts[q] = b.ts[p]; b.dist[q] = b.dist[p] + 1;
                }
            } else {
                if (caps[4 * q + (d ^ 1)] <= 0) continue;
                if (b.tree[q] == T_FREE) {
                    b.tree[q] = T_T; b.par[q] = (int8_t)(d ^ 1);
                    b.ts[q] = b.ts[p]; b.dist[q] = b.dist[p] + 1;
                    bk_activate(&b, q);
                } else if (b.tree[q] == T_S) {
                    ea = q; et = p; edir = d ^ 1;
                    break;
                } else if (b.ts[q] <= b.ts[p] && b.dist[q] > b.dist[p]) {
                    b.par[q] = (int8_t)(d ^ 1);
                    b.ts[q] = b.ts[p]; b.dist[q] = b.dist[p] + 1;
                }
            }
        }
        b.time++;
        if (edir >= 0) {
            bk_augment(&b, ea, et, edir, &flow);
            s.augments++;
            while (b.ocount > 0) {
                int64_t o = b.orph[b.oh];
                b.oh = (b.oh + 1) % b.n;
                b.ocount--;
                if (b.par[o] == P_ORPHAN) bk_adopt(&b, o);
            }
            if (b.tree[p] == T_FREE) cur = -1;
        } else {
            cur = -1;
        }
    }
    free(b.tree); free(b.par); free(b.ts); free(b.dist); free(b.active); free(b.inact); free(b.orph);
    if (st) *st = s;
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Cuts                                                                      */
/* ------------------------------------------------------------------------ */

/* smax: complement of the sink-reachable set (InitLabels + SpreadLabels,
 * GraphCutKernels.cu:228-351, with SPREAD_ZEROS, GraphCut.h:37);
 * smin: nodes reachable from positive-excess nodes along residual edges. */
void or_cuts(int W, int H, const int32_t *caps, const int32_t *excess, uint8_t *smin, uint8_t *smax) {
    int64_t n = (int64_t)W * H;
    int64_t *queue = (int64_t *)malloc((size_t)(n + 1) * sizeof(int64_t));
    uint8_t *mark = (uint8_t *)calloc((size_t)n, 1);
    int64_t qh = 0, qt = 0;
    for (int64_t i = 0; i < n; ++i)
        if (excess[i] < 0) { mark[i] = 1; queue[qt++] = i; }
    while (qh < qt) {
        int64_t v = queue[qh++];
        int x = (int)(v % W), y = (int)(v / W);
        for (int d = 0; d < 4; ++d) {
            if ((d == DL && x == 0) || (d == DR && x == W - 1) || (d == DU && y == 0) || (d == DD && y == H - 1))
                continue;
            int64_t u = nbr(v, d, W);
            if (!mark[u] && caps[4 * u + (d ^ 1)] > 0) { mark[u] = 1; queue[qt++] = u; }
        }
    }
    for (int64_t i = 0; i < n; ++i) {
        int x = (int)(i % W), y = (int)(i / W);
        int inside = x > 0 && y > 0 && x < W - 1 && y < H - 1;
        smax[i] = (uint8_t)(inside && !mark[i]);
    }
    memset(mark, 0, (size_t)n);
    qh = qt = 0;
    for (int64_t i = 0; i < n; ++i)
        if (excess[i] > 0) { mark[i] = 1; queue[qt++] = i; }
    while (qh < qt) {
        int64_t u = queue[qh++];
        int x = (int)(u % W), y = (int)(u / W);
        for (int d = 0; d < 4; ++d) {
            if ((d == DL && x == 0) || (d == DR && x == W - 1) || (d == DU && y == 0) || (d == DD && y == H - 1))
                continue;
            int64_t v = nbr(u, d, W);
            if (!mark[v] && caps[4 * u + d] > 0) { mark[v] = 1; queue[qt++] = v; }
        }
    }
    for (int64_t i = 0; i < n; ++i) smin[i] = mark[i];
    free(queue);
    free(mark);
}

int64_t or_cut_energy(int W, int H, const int32_t *dp, const int32_t *dn, int penalty,
                      const int32_t *up, const int32_t *down, const int32_t *left,
                      const int32_t *right, const uint8_t *label) {
    int64_t n = (int64_t)W * H;
    int32_t *caps = (int32_t *)malloc((size_t)(4 * n) * sizeof(int32_t));
    int32_t *ex = (int32_t *)malloc((size_t)n * sizeof(int32_t));
    or_build(W, H, dp, dn, penalty, up, down, left, right, caps, ex);
    int64_t e = 0;
    for (int y = 1; y < H - 1; ++y)
        for (int x = 1; x < W - 1; ++x) {
            int64_t i = (int64_t)y * W + x;
            if (label[i]) {
                e += dn[i];
                for (int d = 0; d < 4; ++d) {
                    int64_t j = nbr(i, d, W);
                    if (!label[j]) e += caps[4 * i + d];
                }
            } else {
                e += dp[i];
            }
        }
    free(caps);
    free(ex);
    return e;
}

int64_t or_interior_dp(int W, int H, const int32_t *dp) {
    int64_t s = 0;
    for (int y = 1; y < H - 1; ++y)
        for (int x = 1; x < W - 1; ++x) s += dp[(int64_t)y * W + x];
    return s;
}

int32_t or_reference_energy(int W, int H, const int32_t *dp, const int32_t *excess_final) {
    int wex = 32 * ((W + 31) / 32);
    int64_t size = (int64_t)W * H;
    uint32_t init = 0, fin = 0;
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            int64_t t = (int64_t)x + (int64_t)y * wex; /* padded position */
            int32_t v = dp[(int64_t)y * W + x];
            if (t < size && v > 0) init += (uint32_t)v;
        }
    for (int64_t i = 0; i < size; ++i)
        if (excess_final[i] > 0) fin += (uint32_t)excess_final[i];
    return (int32_t)(init - fin);
}

int or_solve(int W, int H, const int32_t *dp, const int32_t *dn, int penalty,
             const int32_t *up, const int32_t *down, const int32_t *left,
             const int32_t *right, int solver, uint8_t *smin, uint8_t *smax,
             int64_t *flow, int32_t *excess_out, or_stats *st) {
    int64_t n = (int64_t)W * H;
    int32_t *caps = (int32_t *)malloc((size_t)(4 * n) * sizeof(int32_t));
    int32_t *ex = (int32_t *)malloc((size_t)n * sizeof(int32_t));
    if (!caps || !ex) { free(caps); free(ex); return -2; }
    or_build(W, H, dp, dn, penalty, up, down, left, right, caps, ex);
    or_stats s;
    int rc = solver == 1 ? or_maxflow_bk(W, H, caps, ex, &s) : or_maxflow_pr(W, H, caps, ex, &s);
    if (rc == 0) {
        int64_t pos = 0;
        for (int64_t i = 0; i < n; ++i) if (ex[i] > 0) pos += ex[i];
        s.flow = or_interior_dp(W, H, dp) - pos;
        if (flow) *flow = s.flow;
        if (smin && smax) or_cuts(W, H, caps, ex, smin, smax);
        if (excess_out) memcpy(excess_out, ex, (size_t)n * sizeof(int32_t));
        if (st) *st = s;
    }
    free(caps);
    free(ex);
    return rc;
}

int or_segment(const uint8_t *rgb, const uint8_t *scrib, int W, int H, double lambda, int solver,
               int32_t *dp, int32_t *dn, int32_t *up, int32_t *down, int32_t *left, int32_t *right,
               uint8_t *smin, uint8_t *smax, int64_t *flow) {
    int32_t hf[4096], hb[4096], dpl[4096], dnl[4096];
    int n = W * H;
    or_histograms(rgb, scrib, n, hf, hb);
    or_tlink_lut(hf, hb, NULL, NULL, dpl, dnl);
    or_tlinks(rgb, n, dpl, dnl, dp, dn);
    or_nlinks(rgb, W, H, lambda, up, down, left, right);
    return or_solve(W, H, dp, dn, 0, up, down, left, right, solver, smin, smax, flow, NULL, NULL);
}

/* ---- batch over host threads ---- */
typedef struct {
    int n_img;
    const int *Ws, *Hs;
    const int64_t *offs;
    const uint8_t *rgb, *scrib;
    const double *lambdas;
    int solver;
    uint8_t *smin, *smax;
    int64_t *flows;
    int next;
    int err;
    pthread_mutex_t mu;
} batch_ctx;

static void *batch_worker(void *arg) {
    batch_ctx *c = (batch_ctx *)arg;
    for (;;) {
        pthread_mutex_lock(&c->mu);
        int k = c->next++;
        pthread_mutex_unlock(&c->mu);
        if (k >= c->n_img) break;
        int W = c->Ws[k], H = c->Hs[k];
        int64_t off = c->offs[k], n = (int64_t)W * H;
        int32_t *buf = (int32_t *)malloc((size_t)(6 * n) * sizeof(int32_t));
        if (!buf) { c->err = -2; continue; }
        int rc = or_segment(c->rgb + 3 * off, c->scrib + off, W, H, c->lambdas[k], c->solver,
                            buf, buf + n, buf + 2 * n, buf + 3 * n, buf + 4 * n, buf + 5 * n,
                            c->smin + off, c->smax + off, c->flows + k);
        if (rc) c->err = rc;
        free(buf);
    }
    return NULL;
}

int or_segment_batch(int n_img, const int *Ws, const int *Hs, const int64_t *offs,
                     const uint8_t *rgb, const uint8_t *scrib, const double *lambdas,
                     int solver, int nthreads, uint8_t *smin, uint8_t *smax, int64_t *flows) {
    batch_ctx c;
    memset(&c, 0, sizeof(c));
    c.n_img = n_img; c.Ws = Ws; c.Hs = Hs; c.offs = offs; c.rgb = rgb; c.scrib = scrib;
    c.lambdas = lambdas; c.solver = solver; c.smin = smin; c.smax = smax; c.flows = flows;
    pthread_mutex_init(&c.mu, NULL);
    if (nthreads < 1) nthreads = 1;
    if (nthreads > 256) nthreads = 256;
    pthread_t th[256];
    for (int t = 0; t < nthreads; ++t) pthread_create(&th[t], NULL, batch_worker, &c);
    for (int t = 0; t < nthreads; ++t) pthread_join(th[t], NULL);
    pthread_mutex_destroy(&c.mu);
    return c.err;
}


/* ---------------------------------------------------------------------------
 * Kernel-density data term of the reference (DataTerm.cpp:97-137,
 * DataTermKernels.cu:19-31, 61-83, 116-161).
 * ------------------------------------------------------------------------- */

void or_kde_gauss(int sigma, float *gauss) {
    /* K_InitGaussian (DataTermKernels.cu:19-31): 1 / (sigma * 2.507) *
     * expf(-0.5 * (x / sigma)^2) with its types: x / sigma in float, the
     * exponent in double rounded to float for expf, the product in double. */
    for (int x = 0; x < 101; ++x) {
        const float xs = (float)x / (float)sigma;
        const double a = -0.5 * (double)xs * (double)xs;
        gauss[x] = (float)(1.0 / ((double)(float)sigma * 2.507) * (double)expf((float)a));
    }
}

int or_kde_select(const uint8_t *img, int W, int H, int x, int y, uint8_t *sel) {
    int k = 0;
    for (int i = 0; i < 5; ++i)
        for (int j = 0; j < 5; ++j) {
            const int px = x + i, py = y + j;
            if (px < 0 || py < 0 || px >= W || py >= H) continue;
            const uint8_t *p = img + 3 * ((size_t)py * W + px);
            sel[3 * k] = p[0];
            sel[3 * k + 1] = p[1];
            sel[3 * k + 2] = p[2];
            ++k;
        }
    return k;
}

void or_kde_terms(const float *gauss, const uint8_t *sel, int n_sel, const uint8_t *img, int n,
                  int32_t *pos, int32_t *neg) {
    for (int i = 0; i < n; ++i) {
        const uint8_t *c = img + 3 * (size_t)i;
        float p = 0.0f;
        for (int k = 0; k < n_sel; ++k) {
            const int d0 = (int)c[0] - sel[3 * k], d1 = (int)c[1] - sel[3 * k + 1], d2 = (int)c[2] - sel[3 * k + 2];
            const int d = d0 * d0 + d1 * d1 + d2 * d2;
            if (d < 101 * 101) {
                int r = (int)sqrt((double)d); /* floor(sqrt(d)), exact for d < 2^26 */
                while (r * r > d) --r;
                while ((r + 1) * (r + 1) <= d) ++r;
                p = p + gauss[r];
            }
        }
        pos[i] = (int32_t)(300000.0 * (double)p);
        neg[i] = (int32_t)(300000.0 * (double)(1.0f - p));
    }
}

/* ---------------------------------------------------------------------------
 * 8-connected graphs (the reference built with NEIGHBORHOOD == 8).
 * Directions: 0 left, 1 right, 2 up, 3 down, 4 up-left, 5 up-right,
 * 6 down-left, 7 down-right; caps8[8 * i + d] is the capacity from pixel i to
 * its neighbour in direction d.
 * ------------------------------------------------------------------------- */

static const int D8X[8] = {-1, 1, 0, 0, -1, 1, -1, 1};
static const int D8Y[8] = {0, 0, -1, 1, -1, -1, 1, 1};
static const int D8OPP[8] = {1, 0, 3, 2, 7, 6, 5, 4};

/* InitGraph / InitGraphVarEdges with NEIGHBORHOOD == 8
 * (GraphCutKernels.cu:112-214): interior nodes only; arrays[d] (or the
 * penalty) per direction; the edges of x == 1 toward the left column, of
 * x == W-2 toward the right, of y == 1 upward and of y == H-2 downward
 * (diagonals included) are zeroed. */
void or8_build(int W, int H, const int32_t *dp, const int32_t *dn, int penalty, const int32_t *const *arrays,
               int32_t *caps8, int32_t *excess) {
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            const int64_t i = (int64_t)y * W + x;
            int32_t *c = caps8 + 8 * i;
            const int inside = x > 0 && y > 0 && x < W - 1 && y < H - 1;
            for (int d = 0; d < 8; ++d) c[d] = inside ? (arrays ? arrays[d][i] : penalty) : 0;
            excess[i] = inside ? dp[i] - dn[i] : 0;
            if (!inside) continue;
            if (x == 1) c[0] = c[4] = c[6] = 0;
            if (x == W - 2) c[1] = c[5] = c[7] = 0;
            if (y == 1) c[2] = c[4] = c[5] = 0;
            if (y == H - 2) c[3] = c[6] = c[7] = 0;
        }
}

static inline int or8_nbr(int W, int H, int64_t i, int d, int64_t *j) {
    const int x = (int)(i % W) + D8X[d], y = (int)(i / W) + D8Y[d];
    if (x < 0 || y < 0 || x >= W || y >= H) return 0;
    *j = (int64_t)y * W + x;
    return 1;
}

/* exact residual BFS distance to the sink-connected nodes (excess < 0) */
static void or8_global_relabel(int W, int H, const int32_t *caps8, const int32_t *excess, int32_t *h, int32_t INF,
                               int64_t *queue) {
    const int64_t n = (int64_t)W * H;
    int64_t qh = 0, qt = 0;
    for (int64_t i = 0; i < n; ++i) {
        h[i] = INF;
        if (excess[i] < 0) { h[i] = 1; queue[qt++] = i; }
    }
    while (qh < qt) {
        const int64_t v = queue[qh++];
        for (int d = 0; d < 8; ++d) {
            int64_t u;
            if (!or8_nbr(W, H, v, d, &u)) continue;
            /* u -> v is u's edge in the direction opposite to d */
            if (h[u] == INF && caps8[8 * u + D8OPP[d]] > 0) {
                h[u] = h[v] + 1;
                queue[qt++] = u;
            }
        }
    }
}

/* FIFO push-relabel with exact global relabels (8 directions). */
int or8_maxflow(int W, int H, int32_t *caps8, int32_t *excess) {
    const int64_t n = (int64_t)W * H;
    const int32_t INF = (int32_t)(n + 1);
    int32_t *h = (int32_t *)malloc((size_t)n * sizeof(int32_t));
    int64_t *queue = (int64_t *)malloc((size_t)(n + 1) * sizeof(int64_t));
    int64_t *fifo = (int64_t *)malloc((size_t)(n + 1) * sizeof(int64_t));
    uint8_t *inq = (uint8_t *)calloc((size_t)n, 1);
    if (!h || !queue || !fifo || !inq) {
        free(h); free(queue); free(fifo); free(inq);
        return -2;
    }
    int64_t fh = 0, fcount = 0, cap_q = n + 1, work = 0;
#define FIFO8_PUSH(v) do { fifo[(fh + fcount) % cap_q] = (v); fcount++; inq[v] = 1; } while (0)
    or8_global_relabel(W, H, caps8, excess, h, INF, queue);
    for (int64_t i = 0; i < n; ++i)
        if (excess[i] > 0 && h[i] < INF) FIFO8_PUSH(i);
    while (fcount > 0) {
        const int64_t u = fifo[fh];
        fh = (fh + 1) % cap_q;
        fcount--;
        inq[u] = 0;
        while (excess[u] > 0 && h[u] < INF) {
            for (int d = 0; d < 8 && excess[u] > 0; ++d) {
                const int32_t r = caps8[8 * u + d];
                int64_t v;
                if (r <= 0 || !or8_nbr(W, H, u, d, &v) || h[u] != h[v] + 1) continue;
                const int32_t f = excess[u] < r ? excess[u] : r;
                caps8[8 * u + d] -= f;
                caps8[8 * v + D8OPP[d]] += f;
                excess[u] -= f;
                const int32_t ev = excess[v];
                excess[v] += f;
                if (ev <= 0 && excess[v] > 0 && !inq[v] && h[v] < INF) FIFO8_PUSH(v);
            }
            if (excess[u] <= 0) break;
            int32_t m = INF;
            for (int d = 0; d < 8; ++d) {
                int64_t v;
                if (caps8[8 * u + d] <= 0 || !or8_nbr(W, H, u, d, &v)) continue;
                if (h[v] < m) m = h[v];
            }
            h[u] = m >= INF - 1 ? INF : m + 1;
            work += 20;
        }
        if (work > 6 * n + 64 && fcount > 0) {
            or8_global_relabel(W, H, caps8, excess, h, INF, queue);
            work = 0;
            fh = 0;
            fcount = 0;
            memset(inq, 0, (size_t)n);
            for (int64_t i = 0; i < n; ++i)
                if (excess[i] > 0 && h[i] < INF) FIFO8_PUSH(i);
        }
    }
#undef FIFO8_PUSH
    or8_global_relabel(W, H, caps8, excess, h, INF, queue);
    int ok = 1;
    for (int64_t i = 0; i < n; ++i)
        if (excess[i] > 0 && h[i] < INF) { ok = 0; break; }
    free(h); free(queue); free(fifo); free(inq);
    return ok ? 0 : -3;
}

/* smax: interior nodes that cannot reach the sink; smin: nodes reachable
 * from positive excess (8-connected residual graph). */
void or8_cuts(int W, int H, const int32_t *caps8, const int32_t *excess, uint8_t *smin, uint8_t *smax) {
    const int64_t n = (int64_t)W * H;
    int64_t *queue = (int64_t *)malloc((size_t)(n + 1) * sizeof(int64_t));
    uint8_t *mark = (uint8_t *)calloc((size_t)n, 1);
    int64_t qh = 0, qt = 0;
    for (int64_t i = 0; i < n; ++i)
        if (excess[i] < 0) { mark[i] = 1; queue[qt++] = i; }
    while (qh < qt) {
        const int64_t v = queue[qh++];
        for (int d = 0; d < 8; ++d) {
            int64_t u;
            if (!or8_nbr(W, H, v, d, &u)) continue;
            if (!mark[u] && caps8[8 * u + D8OPP[d]] > 0) { mark[u] = 1; queue[qt++] = u; }
        }
    }
    for (int64_t i = 0; i < n; ++i) {
        const int x = (int)(i % W), y = (int)(i / W);
        smax[i] = (uint8_t)(x > 0 && y > 0 && x < W - 1 && y < H - 1 && !mark[i]);
    }
    memset(mark, 0, (size_t)n);
    qh = qt = 0;
    for (int64_t i = 0; i < n; ++i)
        if (excess[i] > 0) { mark[i] = 1; queue[qt++] = i; }
    while (qh < qt) {
        const int64_t u = queue[qh++];
        for (int d = 0; d < 8; ++d) {
            int64_t v;
            if (!or8_nbr(W, H, u, d, &v)) continue;
            if (!mark[v] && caps8[8 * u + d] > 0) { mark[v] = 1; queue[qt++] = v; }
        }
    }
    memcpy(smin, mark, (size_t)n);
    free(queue);
    free(mark);
}

int or8_solve(int W, int H, const int32_t *dp, const int32_t *dn, int penalty, const int32_t *const *arrays,
              uint8_t *smin, uint8_t *smax, int64_t *flow, int32_t *excess_out) {
    const int64_t n = (int64_t)W * H;
    int32_t *caps8 = (int32_t *)malloc((size_t)(8 * n) * sizeof(int32_t));
    int32_t *ex = (int32_t *)malloc((size_t)n * sizeof(int32_t));
    if (!caps8 || !ex) { free(caps8); free(ex); return -2; }
    or8_build(W, H, dp, dn, penalty, arrays, caps8, ex);
    const int rc = or8_maxflow(W, H, caps8, ex);
    if (rc == 0) {
        int64_t pos = 0;
        for (int64_t i = 0; i < n; ++i) if (ex[i] > 0) pos += ex[i];
        if (flow) *flow = or_interior_dp(W, H, dp) - pos;
        if (smin && smax) or8_cuts(W, H, caps8, ex, smin, smax);
        if (excess_out) memcpy(excess_out, ex, (size_t)n * sizeof(int32_t));
    }
    free(caps8);
    free(ex);
    return rc;
}
