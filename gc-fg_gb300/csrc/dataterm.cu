// dataterm.cu -- colour-histogram t-links, contrast-sensitive n-links and
// the fused image -> tile-space residual graph build, for a whole batch.
//
// Replaces the reference's data-term module (DataTerm.cpp:52-205,
// DataTermKernels.cu:19-150), whose Gaussian KDE over a 256^3 cube is
// replaced by a 16^3 colour histogram per class:
//   p_k(bin) = (H_k[bin] + 1) / (N_k + 4096),  bin = (r>>4, g>>4, b>>4)
//   dp = round(10 * -log p_bg)   (source / foreground t-link)
//   dn = round(10 * -log p_fg)   (sink / background t-link)
// N-links: w = round(lambda * exp(-||dI||^2 / (2 sigma^2))), sigma^2 = mean
// ||dI||^2 over all horizontally and vertically adjacent pairs.  The
// reference has no n-link kernel; its callers pass per-direction arrays
// (solveMRF.cu:87-90) that InitGraphVarEdges consumes
// (GraphCutKernels.cu:165-214).
//
// Exactness: per image, the -log values of the 4096 bins and the weights of
// every ||dI||^2 that can round to a non-zero capacity are evaluated once in
// double precision into small tables; the per-pixel passes are integer
// gathers, so the int32 capacities match the CPU oracle bit for bit.
#include "dataterm.cuh"

namespace gcfg {

__device__ __forceinline__ int color_bin3(const uint8_t *__restrict__ p) {
    return ((p[0] >> 4) << 8) | ((p[1] >> 4) << 4) | (p[2] >> 4);
}

__device__ __forceinline__ int diff2p(const uint8_t *__restrict__ a, const uint8_t *__restrict__ b) {
    const int d0 = (int)a[0] - b[0], d1 = (int)a[1] - b[1], d2 = (int)a[2] - b[2];
    return d0 * d0 + d1 * d1 + d2 * d2;
}

// Image of a global chunk index (chunk_off: prefix sums of chunks per image).
__device__ __forceinline__ int chunk_image(const long long *__restrict__ chunk_off, int n_img,
                                           long long chunk) {
    int lo = 0, hi = n_img - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldg(chunk_off + mid) <= chunk) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// Scribble histograms: privatised per block in shared memory, with warp
// aggregation of equal bins (__match_any_sync) before the shared atomics.
__global__ void __launch_bounds__(256) k_hist_b(const uint8_t *__restrict__ rgb,
                                                const uint8_t *__restrict__ scrib,
                                                const ImgDesc *__restrict__ img,
                                                const long long *__restrict__ chunk_off, int n_img,
                                                int *__restrict__ hist) {
    __shared__ int sh[2 * NBINS];
    const int im = chunk_image(chunk_off, n_img, blockIdx.x);
    const long long n = (long long)img[im].W * img[im].H;
    const long long first = ((long long)blockIdx.x - chunk_off[im]) * CHUNK_PX;
    const long long last = min(n, first + CHUNK_PX);
    const long long pix0 = img[im].pix0;
    for (int i = threadIdx.x; i < 2 * NBINS; i += blockDim.x) sh[i] = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31;
    for (long long base = first + (threadIdx.x & ~31); base < last; base += blockDim.x) {
        const long long i = base + lane;
        int key = -1;
        if (i < last) {
            const int s = scrib[pix0 + i];
            if (s == 1 || s == 2) key = (s - 1) * NBINS + color_bin3(rgb + 3 * (pix0 + i));
        }
        const unsigned same = __match_any_sync(0xffffffffu, key);
        if (key >= 0 && lane == __ffs(same) - 1) atomicAdd(&sh[key], __popc(same));
    }
    __syncthreads();
    int *dst = hist + (size_t)im * 2 * NBINS;
    for (int i = threadIdx.x; i < 2 * NBINS; i += blockDim.x)
        if (sh[i]) atomicAdd(dst + i, sh[i]);
}

// Sum of ||dI||^2 over all right and down neighbour pairs, exact int64.
__global__ void __launch_bounds__(256) k_sigma_b(const uint8_t *__restrict__ rgb,
                                                 const ImgDesc *__restrict__ img,
                                                 const long long *__restrict__ chunk_off, int n_img,
                                                 ImgState *ist) {
    const int im = chunk_image(chunk_off, n_img, blockIdx.x);
    const int W = img[im].W, H = img[im].H;
    const long long n = (long long)W * H;
    const long long first = ((long long)blockIdx.x - chunk_off[im]) * CHUNK_PX;
    const long long last = min(n, first + CHUNK_PX);
    const uint8_t *base = rgb + 3 * img[im].pix0;
    unsigned long long acc = 0;
    for (long long i = first + threadIdx.x; i < last; i += blockDim.x) {
        const int x = (int)(i % W), y = (int)(i / W);
        const uint8_t *p = base + 3 * i;
        if (x + 1 < W) acc += (unsigned)diff2p(p, p + 3);
        if (y + 1 < H) acc += (unsigned)diff2p(p, p + 3 * (long long)W);
    }
    warp_atomic_add_u64(&ist[im].sigma_sum, acc);
}

// Per-bin t-link tables (one block per image, double precision).
__global__ void __launch_bounds__(1024) k_tlut_b(const int *__restrict__ hist, int *__restrict__ dp_lut,
                                                 int *__restrict__ dn_lut, double *raw_dp,
                                                 double *raw_dn) {
    __shared__ long long part[2][32];
    const int im = blockIdx.x;
    const int *hf = hist + (size_t)im * 2 * NBINS;
    const int *hb = hf + NBINS;
    long long nf = 0, nb = 0;
    for (int b = threadIdx.x; b < NBINS; b += blockDim.x) {
        nf += hf[b];
        nb += hb[b];
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        nf += __shfl_down_sync(0xffffffffu, nf, o);
        nb += __shfl_down_sync(0xffffffffu, nb, o);
    }
    if ((threadIdx.x & 31) == 0) {
        part[0][threadIdx.x >> 5] = nf;
        part[1][threadIdx.x >> 5] = nb;
    }
    __syncthreads();
    if (threadIdx.x < 32) {
        nf = threadIdx.x < (blockDim.x >> 5) ? part[0][threadIdx.x] : 0;
        nb = threadIdx.x < (blockDim.x >> 5) ? part[1][threadIdx.x] : 0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            nf += __shfl_down_sync(0xffffffffu, nf, o);
            nb += __shfl_down_sync(0xffffffffu, nb, o);
        }
        if (threadIdx.x == 0) {
            part[0][0] = nf;
            part[1][0] = nb;
        }
    }
    __syncthreads();
    const double df = (double)(part[0][0] + NBINS), db = (double)(part[1][0] + NBINS);
    for (int b = threadIdx.x; b < NBINS; b += blockDim.x) {
        const double pf = (double)(hf[b] + 1) / df;
        const double pb = (double)(hb[b] + 1) / db;
        const double rdn = 10.0 * -log(pf);
        const double rdp = 10.0 * -log(pb);
        dp_lut[(size_t)im * NBINS + b] = (int)round(rdp);
        dn_lut[(size_t)im * NBINS + b] = (int)round(rdn);
        if (raw_dp) raw_dp[(size_t)im * NBINS + b] = rdp;
        if (raw_dn) raw_dn[(size_t)im * NBINS + b] = rdn;
    }
}

// Length of each image's n-link table: beyond d2lim every weight rounds to 0
// (lambda * exp(-d2 / 2 sigma^2) < 0.5 with a margin far above rounding error).
__global__ void k_d2lim_b(const ImgDesc *__restrict__ img, int n_img, ImgState *ist) {
    const int im = blockIdx.x * blockDim.x + threadIdx.x;
    if (im >= n_img) return;
    const int W = img[im].W, H = img[im].H;
    const double lambda = img[im].lambda;
    const unsigned long long s = ist[im].sigma_sum;
    const long long count = (long long)(W - 1) * H + (long long)W * (H - 1);
    int lim;
    if (s == 0 || count == 0 || lambda < 0.5) {
        lim = 0;
    } else {
        const double s2 = (double)s / (double)count;
        const double x = 2.0 * s2 * (log(2.0 * lambda) + 1e-9) + 2.0;
        lim = x >= (double)MAX_D2 ? MAX_D2 : (int)ceil(x);
    }
    ist[im].d2lim = lim;
}

// N-link weight for every ||dI||^2 up to d2lim (double precision).
__global__ void k_wlut_b(const ImgDesc *__restrict__ img, const ImgState *__restrict__ ist,
                         int *__restrict__ wlut) {
    const int im = blockIdx.y;
    const int d2 = blockIdx.x * blockDim.x + threadIdx.x;
    if (d2 > ist[im].d2lim) return;
    const int W = img[im].W, H = img[im].H;
    const unsigned long long s = ist[im].sigma_sum;
    const long long count = (long long)(W - 1) * H + (long long)W * (H - 1);
    const double lambda = img[im].lambda;
    double w;
    if (s == 0 || count == 0) {
        w = lambda;
    } else {
        const double s2 = (double)s / (double)count;
        const double a = -(double)d2 / (2.0 * s2);
        w = lambda * exp(a);
    }
    wlut[(size_t)im * WLUT_STRIDE + d2] = (int)round(w);
}

__device__ __forceinline__ int nlink_w(const int *__restrict__ wl, int lim, int d2) {
    return d2 <= lim ? __ldg(wl + d2) : 0;
}

// Fused image -> residual graph of one tile: t-link gather, n-link gather,
// the reference's interior/border conventions, tile-major output.
__global__ void __launch_bounds__(TILE_THREADS) k_build_img_b(Batch b, const uint8_t *__restrict__ rgb,
                                                               const int *__restrict__ dp_lut,
                                                               const int *__restrict__ dn_lut,
                                                               const int *__restrict__ wlut) {
    const int t = blockIdx.x;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int im = __ldg(b.tile_img + t);
    const ImgDesc d = b.img[im];
    const int lt = t - d.tile0;
    const int tx = lt % d.tiles_x, ty = lt / d.tiles_x;
    const int W = d.W, H = d.H;
    const int lim = b.ist[im].d2lim;
    const int *wl = wlut + (size_t)im * WLUT_STRIDE;
    const int *dpl = dp_lut + (size_t)im * NBINS;
    const int *dnl = dn_lut + (size_t)im * NBINS;
    const uint8_t *base = rgb + 3 * d.pix0;
    const long long w32 = (long long)((W + 31) / 32) * 32;
    unsigned long long idp = 0, rinit = 0, pos = 0;
#pragma unroll
    for (int k = 0; k < ROWS_PER_WARP; ++k) {
        const int r = warp + 8 * k;
        const int x = tx * TILE_W + lane, y = ty * TILE_H + r;
        int4 c = make_int4(0, 0, 0, 0);
        int e = 0;
        if (x < W && y < H) {
            const long long i = (long long)y * W + x;
            const uint8_t *p = base + 3 * i;
            const int bin = color_bin3(p);
            const int vdp = __ldg(dpl + bin);
            if ((long long)x + (long long)y * w32 < (long long)W * H && vdp > 0) rinit += (unsigned)vdp;
            if (x > 0 && y > 0 && x < W - 1 && y < H - 1) {
                c.x = x == 1 ? 0 : nlink_w(wl, lim, diff2p(p, p - 3));
                c.y = x == W - 2 ? 0 : nlink_w(wl, lim, diff2p(p, p + 3));
                c.z = y == 1 ? 0 : nlink_w(wl, lim, diff2p(p, p - 3 * (long long)W));
                c.w = y == H - 2 ? 0 : nlink_w(wl, lim, diff2p(p, p + 3 * (long long)W));
                e = vdp - __ldg(dnl + bin);
                idp += (unsigned)vdp;
            }
        }
        const size_t q = (size_t)t * TPX + r * 32 + lane;
        b.cap[q] = c;
        b.exc[q] = e;
        write_tile_masks(b, t, r, c, e);
        if (e > 0) pos += (unsigned)e;
    }
    block_store_sum(b.tile_pos + t, pos);
    warp_atomic_add_u64(&b.ist[im].interior_dp, idp);
    warp_atomic_add_u64(&b.ist[im].ref_init, rinit);
}

// Row-major t-link / n-link arrays of image 0 (the stand-alone data-term API).
__global__ void k_tlinks_apply(const uint8_t *__restrict__ rgb, long long n,
                               const int *__restrict__ dp_lut, const int *__restrict__ dn_lut,
                               int *__restrict__ dp, int *__restrict__ dn) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int bin = color_bin3(rgb + 3 * i);
    dp[i] = __ldg(dp_lut + bin);
    dn[i] = __ldg(dn_lut + bin);
}

__global__ void k_nlinks_apply(const uint8_t *__restrict__ rgb, int W, int H, const ImgState *ist,
                               const int *__restrict__ wl, int *__restrict__ up,
                               int *__restrict__ down, int *__restrict__ left,
                               int *__restrict__ right) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= W || y >= H) return;
    const int lim = ist[0].d2lim;
    const long long i = (long long)y * W + x;
    const uint8_t *p = rgb + 3 * i;
    left[i] = x > 0 ? nlink_w(wl, lim, diff2p(p, p - 3)) : 0;
    right[i] = x + 1 < W ? nlink_w(wl, lim, diff2p(p, p + 3)) : 0;
    up[i] = y > 0 ? nlink_w(wl, lim, diff2p(p, p - 3 * (long long)W)) : 0;
    down[i] = y + 1 < H ? nlink_w(wl, lim, diff2p(p, p + 3 * (long long)W)) : 0;
}

// ---------------------------------------------------------------------------
// Host launchers
// ---------------------------------------------------------------------------

gcfg_status dt_tables(const DtArgs &a, cudaStream_t st) {
    // a.scrib == NULL: n-link tables only (the colour histograms need scribbles)
    if (a.scrib) {
        GCFG_CK(cudaMemsetAsync(a.hist, 0, (size_t)a.n_img * 2 * NBINS * sizeof(int), st));
        GCFG_LAUNCH(GCFG_PK_HIST, st,
                    k_hist_b<<<a.total_chunks, 256, 0, st>>>(a.rgb, a.scrib, a.img, a.chunk_off, a.n_img, a.hist));
        GCFG_LAUNCH(GCFG_PK_TLUT, st,
                    k_tlut_b<<<a.n_img, 1024, 0, st>>>(a.hist, a.dp_lut, a.dn_lut, a.raw_dp, a.raw_dn));
    }
    GCFG_LAUNCH(GCFG_PK_SIGMA, st,
                k_sigma_b<<<a.total_chunks, 256, 0, st>>>(a.rgb, a.img, a.chunk_off, a.n_img, a.ist));
    GCFG_LAUNCH(GCFG_PK_WLUT, st, k_d2lim_b<<<div_up(a.n_img, 128), 128, 0, st>>>(a.img, a.n_img, a.ist));
    GCFG_LAUNCH(GCFG_PK_WLUT, st,
                k_wlut_b<<<dim3(div_up(MAX_D2 + 1, 256), a.n_img), 256, 0, st>>>(a.img, a.ist, a.wlut));
    GCFG_CK(cudaGetLastError());
    return GCFG_OK;
}

gcfg_status dt_build(const Batch &b, const DtArgs &a, cudaStream_t st) {
    GCFG_LAUNCH(GCFG_PK_BUILD, st,
                k_build_img_b<<<b.n_tiles, TILE_THREADS, 0, st>>>(b, a.rgb, a.dp_lut, a.dn_lut, a.wlut));
    GCFG_CK(cudaGetLastError());
    return GCFG_OK;
}

gcfg_status dt_apply_tlinks(const DtArgs &a, long long n, int *dp, int *dn, cudaStream_t st) {
    GCFG_LAUNCH(GCFG_PK_OTHER, st,
                k_tlinks_apply<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(a.rgb, n, a.dp_lut, a.dn_lut, dp, dn));
    GCFG_CK(cudaGetLastError());
    return GCFG_OK;
}

gcfg_status dt_apply_nlinks(const DtArgs &a, int W, int H, int *up, int *down, int *left, int *right,
                            cudaStream_t st) {
    dim3 blk(32, 8), grd(div_up(W, 32), div_up(H, 8));
    GCFG_LAUNCH(GCFG_PK_OTHER, st,
                k_nlinks_apply<<<grd, blk, 0, st>>>(a.rgb, W, H, a.ist, a.wlut, up, down, left, right));
    GCFG_CK(cudaGetLastError());
    return GCFG_OK;
}

}  // namespace gcfg
