// dataterm.cu -- colour-histogram t-links, contrast-sensitive n-links, the
// fused image -> residual-graph build, and the one-image segmenter.
//
// Replaces the reference's data-term module (DataTerm.cpp:52-205,
// DataTermKernels.cu:19-150), whose Gaussian KDE over a 256^3 cube is
// replaced by a 16^3 colour histogram per class:
//   p_k(bin) = (H_k[bin] + 1) / (N_k + 4096),  bin = (r>>4, g>>4, b>>4)
//   dp = round(10 * -log p_bg)   (source / foreground t-link)
//   dn = round(10 * -log p_fg)   (sink / background t-link)
// N-links: w = round(lambda * exp(-||dI||^2 / (2 sigma^2))), sigma^2 = mean
// ||dI||^2 over all 4-neighbour pairs.  The reference has no n-link kernel;
// its callers pass per-direction arrays (solveMRF.cu:87-90) that
// InitGraphVarEdges consumes (GraphCutKernels.cu:165-214).
//
// Exactness: the per-bin -log values and the per-||dI||^2 weights are
// computed once per image into small lookup tables in double precision, so
// the quantised int32 capacities match the CPU oracle bit for bit; the
// per-pixel passes are integer gathers.
#include <cstring>

#include "gcfg_internal.cuh"
#include "solver.cuh"

namespace gcfg {

constexpr int NBINS = 4096;
constexpr int MAX_D2 = 3 * 255 * 255;   // largest ||dI||^2 of two RGB pixels

__device__ __forceinline__ int color_bin(const uint8_t *__restrict__ rgb, size_t i) {
    const uint8_t r = rgb[3 * i], g = rgb[3 * i + 1], b = rgb[3 * i + 2];
    return ((r >> 4) << 8) | ((g >> 4) << 4) | (b >> 4);
}

__device__ __forceinline__ int diff2(const uint8_t *__restrict__ rgb, size_t a, size_t b) {
    const int d0 = (int)rgb[3 * a] - rgb[3 * b];
    const int d1 = (int)rgb[3 * a + 1] - rgb[3 * b + 1];
    const int d2 = (int)rgb[3 * a + 2] - rgb[3 * b + 2];
    return d0 * d0 + d1 * d1 + d2 * d2;
}

// Scribble histograms: privatised per block in shared memory, with warp
// aggregation of equal bins (__match_any_sync) before the shared atomics.
__global__ void __launch_bounds__(256) k_hist(const uint8_t *__restrict__ rgb,
                                              const uint8_t *__restrict__ scrib, int n,
                                              int *__restrict__ hist) {
    __shared__ int sh[2 * NBINS];
    for (int i = threadIdx.x; i < 2 * NBINS; i += blockDim.x) sh[i] = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int stride = gridDim.x * blockDim.x;
    // every lane runs the same number of iterations so that the warp
    // collectives see full warps
    for (int base = blockIdx.x * blockDim.x + (threadIdx.x & ~31); base < n; base += stride) {
        const int i = base + lane;
        int key = -1;
        if (i < n) {
            const int s = scrib[i];
            if (s == 1 || s == 2) key = (s - 1) * NBINS + color_bin(rgb, i);
        }
        const unsigned same = __match_any_sync(0xffffffffu, key);
        if (key >= 0 && lane == __ffs(same) - 1) atomicAdd(&sh[key], __popc(same));
    }
    __syncthreads();
    for (int i = threadIdx.x; i < 2 * NBINS; i += blockDim.x)
        if (sh[i]) atomicAdd(&hist[i], sh[i]);
}

// Per-bin t-link table in double precision (one block).
__global__ void __launch_bounds__(1024) k_tlut(const int *__restrict__ hist, int *dp_lut,
                                               int *dn_lut, double *raw_dp, double *raw_dn) {
    __shared__ long long part[2][32];
    long long nf = 0, nb = 0;
    for (int b = threadIdx.x; b < NBINS; b += blockDim.x) {
        nf += hist[b];
        nb += hist[NBINS + b];
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
        const double pf = (double)(hist[b] + 1) / df;
        const double pb = (double)(hist[NBINS + b] + 1) / db;
        const double rdn = 10.0 * -log(pf);
        const double rdp = 10.0 * -log(pb);
        dp_lut[b] = (int)round(rdp);
        dn_lut[b] = (int)round(rdn);
        if (raw_dp) raw_dp[b] = rdp;
        if (raw_dn) raw_dn[b] = rdn;
    }
}

// Sum of ||dI||^2 over all right and down neighbour pairs (exact, int64).
__global__ void __launch_bounds__(256) k_sigma(const uint8_t *__restrict__ rgb, int W, int H,
                                               unsigned long long *sum) {
    const size_t n = (size_t)W * H;
    unsigned long long acc = 0;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    const size_t start = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    const size_t rounds = (n + stride - 1) / stride;
    for (size_t k = 0; k < rounds; ++k) {
        const size_t i = start + k * stride;
        if (i < n) {
            const int x = (int)(i % W), y = (int)(i / W);
            if (x + 1 < W) acc += (unsigned)diff2(rgb, i, i + 1);
            if (y + 1 < H) acc += (unsigned)diff2(rgb, i, i + W);
        }
    }
    warp_atomic_add_u64(sum, acc);
}

// N-link weight for every possible ||dI||^2 (double precision, once per image).
__global__ void k_wlut(const unsigned long long *__restrict__ sum, long long count, double lambda,
                       int *__restrict__ wlut) {
    const int d2 = blockIdx.x * blockDim.x + threadIdx.x;
    if (d2 > MAX_D2) return;
    const unsigned long long s = *sum;
    double w;
    if (s == 0 || count == 0) {
        w = lambda;
    } else {
        const double s2 = (double)s / (double)count;
        const double a = -(double)d2 / (2.0 * s2);
        w = lambda * exp(a);
    }
    wlut[d2] = (int)round(w);
}

__global__ void k_tlinks_apply(const uint8_t *__restrict__ rgb, int n, const int *__restrict__ dp_lut,
                               const int *__restrict__ dn_lut, int *__restrict__ dp,
                               int *__restrict__ dn) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int b = color_bin(rgb, i);
    dp[i] = __ldg(dp_lut + b);
    dn[i] = __ldg(dn_lut + b);
}

__global__ void k_nlinks_apply(const uint8_t *__restrict__ rgb, int W, int H,
                               const int *__restrict__ wlut, int *__restrict__ up,
                               int *__restrict__ down, int *__restrict__ left,
                               int *__restrict__ right) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= W || y >= H) return;
    const size_t i = (size_t)y * W + x;
    left[i] = x > 0 ? __ldg(wlut + diff2(rgb, i, i - 1)) : 0;
    right[i] = x + 1 < W ? __ldg(wlut + diff2(rgb, i, i + 1)) : 0;
    up[i] = y > 0 ? __ldg(wlut + diff2(rgb, i, i - W)) : 0;
    down[i] = y + 1 < H ? __ldg(wlut + diff2(rgb, i, i + W)) : 0;
}

// Fused image -> residual graph: t-link gather + n-link gather + the
// reference's interior/border conventions, straight into the tile layout.
__global__ void k_build_image(GraphDev g, const uint8_t *__restrict__ rgb,
                              const int *__restrict__ dp_lut, const int *__restrict__ dn_lut,
                              const int *__restrict__ wlut, Counters *cnt) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    const int W = g.W, H = g.H;
    int4 c = make_int4(0, 0, 0, 0);
    int e = 0;
    unsigned long long idp = 0, rinit = 0;
    if (x < W && y < H) {
        const size_t i = (size_t)y * W + x;
        const int b = color_bin(rgb, i);
        const int vdp = __ldg(dp_lut + b);
        const long long w32 = (long long)((W + 31) / 32) * 32;
        if ((long long)x + (long long)y * w32 < (long long)W * H && vdp > 0) rinit = (unsigned)vdp;
        if (x > 0 && y > 0 && x < W - 1 && y < H - 1) {
            const int vdn = __ldg(dn_lut + b);
            c.x = x == 1 ? 0 : __ldg(wlut + diff2(rgb, i, i - 1));
            c.y = x == W - 2 ? 0 : __ldg(wlut + diff2(rgb, i, i + 1));
            c.z = y == 1 ? 0 : __ldg(wlut + diff2(rgb, i, i - W));
            c.w = y == H - 2 ? 0 : __ldg(wlut + diff2(rgb, i, i + W));
            e = vdp - vdn;
            idp = (unsigned long long)vdp;
        }
    }
    if (x < g.Wp && y < g.Hp) {
        const size_t p = (size_t)y * g.Wp + x;
        g.cap[p] = c;
        g.exc[p] = e;
    }
    warp_atomic_add_u64(&cnt->interior_dp, idp);
    warp_atomic_add_u64(&cnt->ref_init, rinit);
}

// ---------------------------------------------------------------------------
// Host helpers
// ---------------------------------------------------------------------------

struct DataTermBufs {
    int *hist = nullptr;               // 2 * 4096
    int *dp_lut = nullptr, *dn_lut = nullptr;
    double *raw_dp = nullptr, *raw_dn = nullptr;
    int *wlut = nullptr;               // MAX_D2 + 1
    unsigned long long *sigma = nullptr;

    gcfg_status alloc() {
        if (cudaMalloc(&hist, 2 * NBINS * sizeof(int)) != cudaSuccess) return GCFG_ERR_OOM;
        if (cudaMalloc(&dp_lut, NBINS * sizeof(int)) != cudaSuccess) return GCFG_ERR_OOM;
        if (cudaMalloc(&dn_lut, NBINS * sizeof(int)) != cudaSuccess) return GCFG_ERR_OOM;
        if (cudaMalloc(&raw_dp, NBINS * sizeof(double)) != cudaSuccess) return GCFG_ERR_OOM;
        if (cudaMalloc(&raw_dn, NBINS * sizeof(double)) != cudaSuccess) return GCFG_ERR_OOM;
        if (cudaMalloc(&wlut, (MAX_D2 + 1) * sizeof(int)) != cudaSuccess) return GCFG_ERR_OOM;
        if (cudaMalloc(&sigma, sizeof(unsigned long long)) != cudaSuccess) return GCFG_ERR_OOM;
        return GCFG_OK;
    }
    void release() {
        cudaFree(hist);
        cudaFree(dp_lut);
        cudaFree(dn_lut);
        cudaFree(raw_dp);
        cudaFree(raw_dn);
        cudaFree(wlut);
        cudaFree(sigma);
        *this = DataTermBufs();
    }
};

static int hist_blocks(int n) {
    int b = (n + 255) / 256;
    return b < 1 ? 1 : (b > 152 * 2 ? 152 * 2 : b);
}

static gcfg_status run_tlut(DataTermBufs &b, const uint8_t *rgb, const uint8_t *scrib, int n,
                            cudaStream_t st) {
    GCFG_CK(cudaMemsetAsync(b.hist, 0, 2 * NBINS * sizeof(int), st));
    GCFG_LAUNCH(GCFG_PK_HIST, st, k_hist<<<hist_blocks(n), 256, 0, st>>>(rgb, scrib, n, b.hist));
    GCFG_LAUNCH(GCFG_PK_TLUT, st, k_tlut<<<1, 1024, 0, st>>>(b.hist, b.dp_lut, b.dn_lut, b.raw_dp, b.raw_dn));
    GCFG_CK(cudaGetLastError());
    return GCFG_OK;
}

static gcfg_status run_wlut(DataTermBufs &b, const uint8_t *rgb, int W, int H, double lambda,
                            cudaStream_t st) {
    GCFG_CK(cudaMemsetAsync(b.sigma, 0, sizeof(unsigned long long), st));
    GCFG_LAUNCH(GCFG_PK_SIGMA, st, k_sigma<<<hist_blocks(W * H), 256, 0, st>>>(rgb, W, H, b.sigma));
    const long long count = (long long)(W - 1) * H + (long long)W * (H - 1);
    GCFG_LAUNCH(GCFG_PK_WLUT, st, k_wlut<<<div_up(MAX_D2 + 1, 256), 256, 0, st>>>(b.sigma, count, lambda, b.wlut));
    GCFG_CK(cudaGetLastError());
    return GCFG_OK;
}

}  // namespace gcfg

using namespace gcfg;

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------

struct gcfg_segmenter {
    int max_w = 0, max_h = 0;
    SolverState s;
    DataTermBufs dt;
    uint8_t *d_rgb = nullptr, *d_scrib = nullptr, *d_smin = nullptr, *d_smax = nullptr;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    int push_rounds = 4, max_sweeps = 64;
};

extern "C" {

gcfg_status gcfg_tlinks(const uint8_t *d_rgb, const uint8_t *d_scrib, int n, int32_t *d_dp,
                        int32_t *d_dn, double *h_raw_dp, double *h_raw_dn, void *stream) {
    if (!d_rgb || !d_scrib || !d_dp || !d_dn || n <= 0) return GCFG_ERR_INVALID;
    cudaStream_t st = (cudaStream_t)stream;
    DataTermBufs b;
    gcfg_status rc = b.alloc();
    if (rc == GCFG_OK) rc = run_tlut(b, d_rgb, d_scrib, n, st);
    if (rc == GCFG_OK) {
        GCFG_LAUNCH(GCFG_PK_OTHER, st, k_tlinks_apply<<<div_up(n, 256), 256, 0, st>>>(d_rgb, n, b.dp_lut, b.dn_lut, d_dp, d_dn));
        if (cudaGetLastError() != cudaSuccess) rc = GCFG_ERR_CUDA;
    }
    if (rc == GCFG_OK && h_raw_dp &&
        cudaMemcpyAsync(h_raw_dp, b.raw_dp, NBINS * sizeof(double), cudaMemcpyDeviceToHost, st) != cudaSuccess)
        rc = GCFG_ERR_CUDA;
    if (rc == GCFG_OK && h_raw_dn &&
        cudaMemcpyAsync(h_raw_dn, b.raw_dn, NBINS * sizeof(double), cudaMemcpyDeviceToHost, st) != cudaSuccess)
        rc = GCFG_ERR_CUDA;
    if (cudaStreamSynchronize(st) != cudaSuccess && rc == GCFG_OK) rc = GCFG_ERR_CUDA;
    b.release();
    return rc;
}

gcfg_status gcfg_nlinks(const uint8_t *d_rgb, int w, int h, double lambda, int32_t *d_up,
                        int32_t *d_down, int32_t *d_left, int32_t *d_right, void *stream) {
    if (!d_rgb || !d_up || !d_down || !d_left || !d_right || w <= 0 || h <= 0 || !(lambda >= 0))
        return GCFG_ERR_INVALID;
    if (lambda * 1.0000001 + 1 > (double)GCFG_MAX_CAP) return GCFG_ERR_INVALID;
    cudaStream_t st = (cudaStream_t)stream;
    DataTermBufs b;
    gcfg_status rc = b.alloc();
    if (rc == GCFG_OK) rc = run_wlut(b, d_rgb, w, h, lambda, st);
    if (rc == GCFG_OK) {
        dim3 blk(32, 8), grd(div_up(w, 32), div_up(h, 8));
        GCFG_LAUNCH(GCFG_PK_OTHER, st, k_nlinks_apply<<<grd, blk, 0, st>>>(d_rgb, w, h, b.wlut, d_up, d_down, d_left, d_right));
        if (cudaGetLastError() != cudaSuccess) rc = GCFG_ERR_CUDA;
    }
    if (cudaStreamSynchronize(st) != cudaSuccess && rc == GCFG_OK) rc = GCFG_ERR_CUDA;
    b.release();
    return rc;
}

gcfg_status gcfg_seg_create(int max_w, int max_h, gcfg_segmenter **out) {
    if (!out || max_w < 1 || max_h < 1 || (long long)max_w * max_h > (1LL << 31) - 1)
        return GCFG_ERR_INVALID;
    gcfg_segmenter *s = new gcfg_segmenter();
    s->max_w = max_w;
    s->max_h = max_h;
    const size_t n = (size_t)max_w * max_h;
    gcfg_status rc = solver_alloc(s->s, max_w, max_h);
    if (rc == GCFG_OK) rc = s->dt.alloc();
    if (rc == GCFG_OK && (cudaMalloc(&s->d_rgb, 3 * n) != cudaSuccess ||
                          cudaMalloc(&s->d_scrib, n) != cudaSuccess ||
                          cudaMalloc(&s->d_smin, n) != cudaSuccess ||
                          cudaMalloc(&s->d_smax, n) != cudaSuccess))
        rc = GCFG_ERR_OOM;
    if (rc == GCFG_OK && (cudaEventCreate(&s->ev0) != cudaSuccess ||
                          cudaEventCreate(&s->ev1) != cudaSuccess))
        rc = GCFG_ERR_CUDA;
    if (rc) {
        gcfg_seg_destroy(s);
        return rc;
    }
    *out = s;
    return GCFG_OK;
}

gcfg_status gcfg_seg_set_stream(gcfg_segmenter *s, void *stream) {
    if (!s) return GCFG_ERR_INVALID;
    s->stream = (cudaStream_t)stream;
    return GCFG_OK;
}

gcfg_status gcfg_seg_run(gcfg_segmenter *s, const uint8_t *d_rgb, const uint8_t *d_scrib, int w,
                         int h, double lambda, uint8_t *d_smin, uint8_t *d_smax,
                         gcfg_result *res) {
    if (!s || !d_rgb || !d_scrib || w < 1 || h < 1 || w > s->max_w || h > s->max_h ||
        (long long)w * h > (long long)s->max_w * s->max_h || !(lambda >= 0) ||
        lambda * 1.0000001 + 1 > (double)GCFG_MAX_CAP)
        return GCFG_ERR_INVALID;
    cudaStream_t st = s->stream;
    GCFG_CK(cudaEventRecord(s->ev0, st));
    GraphDev g = solver_view(s->s, w, h);
    GCFG_TRY(run_tlut(s->dt, d_rgb, d_scrib, w * h, st));
    GCFG_TRY(run_wlut(s->dt, d_rgb, w, h, lambda, st));
    GCFG_CK(cudaMemsetAsync(s->s.cnt, 0, sizeof(Counters), st));
    dim3 blk(32, 8), grd(g.Wp / 32, g.Hp / 8);
    GCFG_LAUNCH(GCFG_PK_BUILD, st, k_build_image<<<grd, blk, 0, st>>>(g, d_rgb, s->dt.dp_lut, s->dt.dn_lut, s->dt.wlut, s->s.cnt));
    GCFG_CK(cudaGetLastError());
    gcfg_result r;
    memset(&r, 0, sizeof(r));
    GCFG_TRY(solve(s->s, g, st, s->push_rounds, s->max_sweeps, &r));
    GCFG_TRY(extract(g, d_smin, d_smax, nullptr, st));
    GCFG_CK(cudaEventRecord(s->ev1, st));
    GCFG_CK(cudaEventSynchronize(s->ev1));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, s->ev0, s->ev1);
    r.ms = ms;
    if (res) *res = r;
    return GCFG_OK;
}

gcfg_status gcfg_seg_run_host(gcfg_segmenter *s, const uint8_t *h_rgb, const uint8_t *h_scrib,
                              int w, int h, double lambda, uint8_t *h_smin, uint8_t *h_smax,
                              gcfg_result *res) {
    if (!s || !h_rgb || !h_scrib || w < 1 || h < 1 || w > s->max_w || h > s->max_h)
        return GCFG_ERR_INVALID;
    const size_t n = (size_t)w * h;
    cudaStream_t st = s->stream;
    GCFG_CK(cudaMemcpyAsync(s->d_rgb, h_rgb, 3 * n, cudaMemcpyHostToDevice, st));
    GCFG_CK(cudaMemcpyAsync(s->d_scrib, h_scrib, n, cudaMemcpyHostToDevice, st));
    GCFG_TRY(gcfg_seg_run(s, s->d_rgb, s->d_scrib, w, h, lambda, s->d_smin, s->d_smax, res));
    if (h_smin) GCFG_CK(cudaMemcpyAsync(h_smin, s->d_smin, n, cudaMemcpyDeviceToHost, st));
    if (h_smax) GCFG_CK(cudaMemcpyAsync(h_smax, s->d_smax, n, cudaMemcpyDeviceToHost, st));
    GCFG_CK(cudaStreamSynchronize(st));
    return GCFG_OK;
}

gcfg_status gcfg_seg_destroy(gcfg_segmenter *s) {
    if (!s) return GCFG_ERR_INVALID;
    solver_free(s->s);
    s->dt.release();
    cudaFree(s->d_rgb);
    cudaFree(s->d_scrib);
    cudaFree(s->d_smin);
    cudaFree(s->d_smax);
    if (s->ev0) cudaEventDestroy(s->ev0);
    if (s->ev1) cudaEventDestroy(s->ev1);
    delete s;
    return GCFG_OK;
}

}  // extern "C"
