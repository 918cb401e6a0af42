// dterm_api.cu -- the DataTerm interface (DataTerm.h:9-19) over the
// colour-histogram data term.
//
// The reference keeps one global data-term state per process: an image, a
// selection map and a kernel-density colour model that selectOnMap() splats
// into (DataTerm.cpp:28-165).  Here the state lives in a handle: the image
// (3 bytes per pixel, as given), the selection map (one byte per pixel: 0 none,
// 1 foreground, 2 background) and the two t-link arrays.  The colour model is
// the 16^3-bin histogram pair of the selected pixels, rebuilt from the current
// image and map whenever the t-links are computed (gcfg_dt_compute), so a
// selection made by selectOnMap() and one made by setSelection() both act on
// the model.
//
// The reference's own model is available too (gcfg_dt_set_model,
// GCFG_DT_KDE): a kernel density over the 256^3 colour cube that every
// selectOnMap() adds to (DataTerm.cpp:97-137, DataTermKernels.cu:19-31,
// 61-83, 116-161).  The reference launches one 256^3-thread kernel per
// selected pixel; here one launch per selectOnMap() covers only the bounding
// box of the 25 colours' support balls (|c - s|^2 < 101^2), and each thread
// adds its cube point's terms in the reference's order (pixel after pixel,
// x offset outer), so the float sums are the reference's, bit for bit.
#include <algorithm>
#include <cstring>

#include "engine.cuh"

namespace gcfg {
namespace {

// setSelection: int map -> byte map (K_SetMap, DataTermKernels.cu:86-94).
__global__ void k_sel_from_int(const int32_t *__restrict__ in, uint8_t *__restrict__ map, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        map[i] = (uint8_t)in[i];
}

// selectOnMap: mark a size x size square with corner (x0, y0), clipped to the
// image (DataTerm.cpp:111-123 marks x..x+4, y..y+4 without clipping).
__global__ void k_sel_square(uint8_t *map, int W, int H, int x0, int y0, int size, int cls) {
    const int dx = threadIdx.x, dy = threadIdx.y;
    if (dx >= size || dy >= size) return;
    const int x = x0 + dx, y = y0 + dy;
    if (x < 0 || y < 0 || x >= W || y >= H) return;
    map[(long long)y * W + x] = (uint8_t)cls;
}

// drawSelection: the pixels whose selection-map entry is 1 become
// (0, 0, 255), every other pixel keeps its colour, as K_DrawMap does
// (DataTermKernels.cu:96-113; a map set from labels marks label 1).
__global__ void k_draw_sel(const uint8_t *__restrict__ map, const uint8_t *__restrict__ img,
                           uint8_t *__restrict__ out, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const uint8_t m = map[i];
        uint8_t c0 = img[3 * i + 0], c1 = img[3 * i + 1], c2 = img[3 * i + 2];
        if (m == 1) {
            c0 = 0;
            c1 = 0;
            c2 = 255;
        }
        out[3 * i + 0] = c0;
        out[3 * i + 1] = c1;
        out[3 * i + 2] = c2;
    }
}

// ---- kernel-density model ----

constexpr int KDE_N = 101;            // table entries (distances 0..100)
constexpr int KDE_CUBE = 256;
constexpr int KDE_MAX_SEL = 25;       // colours per selectOnMap (a 5x5 square)

struct KdeSel {
    int n;
    unsigned char c[KDE_MAX_SEL][3];
};

// Table entry x: 1 / (sigma * 2.507) * exp(-0.5 (x / sigma)^2), with the
// reference's types: x / sigma in float, the rest in double, exp in float.
__global__ void k_kde_gauss(float sigma, float *gauss) {
    const int x = threadIdx.x;
    if (x >= KDE_N) return;
    const float xs = x / sigma;
    const double a = -0.5 * xs * xs;
    gauss[x] = (float)(1.0 / (sigma * 2.507) * expf((float)a));
}

// Cube point (c0, c1, c2) of the box lo + (threadIdx/blockIdx offsets): add
// the table entry of each selected colour within the support, in order.
__global__ void k_kde_splat(float *__restrict__ pdf, const float *__restrict__ gauss, KdeSel sel, int lo0,
                            int lo1, int lo2, int n0, int n1, int n2) {
    __shared__ float g[KDE_N];
    for (int i = threadIdx.x; i < KDE_N; i += blockDim.x) g[i] = gauss[i];
    __syncthreads();
    const int d2i = blockIdx.x * blockDim.x + threadIdx.x;
    if (d2i >= n2) return;
    const int c2 = lo2 + d2i, c0 = lo0 + (int)blockIdx.y, c1 = lo1 + (int)blockIdx.z;
    const size_t idx = ((size_t)c1 * KDE_CUBE + c0) * KDE_CUBE + c2;
    float v = 0.f;
    bool touched = false;
    for (int k = 0; k < sel.n; ++k) {
        const int e0 = c0 - sel.c[k][0], e1 = c1 - sel.c[k][1], e2 = c2 - sel.c[k][2];
        const int d = e0 * e0 + e1 * e1 + e2 * e2;
        if (d < KDE_N * KDE_N) {
            if (!touched) v = pdf[idx];
            touched = true;
            v += g[(int)sqrtf((float)d)];  // floor(sqrt(d)): d and sqrtf are exact enough here
        }
    }
    if (touched) pdf[idx] = v;
}

// t-links of the kernel-density model: pos = (int)(300000 p),
// neg = (int)(300000 (1 - p)), p in float, the products in double.
__global__ void k_kde_terms(const uint8_t *__restrict__ img, const float *__restrict__ pdf, int *__restrict__ pos,
                            int *__restrict__ neg, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const uint8_t *c = img + 3 * i;
        const float p = pdf[((size_t)c[1] * KDE_CUBE + c[0]) * KDE_CUBE + c[2]];
        pos[i] = (int)(300000.0 * (double)p);
        neg[i] = (int)(300000.0 * (double)(1.0f - p));
    }
}

int grid_for(long long n) {
    long long b = (n + 255) / 256;
    return (int)(b < 4096 ? (b > 0 ? b : 1) : 4096);
}

}  // namespace
}  // namespace gcfg

using namespace gcfg;

struct gcfg_dataterm {
    int W = 0, H = 0;
    int sigma = 5;
    uint8_t *d_img = nullptr, *d_sel = nullptr;
    int32_t *d_pos = nullptr, *d_neg = nullptr;
    int32_t *d_tmp = nullptr;  // setSelection staging (allocated on first use)
    uint8_t *d_draw = nullptr; // drawSelection output (allocated on first use)
    cudaStream_t st = nullptr;
    int model = GCFG_DT_HISTOGRAM;
    float *d_pdf = nullptr;    // kernel-density model: 256^3 floats (allocated on first use)
    float *d_gauss = nullptr;  // its 101-entry table
};

namespace {
gcfg_status kde_table(gcfg_dataterm *d) {
    k_kde_gauss<<<1, 128, 0, d->st>>>((float)d->sigma, d->d_gauss);
    g_launches.fetch_add(1, std::memory_order_relaxed);
    GCFG_CK(cudaGetLastError());
    return GCFG_OK;
}
}  // namespace

extern "C" {

gcfg_status gcfg_dt_create(int w, int h, gcfg_dataterm **out) {
    if (!out || w <= 0 || h <= 0 || (long long)w * h > (1LL << 31) - 1) return GCFG_ERR_INVALID;
    gcfg_dataterm *d = new gcfg_dataterm();
    d->W = w;
    d->H = h;
    const size_t n = (size_t)w * h;
    if (cudaMalloc(&d->d_img, 3 * n) != cudaSuccess || cudaMalloc(&d->d_sel, n) != cudaSuccess ||
        cudaMalloc(&d->d_pos, n * sizeof(int32_t)) != cudaSuccess ||
        cudaMalloc(&d->d_neg, n * sizeof(int32_t)) != cudaSuccess) {
        cudaFree(d->d_img);
        cudaFree(d->d_sel);
        cudaFree(d->d_pos);
        cudaFree(d->d_neg);
        delete d;
        return GCFG_ERR_OOM;
    }
    // a fresh state has an empty selection (init_data_term calls reset())
    if (cudaMemset(d->d_sel, 0, n) != cudaSuccess || cudaMemset(d->d_img, 0, 3 * n) != cudaSuccess) {
        cudaFree(d->d_img);
        cudaFree(d->d_sel);
        cudaFree(d->d_pos);
        cudaFree(d->d_neg);
        delete d;
        return GCFG_ERR_CUDA;
    }
    *out = d;
    return GCFG_OK;
}

gcfg_status gcfg_dt_destroy(gcfg_dataterm *d) {
    if (!d) return GCFG_ERR_INVALID;
    cudaStreamSynchronize(d->st);
    cudaFree(d->d_img);
    cudaFree(d->d_sel);
    cudaFree(d->d_pos);
    cudaFree(d->d_neg);
    cudaFree(d->d_tmp);
    cudaFree(d->d_draw);
    cudaFree(d->d_pdf);
    cudaFree(d->d_gauss);
    delete d;
    return GCFG_OK;
}

gcfg_status gcfg_dt_set_stream(gcfg_dataterm *d, void *stream) {
    if (!d) return GCFG_ERR_INVALID;
    d->st = (cudaStream_t)stream;
    return GCFG_OK;
}

gcfg_status gcfg_dt_set_image(gcfg_dataterm *d, const uint8_t *h_img) {
    if (!d || !h_img) return GCFG_ERR_INVALID;
    GCFG_CK(cudaMemcpyAsync(d->d_img, h_img, (size_t)3 * d->W * d->H, cudaMemcpyHostToDevice, d->st));
    GCFG_CK(cudaStreamSynchronize(d->st));
    return GCFG_OK;
}

gcfg_status gcfg_dt_set_image_device(gcfg_dataterm *d, const uint8_t *d_img) {
    if (!d || !d_img) return GCFG_ERR_INVALID;
    GCFG_CK(cudaMemcpyAsync(d->d_img, d_img, (size_t)3 * d->W * d->H, cudaMemcpyDeviceToDevice, d->st));
    return GCFG_OK;
}

gcfg_status gcfg_dt_set_selection(gcfg_dataterm *d, const int32_t *h_select) {
    if (!d || !h_select) return GCFG_ERR_INVALID;
    const long long n = (long long)d->W * d->H;
    if (!d->d_tmp && cudaMalloc(&d->d_tmp, (size_t)n * sizeof(int32_t)) != cudaSuccess) return GCFG_ERR_OOM;
    GCFG_CK(cudaMemcpyAsync(d->d_tmp, h_select, (size_t)n * sizeof(int32_t), cudaMemcpyHostToDevice, d->st));
    k_sel_from_int<<<grid_for(n), 256, 0, d->st>>>(d->d_tmp, d->d_sel, n);
    g_launches.fetch_add(1, std::memory_order_relaxed);
    GCFG_CK(cudaGetLastError());
    GCFG_CK(cudaStreamSynchronize(d->st));
    return GCFG_OK;
}

gcfg_status gcfg_dt_set_scribbles_device(gcfg_dataterm *d, const uint8_t *d_scrib) {
    if (!d || !d_scrib) return GCFG_ERR_INVALID;
    GCFG_CK(cudaMemcpyAsync(d->d_sel, d_scrib, (size_t)d->W * d->H, cudaMemcpyDeviceToDevice, d->st));
    return GCFG_OK;
}

gcfg_status gcfg_dt_reset(gcfg_dataterm *d) {
    if (!d) return GCFG_ERR_INVALID;
    GCFG_CK(cudaMemsetAsync(d->d_sel, 0, (size_t)d->W * d->H, d->st));
    if (d->d_pdf) GCFG_CK(cudaMemsetAsync(d->d_pdf, 0, sizeof(float) * KDE_CUBE * KDE_CUBE * KDE_CUBE, d->st));
    return GCFG_OK;
}

gcfg_status gcfg_dt_set_model(gcfg_dataterm *d, int model) {
    if (!d || (model != GCFG_DT_HISTOGRAM && model != GCFG_DT_KDE)) return GCFG_ERR_INVALID;
    if (model == GCFG_DT_KDE && !d->d_pdf) {
        const size_t bytes = sizeof(float) * KDE_CUBE * KDE_CUBE * KDE_CUBE;
        if (cudaMalloc(&d->d_pdf, bytes) != cudaSuccess) return GCFG_ERR_OOM;
        if (cudaMalloc(&d->d_gauss, sizeof(float) * KDE_N) != cudaSuccess) {
            cudaFree(d->d_pdf);
            d->d_pdf = nullptr;
            return GCFG_ERR_OOM;
        }
        GCFG_CK(cudaMemsetAsync(d->d_pdf, 0, bytes, d->st));
        GCFG_TRY(kde_table(d));
    }
    d->model = model;
    return GCFG_OK;
}

gcfg_status gcfg_dt_kde_table(gcfg_dataterm *d, float *h_gauss) {
    if (!d || !h_gauss || !d->d_gauss) return GCFG_ERR_STATE;
    GCFG_CK(cudaMemcpyAsync(h_gauss, d->d_gauss, sizeof(float) * KDE_N, cudaMemcpyDeviceToHost, d->st));
    GCFG_CK(cudaStreamSynchronize(d->st));
    return GCFG_OK;
}

gcfg_status gcfg_dt_select_on_map(gcfg_dataterm *d, int x, int y, int cls) {
    if (!d || (cls != 1 && cls != 2)) return GCFG_ERR_INVALID;
    k_sel_square<<<1, dim3(GCFG_DT_SELECT_SIZE, GCFG_DT_SELECT_SIZE), 0, d->st>>>(d->d_sel, d->W, d->H, x, y,
                                                                               GCFG_DT_SELECT_SIZE, cls);
    g_launches.fetch_add(1, std::memory_order_relaxed);
    GCFG_CK(cudaGetLastError());
    if (d->model != GCFG_DT_KDE || cls != 1) return GCFG_OK;
    // the selected colours, in the reference's order (x offset outer), clipped
    KdeSel sel;
    sel.n = 0;
    unsigned char row[GCFG_DT_SELECT_SIZE][3];
    for (int i = 0; i < GCFG_DT_SELECT_SIZE; ++i) {
        const int px = x + i;
        if (px < 0 || px >= d->W) continue;
        for (int j = 0; j < GCFG_DT_SELECT_SIZE; ++j) {
            const int py = y + j;
            if (py < 0 || py >= d->H) continue;
            GCFG_CK(cudaMemcpyAsync(row[j], d->d_img + 3 * ((size_t)py * d->W + px), 3, cudaMemcpyDeviceToHost,
                                    d->st));
        }
        GCFG_CK(cudaStreamSynchronize(d->st));
        for (int j = 0; j < GCFG_DT_SELECT_SIZE; ++j) {
            const int py = y + j;
            if (py < 0 || py >= d->H) continue;
            memcpy(sel.c[sel.n++], row[j], 3);
        }
    }
    if (!sel.n) return GCFG_OK;
    int lo[3], hi[3];
    for (int ch = 0; ch < 3; ++ch) {
        lo[ch] = 255;
        hi[ch] = 0;
        for (int k = 0; k < sel.n; ++k) {
            lo[ch] = std::min(lo[ch], (int)sel.c[k][ch] - (KDE_N - 1));
            hi[ch] = std::max(hi[ch], (int)sel.c[k][ch] + (KDE_N - 1));
        }
        lo[ch] = std::max(lo[ch], 0);
        hi[ch] = std::min(hi[ch], KDE_CUBE - 1);
    }
    const int n0 = hi[0] - lo[0] + 1, n1 = hi[1] - lo[1] + 1, n2 = hi[2] - lo[2] + 1;
    dim3 grid((n2 + 127) / 128, n0, n1);  // n0, n1 <= 256
    k_kde_splat<<<grid, 128, 0, d->st>>>(d->d_pdf, d->d_gauss, sel, lo[0], lo[1], lo[2], n0, n1, n2);
    g_launches.fetch_add(1, std::memory_order_relaxed);
    GCFG_CK(cudaGetLastError());
    return GCFG_OK;
}

gcfg_status gcfg_dt_set_sigma(gcfg_dataterm *d, int sigma) {
    if (!d || sigma <= 0) return GCFG_ERR_INVALID;
    d->sigma = sigma;  // the histogram model has no kernel width; the kernel density's table changes
    if (d->d_gauss) GCFG_TRY(kde_table(d));
    return GCFG_OK;
}

gcfg_status gcfg_dt_compute(gcfg_dataterm *d) {
    if (!d) return GCFG_ERR_INVALID;
    if (d->model == GCFG_DT_KDE) {
        const long long n = (long long)d->W * d->H;
        k_kde_terms<<<grid_for(n), 256, 0, d->st>>>(d->d_img, d->d_pdf, d->d_pos, d->d_neg, n);
        g_launches.fetch_add(1, std::memory_order_relaxed);
        GCFG_CK(cudaGetLastError());
        GCFG_CK(cudaStreamSynchronize(d->st));
        return GCFG_OK;
    }
    return gcfg_tlinks(d->d_img, d->d_sel, d->W * d->H, d->d_pos, d->d_neg, nullptr, nullptr, d->st);
}

gcfg_status gcfg_dt_nlinks(gcfg_dataterm *d, double lambda, int32_t *d_up, int32_t *d_down, int32_t *d_left,
                           int32_t *d_right) {
    if (!d) return GCFG_ERR_INVALID;
    return gcfg_nlinks(d->d_img, d->W, d->H, lambda, d_up, d_down, d_left, d_right, d->st);
}

int32_t *gcfg_dt_pos(gcfg_dataterm *d) { return d ? d->d_pos : nullptr; }
int32_t *gcfg_dt_neg(gcfg_dataterm *d) { return d ? d->d_neg : nullptr; }
uint8_t *gcfg_dt_image(gcfg_dataterm *d) { return d ? d->d_img : nullptr; }
uint8_t *gcfg_dt_selection(gcfg_dataterm *d) { return d ? d->d_sel : nullptr; }

gcfg_status gcfg_dt_draw_selection(gcfg_dataterm *d, const uint8_t *h_in, uint8_t *h_out) {
    if (!d || !h_in || !h_out) return GCFG_ERR_INVALID;
    const long long n = (long long)d->W * d->H;
    if (!d->d_draw && cudaMalloc(&d->d_draw, (size_t)3 * n) != cudaSuccess) return GCFG_ERR_OOM;
    // as in the reference, the input becomes the current image; the marks go
    // only to the output (the reference also leaves them in its image buffer)
    GCFG_CK(cudaMemcpyAsync(d->d_img, h_in, (size_t)3 * n, cudaMemcpyHostToDevice, d->st));
    k_draw_sel<<<grid_for(n), 256, 0, d->st>>>(d->d_sel, d->d_img, d->d_draw, n);
    g_launches.fetch_add(1, std::memory_order_relaxed);
    GCFG_CK(cudaGetLastError());
    GCFG_CK(cudaMemcpyAsync(h_out, d->d_draw, (size_t)3 * n, cudaMemcpyDeviceToHost, d->st));
    GCFG_CK(cudaStreamSynchronize(d->st));
    return GCFG_OK;
}

}  // extern "C"
