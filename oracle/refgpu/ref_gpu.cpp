/* The reference's CUDA path on the GPU: test and benchmark infrastructure.
 *
 * The device code is the reference's own (GraphCutKernels.cu, compiled from
 * the reference checkout into gc_ref_kernels.cubin, and with its
 * NEIGHBORHOOD switch set to 8 into gc_ref_kernels8.cubin, by
 * build_ref_gpu.sh).  The reference's host code (GraphCut.cu) is compiled
 * into every application and cannot be rebuilt where its sources are absent,
 * so this file restates it, launch for launch, over the cubins' kernels:
 *
 *   refgpu_solve / refgpu_solve8
 *                 = GC_Init (GraphCut.cu:187-263: padded sizes, the graph's
 *                   allocations) + GC_SetGraph (:301-319) + GC_Optimize
 *                   (:385-534) + GC_End (:542-568)
 *   get_energy    = getEnergy (GraphCut.cu:359-376)
 *   refgpu_kde    = DataTerm::init_data_term + setImage + setSigmaGaussian +
 *                   selectOnMap (per point) + getDataTermsMixture
 *                   (DataTerm.cpp:28-137) over the data-term kernels
 *                   (DataTermKernels.cu, gc_ref_dt_kernels.cubin)
 *   refgpu_draw   = DataTerm::drawSelection (DataTerm.cpp:155-165)
 *
 * Differences, all outside the timed arithmetic: every loop is bounded (an
 * iteration cap and a wall-clock cap, reported through the status instead of
 * spinning forever, GraphCut.cu:414,465,517 are unbounded), errors are
 * returned instead of exit(), and nothing is printed.  The launch order, the
 * blocking copies of the alive flag every ACTIVITY_CHECK_FREQUENCY
 * iterations and around every GlobalRelabel / SpreadLabels launch, and the
 * global-relabel schedule are the reference's.
 *
 * The kernels take the reference's KernelWrapper by value; RKernel<NB> below
 * has the same members in the same order (GraphCut.h:60-105), hence the same
 * layout (120 bytes with NEIGHBORHOOD 4, 152 with 8) on every LP64 host and
 * on the device.
 */
#include <cuda_runtime.h>

#include <chrono>
#include <cmath>
#include <cstring>

namespace {

// NodeWrapper / GraphWrapper / KernelWrapper (GraphCut.h:60-105): the edge
// arrays l, r, u, d, then with NEIGHBORHOOD 8 ul, dr, ur, dl
template <int NB>
struct RNode {
    int *edge[NB];
    int *height, *excess, *status, *comp_h, *comp_n, *energy_sum;
};
template <int NB>
struct RGraph {
    int width, height, size, width_ex, height_ex, size_ex;
    RNode<NB> n;
};
template <int NB>
struct RKernel {
    int block_x;
    int *active;
    RGraph<NB> g;
};
static_assert(sizeof(RKernel<4>) == 120, "KernelWrapper layout (GraphCut.h:60-105)");
static_assert(sizeof(RKernel<8>) == 152, "KernelWrapper layout with NEIGHBORHOOD 8");

// GraphCut.h:43-48 and :144-157
constexpr int TX = 32, TY = 8;
constexpr int ACTIVITY_CHECK = 10, GR_FREQUENCY = 100, GR_FIRST = 100;

// The reference's kernels of one NEIGHBORHOOD build (one cubin each).
struct Kernels {
    cudaLibrary_t lib = nullptr;
    cudaKernel_t init, init_var, relabel, push, activity, init_gr, gr, energy, init_labels, spread;
};
Kernels g_k4, g_k8;

// Itanium-mangled names of the reference's kernels (GraphCutKernels.cu);
// InitGraphVarEdges takes 6 int* arrays with NEIGHBORHOOD 4 and 10 with 8.
struct Named {
    cudaKernel_t Kernels::*k;
    const char *name;
};
const Named kNames[] = {
    {&Kernels::init, "_Z9InitGraph13KernelWrapperPiS0_i"},
    {&Kernels::relabel, "_Z7Relabel13KernelWrapperi"},
    {&Kernels::push, "_Z8WavePush13KernelWrapperiPi"},
    {&Kernels::activity, "_Z14UpdateActivityPiS_iiS_"},
    {&Kernels::init_gr, "_Z17InitGlobalRelabel13KernelWrapper"},
    {&Kernels::gr, "_Z13GlobalRelabel13KernelWrapperPi"},
    {&Kernels::energy, "_Z11EnergyLevel13KernelWrapperiiPiS0_b"},
    {&Kernels::init_labels, "_Z10InitLabels13KernelWrapperPi"},
    {&Kernels::spread, "_Z12SpreadLabels13KernelWrapperPiS0_"},
};
const char *const kInitVar4 = "_Z17InitGraphVarEdges13KernelWrapperPiS0_S0_S0_S0_S0_";
const char *const kInitVar8 = "_Z17InitGraphVarEdges13KernelWrapperPiS0_S0_S0_S0_S0_S0_S0_S0_S0_";

enum { OK = 0, ERR_INVALID = 1, ERR_CUDA = 2, ERR_CAP = 3, ERR_NOT_LOADED = 4 };

int load(Kernels &K, const char *path, const char *init_var_name) {
    if (K.lib) return OK;
    if (!path) return ERR_INVALID;
    cudaLibrary_t lib;
    if (cudaLibraryLoadFromFile(&lib, path, nullptr, nullptr, 0, nullptr, nullptr, 0) != cudaSuccess)
        return ERR_CUDA;
    bool ok = cudaLibraryGetKernel(&K.init_var, lib, init_var_name) == cudaSuccess;
    for (const Named &n : kNames) ok = ok && cudaLibraryGetKernel(&(K.*n.k), lib, n.name) == cudaSuccess;
    if (!ok) {
        cudaLibraryUnload(lib);
        return ERR_CUDA;
    }
    K.lib = lib;
    return OK;
}

// GraphCut.cu:165-170 (float ceil, as the reference computes it)
int round_up(int a, int b) { return (int)std::ceil((float)a / (float)b); }

using Clock = std::chrono::steady_clock;
double ms_since(Clock::time_point t) {
    return std::chrono::duration<double, std::milli>(Clock::now() - t).count();
}

cudaError_t launch(cudaKernel_t k, dim3 grid, void **args) {
    return cudaLaunchKernel((const void *)k, grid, dim3(TX, TY, 1), args, 0, 0);
}

#define TRY(x)                         \
    do {                               \
        if ((x) != cudaSuccess) {      \
            rc = ERR_CUDA;             \
            goto done;                 \
        }                              \
    } while (0)

// getEnergy (GraphCut.cu:359-376): tree sum of the positive part of source
// in energy_sum; the first 8 ints are copied to dest.
template <int NB>
cudaError_t get_energy(const Kernels &K, RKernel<NB> k, dim3 grid, int *source, int *dest, bool limited) {
    int odd = 0;
    int stride = limited ? k.g.size : k.g.size_ex;
    int *out = k.g.n.energy_sum;
    for (;; odd = stride % 2, stride = (stride + 1) / 2) {
        if (stride == 1) odd = 0;
        void *a[] = {&k, &stride, &odd, &source, &out, &limited};
        cudaError_t e = launch(K.energy, grid, a);
        if (e != cudaSuccess) return e;
        if (stride == 1) return cudaMemcpy(dest, out, 8 * sizeof(int), cudaMemcpyDeviceToHost);
    }
}

}  // namespace

extern "C" {

struct refgpu_stats {
    long long iterations;       // main-loop iterations (the reference's counter)
    long long global_relabels;  // global relabels started
    long long gr_launches;      // GlobalRelabel launches
    long long spread_launches;  // SpreadLabels launches
    int initial_energy;         // "Initial energy level" (GraphCut.cu:400)
    int final_energy;           // "Final energy level" = initial - sum+ excess (:456)
    int converged;              // 1 when the reference's own termination test ended the loop
    int pad;
    double ms_init;             // GC_Init's allocations
    double ms_solve;            // GC_SetGraph + GC_Optimize, wall clock
    double ms_loop;             // the reference's internal timer (the push-relabel loop)
    double ms_end;              // GC_End's frees
};

}  // extern "C"

namespace {

// One solve: edges == NULL selects the constant penalty (InitGraph), else
// edges[0 .. NB-1] are the NB host arrays in InitGraphVarEdges' order (up,
// down, left, right, then upleft, upright, downleft, downright).
template <int NB>
int solve(const Kernels &K, int w, int h, const int *dp, const int *dn, int penalty, const int *const *edges,
          int *label, long long max_iters, double max_seconds, refgpu_stats *st) {
    if (!K.lib) return ERR_NOT_LOADED;
    if (w < 1 || h < 1 || !dp || !dn || !label || !st) return ERR_INVALID;
    if ((long long)w * h > (1LL << 28)) return ERR_INVALID;
    std::memset(st, 0, sizeof(*st));
    const bool var = edges != nullptr;
    if (var)
        for (int i = 0; i < NB; ++i)
            if (!edges[i]) return ERR_INVALID;
    const size_t n = (size_t)w * h;
    const int n_in = var ? 2 + NB : 2;
    int rc = OK;
    int *d_in[2 + NB] = {};
    int *owned[NB + 7] = {};
    int *d_alive = nullptr, *d_label = nullptr;
    int zero_arr[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    int h_alive[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    RKernel<NB> k;
    std::memset(&k, 0, sizeof(k));
    dim3 grid;
    Clock::time_point t0;

    for (int i = 0; i < n_in; ++i) {
        const int *src = i == 0 ? dp : i == 1 ? dn : edges[i - 2];
        TRY(cudaMalloc((void **)&d_in[i], n * sizeof(int)));
        TRY(cudaMemcpy(d_in[i], src, n * sizeof(int), cudaMemcpyHostToDevice));
    }
    TRY(cudaDeviceSynchronize());

    // ---- GC_Init (GraphCut.cu:187-263)
    t0 = Clock::now();
    k.g.width = w;
    k.g.height = h;
    k.g.size = w * h;
    k.g.width_ex = TX * round_up(w, TX);
    k.g.height_ex = TY * round_up(h, TY);
    k.g.size_ex = k.g.width_ex * k.g.height_ex;
    k.block_x = round_up(k.g.width_ex, TX);
    {
        const int block_y = round_up(k.g.height_ex, TY);
        const int block_count = round_up(k.g.size_ex, TX * TY);
        grid = dim3(k.block_x, block_y, 1);
        int **fields[NB + 6];
        for (int i = 0; i < NB; ++i) fields[i] = &k.g.n.edge[i];
        fields[NB + 0] = &k.g.n.height;
        fields[NB + 1] = &k.g.n.excess;
        fields[NB + 2] = &k.g.n.status;
        fields[NB + 3] = &k.g.n.comp_h;
        fields[NB + 4] = &k.g.n.comp_n;
        fields[NB + 5] = &k.g.n.energy_sum;
        for (int i = 0; i < NB + 6; ++i) {
            TRY(cudaMalloc((void **)fields[i], sizeof(int) * k.g.size_ex));
            owned[i] = *fields[i];
        }
        TRY(cudaMalloc((void **)&k.active, sizeof(int) * block_count));
        owned[NB + 6] = k.active;
    }
    TRY(cudaDeviceSynchronize());
    st->ms_init = ms_since(t0);

    // ---- GC_SetGraph (GraphCut.cu:301-319) + GC_Optimize (:385-534)
    t0 = Clock::now();
    if (var) {
        void *a[3 + NB] = {&k, &d_in[0], &d_in[1]};
        for (int i = 0; i < NB; ++i) a[3 + i] = &d_in[2 + i];
        TRY(launch(K.init_var, grid, a));
    } else {
        void *a[] = {&k, &d_in[0], &d_in[1], &penalty};
        TRY(launch(K.init, grid, a));
    }
    TRY(cudaMalloc((void **)&d_alive, 8 * sizeof(int)));
    TRY(get_energy(K, k, grid, d_in[0], h_alive, true));
    st->initial_energy = h_alive[0];
    {
        const Clock::time_point t_loop = Clock::now();
        long long counter = 0;
        for (;;) {
            const int skip = (int)(counter % ACTIVITY_CHECK);
            ++counter;
            if (!skip) TRY(cudaMemcpy(d_alive, zero_arr, 8 * sizeof(int), cudaMemcpyHostToDevice));
            {
                int s = skip;
                void *a[] = {&k, &s};
                TRY(launch(K.relabel, grid, a));
            }
            {
                int s = skip;
                void *a[] = {&k, &s, &d_alive};
                TRY(launch(K.push, grid, a));
            }
            if (!skip) {
                int bx = k.block_x, wex = k.g.width_ex;
                void *a[] = {&k.g.n.status, &k.active, &bx, &wex, &d_alive};
                TRY(launch(K.activity, grid, a));
                TRY(cudaMemcpy(h_alive, d_alive, 8 * sizeof(int), cudaMemcpyDeviceToHost));
            }
            if (!h_alive[0]) {
                TRY(cudaDeviceSynchronize());
                st->ms_loop = ms_since(t_loop);
                TRY(get_energy(K, k, grid, k.g.n.excess, h_alive, false));
                st->final_energy = st->initial_energy - h_alive[0];
                st->converged = 1;
                break;
            }
            if (!((counter - GR_FIRST) % GR_FREQUENCY)) {
                void *a0[] = {&k};
                TRY(launch(K.init_gr, grid, a0));
                st->global_relabels++;
                for (;;) {
                    TRY(cudaMemcpy(d_alive, zero_arr, 8 * sizeof(int), cudaMemcpyHostToDevice));
                    void *a[] = {&k, &d_alive};
                    TRY(launch(K.gr, grid, a));
                    st->gr_launches++;
                    TRY(cudaMemcpy(h_alive, d_alive, 8 * sizeof(int), cudaMemcpyDeviceToHost));
                    if (!h_alive[0]) break;
                    if (ms_since(t0) > max_seconds * 1e3) {
                        rc = ERR_CAP;
                        goto done;
                    }
                }
                h_alive[0] = 1;
            }
            if (counter >= max_iters || ((counter & 63) == 0 && ms_since(t0) > max_seconds * 1e3)) {
                st->iterations = counter;
                rc = ERR_CAP;
                goto done;
            }
        }
        st->iterations = counter;
    }
    // labels (GraphCut.cu:507-529): the caller's array goes in, InitLabels
    // overwrites it, SpreadLabels runs until nothing changes
    TRY(cudaMalloc((void **)&d_label, sizeof(int) * n));
    TRY(cudaMemcpy(d_label, label, sizeof(int) * n, cudaMemcpyHostToDevice));
    {
        void *a[] = {&k, &d_label};
        TRY(launch(K.init_labels, grid, a));
    }
    for (;;) {
        TRY(cudaMemcpy(d_alive, zero_arr, 8 * sizeof(int), cudaMemcpyHostToDevice));
        void *a[] = {&k, &d_label, &d_alive};
        TRY(launch(K.spread, grid, a));
        st->spread_launches++;
        TRY(cudaMemcpy(h_alive, d_alive, 8 * sizeof(int), cudaMemcpyDeviceToHost));
        if (!h_alive[0]) break;
        if (ms_since(t0) > max_seconds * 1e3) {
            rc = ERR_CAP;
            goto done;
        }
    }
    TRY(cudaMemcpy(label, d_label, sizeof(int) * n, cudaMemcpyDeviceToHost));
    TRY(cudaFree(d_label));
    d_label = nullptr;
    TRY(cudaFree(d_alive));
    d_alive = nullptr;
    st->ms_solve = ms_since(t0);

done:
    if (d_label) cudaFree(d_label);
    if (d_alive) cudaFree(d_alive);
    {
        // ---- GC_End (GraphCut.cu:542-568): the graph's arrays, never the inputs
        const Clock::time_point t_end = Clock::now();
        for (int *p : owned)
            if (p) cudaFree(p);
        st->ms_end = ms_since(t_end);
    }
    for (int *p : d_in)
        if (p) cudaFree(p);
    if (rc == OK && cudaGetLastError() != cudaSuccess) rc = ERR_CUDA;
    return rc;
}

}  // namespace

extern "C" {

/* Loads the reference's kernels (NEIGHBORHOOD 4) from the cubin.  Returns 0,
 * or 2 when the file cannot be loaded or a kernel is missing. */
int refgpu_load(const char *cubin_path) { return load(g_k4, cubin_path, kInitVar4); }

/* The same for the NEIGHBORHOOD 8 build of the kernels. */
int refgpu_load8(const char *cubin_path) { return load(g_k8, cubin_path, kInitVar8); }

/* One solve through the reference's CUDA path.  dp/dn (and up/down/left/right
 * when up != NULL, else the constant penalty) are HOST arrays of w*h int32,
 * row-major; they are uploaded first (outside every timed span, as the
 * reference's callers do before GC_Init, solveMRF.cu:70-86).  label (host,
 * w*h int32) receives the reference's labels.  Returns 0 when the
 * reference's termination test ended the solve, 3 when max_iters main-loop
 * iterations or max_seconds passed first (labels then not computed), 4 when
 * the kernels were not loaded. */
int refgpu_solve(int w, int h, const int *dp, const int *dn, int penalty, const int *up, const int *down,
                 const int *left, const int *right, int *label, long long max_iters, double max_seconds,
                 refgpu_stats *st) {
    const int *edges[4] = {up, down, left, right};
    return solve<4>(g_k4, w, h, dp, dn, penalty, up ? edges : nullptr, label, max_iters, max_seconds, st);
}

/* The same with NEIGHBORHOOD 8: edges8 == NULL selects the constant penalty,
 * else it points to the eight host arrays up, down, left, right, upleft,
 * upright, downleft, downright (GraphCut.cu:187-194). */
int refgpu_solve8(int w, int h, const int *dp, const int *dn, int penalty, const int *const *edges8, int *label,
                  long long max_iters, double max_seconds, refgpu_stats *st) {
    return solve<8>(g_k8, w, h, dp, dn, penalty, edges8, label, max_iters, max_seconds, st);
}

}  // extern "C"

namespace {

// The data-term kernels (DataTermKernels.cu) and the launch shapes
// DataTerm::init_data_term sets up (DataTerm.cpp:34-50).
struct DtKernels {
    cudaLibrary_t lib = nullptr;
    cudaKernel_t gauss, init_map, init_cs, select, calc, draw;
};
DtKernels g_dt;
constexpr int DT_N_PDF = 256;

int dt_ready() { return g_dt.lib ? OK : ERR_NOT_LOADED; }

}  // namespace

extern "C" {

/* Loads the reference's data-term kernels from their cubin. */
int refgpu_load_dt(const char *cubin_path) {
    if (g_dt.lib) return OK;
    if (!cubin_path) return ERR_INVALID;
    cudaLibrary_t lib;
    if (cudaLibraryLoadFromFile(&lib, cubin_path, nullptr, nullptr, 0, nullptr, nullptr, 0) != cudaSuccess)
        return ERR_CUDA;
    bool ok = cudaLibraryGetKernel(&g_dt.gauss, lib, "_Z14K_InitGaussianfPf") == cudaSuccess;
    ok = ok && cudaLibraryGetKernel(&g_dt.init_map, lib, "_Z18K_InitSelectionMapPhi") == cudaSuccess;
    ok = ok && cudaLibraryGetKernel(&g_dt.init_cs, lib, "_Z16K_InitColorSpacePfi") == cudaSuccess;
    ok = ok && cudaLibraryGetKernel(&g_dt.select, lib, "_Z16K_SelectAndGaussPhS_PfS0_iiii") == cudaSuccess;
    ok = ok && cudaLibraryGetKernel(&g_dt.calc, lib, "_Z11K_CalcTermsPhPfPiS1_i") == cudaSuccess;
    ok = ok && cudaLibraryGetKernel(&g_dt.draw, lib, "_Z9K_DrawMapPhS_i") == cudaSuccess;
    if (!ok) {
        cudaLibraryUnload(lib);
        return ERR_CUDA;
    }
    g_dt.lib = lib;
    return OK;
}

/* The reference's kernel-density data term on the GPU, driven as
 * DataTerm.cpp does: init_data_term (K_InitGaussian with the default sigma 5,
 * reset = K_InitSelectionMap + K_InitColorSpace), setImage, then
 * setSigmaGaussian(sigma) when sigma > 0, selectOnMap for every point
 * (25 K_SelectAndGauss launches over the 256^3 colour cube, one per pixel of
 * the 5x5 square at (x, y)), getDataTermsMixture (K_CalcTerms).  Host
 * buffers: img (h*w*3 bytes, the reference's channel order), pts (npts (x, y)
 * pairs); outputs pos, neg (w*h int32), gauss (the 101 table entries) and map
 * (w*h bytes, the selection map).
 * The reference's kernels cover floor(w/16)*16 x floor(h/16)*16 pixels and
 * selectOnMap writes past the image when the square does not fit, so w and
 * h must be multiples of 16 and every square must lie inside the image
 * (else 1, before any GPU work). */
int refgpu_kde(int w, int h, const unsigned char *img, int sigma, int npts, const int *pts, int *pos, int *neg,
               float *gauss, unsigned char *map) {
    if (dt_ready() != OK) return ERR_NOT_LOADED;
    if (w < 16 || h < 16 || w % 16 || h % 16 || !img || npts < 0 || (npts && !pts) || !pos || !neg) return ERR_INVALID;
    for (int k = 0; k < npts; ++k)
        if (pts[2 * k] < 0 || pts[2 * k + 1] < 0 || pts[2 * k] + 5 > w || pts[2 * k + 1] + 5 > h) return ERR_INVALID;
    const size_t n = (size_t)w * h;
    unsigned char *d_img = nullptr, *d_map = nullptr;
    float *d_gauss = nullptr, *d_pdf = nullptr;
    int *d_pos = nullptr, *d_neg = nullptr;
    int rc = OK;
    const dim3 t3(8, 8, 8), b3(DT_N_PDF / 8, DT_N_PDF / 8, DT_N_PDF / 8);  // DataTerm.cpp:34-40
    const dim3 t2(16, 16, 1), b2(w / 16, h / 16, 1);                       // :42-49
    const dim3 blin(256 * 3 / 16, 1, 1);                                    // :51-52
    TRY(cudaMalloc(&d_img, 3 * n));
    TRY(cudaMalloc(&d_gauss, sizeof(float) * DT_N_PDF));
    TRY(cudaMalloc(&d_pdf, sizeof(float) * DT_N_PDF * DT_N_PDF * DT_N_PDF));
    TRY(cudaMalloc(&d_map, n));
    TRY(cudaMalloc(&d_pos, sizeof(int) * n));
    TRY(cudaMalloc(&d_neg, sizeof(int) * n));
    {
        float s0 = 5.0f;  // DEFAULT_SIGMA (DataTerm.cpp:6)
        int npdf = DT_N_PDF, width = w;
        void *ag[] = {&s0, &d_gauss};
        TRY(cudaLaunchKernel((const void *)g_dt.gauss, blin, t2, ag, 0, 0));
        void *am[] = {&d_map, &width};
        TRY(cudaLaunchKernel((const void *)g_dt.init_map, b2, t2, am, 0, 0));
        void *ac[] = {&d_pdf, &npdf};
        TRY(cudaLaunchKernel((const void *)g_dt.init_cs, b3, t3, ac, 0, 0));
        TRY(cudaMemcpy(d_img, img, 3 * n, cudaMemcpyHostToDevice));
        if (sigma > 0) {
            float sg = (float)sigma;
            void *as[] = {&sg, &d_gauss};
            TRY(cudaLaunchKernel((const void *)g_dt.gauss, blin, t2, as, 0, 0));
        }
        int rect = 8;
        for (int k = 0; k < npts; ++k)
            for (int i = 0; i < 5; ++i)
                for (int j = 0; j < 5; ++j) {
                    int x1 = pts[2 * k] + i, y1 = pts[2 * k + 1] + j;
                    void *a[] = {&d_map, &d_img, &d_pdf, &d_gauss, &x1, &y1, &rect, &width};
                    TRY(cudaLaunchKernel((const void *)g_dt.select, b3, t3, a, 0, 0));
                }
        void *at[] = {&d_img, &d_pdf, &d_pos, &d_neg, &width};
        TRY(cudaLaunchKernel((const void *)g_dt.calc, b2, t2, at, 0, 0));
        TRY(cudaMemcpy(pos, d_pos, sizeof(int) * n, cudaMemcpyDeviceToHost));
        TRY(cudaMemcpy(neg, d_neg, sizeof(int) * n, cudaMemcpyDeviceToHost));
        if (gauss) TRY(cudaMemcpy(gauss, d_gauss, sizeof(float) * 101, cudaMemcpyDeviceToHost));
        if (map) TRY(cudaMemcpy(map, d_map, n, cudaMemcpyDeviceToHost));
    }
done:
    cudaFree(d_img);
    cudaFree(d_gauss);
    cudaFree(d_pdf);
    cudaFree(d_map);
    cudaFree(d_pos);
    cudaFree(d_neg);
    if (rc == OK && cudaGetLastError() != cudaSuccess) rc = ERR_CUDA;
    return rc;
}

/* DataTerm::drawSelection (DataTerm.cpp:155-165): the input image is copied
 * to the device, K_DrawMap paints the pixels whose selection-map entry is 1,
 * and the result comes back.  map: w*h bytes (host), in, out: h*w*3 bytes;
 * w and h multiples of 16 as for refgpu_kde. */
int refgpu_draw(int w, int h, const unsigned char *map, const unsigned char *in, unsigned char *out) {
    if (dt_ready() != OK) return ERR_NOT_LOADED;
    if (w < 16 || h < 16 || w % 16 || h % 16 || !map || !in || !out) return ERR_INVALID;
    const size_t n = (size_t)w * h;
    unsigned char *d_img = nullptr, *d_map = nullptr;
    int rc = OK;
    int width = w;
    const dim3 t2(16, 16, 1), b2(w / 16, h / 16, 1);
    TRY(cudaMalloc(&d_img, 3 * n));
    TRY(cudaMalloc(&d_map, n));
    TRY(cudaMemcpy(d_map, map, n, cudaMemcpyHostToDevice));
    TRY(cudaMemcpy(d_img, in, 3 * n, cudaMemcpyHostToDevice));
    {
        void *a[] = {&d_map, &d_img, &width};
        TRY(cudaLaunchKernel((const void *)g_dt.draw, b2, t2, a, 0, 0));
    }
    TRY(cudaMemcpy(out, d_img, 3 * n, cudaMemcpyDeviceToHost));
done:
    cudaFree(d_img);
    cudaFree(d_map);
    if (rc == OK && cudaGetLastError() != cudaSuccess) rc = ERR_CUDA;
    return rc;
}

}  // extern "C"
