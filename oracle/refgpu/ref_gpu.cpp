/* The reference's CUDA path on the GPU: test and benchmark infrastructure.
 *
 * The device code is the reference's own (GraphCutKernels.cu, compiled from
 * the reference checkout into gc_ref_kernels.cubin by build_ref_gpu.sh).  The
 * reference's host code (GraphCut.cu) is compiled into every application
 * and cannot be rebuilt where its sources are absent, so this file restates
 * it, launch for launch, over the cubin's kernels:
 *
 *   refgpu_solve  = GC_Init (GraphCut.cu:187-263: padded sizes, eleven
 *                   allocations) + GC_SetGraph (:301-319) + GC_Optimize
 *                   (:385-534) + GC_End (:542-568)
 *   get_energy    = getEnergy (GraphCut.cu:359-376)
 *
 * Differences, all outside the timed arithmetic: every loop is bounded (an
 * iteration cap and a wall-clock cap, reported through the status instead of
 * spinning forever, GraphCut.cu:414,465,517 are unbounded), errors are
 * returned instead of exit(), and nothing is printed.  The launch order, the
 * blocking copies of the alive flag every ACTIVITY_CHECK_FREQUENCY
 * iterations and around every GlobalRelabel / SpreadLabels launch, and the
 * global-relabel schedule are the reference's.
 *
 * The kernels take the reference's KernelWrapper by value; RKernel below has
 * the same members in the same order (GraphCut.h:60-105, NEIGHBORHOOD 4),
 * hence the same 120-byte layout on every LP64 host and on the device.
 */
#include <cuda_runtime.h>

#include <chrono>
#include <cmath>
#include <cstring>

namespace {

struct RNode {
    int *edge_l, *edge_r, *edge_u, *edge_d;
    int *height, *excess, *status, *comp_h, *comp_n, *energy_sum;
};
struct RGraph {
    int width, height, size, width_ex, height_ex, size_ex;
    RNode n;
};
struct RKernel {
    int block_x;
    int *active;
    RGraph g;
};
static_assert(sizeof(RKernel) == 120, "KernelWrapper layout (GraphCut.h:60-105)");

// GraphCut.h:43-48 and :144-157
constexpr int TX = 32, TY = 8;
constexpr int ACTIVITY_CHECK = 10, GR_FREQUENCY = 100, GR_FIRST = 100;

cudaLibrary_t g_lib = nullptr;
cudaKernel_t k_init, k_init_var, k_relabel, k_push, k_activity, k_init_gr, k_gr, k_energy,
    k_init_labels, k_spread;

// Itanium-mangled names of the reference's kernels (GraphCutKernels.cu)
struct Named {
    cudaKernel_t *k;
    const char *name;
};
const Named kNames[] = {
    {&k_init, "_Z9InitGraph13KernelWrapperPiS0_i"},
    {&k_init_var, "_Z17InitGraphVarEdges13KernelWrapperPiS0_S0_S0_S0_S0_"},
    {&k_relabel, "_Z7Relabel13KernelWrapperi"},
    {&k_push, "_Z8WavePush13KernelWrapperiPi"},
    {&k_activity, "_Z14UpdateActivityPiS_iiS_"},
    {&k_init_gr, "_Z17InitGlobalRelabel13KernelWrapper"},
    {&k_gr, "_Z13GlobalRelabel13KernelWrapperPi"},
    {&k_energy, "_Z11EnergyLevel13KernelWrapperiiPiS0_b"},
    {&k_init_labels, "_Z10InitLabels13KernelWrapperPi"},
    {&k_spread, "_Z12SpreadLabels13KernelWrapperPiS0_"},
};

enum { OK = 0, ERR_INVALID = 1, ERR_CUDA = 2, ERR_CAP = 3, ERR_NOT_LOADED = 4 };

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
cudaError_t get_energy(RKernel k, dim3 grid, int *source, int *dest, bool limited) {
    int odd = 0;
    int stride = limited ? k.g.size : k.g.size_ex;
    int *out = k.g.n.energy_sum;
    for (;; odd = stride % 2, stride = (stride + 1) / 2) {
        if (stride == 1) odd = 0;
        void *a[] = {&k, &stride, &odd, &source, &out, &limited};
        cudaError_t e = launch(k_energy, grid, a);
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

/* Loads the reference's kernels from the cubin.  Returns 0, or 2 when the
 * file cannot be loaded or a kernel is missing. */
int refgpu_load(const char *cubin_path) {
    if (g_lib) return OK;
    if (!cubin_path) return ERR_INVALID;
    cudaLibrary_t lib;
    if (cudaLibraryLoadFromFile(&lib, cubin_path, nullptr, nullptr, 0, nullptr, nullptr, 0) != cudaSuccess)
        return ERR_CUDA;
    for (const Named &n : kNames) {
        if (cudaLibraryGetKernel(n.k, lib, n.name) != cudaSuccess) {
            cudaLibraryUnload(lib);
            return ERR_CUDA;
        }
    }
    g_lib = lib;
    return OK;
}

/* One solve through the reference's CUDA path.  dp/dn (and up/down/left/right
 * when up != NULL, else the constant penalty) are HOST arrays of w*h int32,
 * row-major; they are uploaded first (outside every timed span, as the
 * reference's callers do before GC_Init, solveMRF.cu:70-86).  label (host,
 * w*h int32) receives the reference's labels.  Returns 0 when the
 * reference's termination test ended the solve, 3 when max_iters main-loop
 * iterations or max_seconds passed first (labels then not computed). */
int refgpu_solve(int w, int h, const int *dp, const int *dn, int penalty, const int *up,
                 const int *down, const int *left, const int *right, int *label,
                 long long max_iters, double max_seconds, refgpu_stats *st) {
    if (!g_lib) return ERR_NOT_LOADED;
    if (w < 1 || h < 1 || !dp || !dn || !label || !st) return ERR_INVALID;
    if ((long long)w * h > (1LL << 28)) return ERR_INVALID;
    std::memset(st, 0, sizeof(*st));
    const bool var = up != nullptr;
    if (var && (!down || !left || !right)) return ERR_INVALID;
    const size_t n = (size_t)w * h;
    int rc = OK;
    int *d_in[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    const int *h_in[6] = {dp, dn, up, down, left, right};
    int *owned[11] = {};
    int *d_alive = nullptr, *d_label = nullptr;
    int zero_arr[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    int h_alive[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    RKernel k;
    std::memset(&k, 0, sizeof(k));
    dim3 grid;
    Clock::time_point t0;

    for (int i = 0; i < (var ? 6 : 2); ++i) {
        TRY(cudaMalloc((void **)&d_in[i], n * sizeof(int)));
        TRY(cudaMemcpy(d_in[i], h_in[i], n * sizeof(int), cudaMemcpyHostToDevice));
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
        int **fields[10] = {&k.g.n.edge_u, &k.g.n.edge_d, &k.g.n.edge_l, &k.g.n.edge_r, &k.g.n.height,
                            &k.g.n.excess, &k.g.n.status, &k.g.n.comp_h, &k.g.n.comp_n, &k.g.n.energy_sum};
        for (int i = 0; i < 10; ++i) {
            TRY(cudaMalloc((void **)fields[i], sizeof(int) * k.g.size_ex));
            owned[i] = *fields[i];
        }
        TRY(cudaMalloc((void **)&k.active, sizeof(int) * block_count));
        owned[10] = k.active;
    }
    TRY(cudaDeviceSynchronize());
    st->ms_init = ms_since(t0);

    // ---- GC_SetGraph (GraphCut.cu:301-319) + GC_Optimize (:385-534)
    t0 = Clock::now();
    if (var) {
        void *a[] = {&k, &d_in[0], &d_in[1], &d_in[2], &d_in[3], &d_in[4], &d_in[5]};
        TRY(launch(k_init_var, grid, a));
    } else {
        void *a[] = {&k, &d_in[0], &d_in[1], &penalty};
        TRY(launch(k_init, grid, a));
    }
    TRY(cudaMalloc((void **)&d_alive, 8 * sizeof(int)));
    TRY(get_energy(k, grid, d_in[0], h_alive, true));
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
                TRY(launch(k_relabel, grid, a));
            }
            {
                int s = skip;
                void *a[] = {&k, &s, &d_alive};
                TRY(launch(k_push, grid, a));
            }
            if (!skip) {
                int bx = k.block_x, wex = k.g.width_ex;
                void *a[] = {&k.g.n.status, &k.active, &bx, &wex, &d_alive};
                TRY(launch(k_activity, grid, a));
                TRY(cudaMemcpy(h_alive, d_alive, 8 * sizeof(int), cudaMemcpyDeviceToHost));
            }
            if (!h_alive[0]) {
                TRY(cudaDeviceSynchronize());
                st->ms_loop = ms_since(t_loop);
                TRY(get_energy(k, grid, k.g.n.excess, h_alive, false));
                st->final_energy = st->initial_energy - h_alive[0];
                st->converged = 1;
                break;
            }
            if (!((counter - GR_FIRST) % GR_FREQUENCY)) {
                void *a0[] = {&k};
                TRY(launch(k_init_gr, grid, a0));
                st->global_relabels++;
                for (;;) {
                    TRY(cudaMemcpy(d_alive, zero_arr, 8 * sizeof(int), cudaMemcpyHostToDevice));
                    void *a[] = {&k, &d_alive};
                    TRY(launch(k_gr, grid, a));
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
        TRY(launch(k_init_labels, grid, a));
    }
    for (;;) {
        TRY(cudaMemcpy(d_alive, zero_arr, 8 * sizeof(int), cudaMemcpyHostToDevice));
        void *a[] = {&k, &d_label, &d_alive};
        TRY(launch(k_spread, grid, a));
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

}  // extern "C"
