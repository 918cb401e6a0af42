// noalloc.cu -- gcfg_solve_noalloc: the graph solve without any allocation.
//
// Some callers cannot allocate device memory when they solve: a host
// framework that owns all of the GPU's memory and forbids its plug-ins to
// call cudaMalloc, a process that is already at its device-memory limit, or a
// latency-bound loop that cannot afford cudaMalloc/cudaFree (both can
// synchronise the whole device).  This entry point solves one graph with all
// of its working memory (tile arena, work queues, counters) in one fixed
// file-scope device array.  It runs the same kernels as gcfg_init +
// gcfg_optimize; only where the working memory comes from differs.
//
// Limits and rules:
//   * the image may have at most GCFG_NOALLOC_MAX_TILES 32x32 tiles
//     (ceil(w/32) * ceil(h/32) <= 640, e.g. 1024x640 or 800x800 pixels);
//     larger sizes are refused with GCFG_ERR_TOO_LARGE;
//   * the array (GCFG_NOALLOC_SCRATCH_BYTES, 16 MiB) exists on every GPU that
//     loads the library, until the process exits;
//   * every call shares the array and leaves its contents behind; the parts
//     that must start from zero are cleared by each call;
//   * two calls whose GPU work overlaps (e.g. on two streams) race on the
//     array: serialise them;
//   * every call looks up the array's device address on the current device
//     (cudaGetSymbolAddress, which allocates nothing), so a context that was
//     reset or recreated since the last call never receives a stale address;
//   * the call synchronises its stream twice (it reads back the capacity
//     check after the build and the flow after the solve) and returns after
//     the solve has finished.
#include "engine.cuh"

namespace gcfg {

namespace {

constexpr size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

constexpr size_t T = GCFG_NOALLOC_MAX_TILES;
// carve-up of the array (offsets in bytes, each 256-byte aligned)
constexpr size_t OFF_CAP = 0;
constexpr size_t OFF_EXC = OFF_CAP + align256(T * TPX * sizeof(int4));
constexpr size_t OFF_H = OFF_EXC + align256(T * TPX * sizeof(int));
constexpr size_t OFF_HB = OFF_H + align256(T * TPX * sizeof(int));
constexpr size_t OFF_TNB = OFF_HB + align256(T * 4 * 32 * sizeof(int));
constexpr size_t OFF_HFIN = OFF_TNB + align256(T * sizeof(int4));
constexpr size_t OFF_REACH = OFF_HFIN + align256(T * 32 * sizeof(unsigned));
constexpr size_t OFF_TMASK = OFF_REACH + align256(T * 32 * sizeof(unsigned));
constexpr size_t OFF_TACT = OFF_TMASK + align256(T * 6 * 32 * sizeof(unsigned));
constexpr size_t OFF_TPOS = OFF_TACT + align256(T * sizeof(int));
constexpr size_t OFF_LISTS = OFF_TPOS + align256(T * sizeof(unsigned long long));
constexpr size_t OFF_MPUSH = OFF_LISTS + align256((size_t)L_NLISTS * T * sizeof(int));
constexpr size_t OFF_MGR = OFF_MPUSH + align256(T * sizeof(int));
constexpr size_t OFF_TIMG = OFF_MGR + align256(T * sizeof(int));
constexpr size_t OFF_IMG = OFF_TIMG + align256(T * sizeof(int));
constexpr size_t OFF_IST = OFF_IMG + align256(sizeof(ImgDesc));
constexpr size_t OFF_CTL = OFF_IST + align256(sizeof(ImgState));
constexpr size_t NEEDED = OFF_CTL + align256(sizeof(Ctl));
static_assert(NEEDED <= GCFG_NOALLOC_SCRATCH_BYTES, "scratch array too small for its tile limit");

// The working memory.  In host code this name is only a handle for
// cudaGetSymbolAddress, never an address the GPU can use.
static __device__ __align__(256) unsigned char g_noalloc_scratch[GCFG_NOALLOC_SCRATCH_BYTES];

// Device address of the array in the current device's context.  Looked up
// on every call, not cached: after cudaDeviceReset or a recreated primary
// context the module is loaded again and the array may move.
gcfg_status scratch_address(unsigned char **out) {
    void *p = nullptr;
    GCFG_CK(cudaGetSymbolAddress(&p, g_noalloc_scratch));
    if (!p) return GCFG_ERR_CUDA;
    *out = static_cast<unsigned char *>(p);
    return GCFG_OK;
}

// Descriptor of the single image and its tile -> image map, written on the
// device so that the call needs no host staging buffer.
__global__ void k_noalloc_layout(ImgDesc *img, int *tile_img, int W, int H) {
    const int tiles_x = (W + TILE_W - 1) / TILE_W, tiles_y = (H + TILE_H - 1) / TILE_H;
    const int n = tiles_x * tiles_y;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        ImgDesc d;
        d.W = W;
        d.H = H;
        d.tiles_x = tiles_x;
        d.tiles_y = tiles_y;
        d.tile0 = 0;
        d.n_tiles = n;
        d.pix0 = 0;
        d.lambda = 0.0;
        d.out0 = 0;
        *img = d;
    }
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) tile_img[t] = 0;
}

}  // namespace
}  // namespace gcfg

using namespace gcfg;

extern "C" gcfg_status gcfg_solve_noalloc(int w, int h, const int32_t *d_dp, const int32_t *d_dn,
                                          int32_t penalty, const int32_t *d_up, const int32_t *d_down,
                                          const int32_t *d_left, const int32_t *d_right, int32_t *d_label,
                                          int64_t *h_flow, void *stream) {
    if (w <= 0 || h <= 0 || !d_dp || !d_dn || !d_label) return GCFG_ERR_INVALID;
    if (d_up && (!d_down || !d_left || !d_right)) return GCFG_ERR_INVALID;
    if (penalty < 0 || penalty > GCFG_MAX_CAP) return GCFG_ERR_INVALID;
    const long long tiles = (long long)((w + TILE_W - 1) / TILE_W) * ((h + TILE_H - 1) / TILE_H);
    if (tiles > GCFG_NOALLOC_MAX_TILES) return GCFG_ERR_TOO_LARGE;
    cudaStream_t st = (cudaStream_t)stream;
    unsigned char *base = nullptr;
    GCFG_TRY(scratch_address(&base));

    Batch b;
    b.n_img = 1;
    b.n_tiles = (int)tiles;
    b.tlist = nullptr;
    b.n_tlist = 0;
    b.ilist = nullptr;
    b.n_ilist = 0;
    b.img = reinterpret_cast<const ImgDesc *>(base + OFF_IMG);
    b.ist = reinterpret_cast<ImgState *>(base + OFF_IST);
    b.tile_img = reinterpret_cast<const int *>(base + OFF_TIMG);
    b.cap = reinterpret_cast<int4 *>(base + OFF_CAP);
    b.exc = reinterpret_cast<int *>(base + OFF_EXC);
    b.h = reinterpret_cast<int *>(base + OFF_H);
    b.hb = reinterpret_cast<int *>(base + OFF_HB);
    b.tile_nb = reinterpret_cast<int4 *>(base + OFF_TNB);
    b.hfin = reinterpret_cast<unsigned *>(base + OFF_HFIN);
    b.reach = reinterpret_cast<unsigned *>(base + OFF_REACH);
    b.tmask = reinterpret_cast<unsigned *>(base + OFF_TMASK);
    b.tile_act = reinterpret_cast<int *>(base + OFF_TACT);
    b.tile_pos = reinterpret_cast<unsigned long long *>(base + OFF_TPOS);
    b.lists = reinterpret_cast<int *>(base + OFF_LISTS);
    b.list_cap = (int)GCFG_NOALLOC_MAX_TILES;
    b.mark_push = reinterpret_cast<int *>(base + OFF_MPUSH);
    b.mark_gr = reinterpret_cast<int *>(base + OFF_MGR);
    b.ctl = reinterpret_cast<Ctl *>(base + OFF_CTL);

    // what must start from zero: the image's counters and the control block
    GCFG_CK(cudaMemsetAsync(base + OFF_IST, 0, sizeof(ImgState), st));
    GCFG_CK(cudaMemsetAsync(base + OFF_CTL, 0, sizeof(Ctl), st));
    k_noalloc_layout<<<1, 256, 0, st>>>(reinterpret_cast<ImgDesc *>(base + OFF_IMG),
                                        reinterpret_cast<int *>(base + OFF_TIMG), w, h);
    g_launches.fetch_add(1, std::memory_order_relaxed);
    GCFG_CK(cudaGetLastError());
    GCFG_TRY(launch_build_arrays(b, d_dp, d_dn, penalty, d_up, d_down, d_left, d_right, st));
    int err = 0;
    GCFG_CK(cudaMemcpyAsync(&err, base + OFF_CTL + offsetof(Ctl, err), sizeof(int), cudaMemcpyDeviceToHost, st));
    GCFG_CK(cudaStreamSynchronize(st));
    if (err) return GCFG_ERR_INVALID;  // capacities outside [0, GCFG_MAX_CAP]

    GCFG_CK(cudaMemsetAsync(base + OFF_CTL, 0, sizeof(Ctl), st));
    SolveParams prm = kDefaultSolveParams;
    GCFG_TRY(launch_solve(b, prm, (int)tiles, st));
    GCFG_TRY(launch_extract(b, nullptr, nullptr, d_label, st));
    ImgState s;
    GCFG_CK(cudaMemcpyAsync(&err, base + OFF_CTL + offsetof(Ctl, err), sizeof(int), cudaMemcpyDeviceToHost, st));
    GCFG_CK(cudaMemcpyAsync(&s, base + OFF_IST, sizeof(ImgState), cudaMemcpyDeviceToHost, st));
    GCFG_CK(cudaStreamSynchronize(st));
    if (err) return GCFG_ERR_NOT_CONVERGED;
    if (h_flow) *h_flow = (long long)s.interior_dp - (long long)s.pos_excess;
    return GCFG_OK;
}
