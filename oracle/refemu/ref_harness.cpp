/*
 * ref_harness.cpp -- drives the reference's own host API (GC_Init,
 * GC_Optimize, GC_End from GraphCut.cu:187-568) on one instance, the way the
 * reference's solveMRF.cu:105-111 and Debug.cu:83-88 do, and writes the
 * label array it returns.  Linked against the reference's GraphCut.cu
 * compiled for the CPU thread emulator.  Test infrastructure only.
 *
 * Input file (little-endian int32): W, H, mode (0 = constant penalty,
 * 1 = per-direction arrays), penalty, dp[W*H], dn[W*H], and in mode 1
 * up[W*H], down[W*H], left[W*H], right[W*H].
 * Output file: label[W*H] int32.  The reference's own printf output
 * ("Final energy level: ...") goes to stdout.
 */
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "GraphCut.h"

GlobalWrapper GC_Init(int width, int height, int *data_positive, int *data_negative, int penalty,
                      int *up, int *down, int *left, int *right);
void GC_Optimize(GlobalWrapper gw, int *label);
void GC_End(GlobalWrapper *gw);

static bool read_ints(FILE *f, int *dst, size_t n) { return std::fread(dst, sizeof(int), n, f) == n; }

int main(int argc, char **argv) {
    if (argc != 3) {
        std::fprintf(stderr, "usage: %s instance.bin labels.bin\n", argv[0]);
        return 1;
    }
    FILE *f = std::fopen(argv[1], "rb");
    if (!f) return 1;
    int hdr[4];
    if (!read_ints(f, hdr, 4)) return 1;
    int W = hdr[0], H = hdr[1], mode = hdr[2], penalty = hdr[3];
    size_t n = (size_t)W * H;
    std::vector<int> dp(n), dn(n), up, down, left, right;
    if (!read_ints(f, dp.data(), n) || !read_ints(f, dn.data(), n)) return 1;
    if (mode == 1) {
        up.resize(n); down.resize(n); left.resize(n); right.resize(n);
        if (!read_ints(f, up.data(), n) || !read_ints(f, down.data(), n) ||
            !read_ints(f, left.data(), n) || !read_ints(f, right.data(), n))
            return 1;
    }
    std::fclose(f);
    /* "device" copies, as the reference's callers make (solveMRF.cu:79-90) */
    int *d_dp, *d_dn, *d_up = nullptr, *d_down = nullptr, *d_left = nullptr, *d_right = nullptr;
    cudaMalloc((void **)&d_dp, n * sizeof(int));
    cudaMalloc((void **)&d_dn, n * sizeof(int));
    cudaMemcpy(d_dp, dp.data(), n * sizeof(int), cudaMemcpyHostToDevice);
    cudaMemcpy(d_dn, dn.data(), n * sizeof(int), cudaMemcpyHostToDevice);
    if (mode == 1) {
        cudaMalloc((void **)&d_up, n * sizeof(int));
        cudaMalloc((void **)&d_down, n * sizeof(int));
        cudaMalloc((void **)&d_left, n * sizeof(int));
        cudaMalloc((void **)&d_right, n * sizeof(int));
        cudaMemcpy(d_up, up.data(), n * sizeof(int), cudaMemcpyHostToDevice);
        cudaMemcpy(d_down, down.data(), n * sizeof(int), cudaMemcpyHostToDevice);
        cudaMemcpy(d_left, left.data(), n * sizeof(int), cudaMemcpyHostToDevice);
        cudaMemcpy(d_right, right.data(), n * sizeof(int), cudaMemcpyHostToDevice);
    }
    GlobalWrapper gw = GC_Init(W, H, d_dp, d_dn, penalty, d_up, d_down, d_left, d_right);
    std::vector<int> label(n, 0);
    GC_Optimize(gw, label.data());
    GC_End(&gw);
    std::printf("emu: launches %lld barriers %lld\n", emu_launch_count, emu_barrier_count);
    FILE *o = std::fopen(argv[2], "wb");
    if (!o) return 1;
    std::fwrite(label.data(), sizeof(int), n, o);
    std::fclose(o);
    return 0;
}
