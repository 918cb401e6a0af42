/*
 * ref_harness8.cpp -- drives the reference's host API (GC_Init, GC_Optimize,
 * GC_End, GraphCut.cu:187-568) built with NEIGHBORHOOD == 8 on one instance
 * and writes the labels it returns.  Compiled after the reference's
 * GraphCut.h with its NEIGHBORHOOD switched to 8 (see build_ref.sh), so that
 * the wrapper structs match the solver's.  Test infrastructure only.
 *
 * Input file (little-endian int32): W, H, mode (0 = constant penalty,
 * 1 = per-direction arrays), penalty, dp[W*H], dn[W*H], and in mode 1 the
 * eight arrays up, down, left, right, upleft, upright, downleft, downright
 * (W*H each).  Output file: label[W*H] int32.
 */
#include <cstdio>
#include <vector>

#include "GraphCut.h"

GlobalWrapper GC_Init(int width, int height, int *data_positive, int *data_negative, int penalty, int *up,
                      int *down, int *left, int *right, int *upleft, int *upright, int *downleft, int *downright);
void GC_Optimize(GlobalWrapper gw, int *label);
void GC_End(GlobalWrapper *gw);

int main(int argc, char **argv) {
    if (argc != 3) {
        std::fprintf(stderr, "usage: %s instance.bin labels.bin\n", argv[0]);
        return 1;
    }
    FILE *f = std::fopen(argv[1], "rb");
    if (!f) return 1;
    int hdr[4];
    if (std::fread(hdr, sizeof(int), 4, f) != 4) return 1;
    const int W = hdr[0], H = hdr[1], mode = hdr[2], penalty = hdr[3];
    const size_t n = (size_t)W * H;
    std::vector<int> host((2 + (mode == 1 ? 8 : 0)) * n);
    if (std::fread(host.data(), sizeof(int), host.size(), f) != host.size()) return 1;
    std::fclose(f);
    std::vector<int *> dev(10, nullptr);
    for (size_t k = 0; k * n < host.size(); ++k) {
        cudaMalloc((void **)&dev[k], n * sizeof(int));
        cudaMemcpy(dev[k], host.data() + k * n, n * sizeof(int), cudaMemcpyHostToDevice);
    }
    GlobalWrapper gw = GC_Init(W, H, dev[0], dev[1], penalty, dev[2], dev[3], dev[4], dev[5], dev[6], dev[7],
                               dev[8], dev[9]);
    std::vector<int> label(n, 0);
    GC_Optimize(gw, label.data());
    GC_End(&gw);
    FILE *o = std::fopen(argv[2], "wb");
    if (!o) return 1;
    std::fwrite(label.data(), sizeof(int), n, o);
    std::fclose(o);
    return 0;
}
