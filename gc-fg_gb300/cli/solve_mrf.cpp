// solve_mrf -- solve a two-label MRF file on the GPU, the way the
// reference's solveMRF program does (solveMRF.cu:69-141): the same input
// format, the same graph (up = down = vertical cue, left = right = horizontal
// cue of each pixel), the same console lines and the same labelMRF.ppm.
// Written against the GraphCut.h front end, so it is also a reference-style
// caller of this library.
//
//   solve_mrf MRF_file [output.ppm]      (default output: labelMRF.ppm)
#include <cstdio>
#include <vector>

#include "GraphCut.h"
#include "mrf_io.hpp"

int main(int argc, char **argv) {
    if (argc != 2 && argc != 3) {
        std::printf("Usage: %s MRF_file [output.ppm]\n", argv[0]);
        return 1;
    }
    gcfg_cli::Mrf m;
    try {
        m = gcfg_cli::read_mrf(argv[1]);
    } catch (const std::exception &e) {
        std::fprintf(stderr, "%s\n", e.what());
        return 1;
    }
    const size_t n = (size_t)m.W * m.H;
    int *d[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    const std::vector<int> *src[6] = {&m.dp, &m.dn, &m.vcue, &m.vcue, &m.hcue, &m.hcue};
    for (int k = 0; k < 6; ++k) {
        CUDA_SAFE_CALL(cudaMalloc((void **)&d[k], sizeof(int) * n));
        CUDA_SAFE_CALL(cudaMemcpy(d[k], src[k]->data(), sizeof(int) * n, cudaMemcpyHostToDevice));
    }
    std::printf("Solving a %d x %d MRF problem...\n", m.H, m.W);
    GlobalWrapper gw = GC_Init(m.W, m.H, d[0], d[1], 0, d[2], d[3], d[4], d[5]);
    std::vector<int> label(n);
    GC_Optimize(gw, label.data());
    try {
        gcfg_cli::write_label_ppm(argc == 3 ? argv[2] : "labelMRF.ppm", label, m.W, m.H);
    } catch (const std::exception &e) {
        std::fprintf(stderr, "%s\n", e.what());
        return 1;
    }
    for (int k = 0; k < 6; ++k) CUDA_SAFE_CALL(cudaFree(d[k]));
    GC_End(&gw);
    return 0;
}
