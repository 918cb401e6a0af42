// segment_dat -- the reference's demo application (Application.cu:9-86) on
// the GPU: t-links from a ".dat" file ("H W", W*H sink then W*H source
// t-links), a constant n-link penalty, and an overlay of the result on an
// ASCII PPM image (the image's colour where the label is 1, black elsewhere).
//
//   segment_dat [t-links.dat [image.ppm [penalty [output.ppm]]]]
//   defaults: rihanna.dat rihanna.ppm 600 label.ppm, as the reference uses
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "GraphCut.h"
#include "mrf_io.hpp"

int main(int argc, char **argv) {
    const std::string dat = argc > 1 ? argv[1] : "rihanna.dat";
    const std::string ppm = argc > 2 ? argv[2] : "rihanna.ppm";
    const int penalty = argc > 3 ? std::atoi(argv[3]) : 600;
    const std::string out = argc > 4 ? argv[4] : "label.ppm";
    int W = 0, H = 0, iw = 0, ih = 0;
    std::vector<int> dp, dn, rgb;
    try {
        gcfg_cli::read_dat(dat, W, H, dp, dn);
        rgb = gcfg_cli::read_ppm_ascii(ppm, iw, ih);
    } catch (const std::exception &e) {
        std::fprintf(stderr, "%s\n", e.what());
        return 1;
    }
    if (iw != W || ih != H) {
        std::fprintf(stderr, "%s is %dx%d but %s is %dx%d\n", ppm.c_str(), iw, ih, dat.c_str(), W, H);
        return 1;
    }
    const size_t n = (size_t)W * H;
    int *d_dp = nullptr, *d_dn = nullptr;
    CUDA_SAFE_CALL(cudaMalloc((void **)&d_dp, sizeof(int) * n));
    CUDA_SAFE_CALL(cudaMalloc((void **)&d_dn, sizeof(int) * n));
    CUDA_SAFE_CALL(cudaMemcpy(d_dp, dp.data(), sizeof(int) * n, cudaMemcpyHostToDevice));
    CUDA_SAFE_CALL(cudaMemcpy(d_dn, dn.data(), sizeof(int) * n, cudaMemcpyHostToDevice));
    GlobalWrapper gw = GC_Init(W, H, d_dp, d_dn, penalty);
    std::vector<int> label(n);
    GC_Optimize(gw, label.data());
    try {
        gcfg_cli::write_overlay_ppm(out, label, rgb, W, H);
    } catch (const std::exception &e) {
        std::fprintf(stderr, "%s\n", e.what());
        return 1;
    }
    CUDA_SAFE_CALL(cudaFree(d_dp));
    CUDA_SAFE_CALL(cudaFree(d_dn));
    GC_End(&gw);
    return 0;
}
