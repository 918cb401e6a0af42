/*
 * dt_harness.cpp -- drives the reference's DataTerm namespace (DataTerm.cpp,
 * with DataTermKernels.cu, compiled for the CPU thread emulator) the way its
 * applications do: init_data_term, setSigmaGaussian, setImage, selectOnMap
 * (a list of points, in order), getDataTermsMixture, getPos/getNeg.
 * Test infrastructure only.
 *
 * Input file (little-endian int32 header): W, H, sigma, n_points; then
 * 3*W*H image bytes; then n_points (x, y) int32 pairs.
 * Output file: the 101 float entries of the Gaussian table, then pos[W*H] and
 * neg[W*H] int32.
 */
#include <cstdint>
#include <cstdio>
#include <vector>

#include "cuda_emu.h"

namespace DataTerm {
int *getPos();
int *getNeg();
void init_data_term(int w, int h);
void setImage(unsigned char *h_img);
void selectOnMap(int x, int y, int sigma);
void getDataTermsMixture();
void setSigmaGaussian(int sigma);
extern float *d_gaussian;
}  // namespace DataTerm

int main(int argc, char **argv) {
    if (argc != 3) {
        std::fprintf(stderr, "usage: %s input.bin output.bin\n", argv[0]);
        return 1;
    }
    FILE *f = std::fopen(argv[1], "rb");
    if (!f) return 1;
    int hdr[4];
    if (std::fread(hdr, sizeof(int), 4, f) != 4) return 1;
    const int W = hdr[0], H = hdr[1], sigma = hdr[2], n = hdr[3];
    std::vector<unsigned char> img((size_t)3 * W * H);
    std::vector<int> pts((size_t)2 * n);
    if (std::fread(img.data(), 1, img.size(), f) != img.size()) return 1;
    if (n && std::fread(pts.data(), sizeof(int), pts.size(), f) != pts.size()) return 1;
    std::fclose(f);
    DataTerm::init_data_term(W, H);
    DataTerm::setSigmaGaussian(sigma);
    DataTerm::setImage(img.data());
    for (int k = 0; k < n; ++k) DataTerm::selectOnMap(pts[2 * k], pts[2 * k + 1], sigma);
    DataTerm::getDataTermsMixture();
    std::vector<float> gauss(101);
    std::vector<int> pos((size_t)W * H), neg((size_t)W * H);
    cudaMemcpy(gauss.data(), DataTerm::d_gaussian, 101 * sizeof(float), cudaMemcpyDeviceToHost);
    cudaMemcpy(pos.data(), DataTerm::getPos(), pos.size() * sizeof(int), cudaMemcpyDeviceToHost);
    cudaMemcpy(neg.data(), DataTerm::getNeg(), neg.size() * sizeof(int), cudaMemcpyDeviceToHost);
    FILE *o = std::fopen(argv[2], "wb");
    if (!o) return 1;
    std::fwrite(gauss.data(), sizeof(float), gauss.size(), o);
    std::fwrite(pos.data(), sizeof(int), pos.size(), o);
    std::fwrite(neg.data(), sizeof(int), neg.size(), o);
    std::fclose(o);
    return 0;
}
