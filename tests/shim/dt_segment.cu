// A caller of the reference's DataTerm namespace plus GraphCut API
// (DataTerm.h:9-19 feeding GC_Init through getPos/getNeg), compiled
// unchanged against include/DataTerm.h and include/GraphCut.cu.
//
//   dt_segment <input> <out-prefix>
//
// input (little-endian int32 header): W, H, penalty, n_ops; then rgb
// [3*W*H bytes]; selection [W*H int32] for setSelection; then n_ops triples
// (x, y, cls) of selectOnMap (cls 1) / selectBackgroundOnMap (cls 2).
// Writes <out-prefix>.pos / .neg (W*H int32 t-links from getPos/getNeg),
// .label (W*H int32 from GC_Optimize) and .draw (3*W*H bytes from
// drawSelection of the input image).
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "DataTerm.h"
#include "GraphCut.cu"

template <typename T>
static void read_into(FILE *f, T *p, size_t n) {
    if (n && fread(p, sizeof(T), n, f) != n) {
        fprintf(stderr, "short input file\n");
        exit(2);
    }
}

template <typename T>
static void write_file(const std::string &path, const T *p, size_t n) {
    FILE *o = fopen(path.c_str(), "wb");
    if (!o || fwrite(p, sizeof(T), n, o) != n) exit(2);
    fclose(o);
}

int main(int argc, char **argv) {
    if (argc != 3) {
        fprintf(stderr, "usage: dt_segment <input> <out-prefix>\n");
        return 2;
    }
    FILE *f = fopen(argv[1], "rb");
    if (!f) return 2;
    int hdr[4];
    read_into(f, hdr, 4);
    const int width = hdr[0], height = hdr[1], penalty = hdr[2], n_ops = hdr[3];
    const size_t n = (size_t)width * height;
    std::vector<unsigned char> img(3 * n);
    std::vector<int> sel(n), ops(3 * (size_t)n_ops);
    read_into(f, img.data(), 3 * n);
    read_into(f, sel.data(), n);
    read_into(f, ops.data(), ops.size());
    fclose(f);

    DataTerm::init_data_term(width, height);
    DataTerm::setSigmaGaussian(5);
    DataTerm::setImage(img.data());
    DataTerm::setSelection(sel.data());
    for (int k = 0; k < n_ops; ++k) {
        if (ops[3 * k + 2] == 1)
            DataTerm::selectOnMap(ops[3 * k], ops[3 * k + 1], 5);
        else
            DataTerm::selectBackgroundOnMap(ops[3 * k], ops[3 * k + 1]);
    }
    DataTerm::getDataTermsMixture();

    std::vector<int> pos(n), neg(n);
    CUDA_SAFE_CALL(cudaMemcpy(pos.data(), DataTerm::getPos(), sizeof(int) * n, cudaMemcpyDeviceToHost));
    CUDA_SAFE_CALL(cudaMemcpy(neg.data(), DataTerm::getNeg(), sizeof(int) * n, cudaMemcpyDeviceToHost));
    const std::string pre = argv[2];
    write_file(pre + ".pos", pos.data(), n);
    write_file(pre + ".neg", neg.data(), n);

    GlobalWrapper gw = GC_Init(width, height, DataTerm::getPos(), DataTerm::getNeg(), penalty);
    std::vector<int> label(n);
    GC_Optimize(gw, label.data());
    GC_End(&gw);
    write_file(pre + ".label", label.data(), n);

    std::vector<unsigned char> drawn(3 * n);
    DataTerm::drawSelection(img.data(), drawn.data());
    write_file(pre + ".draw", drawn.data(), 3 * n);
    DataTerm::free_data_term();
    return 0;
}
