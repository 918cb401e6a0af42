// A caller of the reference's GraphCut API built with NEIGHBORHOOD == 8
// (GC_Init with the four diagonal arrays, GraphCut.cu:187-194), compiled
// unchanged against include/GraphCut.cu.
//
//   gc_solve8 <instance> <labels-out> [<instance> <labels-out> ...]
//
// instance (little-endian int32): W, H, penalty, arrays (0/1), dp[W*H],
// dn[W*H], and when arrays == 1 up, down, left, right, upleft, upright,
// downleft, downright [W*H each].  labels-out: W*H int32 from GC_Optimize.
#define NEIGHBORHOOD 8
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "GraphCut.cu"

static int run_one(const char *in_path, const char *out_path) {
    FILE *f = fopen(in_path, "rb");
    if (!f) return 2;
    int hdr[4];
    if (fread(hdr, sizeof(int), 4, f) != 4) return 2;
    const int width = hdr[0], height = hdr[1], penalty = hdr[2], arrays = hdr[3];
    const size_t n = (size_t)width * height;
    const int k = 2 + (arrays ? 8 : 0);
    std::vector<int> host(k * n);
    if (fread(host.data(), sizeof(int), host.size(), f) != host.size()) return 2;
    fclose(f);
    std::vector<int *> d(10, (int *)NULL);
    for (int a = 0; a < k; ++a) {
        CUDA_SAFE_CALL(cudaMalloc((void **)&d[a], sizeof(int) * n));
        CUDA_SAFE_CALL(cudaMemcpy(d[a], host.data() + a * n, sizeof(int) * n, cudaMemcpyHostToDevice));
    }
    GlobalWrapper gw = arrays ? GC_Init(width, height, d[0], d[1], 0, d[2], d[3], d[4], d[5], d[6], d[7], d[8], d[9])
                              : GC_Init(width, height, d[0], d[1], penalty);
    std::vector<int> label(n);
    GC_Optimize(gw, label.data());
    GC_End(&gw);
    FILE *o = fopen(out_path, "wb");
    if (!o || fwrite(label.data(), sizeof(int), n, o) != n) return 2;
    fclose(o);
    for (int a = 0; a < k; ++a) CUDA_SAFE_CALL(cudaFree(d[a]));
    return 0;
}

int main(int argc, char **argv) {
    if (argc < 3 || (argc - 1) % 2 != 0) {
        fprintf(stderr, "usage: gc_solve8 <instance> <labels-out> [...]\n");
        return 2;
    }
    for (int a = 1; a + 1 < argc; a += 2) {
        const int rc = run_one(argv[a], argv[a + 1]);
        if (rc) return rc;
        fflush(stdout);
    }
    return 0;
}
