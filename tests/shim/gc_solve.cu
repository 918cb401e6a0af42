// A caller written against the reference's GraphCut API (the same calls and
// order as solveMRF.cu:105-138 and Debug.cu:83-101), compiled unchanged
// against include/GraphCut.cu.
//
//   gc_solve once|resolve <instance> <labels-out> [<instance> <labels-out> ...]
//
// instance (little-endian int32): W, H, penalty, arrays (0/1), dp[W*H],
// dn[W*H], and when arrays == 1 up, down, left, right [W*H each].
// labels-out: W*H int32 from GC_Optimize.  With "resolve" the graph is
// allocated empty (GC_Init(w, h)), filled by GC_SetDataterms + GC_SetPenalty
// or GC_SetEdges + GC_SetGraph, solved, then rebuilt and solved again; the
// two label maps must agree.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "GraphCut.cu"

static std::vector<int> read_ints(FILE *f, size_t n) {
    std::vector<int> v(n);
    if (n && fread(v.data(), sizeof(int), n, f) != n) {
        fprintf(stderr, "short instance file\n");
        exit(2);
    }
    return v;
}

static int *to_device(const std::vector<int> &v) {
    int *d = NULL;
    CUDA_SAFE_CALL(cudaMalloc((void **)&d, sizeof(int) * v.size()));
    CUDA_SAFE_CALL(cudaMemcpy(d, v.data(), sizeof(int) * v.size(), cudaMemcpyHostToDevice));
    return d;
}

static int run_one(const char *in_path, const char *out_path, bool resolve) {
    FILE *f = fopen(in_path, "rb");
    if (!f) return 2;
    std::vector<int> hdr = read_ints(f, 4);
    const int width = hdr[0], height = hdr[1], penalty = hdr[2], arrays = hdr[3];
    const size_t n = (size_t)width * height;
    std::vector<int> dp = read_ints(f, n), dn = read_ints(f, n);
    std::vector<int> up, down, left, right;
    if (arrays) {
        up = read_ints(f, n);
        down = read_ints(f, n);
        left = read_ints(f, n);
        right = read_ints(f, n);
    }
    fclose(f);

    int *d_data_positive = to_device(dp), *d_data_negative = to_device(dn);
    int *d_up = NULL, *d_down = NULL, *d_left = NULL, *d_right = NULL;
    if (arrays) {
        d_up = to_device(up);
        d_down = to_device(down);
        d_left = to_device(left);
        d_right = to_device(right);
    }
    int *label = (int *)malloc(sizeof(int) * n);

    if (!resolve) {
        GlobalWrapper gw = arrays ? GC_Init(width, height, d_data_positive, d_data_negative, 0, d_up, d_down,
                                            d_left, d_right)
                                  : GC_Init(width, height, d_data_positive, d_data_negative, penalty);
        GC_Optimize(gw, label);
        GC_End(&gw);
    } else {
        GlobalWrapper gw = GC_Init(width, height);
        GC_SetDataterms(&gw, d_data_positive, d_data_negative);
        if (arrays)
            GC_SetEdges(&gw, d_up, d_down, d_left, d_right);
        else
            GC_SetPenalty(&gw, penalty);
        GC_SetGraph(gw);
        GC_Optimize(gw, label);
        int *again = (int *)malloc(sizeof(int) * n);
        GC_SetGraph(gw);  // the graph is consumed by a solve
        GC_Optimize(gw, again);
        if (memcmp(label, again, sizeof(int) * n) != 0) {
            fprintf(stderr, "re-solve differs\n");
            return 1;
        }
        free(again);
        GC_End(&gw);
    }

    FILE *o = fopen(out_path, "wb");
    if (!o || fwrite(label, sizeof(int), n, o) != n) return 2;
    fclose(o);
    free(label);
    CUDA_SAFE_CALL(cudaFree(d_data_positive));
    CUDA_SAFE_CALL(cudaFree(d_data_negative));
    if (arrays) {
        CUDA_SAFE_CALL(cudaFree(d_up));
        CUDA_SAFE_CALL(cudaFree(d_down));
        CUDA_SAFE_CALL(cudaFree(d_left));
        CUDA_SAFE_CALL(cudaFree(d_right));
    }
    return 0;
}

int main(int argc, char **argv) {
    if (argc < 4 || (argc - 2) % 2 != 0) {
        fprintf(stderr, "usage: gc_solve once|resolve <instance> <labels-out> [...]\n");
        return 2;
    }
    const bool resolve = strcmp(argv[1], "resolve") == 0;
    for (int k = 2; k + 1 < argc; k += 2) {
        const int rc = run_one(argv[k], argv[k + 1], resolve);
        if (rc) return rc;
        fflush(stdout);
    }
    return 0;
}
