// solver.cuh -- host-side interface of the tile push-relabel solver.
#pragma once

#include "gcfg_internal.cuh"

namespace gcfg {

// Device buffers of one residual graph (sized for a maximum image).
struct SolverState {
    size_t max_pixels = 0;
    int max_tiles = 0;
    int4 *cap = nullptr;
    int *exc = nullptr;
    int *h = nullptr;
    uint8_t *mark = nullptr;
    int *tile_active = nullptr;
    Counters *cnt = nullptr;
    Counters *h_cnt = nullptr;   // pinned host mirror
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    long long interior_dp = 0;   // sum of dp over interior pixels (from the build)
    unsigned ref_init = 0;       // reference's initial energy (int32 wrap)
};

gcfg_status solver_alloc(SolverState &s, int max_w, int max_h);
void solver_free(SolverState &s);
GraphDev solver_view(SolverState &s, int W, int H);
gcfg_status build_from_arrays(SolverState &s, const GraphDev &g, const int *dp, const int *dn,
                              int penalty, const int *up, const int *down, const int *left,
                              const int *right, cudaStream_t st);
gcfg_status solve(SolverState &s, const GraphDev &g, cudaStream_t st, int push_rounds,
                  int max_sweeps, gcfg_result *res);
gcfg_status extract(const GraphDev &g, uint8_t *smin, uint8_t *smax, int *label, cudaStream_t st);

}  // namespace gcfg
