/* GraphCut.h -- source-compatible C++ front end of gcfg.h for programs written
 * against the reference's GraphCut.cu (GC_* free functions with default
 * arguments and a GlobalWrapper handle passed by value; GraphCut.cu:187-542,
 * GraphCut.h:60-128).
 *
 * A caller such as solveMRF.cu, Application.cu or Debug.cu compiles unchanged
 * with `nvcc -I include caller.cu -L gc-fg_gb300 -lgcfg`: `#include "GraphCut.cu"`
 * resolves to include/GraphCut.cu, which includes this file.
 *
 * Same names, argument meaning and ownership as the reference: dp/dn and the
 * four n-link arrays are caller-owned device int32 arrays of W*H; `label` is a
 * caller-owned host int array of W*H that receives 1 for pixels that cannot
 * reach the sink and 0 elsewhere (the 1-pixel border included); the graph is
 * consumed by GC_Optimize, so a re-solve calls GC_SetGraph first.  Errors
 * behave like the reference's cutil checks: a message on stderr and exit().
 * GC_Optimize prints the reference's "Final energy level: %d" line unless
 * GCFG_GRAPHCUT_QUIET is defined.  NEIGHBORHOOD may be defined as 4 (the
 * default, as in the reference's GraphCut.h:22) or 8 before this header; with
 * 8, GC_Init and GC_SetEdges take the four diagonal arrays too, as the
 * reference's do (GraphCut.cu:187-194, 271-289). */
#ifndef GCFG_GRAPHCUT_H_
#define GCFG_GRAPHCUT_H_

#include <cstdio>
#include <cstdlib>

#include <cuda_runtime.h>

#include "gcfg.h"

#ifndef NEIGHBORHOOD
#define NEIGHBORHOOD 4
#endif
#if NEIGHBORHOOD != 4 && NEIGHBORHOOD != 8
#error "NEIGHBORHOOD must be 4 or 8"
#endif

/* cutil's checking macros as the reference's callers use them. */
#ifndef CUDA_SAFE_CALL
#define CUDA_SAFE_CALL(call)                                                                   \
    do {                                                                                       \
        cudaError_t gcfg_err_ = (call);                                                        \
        if (gcfg_err_ != cudaSuccess) {                                                        \
            fprintf(stderr, "Cuda error in file '%s' in line %i : %s.\n", __FILE__, __LINE__, \
                    cudaGetErrorString(gcfg_err_));                                            \
            exit(EXIT_FAILURE);                                                                \
        }                                                                                      \
    } while (0)
#endif

/* The handle.  Copies share one graph (the reference's copies shared its
 * device arrays the same way). */
#if NEIGHBORHOOD == 8
typedef gcfg_graph8 gcfg_graphcut_handle;
#else
typedef gcfg_graph gcfg_graphcut_handle;
#endif
struct GlobalWrapper {
    gcfg_graphcut_handle *graph;
    int width, height;
    int penalty;
    bool varying_edges;
};

namespace gcfg_graphcut_detail {
inline void check(gcfg_status s, const char *what) {
    if (s != GCFG_OK) {
        fprintf(stderr, "%s failed: %s\n", what, gcfg_strerror(s));
        exit(EXIT_FAILURE);
    }
}
}  // namespace gcfg_graphcut_detail

#if NEIGHBORHOOD == 8
#define GCFG_GC_(name) name##8
#else
#define GCFG_GC_(name) name
#endif

/* GraphCut.cu:265 */
inline void GC_SetDataterms(GlobalWrapper *gw, int *data_positive, int *data_negative) {
    gcfg_graphcut_detail::check(GCFG_GC_(gcfg_set_dataterms)(gw->graph, data_positive, data_negative),
                                "GC_SetDataterms");
}

/* GraphCut.cu:271 */
#if NEIGHBORHOOD == 8
inline void GC_SetEdges(GlobalWrapper *gw, int *up, int *down, int *left, int *right, int *upleft, int *upright,
                        int *downleft, int *downright) {
    gcfg_graphcut_detail::check(
        gcfg_set_edges8(gw->graph, up, down, left, right, upleft, upright, downleft, downright), "GC_SetEdges");
    gw->varying_edges = up != NULL;
}
#else
inline void GC_SetEdges(GlobalWrapper *gw, int *up, int *down, int *left, int *right) {
    gcfg_graphcut_detail::check(gcfg_set_edges(gw->graph, up, down, left, right), "GC_SetEdges");
    gw->varying_edges = up != NULL;
}
#endif

/* GraphCut.cu:296 */
inline void GC_SetPenalty(GlobalWrapper *gw, int p) {
    gcfg_graphcut_detail::check(GCFG_GC_(gcfg_set_penalty)(gw->graph, p), "GC_SetPenalty");
    gw->varying_edges = false;
    gw->penalty = p;
}

/* GraphCut.cu:301 */
inline void GC_SetGraph(GlobalWrapper gw) {
    gcfg_graphcut_detail::check(GCFG_GC_(gcfg_set_graph)(gw.graph), "GC_SetGraph");
}

/* GraphCut.cu:187-263: allocate; with data terms, also build the graph. */
#if NEIGHBORHOOD == 8
inline GlobalWrapper GC_Init(int width, int height, int *data_positive = NULL, int *data_negative = NULL,
                             int penalty = 0, int *up = NULL, int *down = NULL, int *left = NULL,
                             int *right = NULL, int *upleft = NULL, int *upright = NULL, int *downleft = NULL,
                             int *downright = NULL) {
    GlobalWrapper gw;
    gw.width = width;
    gw.height = height;
    gw.penalty = penalty;
    gw.varying_edges = up != NULL;
    gw.graph = NULL;
    gcfg_graphcut_detail::check(gcfg_init8(width, height, data_positive, data_negative, penalty, up, down, left,
                                           right, upleft, upright, downleft, downright, &gw.graph),
                                "GC_Init");
    return gw;
}
#else
inline GlobalWrapper GC_Init(int width, int height, int *data_positive = NULL, int *data_negative = NULL,
                             int penalty = 0, int *up = NULL, int *down = NULL, int *left = NULL,
                             int *right = NULL) {
    GlobalWrapper gw;
    gw.width = width;
    gw.height = height;
    gw.penalty = penalty;
    gw.varying_edges = up != NULL;
    gw.graph = NULL;
    gcfg_graphcut_detail::check(
        gcfg_init(width, height, data_positive, data_negative, penalty, up, down, left, right, &gw.graph), "GC_Init");
    return gw;
}
#endif

/* GraphCut.cu:385-534 */
inline void GC_Optimize(GlobalWrapper gw, int *label) {
    gcfg_result r;
    gcfg_graphcut_detail::check(GCFG_GC_(gcfg_optimize)(gw.graph, label, &r), "GC_Optimize");
#ifndef GCFG_GRAPHCUT_QUIET
    printf("Final energy level: %d\n", r.ref_energy);
#endif
}

/* GraphCut.cu:542-569 */
inline void GC_End(GlobalWrapper *gw) {
    if (gw->graph) gcfg_graphcut_detail::check(GCFG_GC_(gcfg_end)(gw->graph), "GC_End");
    gw->graph = NULL;
    gw->width = gw->height = 0;
}

#undef GCFG_GC_

#endif /* GCFG_GRAPHCUT_H_ */
