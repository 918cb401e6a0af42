/* Stand-in for the retired CUDA-SDK <cutil.h> when the reference's kernels
 * (GraphCutKernels.cu) are compiled for the GPU: the kernels use none of
 * cutil's macros, so nothing is needed here.  Test infrastructure only. */
#ifndef GCFG_REFGPU_CUTIL_H
#define GCFG_REFGPU_CUTIL_H
#endif
