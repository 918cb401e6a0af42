/* The reference's own CUDA kernels, unmodified, compiled for the GPU as one
 * cubin: GraphCut.h (the NodeWrapper / GraphWrapper / KernelWrapper structs
 * and the solver constants, GraphCut.h:55-171) and GraphCutKernels.cu (every
 * kernel of the 4-neighbourhood solver, GraphCutKernels.cu:112-898) are read
 * from the reference checkout by the include path of build_ref_gpu.sh.  This
 * file adds no code: ref_gpu.cpp drives the kernels.  Test infrastructure
 * only (the reference's CUDA path, timed beside this repository's). */
#include "GraphCut.h"
#include "GraphCutKernels.cu"
