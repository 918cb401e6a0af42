/* The reference's data-term kernels, unmodified, compiled for the GPU as one
 * cubin: DataTermKernels.cu (K_InitGaussian, K_InitSelectionMap,
 * K_InitColorSpace, K_CalcTerms, K_SetMap, K_DrawMap, K_SelectAndGauss,
 * DataTermKernels.cu:19-150) is read from the reference checkout by the
 * include path of build_ref_gpu.sh.  The two definitions below are the ones
 * DataTerm.cpp makes before it includes the file (N_PDF, DataTerm.cpp:5) and
 * the uchar type its callers get from OpenCV.  ref_gpu.cpp drives the
 * kernels as DataTerm.cpp:28-165 does.  Test infrastructure only. */
#define N_PDF 256
typedef unsigned char uchar;
#include "DataTermKernels.cu"
