/*
 * Stand-in for the reference's GraphCut.cu when one of the reference's
 * applications (solveMRF.cu, Application.cu) is compiled for the CPU thread
 * emulator: the application's `#include "GraphCut.cu"` lands here, and the
 * solver itself (the reference's GraphCut.cu, compiled once) is linked from
 * graphcut_ref.o.  Declares the host API with the reference's default
 * arguments (GraphCut.cu:187-194).  Test infrastructure only.
 */
#include "GraphCut.h"

GlobalWrapper GC_Init(int width, int height, int *data_positive = NULL, int *data_negative = NULL,
                      int penalty = 0, int *up = NULL, int *down = NULL, int *left = NULL, int *right = NULL);
void GC_Optimize(GlobalWrapper gw, int *label);
void GC_End(GlobalWrapper *gw);
