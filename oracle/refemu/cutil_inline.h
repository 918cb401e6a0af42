/* Stand-in for the retired CUDA-SDK <cutil_inline.h> (test infrastructure only). */
#include "cutil.h"
