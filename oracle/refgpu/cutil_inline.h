/* Stand-in for the retired CUDA-SDK <cutil_inline.h>; see cutil.h here. */
