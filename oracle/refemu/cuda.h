/* Stand-in for <cuda.h> when the reference sources are compiled for the CPU
 * thread emulator (test infrastructure only). */
#include "cuda_emu.h"
