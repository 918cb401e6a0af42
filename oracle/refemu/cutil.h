/* Stand-in for the retired CUDA-SDK <cutil.h>: the error and timer macros
 * that the reference's GraphCut.cu uses (GraphCut.cu:215-246, 412-414,
 * 498-505), with the same meaning (abort on error, wall-clock timer).
 * Test infrastructure only. */
#ifndef GCFG_CUTIL_SHIM_H
#define GCFG_CUTIL_SHIM_H
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include "cuda_emu.h"

typedef bool CUTBoolean;
#define CUTTrue true

#define CUDA_SAFE_CALL(call)                                                   \
    do {                                                                       \
        cudaError_t e_ = (call);                                               \
        if (e_ != cudaSuccess) {                                               \
            std::fprintf(stderr, "CUDA error %d at %s:%d\n", (int)e_, __FILE__, \
                         __LINE__);                                            \
            std::exit(2);                                                      \
        }                                                                      \
    } while (0)
#define CUT_SAFE_CALL(call) (void)(call)
#define cutilCheckMsg(msg) (void)(msg)
#define cutilSafeCall(call) CUDA_SAFE_CALL(call)

inline std::chrono::steady_clock::time_point &emu_timer_slot(unsigned t) {
    static std::chrono::steady_clock::time_point slots[64];
    return slots[t % 64];
}
inline double &emu_timer_acc(unsigned t) {
    static double acc[64];
    return acc[t % 64];
}
inline CUTBoolean cutCreateTimer(unsigned *t) {
    static unsigned next = 1;
    *t = next++;
    emu_timer_acc(*t) = 0.0;
    return true;
}
inline CUTBoolean cutStartTimer(unsigned t) {
    emu_timer_slot(t) = std::chrono::steady_clock::now();
    return true;
}
inline CUTBoolean cutStopTimer(unsigned t) {
    emu_timer_acc(t) += std::chrono::duration<double, std::milli>(
                            std::chrono::steady_clock::now() - emu_timer_slot(t)).count();
    return true;
}
inline float cutGetTimerValue(unsigned t) { return (float)emu_timer_acc(t); }
inline CUTBoolean cutDeleteTimer(unsigned) { return true; }
#endif
