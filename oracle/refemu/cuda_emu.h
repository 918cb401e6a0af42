/*
 * cuda_emu.h -- a CPU emulation of the small subset of CUDA C++ that the
 * reference solver's sources use (GraphCut.cu, GraphCutKernels.cu), so that
 * the reference's own kernels and host driver can run unmodified on a host
 * without a GPU and produce golden outputs for the oracle.
 *
 * TEST INFRASTRUCTURE ONLY (the oracle's pinning harness).
 *
 * Model: one CUDA block runs at a time; each CUDA thread of the block is a
 * cooperative fiber; __syncthreads*() is a yield point and the barrier
 * completes when every live fiber of the block has arrived (exited fibers
 * count as arrived).  Blocks run in blockIdx order.  __shared__ arrays become
 * function-static storage, which is correct because only one block is live.
 * Atomics are plain read-modify-writes: fibers never preempt one another.
 * This yields one legal schedule of the reference's kernels.
 */
#ifndef GCFG_CUDA_EMU_H
#define GCFG_CUDA_EMU_H

#include <cmath>
#include <cstddef>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <tuple>
#include <utility>

struct dim3 {
    unsigned x, y, z;
    dim3(unsigned x_ = 1, unsigned y_ = 1, unsigned z_ = 1) : x(x_), y(y_), z(z_) {}
};
struct uint3 {
    unsigned x, y, z;
};

extern uint3 threadIdx;
extern uint3 blockIdx;
extern dim3 blockDim;
extern dim3 gridDim;

#define __global__
#define __device__
#define __host__
#define __shared__ static
#define __forceinline__ inline

void emu_syncthreads_pred(int kind, int pred);
int emu_barrier_result(int kind);

inline void __syncthreads() { emu_syncthreads_pred(0, 0); }
inline int __syncthreads_and(int p) { emu_syncthreads_pred(1, p != 0); return emu_barrier_result(1); }
inline int __syncthreads_or(int p) { emu_syncthreads_pred(2, p != 0); return emu_barrier_result(2); }
inline int __syncthreads_count(int p) { emu_syncthreads_pred(3, p != 0); return emu_barrier_result(3); }
inline void __threadfence_block() {}
inline void __threadfence() {}

inline int atomicAdd(int *p, int v) { int o = *p; *p = o + v; return o; }
inline unsigned atomicAdd(unsigned *p, unsigned v) { unsigned o = *p; *p = o + v; return o; }
inline float atomicAdd(float *p, float v) { float o = *p; *p = o + v; return o; }
inline int atomicSub(int *p, int v) { int o = *p; *p = o - v; return o; }
inline int atomicExch(int *p, int v) { int o = *p; *p = v; return o; }
inline int atomicMin(int *p, int v) { int o = *p; if (v < o) *p = v; return o; }
inline int atomicMax(int *p, int v) { int o = *p; if (v > o) *p = v; return o; }

/* ---- runtime API subset ---- */
typedef enum { cudaSuccess = 0, cudaErrorMemoryAllocation = 2 } cudaError_t;
typedef enum {
    cudaMemcpyHostToHost = 0,
    cudaMemcpyHostToDevice = 1,
    cudaMemcpyDeviceToHost = 2,
    cudaMemcpyDeviceToDevice = 3
} cudaMemcpyKind;

cudaError_t cudaMalloc(void **p, size_t n);
cudaError_t cudaFree(void *p);
inline cudaError_t cudaMemcpy(void *d, const void *s, size_t n, cudaMemcpyKind) {
    std::memmove(d, s, n);
    return cudaSuccess;
}
inline cudaError_t cudaMemset(void *d, int v, size_t n) { std::memset(d, v, n); return cudaSuccess; }
inline cudaError_t cudaThreadSynchronize() { return cudaSuccess; }
inline cudaError_t cudaDeviceSynchronize() { return cudaSuccess; }
inline cudaError_t cudaPeekAtLastError() { return cudaSuccess; }
inline cudaError_t cudaGetLastError() { return cudaSuccess; }
inline const char *cudaGetErrorString(cudaError_t e) { return e == cudaSuccess ? "no error" : "error"; }

/* ---- kernel launch: Kernel<<<g,b>>>(args) is rewritten to
 *      emu_launch(g, b, Kernel, args) by the build recipe ---- */
void emu_run_grid(dim3 grid, dim3 block, const std::function<void()> &body);

template <typename... KArgs, typename... Args>
void emu_launch(dim3 grid, dim3 block, void (*k)(KArgs...), Args &&...args) {
    std::tuple<typename std::decay<KArgs>::type...> targs(std::forward<Args>(args)...);
    emu_run_grid(grid, block, [&]() { std::apply(k, targs); });
}

/* statistics of the emulated run */
extern long long emu_launch_count;
extern long long emu_barrier_count;

#endif
