/*
 * cuda_emu.cpp -- fiber scheduler behind cuda_emu.h.
 *
 * TEST INFRASTRUCTURE ONLY (the oracle's pinning harness; runs on the
 * development host, never shipped).
 *
 * Fibers are created with makecontext and entered once with setcontext; all
 * later switches use _setjmp/_longjmp, which do not touch the signal mask
 * and are therefore cheap.  Build with -U_FORTIFY_SOURCE (the fortified
 * longjmp refuses to jump between stacks).
 */
#include "cuda_emu.h"

#include <setjmp.h>
#include <ucontext.h>

#include <vector>

uint3 threadIdx;
uint3 blockIdx;
dim3 blockDim;
dim3 gridDim;
long long emu_launch_count = 0;
long long emu_barrier_count = 0;

namespace {

enum { F_READY = 0, F_BARRIER = 1, F_DONE = 2 };

struct Fiber {
    ucontext_t uc;
    jmp_buf jb;
    char *stack;
    int state;
    int started;
    int pred;
    uint3 tid;
};

const size_t kStack = 256 * 1024;
std::vector<Fiber> g_fibers;
int g_cur = -1;
jmp_buf g_sched;
const std::function<void()> *g_body = nullptr;
int g_res_and = 0, g_res_or = 0, g_res_count = 0;

void fiber_main() {
    (*g_body)();
    g_fibers[g_cur].state = F_DONE;
    _longjmp(g_sched, 1);
}

void ensure_fibers(int n) {
    while ((int)g_fibers.size() < n) {
        Fiber f;
        std::memset(&f, 0, sizeof(f));
        f.stack = (char *)std::malloc(kStack);
        if (!f.stack) {
            std::fprintf(stderr, "cuda_emu: out of memory for fiber stacks\n");
            std::exit(3);
        }
        g_fibers.push_back(f);
    }
}

void run_block(int nthreads) {
    for (int t = 0; t < nthreads; ++t) {
        Fiber &f = g_fibers[t];
        f.state = F_READY;
        f.started = 0;
        f.pred = 0;
        f.tid.x = t % blockDim.x;
        f.tid.y = (t / blockDim.x) % blockDim.y;
        f.tid.z = t / (blockDim.x * blockDim.y);
    }
    for (;;) {
        for (int t = 0; t < nthreads; ++t) {
            Fiber &f = g_fibers[t];
            if (f.state != F_READY) continue;
            g_cur = t;
            threadIdx = f.tid;
            if (_setjmp(g_sched) == 0) {
                if (!f.started) {
                    f.started = 1;
                    getcontext(&f.uc);
                    f.uc.uc_stack.ss_sp = f.stack;
                    f.uc.uc_stack.ss_size = kStack;
                    f.uc.uc_link = nullptr;
                    makecontext(&f.uc, fiber_main, 0);
                    setcontext(&f.uc);
                } else {
                    _longjmp(f.jb, 1);
                }
            }
        }
        int at_barrier = 0, all_and = 1, any_or = 0, cnt = 0;
        for (int t = 0; t < nthreads; ++t) {
            Fiber &f = g_fibers[t];
            if (f.state == F_BARRIER) {
                at_barrier++;
                all_and &= f.pred != 0;
                any_or |= f.pred != 0;
                cnt += f.pred != 0;
            }
        }
        if (at_barrier == 0) break;
        emu_barrier_count++;
        g_res_and = all_and;
        g_res_or = any_or;
        g_res_count = cnt;
        for (int t = 0; t < nthreads; ++t)
            if (g_fibers[t].state == F_BARRIER) g_fibers[t].state = F_READY;
    }
}

} // namespace

void emu_syncthreads_pred(int, int pred) {
    Fiber &f = g_fibers[g_cur];
    f.pred = pred;
    f.state = F_BARRIER;
    if (_setjmp(f.jb) == 0) _longjmp(g_sched, 1);
    /* resumed after the barrier completed */
    threadIdx = g_fibers[g_cur].tid;
}

int emu_barrier_result(int kind) {
    switch (kind) {
    case 1: return g_res_and;
    case 2: return g_res_or;
    case 3: return g_res_count;
    default: return 0;
    }
}

void emu_run_grid(dim3 grid, dim3 block, const std::function<void()> &body) {
    emu_launch_count++;
    gridDim = grid;
    blockDim = block;
    int nthreads = (int)(block.x * block.y * block.z);
    ensure_fibers(nthreads);
    const std::function<void()> *saved = g_body;
    g_body = &body;
    for (unsigned bz = 0; bz < grid.z; ++bz)
        for (unsigned by = 0; by < grid.y; ++by)
            for (unsigned bx = 0; bx < grid.x; ++bx) {
                blockIdx.x = bx;
                blockIdx.y = by;
                blockIdx.z = bz;
                run_block(nthreads);
            }
    g_body = saved;
}

/* Device allocations are host allocations filled with a non-zero pattern,
 * so that reads of never-written device memory stay visible as garbage the
 * way they would on a GPU. */
cudaError_t cudaMalloc(void **p, size_t n) {
    void *q = std::malloc(n ? n : 1);
    if (!q) return cudaErrorMemoryAllocation;
    std::memset(q, 0x5A, n);
    *p = q;
    return cudaSuccess;
}

cudaError_t cudaFree(void *p) {
    std::free(p);
    return cudaSuccess;
}
