/*
 * emu.cpp -- the block scheduler behind cuda_emu/cuda_runtime.h.
 *
 * TEST INFRASTRUCTURE ONLY (the reference build of the checker).
 *
 * A block's threads run as ucontext fibers on one host thread.  The
 * scheduler resumes every live fiber in thread order; a fiber runs until it
 * calls __syncthreads() or returns, so after one pass every live thread of
 * the block waits at the same barrier, and the next pass releases them.
 * Blocks are independent and are spread over host threads with OpenMP.
 *
 * Block 0 of each launch always runs as fibers.  If none of its threads
 * reached a barrier, the remaining blocks run their threads as plain calls
 * one after another (much cheaper than a context switch per thread); a
 * __syncthreads() met in that mode aborts the process, so a kernel whose
 * barrier only some blocks reach can never be mis-scheduled silently.
 */
#include "cuda_runtime.h"

#include <ucontext.h>

#include <vector>

thread_local uint3 threadIdx;
thread_local uint3 blockIdx;
thread_local dim3 blockDim;
thread_local dim3 gridDim;

namespace psemu {
namespace {

enum { kReady = 0, kBarrier = 1, kDone = 2 };
constexpr size_t kStack = 64 * 1024;

struct Fiber {
    ucontext_t ctx;
    char* stack = nullptr;
    uint3 tid;
    int state = kReady;
};

struct Worker {
    ucontext_t sched;
    std::vector<Fiber> fibers;
    Fiber* cur = nullptr;
    void (*body)(void*) = nullptr;
    void* arg = nullptr;
    bool fiber_mode = false;
    bool saw_barrier = false;
    ~Worker()
    {
        for (Fiber& f : fibers) std::free(f.stack);
    }
};

thread_local Worker t_worker;

void fiber_entry()
{
    Worker& w = t_worker;
    w.body(w.arg);
    w.cur->state = kDone;
    /* returning resumes uc_link, the scheduler */
}

uint3 thread_of(unsigned t, dim3 b)
{
    uint3 r;
    r.x = t % b.x;
    r.y = (t / b.x) % b.y;
    r.z = t / (b.x * b.y);
    return r;
}

void run_block_fibers(Worker& w, unsigned nthreads, dim3 block)
{
    if (w.fibers.size() < nthreads) w.fibers.resize(nthreads);
    for (unsigned t = 0; t < nthreads; ++t) {
        Fiber& f = w.fibers[t];
        if (!f.stack) {
            f.stack = static_cast<char*>(std::malloc(kStack));
            if (!f.stack) { std::fprintf(stderr, "psemu: out of memory\n"); std::abort(); }
        }
        getcontext(&f.ctx);
        f.ctx.uc_stack.ss_sp = f.stack;
        f.ctx.uc_stack.ss_size = kStack;
        f.ctx.uc_link = &w.sched;
        makecontext(&f.ctx, fiber_entry, 0);
        f.tid = thread_of(t, block);
        f.state = kReady;
    }
    w.fiber_mode = true;
    bool live = true;
    while (live) {
        live = false;
        for (unsigned t = 0; t < nthreads; ++t) {
            Fiber& f = w.fibers[t];
            if (f.state == kDone) continue;
            threadIdx = f.tid;
            w.cur = &f;
            f.state = kReady;
            swapcontext(&w.sched, &f.ctx);
            if (f.state != kDone) live = true;
        }
    }
    w.fiber_mode = false;
}

void run_block_direct(Worker& w, unsigned nthreads, dim3 block)
{
    for (unsigned t = 0; t < nthreads; ++t) {
        threadIdx = thread_of(t, block);
        w.body(w.arg);
    }
}

uint3 block_of(unsigned long long b, dim3 g)
{
    uint3 r;
    r.x = unsigned(b % g.x);
    r.y = unsigned((b / g.x) % g.y);
    r.z = unsigned(b / (unsigned long long)(g.x * g.y));
    return r;
}

}  // namespace

void run_grid(dim3 grid, dim3 block, void (*body)(void*), void* arg)
{
    const unsigned nthreads = block.x * block.y * block.z;
    const unsigned long long nblocks = (unsigned long long)grid.x * grid.y * grid.z;
    if (nthreads == 0 || nblocks == 0) return;

    Worker& w0 = t_worker;
    w0.body = body;
    w0.arg = arg;
    w0.saw_barrier = false;
    gridDim = grid;
    blockDim = block;
    blockIdx = block_of(0, grid);
    run_block_fibers(w0, nthreads, block);
    const bool fibers = w0.saw_barrier;

#pragma omp parallel for schedule(dynamic, 16)
    for (long long b = 1; b < (long long)nblocks; ++b) {
        Worker& w = t_worker;
        w.body = body;
        w.arg = arg;
        gridDim = grid;
        blockDim = block;
        blockIdx = block_of((unsigned long long)b, grid);
        if (fibers) run_block_fibers(w, nthreads, block);
        else run_block_direct(w, nthreads, block);
    }
}

}  // namespace psemu

void __syncthreads()
{
    psemu::Worker& w = psemu::t_worker;
    if (!w.fiber_mode) {
        std::fprintf(stderr, "psemu: __syncthreads() in a block run without fibers "
                             "(block 0 of this launch reached no barrier)\n");
        std::abort();
    }
    w.saw_barrier = true;
    w.cur->state = psemu::kBarrier;
    swapcontext(&w.cur->ctx, &w.sched);
}
