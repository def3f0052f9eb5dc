// af_emu.cpp -- launch loops for host-executed CUDA kernel sources (test build only).
#include "include/af_emu.h"

#include <ucontext.h>

#include <vector>

thread_local uint3 threadIdx;
thread_local uint3 blockIdx;
thread_local dim3 blockDim;
thread_local dim3 gridDim;

namespace {

std::vector<char> g_smem;

struct Fiber {
    ucontext_t ctx;
    std::vector<char> stack;
    bool done = false;
    uint3 tid;
};

ucontext_t g_sched;
Fiber* g_current = nullptr;
const std::function<void()>* g_body = nullptr;

void fiber_entry(int lo, int hi) {
    (void)lo;
    (void)hi;
    (*g_body)();
    g_current->done = true;
    // return to the scheduler through uc_link
}

void set_block(dim3 grid, dim3 block, unsigned bx, unsigned by, unsigned bz) {
    gridDim = grid;
    blockDim = block;
    blockIdx = uint3{bx, by, bz};
}

}  // namespace

void __syncthreads() {
    if (!g_current) return;  // plain launch: nothing to wait for
    Fiber* me = g_current;
    swapcontext(&me->ctx, &g_sched);
}

namespace af_emu {

void* dynamic_smem() { return g_smem.data(); }

void launch(dim3 grid, dim3 block, size_t smem, const std::function<void()>& body) {
    g_smem.assign(smem + 16, 0);
    for (unsigned bz = 0; bz < grid.z; ++bz)
        for (unsigned by = 0; by < grid.y; ++by)
            for (unsigned bx = 0; bx < grid.x; ++bx) {
                set_block(grid, block, bx, by, bz);
                for (unsigned tz = 0; tz < block.z; ++tz)
                    for (unsigned ty = 0; ty < block.y; ++ty)
                        for (unsigned tx = 0; tx < block.x; ++tx) {
                            threadIdx = uint3{tx, ty, tz};
                            body();
                        }
            }
}

void launch_sync(dim3 grid, dim3 block, size_t smem, const std::function<void()>& body) {
    const unsigned nt = block.x * block.y * block.z;
    static std::vector<Fiber> fibers;
    if (fibers.size() < nt) fibers.resize(nt);
    for (auto& f : fibers)
        if (f.stack.empty()) f.stack.resize(256 * 1024);
    g_smem.assign(smem + 16, 0);
    g_body = &body;
    for (unsigned bz = 0; bz < grid.z; ++bz)
        for (unsigned by = 0; by < grid.y; ++by)
            for (unsigned bx = 0; bx < grid.x; ++bx) {
                set_block(grid, block, bx, by, bz);
                std::fill(g_smem.begin(), g_smem.end(), 0);
                unsigned i = 0;
                for (unsigned tz = 0; tz < block.z; ++tz)
                    for (unsigned ty = 0; ty < block.y; ++ty)
                        for (unsigned tx = 0; tx < block.x; ++tx, ++i) {
                            Fiber& f = fibers[i];
                            f.done = false;
                            f.tid = uint3{tx, ty, tz};
                            getcontext(&f.ctx);
                            f.ctx.uc_stack.ss_sp = f.stack.data();
                            f.ctx.uc_stack.ss_size = f.stack.size();
                            f.ctx.uc_link = &g_sched;
                            makecontext(&f.ctx, (void (*)())fiber_entry, 2, 0, 0);
                        }
                // passes: each live fiber runs until its next barrier or its end
                for (;;) {
                    bool any = false;
                    for (unsigned k = 0; k < nt; ++k) {
                        Fiber& f = fibers[k];
                        if (f.done) continue;
                        any = true;
                        threadIdx = f.tid;
                        g_current = &f;
                        swapcontext(&g_sched, &f.ctx);
                        g_current = nullptr;
                    }
                    if (!any) break;
                }
            }
    g_body = nullptr;
}

}  // namespace af_emu
