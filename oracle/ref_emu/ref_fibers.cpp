/*
 * ref_fibers.cpp -- runs a CUDA-style kernel body on the CPU, one fiber per
 * thread of a block, blocks one after another.  __syncthreads() switches back
 * to the scheduler; a round resumes every live thread once, so all threads of
 * the block pass each barrier together.  TEST INFRASTRUCTURE.
 */
#include "cuda_shim.h"
#include "ref_emu.h"

#include <ucontext.h>
#include <vector>

uint3 threadIdx, blockIdx;
dim3 blockDim, gridDim;

namespace {
const size_t kStack = 64 * 1024;
ucontext_t g_sched;
std::vector<ucontext_t> g_ctx;
std::vector<char> g_stacks;
std::vector<int> g_done;
int g_cur = 0;
const std::function<void()> *g_body = nullptr;

void fiber_entry()
{
    (*g_body)();
    g_done[g_cur] = 1;
    swapcontext(&g_ctx[g_cur], &g_sched);
}
}  // namespace

void __syncthreads(void) { swapcontext(&g_ctx[g_cur], &g_sched); }

void emu_launch(unsigned grid, unsigned block, const std::function<void()> &body)
{
    gridDim = dim3(grid, 1, 1);
    blockDim = dim3(block, 1, 1);
    g_ctx.resize(block);
    g_stacks.resize(kStack * block);
    g_done.assign(block, 0);
    g_body = &body;
    for (unsigned b = 0; b < grid; b++) {
        blockIdx = make_uint3(b, 0, 0);
        for (unsigned t = 0; t < block; t++) {
            getcontext(&g_ctx[t]);
            g_ctx[t].uc_stack.ss_sp = &g_stacks[kStack * t];
            g_ctx[t].uc_stack.ss_size = kStack;
            g_ctx[t].uc_link = &g_sched;
            makecontext(&g_ctx[t], fiber_entry, 0);
            g_done[t] = 0;
        }
        bool alive = true;
        while (alive) {
            alive = false;
            for (unsigned t = 0; t < block; t++) {
                if (g_done[t]) continue;
                g_cur = (int)t;
                threadIdx = make_uint3(t, 0, 0);
                swapcontext(&g_sched, &g_ctx[t]);
                alive = true;
            }
        }
    }
}
