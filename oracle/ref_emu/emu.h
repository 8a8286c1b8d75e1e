/*
 * emu.h -- TEST INFRASTRUCTURE ONLY.
 *
 * A minimal CUDA execution-model emulator for the host, used to run the
 * reference's own kernel source (src/gcoo_spdm_kernels.cu of
 * hclhkbu/gcoospdm, compiled straight from where it lies) on the CPU so that
 * its exact outputs can be recorded as golden vectors.
 *
 * Model: thread blocks run one after another; the threads of a block are
 * cooperative fibers (ucontext) scheduled round-robin, and __syncthreads()
 * yields to the scheduler until every live thread of the block has reached
 * the barrier. `__shared__` variables become function-local statics, which is
 * exactly block-shared storage because only one block is live at a time.
 * The reference kernels use no atomics, warp intrinsics or cross-block
 * communication, so this schedule computes what the GPU computes.
 */
#ifndef GCOO_REF_EMU_H
#define GCOO_REF_EMU_H

#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <ucontext.h>

#include <functional>
#include <vector>

struct dim3 {
    unsigned x, y, z;
    dim3(unsigned a = 1, unsigned b = 1, unsigned c = 1) : x(a), y(b), z(c) {}
};

namespace emu {

struct Fiber {
    ucontext_t ctx;
    unsigned tid;
    bool done;
    bool at_barrier;
};

extern dim3 g_block_idx;
extern dim3 g_block_dim;
extern Fiber *g_cur;

void sync();
inline dim3 thread_idx() { return dim3(g_cur->tid, 0, 0); }

/* Runs `body` once per thread for every block of `grid` (1-D blocks). */
void launch(dim3 grid, dim3 block, const std::function<void()> &body);

} // namespace emu

#define __global__
#define __device__
#define __host__
#define __forceinline__ inline
#define __shared__ static
#define threadIdx (emu::thread_idx())
#define blockIdx (emu::g_block_idx)
#define blockDim (emu::g_block_dim)
#define __syncthreads() emu::sync()

#endif
