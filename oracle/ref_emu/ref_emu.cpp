/*
 * ref_emu.cpp -- TEST INFRASTRUCTURE ONLY.
 *
 * Compiles the reference's kernel file (src/gcoo_spdm_kernels.cu, included
 * from the reference tree by the build recipe in oracle/Makefile) for the host
 * under the emulator in emu.h, and drives its four kernels with the same
 * launch shapes and the same host orchestration as the reference plugin
 * (src/ShGCOOSpDM.cu:19-126 for the conversion, :153-167 for the multiply).
 * The tile constants come from the reference's own src/constants.h.
 *
 * Output: a shared library used by tests/golden/make_golden.py to record the
 * reference's exact results as fixtures. Nothing in the product uses it.
 */
#include "emu.h"

#include <string.h>

#include "gcoo_spdm_kernels.cu" /* the reference kernels, unmodified */
#include "constants.h"          /* COLUMN_PER_GROUP, BS */

namespace emu {

dim3 g_block_idx;
dim3 g_block_dim;
Fiber *g_cur = nullptr;
static ucontext_t g_sched;
static const std::function<void()> *g_body = nullptr;
static const size_t kStack = 64 * 1024;

void sync()
{
    g_cur->at_barrier = true;
    swapcontext(&g_cur->ctx, &g_sched);
}

static void trampoline()
{
    (*g_body)();
    g_cur->done = true;
    swapcontext(&g_cur->ctx, &g_sched);
}

void launch(dim3 grid, dim3 block, const std::function<void()> &body)
{
    const unsigned nt = block.x;
    std::vector<Fiber> fibers(nt);
    std::vector<char> stacks((size_t)nt * kStack);
    g_body = &body;
    g_block_dim = block;
    for (unsigned bz = 0; bz < grid.z; ++bz)
        for (unsigned by = 0; by < grid.y; ++by)
            for (unsigned bx = 0; bx < grid.x; ++bx) {
                g_block_idx = dim3(bx, by, bz);
                for (unsigned t = 0; t < nt; ++t) {
                    Fiber &f = fibers[t];
                    f.tid = t;
                    f.done = false;
                    f.at_barrier = false;
                    getcontext(&f.ctx);
                    f.ctx.uc_stack.ss_sp = stacks.data() + (size_t)t * kStack;
                    f.ctx.uc_stack.ss_size = kStack;
                    f.ctx.uc_link = nullptr;
                    makecontext(&f.ctx, trampoline, 0);
                }
                for (;;) {
                    unsigned live = 0, waiting = 0;
                    for (unsigned t = 0; t < nt; ++t) {
                        Fiber &f = fibers[t];
                        if (f.done)
                            continue;
                        f.at_barrier = false;
                        g_cur = &f;
                        swapcontext(&g_sched, &f.ctx);
                        if (!f.done) {
                            ++live;
                            waiting += f.at_barrier;
                        }
                    }
                    if (live == 0)
                        break;
                    if (waiting != live || live != nt) {
                        fprintf(stderr, "ref_emu: divergent __syncthreads in block (%u,%u)\n", bx, by);
                        abort();
                    }
                }
            }
    g_cur = nullptr;
}

} // namespace emu

template <int CPG>
static long long convert_impl(float *A, int m, int k, int *groupIndex, int *nnzPerGroup,
                              float *vals, int *rows, int *cols, long long cap)
{
    const int nGroup = (m + CPG - 1) / CPG;
    const int BS_OF_CAL = 512; /* src/ShGCOOSpDM.cu:44 */
    memset(nnzPerGroup, 0, sizeof(int) * (size_t)(nGroup + 1));
    emu::launch(dim3(nGroup), dim3(BS_OF_CAL), [&] {
        cal_group_coo_format_nnz_kernel_cm<BS_OF_CAL, CPG>(A, m, k, nnzPerGroup);
    });
    emu::launch(dim3(1), dim3(1), [&] { prefix_sum_kernel2(nnzPerGroup, groupIndex, nGroup + 1); });
    const long long nnz = groupIndex[nGroup];
    if (nnz > cap)
        return -1 - nnz;
    emu::launch(dim3(nGroup), dim3(BS_OF_CAL), [&] {
        convert_to_group_coo_format_kernel_cm<BS_OF_CAL, CPG>(A, m, k, vals, rows, cols, groupIndex,
                                                              nnzPerGroup);
    });
    return nnz;
}

extern "C" {

/* Reference conversion (count -> serial scan -> scatter) with template
 * parameter CPG in {1,2,4,8,16}. Returns nnz, -1 for an unsupported CPG, or
 * (-1 - nnz) if the output capacity is too small. */
long long ref_emu_convert(float *A, int m, int k, int cpg, int *groupIndex, int *nnzPerGroup,
                          float *vals, int *rows, int *cols, long long cap)
{
    switch (cpg) {
    case 1: return convert_impl<1>(A, m, k, groupIndex, nnzPerGroup, vals, rows, cols, cap);
    case 2: return convert_impl<2>(A, m, k, groupIndex, nnzPerGroup, vals, rows, cols, cap);
    case 4: return convert_impl<4>(A, m, k, groupIndex, nnzPerGroup, vals, rows, cols, cap);
    case 8: return convert_impl<8>(A, m, k, groupIndex, nnzPerGroup, vals, rows, cols, cap);
    case 16: return convert_impl<16>(A, m, k, groupIndex, nnzPerGroup, vals, rows, cols, cap);
    default: return -1;
    }
}

/* Reference multiply with the reference's compiled constants
 * (COLUMN_PER_GROUP, BS); grid (nGroup, ceil(n/BS)), block BS. */
void ref_emu_spdm(float *vals, int *cols, int *rows, int *groupIndex, int *nnzPerGroup, int m,
                  int k, float *B, int n, float *C)
{
    const int nGroup = (m + COLUMN_PER_GROUP - 1) / COLUMN_PER_GROUP;
    emu::launch(dim3(nGroup, (n + BS - 1) / BS), dim3(BS), [&] {
        sparse_dense_groupcoo_mat_mul_kernel<BS, COLUMN_PER_GROUP>(vals, cols, rows, groupIndex,
                                                                  nnzPerGroup, k, m, B, n, k, C);
    });
}

int ref_emu_column_per_group(void) { return COLUMN_PER_GROUP; }
int ref_emu_bs(void) { return BS; }
}
