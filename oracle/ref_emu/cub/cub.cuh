/*
 * cub/cub.cuh -- TEST INFRASTRUCTURE ONLY: host stand-in for the two CUB
 * block primitives the reference kernels use (BlockReduce::Sum,
 * BlockScan::InclusiveSum / ExclusiveSum), for running those kernels under
 * the fiber emulator in emu.h. The reference pins NVlabs/cub at no commit
 * (.gitmodules, branch master); for integer sums every correct reduction or
 * scan gives the same result, so a direct serial formulation over a shared
 * array reproduces CUB's outputs exactly.
 */
#ifndef GCOO_REF_EMU_CUB_SHIM
#define GCOO_REF_EMU_CUB_SHIM

#include "../emu.h"

namespace cub {

template <typename T, int BLOCK_DIM_X>
class BlockReduce {
  public:
    struct TempStorage {
        T v[BLOCK_DIM_X];
    };
    explicit BlockReduce(TempStorage &s) : s_(s) {}
    /* CUB returns the aggregate in thread 0; every thread gets it here. */
    T Sum(T x)
    {
        s_.v[threadIdx.x] = x;
        __syncthreads();
        T acc = T();
        for (int i = 0; i < BLOCK_DIM_X; ++i)
            acc += s_.v[i];
        __syncthreads();
        return acc;
    }

  private:
    TempStorage &s_;
};

template <typename T, int BLOCK_DIM_X>
class BlockScan {
  public:
    struct TempStorage {
        T v[BLOCK_DIM_X];
    };
    explicit BlockScan(TempStorage &s) : s_(s) {}
    void InclusiveSum(T in, T &out)
    {
        const unsigned t = threadIdx.x;
        s_.v[t] = in;
        __syncthreads();
        T acc = T();
        for (unsigned i = 0; i <= t; ++i)
            acc += s_.v[i];
        __syncthreads();
        out = acc;
    }
    void ExclusiveSum(T in, T &out)
    {
        const unsigned t = threadIdx.x;
        s_.v[t] = in;
        __syncthreads();
        T acc = T();
        for (unsigned i = 0; i < t; ++i)
            acc += s_.v[i];
        __syncthreads();
        out = acc;
    }

  private:
    TempStorage &s_;
};

} // namespace cub

#endif
