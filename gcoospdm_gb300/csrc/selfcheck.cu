// selfcheck.cu -- gcoo_check_bounded_wait: exercises the bounded mbarrier
// wait every staged kernel of the library uses, on a barrier that nothing ever
// arrives on, so that the give-up path (status word set, kernel returns,
// context stays usable) can be tested without faulting or hanging a GPU.
#include "handle.hpp"

namespace gcoo {
namespace {

__global__ void wait_never_kernel(uint64_t limit_ns, uint32_t *status)
{
    __shared__ uint64_t bar;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        fence_mbar_init();
    }
    __syncthreads();
    // No thread arrives on `bar`: the wait must give up after limit_ns.
    const bool done = mbar_wait_ns(&bar, 0, limit_ns);
    if (!done && threadIdx.x == 0)
        atomicOr(status, kStatusWaitTimeout);
}

} // namespace
} // namespace gcoo

using namespace gcoo;

extern "C" gcoo_status gcoo_check_bounded_wait(uint64_t limit_ns, void *stream)
{
    if (limit_ns == 0 || limit_ns > kWaitNs)
        return fail(GCOO_ERROR_INVALID_VALUE, "limit_ns must be in (0, 2e9]");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    DevBuf<uint32_t> status;
    if (!status.ensure(1))
        return fail(GCOO_ERROR_ALLOC, "device allocation failed");
    GCOO_CUDA(cudaMemsetAsync(status.ptr, 0, sizeof(uint32_t), st));
    wait_never_kernel<<<1, 32, 0, st>>>(limit_ns, status.ptr);
    count_launches(1);
    GCOO_LAUNCH("wait_never_kernel");
    uint32_t s = 0;
    GCOO_CUDA(cudaMemcpyAsync(&s, status.ptr, sizeof(s), cudaMemcpyDeviceToHost, st));
    GCOO_CUDA(cudaStreamSynchronize(st));
    if (s & kStatusWaitTimeout)
        return fail(GCOO_ERROR_TIMEOUT, "the bounded wait gave up as designed");
    return GCOO_SUCCESS;
}
