// errnorm.cu -- FP64 error-norm check kernel (the only FP64 work in the
// library): accumulates sum (C - A*B)^2 and sum (A*B)^2 with A*B evaluated in
// FP64 from the packed row layout. FP32 products of the inputs are exact in
// FP64, so the reference value has only FP64 summation error.
#include "internal.cuh"

namespace gcoo {

namespace {

constexpr int kThreads = 128;

__global__ void __launch_bounds__(kThreads)
error_norm_kernel(const Entry *__restrict__ packed, const int32_t *__restrict__ row_ptr, int64_t m,
                  const float *__restrict__ B, int64_t n, const float *__restrict__ C,
                  double *__restrict__ acc2)
{
    __shared__ double s_e[kThreads / 32], s_r[kThreads / 32];
    const int64_t j = static_cast<int64_t>(blockIdx.y) * kThreads + threadIdx.x;
    double err = 0.0, ref = 0.0;
    for (int64_t r = blockIdx.x; r < m; r += gridDim.x) {
        if (j < n) {
            double d = 0.0;
            const int64_t e1 = row_ptr[r + 1];
            for (int64_t e = row_ptr[r]; e < e1; ++e) {
                const Entry t = packed[e];
                d = fma(static_cast<double>(t.val), static_cast<double>(__ldg(B + t.col * n + j)), d);
            }
            const double c = static_cast<double>(C[r * n + j]);
            err += (c - d) * (c - d);
            ref += d * d;
        }
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) {
        err += __shfl_xor_sync(0xffffffffu, err, o);
        ref += __shfl_xor_sync(0xffffffffu, ref, o);
    }
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) {
        s_e[warp] = err;
        s_r[warp] = ref;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0.0, b = 0.0;
        for (int w = 0; w < kThreads / 32; ++w) {
            a += s_e[w];
            b += s_r[w];
        }
        atomicAdd(acc2, a);
        atomicAdd(acc2 + 1, b);
    }
}

} // namespace

cudaError_t launch_error_norm(const Entry *packed, const int32_t *row_ptr, int64_t m, const float *B,
                              int64_t n, const float *C, double *acc2, cudaStream_t st)
{
    const int64_t ny = (n + kThreads - 1) / kThreads;
    if (m <= 0 || ny <= 0)
        return cudaSuccess;
    if (ny > 65535)
        return cudaErrorInvalidConfiguration;
    const int64_t gx = m < 16384 ? m : 16384;
    error_norm_kernel<<<dim3(static_cast<unsigned>(gx), static_cast<unsigned>(ny)), kThreads, 0, st>>>(
        packed, row_ptr, m, B, n, C, acc2);
    count_launches(1);
    return cudaGetLastError();
}

} // namespace gcoo
