// baseline_l2peak.cu -- the L2 -> SM read peak of this GPU, measured: the
// roofline denominator for multiplies whose B gathers are served by L2 (every
// FP32 point with more than a few entries per row reads nnz * n * 4 bytes of
// B rows from L2, several times B's size, so that path binds before HBM).
//
// The probe reads 512-byte segments (one 16-byte load per lane, a warp-wide
// contiguous piece, the shape of a B-row load of the multiply) at
// pseudo-random segment offsets inside a 32 MB region that stays resident in
// L2, four segments in flight per warp, 8 CTAs of 256 threads per SM. No
// waits, no atomics: a plain streaming kernel timed with CUDA events.
// Comparison infrastructure like the cuBLAS / cuSPARSE plugins beside it
// (libgcoo_baselines.so); nothing in libgcoo.so calls it.
#include <cuda_runtime.h>
#include <stdint.h>

namespace {

constexpr int kInFlight = 4;

__global__ void __launch_bounds__(256) l2_gather_kernel(const float4 *__restrict__ src, uint32_t seg_mask, int iters,
                                                        float *__restrict__ sink)
{
    const int lane = threadIdx.x & 31;
    uint32_t h = ((blockIdx.x * blockDim.x + threadIdx.x) >> 5) * 2654435761u + 12345u;
    float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int it = 0; it < iters; ++it) {
        float4 v[kInFlight];
#pragma unroll
        for (int u = 0; u < kInFlight; ++u) {
            h = h * 1664525u + 1013904223u; // a linear congruential walk over segments
            const uint32_t seg = (h >> 7) & seg_mask;
            v[u] = __ldg(src + static_cast<size_t>(seg) * 32 + lane);
        }
#pragma unroll
        for (int u = 0; u < kInFlight; ++u) {
            acc.x += v[u].x;
            acc.y += v[u].y;
            acc.z += v[u].z;
            acc.w += v[u].w;
        }
    }
    if (acc.x + acc.y + acc.z + acc.w == 1234.5f) // never true for the zeroed source: keeps the loads live
        sink[0] = acc.x;
}

} // namespace

extern "C" {

// Best of `reps` timed launches (after one warm-up), in GB/s of bytes read
// by the SMs; 0 on any CUDA error (the message is not kept).
double gcoo_measure_l2_read_gbs(int reps)
{
    const size_t region = 32ull << 20;
    const uint32_t segs = static_cast<uint32_t>(region / 512);
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return 0.0;
    float4 *src = nullptr;
    float *sink = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    double best = 0.0;
    const int blocks = sms * 8, iters = 256;
    if (cudaMalloc(&src, region) == cudaSuccess && cudaMalloc(&sink, 16) == cudaSuccess &&
        cudaMemset(src, 0, region) == cudaSuccess && cudaEventCreate(&e0) == cudaSuccess &&
        cudaEventCreate(&e1) == cudaSuccess) {
        const double bytes = static_cast<double>(blocks) * 8 * iters * kInFlight * 512;
        for (int r = 0; r <= reps; ++r) {
            cudaEventRecord(e0);
            l2_gather_kernel<<<blocks, 256>>>(src, segs - 1, iters, sink);
            cudaEventRecord(e1);
            if (cudaEventSynchronize(e1) != cudaSuccess)
                break;
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            if (r > 0 && ms > 0.f && bytes / ms / 1e6 > best)
                best = bytes / ms / 1e6;
        }
        if (cudaGetLastError() != cudaSuccess)
            best = 0.0;
    }
    if (e0)
        cudaEventDestroy(e0);
    if (e1)
        cudaEventDestroy(e1);
    cudaFree(src);
    cudaFree(sink);
    return best;
}

} // extern "C"
