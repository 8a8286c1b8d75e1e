// baseline_refalgo.cu -- BASELINE ONLY: the reference's GCOO algorithm
// (hclhkbu/gcoospdm src/gcoo_spdm_kernels.cu, orchestrated by
// src/ShGCOOSpDM.cu:19-180) restated for the GPU so it can be timed next to
// this library on the same GB300. The reference's own sources cannot be built
// where the benchmark runs, so this is a restatement of its algorithm, not its
// code:
//   * count: one 512-thread CTA per group of 4 rows, each thread counting a
//     strided set of columns, block reduction;
//   * scan: one thread walks the group counts serially (<<<1,1>>>);
//   * the host reads the total back and allocates the entry arrays per call;
//   * scatter: one 512-thread CTA per group, one column per thread per tile,
//     block scan for the column offsets;
//   * multiply: one 128-thread CTA per (group, 128 columns), entries staged in
//     chunks of 128 through shared memory, one thread per output column with
//     four accumulators picked by row & 3, a scalar B load whenever the column
//     changes.
// Its results are bit-identical to the library's (same fmaf chains).
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>

namespace {

constexpr int kCpg = 4;
constexpr int kConvThreads = 512;
constexpr int kMulThreads = 128;

__device__ int block_sum_512(int v, int *s)
{
    s[threadIdx.x] = v;
    __syncthreads();
    for (int d = kConvThreads / 2; d > 0; d >>= 1) {
        if (threadIdx.x < d)
            s[threadIdx.x] += s[threadIdx.x + d];
        __syncthreads();
    }
    const int t = s[0];
    __syncthreads();
    return t;
}

__global__ void ref_count(const float *A, int64_t m, int64_t k, int *cnt)
{
    __shared__ int s[kConvThreads];
    const int64_t r0 = static_cast<int64_t>(blockIdx.x) * kCpg;
    int c = 0;
    for (int64_t col = threadIdx.x; col < k; col += kConvThreads)
        for (int j = 0; j < kCpg && r0 + j < m; ++j)
            c += A[(r0 + j) * k + col] != 0.0f;
    const int t = block_sum_512(c, s);
    if (threadIdx.x == 0)
        cnt[blockIdx.x] = t;
}

__global__ void ref_serial_scan(const int *cnt, int *gi, int64_t n)
{
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        gi[0] = 0;
        for (int64_t i = 1; i < n; ++i)
            gi[i] = gi[i - 1] + cnt[i - 1];
    }
}

__global__ void ref_scatter(const float *A, int64_t m, int64_t k, const int *gi, float *vals, int *rows, int *cols)
{
    __shared__ int s[kConvThreads];
    const int64_t r0 = static_cast<int64_t>(blockIdx.x) * kCpg;
    int64_t base = gi[blockIdx.x];
    for (int64_t t0 = 0; t0 < k; t0 += kConvThreads) {
        const int64_t col = t0 + threadIdx.x;
        float v[kCpg];
        int c = 0;
        for (int j = 0; j < kCpg; ++j) {
            v[j] = (col < k && r0 + j < m) ? A[(r0 + j) * k + col] : 0.0f;
            c += v[j] != 0.0f;
        }
        // inclusive scan of the per-column counts (Hillis-Steele in shared memory)
        s[threadIdx.x] = c;
        __syncthreads();
        for (int d = 1; d < kConvThreads; d <<= 1) {
            const int x = threadIdx.x >= d ? s[threadIdx.x - d] : 0;
            __syncthreads();
            s[threadIdx.x] += x;
            __syncthreads();
        }
        int64_t pos = base + s[threadIdx.x] - c;
        const int tile_total = s[kConvThreads - 1];
        for (int j = 0; j < kCpg; ++j)
            if (v[j] != 0.0f) {
                vals[pos] = v[j];
                rows[pos] = static_cast<int>(r0 + j);
                cols[pos] = static_cast<int>(col);
                ++pos;
            }
        base += tile_total;
        __syncthreads();
    }
}

__global__ void ref_multiply(const float *vals, const int *cols, const int *rows, const int *gi, int64_t m,
                             const float *B, int64_t n, float *C)
{
    __shared__ float s_v[kMulThreads];
    __shared__ int s_c[kMulThreads];
    __shared__ int s_r[kMulThreads];
    const int64_t j = static_cast<int64_t>(blockIdx.y) * kMulThreads + threadIdx.x;
    const int64_t r0 = static_cast<int64_t>(blockIdx.x) * kCpg;
    const int64_t e0 = gi[blockIdx.x], e1 = gi[blockIdx.x + 1];
    float acc[kCpg] = {0.0f, 0.0f, 0.0f, 0.0f};
    for (int64_t ch = e0; ch < e1; ch += kMulThreads) {
        const int64_t e = ch + threadIdx.x;
        if (e < e1) {
            s_v[threadIdx.x] = vals[e];
            s_c[threadIdx.x] = cols[e];
            s_r[threadIdx.x] = rows[e];
        }
        __syncthreads();
        const int len = static_cast<int>(e1 - ch < kMulThreads ? e1 - ch : kMulThreads);
        if (j < n) {
            int prev = -1;
            float b = 0.0f;
            for (int i = 0; i < len; ++i) {
                if (s_c[i] != prev) {
                    prev = s_c[i];
                    b = B[static_cast<int64_t>(prev) * n + j];
                }
                const int lr = s_r[i] & (kCpg - 1);
                acc[lr] = fmaf(s_v[i], b, acc[lr]);
            }
        }
        __syncthreads();
    }
    if (j < n)
        for (int i = 0; i < kCpg; ++i)
            if (r0 + i < m)
                C[(r0 + i) * n + j] = acc[i];
}

struct RefAlgo {
    const float *A = nullptr;
    int64_t m = 0, k = 0;
    int *gi = nullptr, *cnt = nullptr; // built (kernel-only path)
    float *vals = nullptr;
    int *rc = nullptr;
    int64_t nnz = 0;
};

bool ck(cudaError_t e, const char *w)
{
    if (e != cudaSuccess) {
        fprintf(stderr, "refalgo %s: %s\n", w, cudaGetErrorString(e));
        return false;
    }
    return true;
}

// convertToGroupCOOFormat: allocates per call, like the reference.
bool convert(RefAlgo &r, int *&gi, float *&vals, int *&rc, int64_t &nnz)
{
    const int64_t ng = (r.m + kCpg - 1) / kCpg;
    int *cnt = nullptr;
    if (!ck(cudaMalloc(&gi, sizeof(int) * (ng + 1) * 2), "malloc"))
        return false;
    cnt = gi + ng + 1;
    cudaMemset(cnt, 0, sizeof(int) * (ng + 1));
    ref_count<<<static_cast<unsigned>(ng), kConvThreads>>>(r.A, r.m, r.k, cnt);
    cudaDeviceSynchronize();
    ref_serial_scan<<<1, 1>>>(cnt, gi, ng + 1);
    cudaDeviceSynchronize();
    int total = 0;
    if (!ck(cudaMemcpy(&total, gi + ng, sizeof(int), cudaMemcpyDeviceToHost), "readback"))
        return false;
    nnz = total;
    if (!ck(cudaMalloc(&vals, sizeof(float) * (nnz > 0 ? nnz : 1)), "malloc") ||
        !ck(cudaMalloc(&rc, sizeof(int) * (nnz > 0 ? nnz : 1) * 2), "malloc"))
        return false;
    ref_scatter<<<static_cast<unsigned>(ng), kConvThreads>>>(r.A, r.m, r.k, gi, vals, rc, rc + nnz);
    cudaDeviceSynchronize();
    return ck(cudaGetLastError(), "convert");
}

bool multiply(RefAlgo &r, const int *gi, const float *vals, const int *rc, int64_t nnz, const float *B, int64_t n,
              float *C)
{
    const int64_t ng = (r.m + kCpg - 1) / kCpg;
    dim3 grid(static_cast<unsigned>(ng), static_cast<unsigned>((n + kMulThreads - 1) / kMulThreads));
    ref_multiply<<<grid, kMulThreads>>>(vals, rc + nnz, rc, gi, r.m, B, n, C);
    cudaDeviceSynchronize();
    return ck(cudaGetLastError(), "multiply");
}

} // namespace

extern "C" {

void *gcoo_refalgo_create(const float *dA, int64_t m, int64_t k)
{
    RefAlgo *r = new RefAlgo();
    r->A = dA;
    r->m = m;
    r->k = k;
    return r;
}

// mutiplyBy: convert (allocating) + multiply + free, all synchronous.
int gcoo_refalgo_multiply_by(void *h, const float *dB, int64_t n, float *dC)
{
    RefAlgo &r = *static_cast<RefAlgo *>(h);
    int *gi = nullptr, *rc = nullptr;
    float *vals = nullptr;
    int64_t nnz = 0;
    bool ok = convert(r, gi, vals, rc, nnz) && multiply(r, gi, vals, rc, nnz, dB, n, dC);
    cudaFree(vals);
    cudaFree(rc);
    cudaFree(gi);
    return ok ? 0 : 3;
}

// build + runKernelTest
int gcoo_refalgo_build(void *h)
{
    RefAlgo &r = *static_cast<RefAlgo *>(h);
    cudaFree(r.vals);
    cudaFree(r.rc);
    cudaFree(r.gi);
    r.vals = nullptr;
    r.rc = r.gi = nullptr;
    return convert(r, r.gi, r.vals, r.rc, r.nnz) ? 0 : 3;
}

int gcoo_refalgo_run_kernel(void *h, const float *dB, int64_t n, float *dC)
{
    RefAlgo &r = *static_cast<RefAlgo *>(h);
    return multiply(r, r.gi, r.vals, r.rc, r.nnz, dB, n, dC) ? 0 : 3;
}

void gcoo_refalgo_destroy(void *h)
{
    RefAlgo *r = static_cast<RefAlgo *>(h);
    cudaFree(r->vals);
    cudaFree(r->rc);
    cudaFree(r->gi);
    delete r;
}
}
