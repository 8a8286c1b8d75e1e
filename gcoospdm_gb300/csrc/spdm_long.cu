// spdm_long.cu -- the FP32 multiply of the long rows of a skewed matrix.
//
// A row is one sequential fmaf chain per output element (the reference's
// accumulation order, src/gcoo_spdm_kernels.cu:92-158), so a row of a few
// thousand entries is a long dependent chain; in the row kernel it keeps
// only a handful of B loads in flight and sets the whole launch's length.
// Here one warp owns (long row, 32-column tile) and keeps a deep ring of the
// row's B pieces in flight in shared memory with 16-byte cp.async:
//   * the row's entries arrive kEntryDepth batches of 32 ahead (an 8-byte
//     copy per entry), so the columns of the B pieces are on chip when their
//     copies are issued;
//   * the B pieces (32 columns = 128 bytes of a B row per entry) arrive
//     kDepth batches ahead;
//   * each lane then runs its column's chain over the batch from shared
//     memory, in the row's column order starting from 0.0f -- the same fmaf
//     chain as the row kernel and the reference, so results are bit-identical.
// Rows of at least long_row_min() = 256 entries come here; the others go to
// spdm_short_kernel (spdm_fp32.cu), which runs beside this kernel on the
// caller's stream while this one runs on the handle's side stream.
#include "internal.cuh"

namespace gcoo {

namespace {

constexpr int kBatch = 32;              // entries per batch: one per lane
constexpr int kDepth = 4;               // B batches in flight
constexpr int kEntryDepth = 2 * kDepth; // entry batches on chip
constexpr int kTileCols = 32;           // one column per lane
static_assert(kEntryDepth >= 2 * kDepth - 1, "entries must land before their B pieces are requested");

__device__ __forceinline__ void cp_async16(void *dst, const void *src)
{
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async8(void *dst, const void *src)
{
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

__global__ void collect_long_kernel(const int32_t *__restrict__ row_ptr, int64_t m, int32_t min_len,
                                    int32_t *__restrict__ list, int64_t cap, unsigned long long *__restrict__ count)
{
    for (int64_t r = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; r < m;
         r += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const int32_t len = row_ptr[r + 1] - row_ptr[r];
        if (len >= min_len) {
            const unsigned long long i = atomicAdd(count, 1ull);
            atomicAdd(count + 1, static_cast<unsigned long long>(len)); // the long rows' entries
            if (static_cast<int64_t>(i) < cap)
                list[i] = static_cast<int32_t>(r);
        }
    }
}

__global__ void __launch_bounds__(32)
spdm_long_kernel(const Entry *__restrict__ packed, const int32_t *__restrict__ row_ptr,
                 const int32_t *__restrict__ list, const float *__restrict__ B, int64_t n, float *__restrict__ C)
{
    __shared__ __align__(16) float s_b[kDepth][kBatch][kTileCols];
    __shared__ __align__(16) Entry s_e[kEntryDepth][kBatch];
    const int lane = threadIdx.x;
    const int64_t r = list[blockIdx.x];
    const int64_t j0 = static_cast<int64_t>(blockIdx.y) * kTileCols;
    const Entry *row = packed + row_ptr[r];
    const int cnt = row_ptr[r + 1] - row_ptr[r]; // < 2^31 (int32 format)
    const int nb = (cnt + kBatch - 1) / kBatch;
    // 8 lanes per entry, one 16-byte chunk each: a copy instruction moves four
    // whole 128-byte B pieces; chunks past n are not copied (n % 4 == 0)
    const int sub = lane >> 3, chunk = lane & 7;
    const bool chunk_in = j0 + 4 * chunk < n;
    const float *b_lane = B + j0 + 4 * chunk;

    // step g (g = -(kEntryDepth-1) .. nb-1) commits one group: the entries of
    // batch g + kEntryDepth - 1 and the B pieces of batch g + kDepth - 1
    auto issue = [&](int g) {
        const int be = g + kEntryDepth - 1;
        if (be >= 0 && be * kBatch + lane < cnt)
            cp_async8(&s_e[be % kEntryDepth][lane], row + be * kBatch + lane);
        const int bb = g + kDepth - 1;
        if (bb >= 0 && bb < nb && chunk_in) {
            const Entry *es = s_e[bb % kEntryDepth];
            float *dst = &s_b[bb % kDepth][0][4 * chunk];
#pragma unroll
            for (int it = 0; it < kBatch / 4; ++it) {
                const int e = 4 * it + sub;
                if (bb * kBatch + e < cnt)
                    cp_async16(dst + e * kTileCols, b_lane + static_cast<int64_t>(es[e].col) * n);
            }
        }
        cp_async_commit();
    };

    // before step g requests B pieces, the entries they need (step
    // g - (kEntryDepth - kDepth)) have landed: at most kDepth - 2 steps pending
    for (int g = -(kEntryDepth - 1); g < 0; ++g) {
        cp_async_wait<kDepth - 2>();
        __syncwarp();
        issue(g);
    }
    float acc = 0.0f;
    for (int b = 0; b < nb; ++b) {
        // step b - (kDepth - 1), which carried B batch b, has landed
        cp_async_wait<kDepth - 2>();
        __syncwarp();
        issue(b);
        const Entry *es = s_e[b % kEntryDepth];
        const float *bs = &s_b[b % kDepth][0][lane];
        if (cnt - b * kBatch >= kBatch) {
#pragma unroll
            for (int e = 0; e < kBatch; ++e)
                acc = fmaf(es[e].val, bs[e * kTileCols], acc);
        } else {
            const int len = cnt - b * kBatch;
            for (int e = 0; e < len; ++e)
                acc = fmaf(es[e].val, bs[e * kTileCols], acc);
        }
    }
    cp_async_wait<0>();
    if (j0 + lane < n)
        C[r * n + j0 + lane] = acc;
}

} // namespace

int32_t long_row_min() { return 256; }

bool long_rows_ok(int64_t n, const float *B)
{
    return n % 4 == 0 && (reinterpret_cast<uintptr_t>(B) & 15) == 0 && (n + kTileCols - 1) / kTileCols <= 65535;
}

cudaError_t launch_collect_long(const int32_t *row_ptr, int64_t m, int32_t *list, int64_t cap,
                                unsigned long long *count, cudaStream_t st)
{
    if (m <= 0)
        return cudaSuccess;
    int64_t blocks = (m + 255) / 256;
    if (blocks > 4096)
        blocks = 4096;
    collect_long_kernel<<<static_cast<unsigned>(blocks), 256, 0, st>>>(row_ptr, m, long_row_min(), list, cap, count);
    count_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_spdm_long(const Entry *packed, const int32_t *row_ptr, const int32_t *list, int64_t n_long,
                             const float *B, int64_t n, float *C, cudaStream_t st)
{
    if (n_long <= 0 || n <= 0)
        return cudaSuccess;
    dim3 grid(static_cast<unsigned>(n_long), static_cast<unsigned>((n + kTileCols - 1) / kTileCols));
    spdm_long_kernel<<<grid, 32, 0, st>>>(packed, row_ptr, list, B, n, C);
    count_launches(1);
    return cudaGetLastError();
}

} // namespace gcoo
