// spdm_split.cu -- the FP32 multiply's long rows summed in pieces
// (gcoo_params.fp32_sum = GCOO_SUM_SPLIT).
//
// The default FP32 multiply keeps every output element one sequential fmaf
// chain over its row in column order (src/gcoo_spdm_kernels.cu:129-139), so
// a row of 4096 entries is a 4096-long dependent chain and the long rows of
// a skewed matrix set the multiply's length. This mode relaxes that order
// for the rows of at least long_row_min() = 256 entries only:
//   * each long row is cut into pieces of kPiece consecutive entries (its
//     column order); one warp sums a piece as a sequential fmaf chain from
//     0.0f for 256 output columns (two 128-column tiles, 16-byte B loads)
//     into a partial row of a handle-owned buffer;
//   * one thread per (long row, column) then adds the row's partials from
//     0.0f in piece order.
// Every piece and every combine has a fixed order, so results are
// deterministic (the same bits on every run and for every launch order),
// but not bit-identical to the sequential chain: the sum of a long row is
// regrouped. The error stays at FP32 rounding level (chains of at most
// kPiece terms plus a sum of ceil(len / kPiece) partials).
//
// The piece plan (piece -> long row, long row -> first piece) is built on
// the device once per build by one CTA, from the long-row list, its length
// and the row pointers, before the build's one readback; the partial-sum
// buffer is sized from the long rows' entry total read back with the list's
// length, so the plan needs no readback of its own.
#include "internal.cuh"

namespace gcoo {

namespace {

constexpr int kPiece = 32;         // entries per piece: one 32-entry window per warp
static_assert(kPiece <= 32, "a piece's entries are one warp-wide window");
constexpr int kPieceCols = 256;    // output columns per piece warp: two 128-column tiles
constexpr int kPlanThreads = 1024; // the plan kernel's single CTA
constexpr int kPieceBatch = 4;     // entries per batch: 2 x kPieceBatch 16-byte B loads in flight

__global__ void __launch_bounds__(kPlanThreads)
split_plan_kernel(const int32_t *__restrict__ row_ptr, const int32_t *__restrict__ list,
                  const unsigned long long *__restrict__ count, int64_t list_cap, int32_t *__restrict__ piece_first,
                  int32_t *__restrict__ piece_row, int64_t cap, int32_t *__restrict__ total)
{
    __shared__ int32_t warp_sums[kPlanThreads / 32];
    __shared__ int32_t carry;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int64_t n_long = static_cast<int64_t>(count[0]) < list_cap ? static_cast<int64_t>(count[0]) : list_cap;
    if (tid == 0)
        carry = 0;
    __syncthreads();
    for (int64_t base = 0; base < n_long; base += kPlanThreads) {
        const int64_t li = base + tid;
        int32_t pieces = 0;
        if (li < n_long) {
            const int32_t r = list[li];
            pieces = (row_ptr[r + 1] - row_ptr[r] + kPiece - 1) / kPiece;
        }
        // block-wide inclusive scan of the piece counts
        int32_t x = pieces;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const int32_t y = __shfl_up_sync(0xffffffffu, x, d);
            if (lane >= d)
                x += y;
        }
        if (lane == 31)
            warp_sums[warp] = x;
        __syncthreads();
        if (warp == 0) {
            int32_t w = warp_sums[lane];
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const int32_t y = __shfl_up_sync(0xffffffffu, w, d);
                if (lane >= d)
                    w += y;
            }
            warp_sums[lane] = w; // inclusive over warps
        }
        __syncthreads();
        const int32_t first = carry + (warp > 0 ? warp_sums[warp - 1] : 0) + x - pieces;
        if (li < n_long) {
            piece_first[li] = first;
            for (int32_t q = 0; q < pieces; ++q)
                if (first + q < cap)
                    piece_row[first + q] = static_cast<int32_t>(li);
        }
        __syncthreads();
        if (tid == 0)
            carry += warp_sums[kPlanThreads / 32 - 1];
        __syncthreads();
    }
    if (tid == 0)
        *total = carry < cap ? carry : static_cast<int32_t>(cap);
}

// One warp per (piece, 256-column group): the piece's entries (lane i holds
// entry i), B rows of kPieceBatch entries at a time for both 128-column
// tiles, each column's chain over the piece in column order.
__global__ void __launch_bounds__(64)
spdm_piece_kernel(const Entry *__restrict__ packed, const int32_t *__restrict__ row_ptr,
                  const int32_t *__restrict__ list, const int32_t *__restrict__ piece_first,
                  const int32_t *__restrict__ piece_row, const int32_t *__restrict__ total, const float *__restrict__ B,
                  int64_t n, int32_t groups, float *__restrict__ part)
{
    const int lane = threadIdx.x & 31;
    const int64_t gw = (static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const int64_t p = gw / groups;
    if (p >= *total)
        return; // warp-uniform
    const int g = static_cast<int>(gw - p * groups);
    const int32_t li = piece_row[p];
    const int32_t r = list[li];
    const int32_t rs = row_ptr[r], re = row_ptr[r + 1];
    const int32_t e0 = rs + (static_cast<int32_t>(p) - piece_first[li]) * kPiece;
    const int nw = re - e0 < kPiece ? re - e0 : kPiece; // >= 1 by construction
    const int64_t ja = static_cast<int64_t>(g) * kPieceCols + lane * 4, jb = ja + 128;
    const bool has_a = ja < n, has_b = jb < n;
    Entry my;
    my.col = 0;
    my.val = 0.0f;
    if (lane < nw)
        my = packed[e0 + lane];
    float acc_a[4] = {0.f, 0.f, 0.f, 0.f}, acc_b[4] = {0.f, 0.f, 0.f, 0.f};
    for (int u0 = 0; u0 < nw; u0 += kPieceBatch) {
        float a[kPieceBatch], ba[kPieceBatch][4], bb[kPieceBatch][4];
#pragma unroll
        for (int u = 0; u < kPieceBatch; ++u) {
            const int col = __shfl_sync(0xffffffffu, my.col, (u0 + u) & 31);
            a[u] = __shfl_sync(0xffffffffu, my.val, (u0 + u) & 31);
            const float *Bc = B + static_cast<int64_t>(col) * n;
            float4 x = make_float4(0.f, 0.f, 0.f, 0.f), y = x;
            if (u0 + u < nw && has_a)
                x = __ldg(reinterpret_cast<const float4 *>(Bc + ja));
            if (u0 + u < nw && has_b)
                y = __ldg(reinterpret_cast<const float4 *>(Bc + jb));
            ba[u][0] = x.x; ba[u][1] = x.y; ba[u][2] = x.z; ba[u][3] = x.w;
            bb[u][0] = y.x; bb[u][1] = y.y; bb[u][2] = y.z; bb[u][3] = y.w;
        }
#pragma unroll
        for (int u = 0; u < kPieceBatch; ++u)
            if (u0 + u < nw)
#pragma unroll
                for (int v = 0; v < 4; ++v) {
                    acc_a[v] = fmaf(a[u], ba[u][v], acc_a[v]);
                    acc_b[v] = fmaf(a[u], bb[u][v], acc_b[v]);
                }
    }
    float *out = part + p * n;
    if (has_a)
        *reinterpret_cast<float4 *>(out + ja) = make_float4(acc_a[0], acc_a[1], acc_a[2], acc_a[3]);
    if (has_b)
        *reinterpret_cast<float4 *>(out + jb) = make_float4(acc_b[0], acc_b[1], acc_b[2], acc_b[3]);
}

// C[row][j] = the row's partials added from 0.0f in piece order.
__global__ void __launch_bounds__(256)
split_combine_kernel(const int32_t *__restrict__ row_ptr, const int32_t *__restrict__ list,
                     const int32_t *__restrict__ piece_first, const int32_t *__restrict__ total,
                     const float *__restrict__ part, int64_t n, float *__restrict__ C)
{
    const int64_t li = blockIdx.x;
    const int64_t j = static_cast<int64_t>(blockIdx.y) * blockDim.x + threadIdx.x;
    if (j >= n)
        return;
    const int32_t r = list[li];
    const int32_t pieces = (row_ptr[r + 1] - row_ptr[r] + kPiece - 1) / kPiece;
    const int32_t first = piece_first[li];
    const int32_t end = first + pieces < *total ? first + pieces : *total;
    // eight partials' loads in flight at a time, added one by one in piece order
    float sum = 0.0f;
    int32_t q = first;
    for (; q + 8 <= end; q += 8) {
        float x[8];
#pragma unroll
        for (int u = 0; u < 8; ++u)
            x[u] = part[static_cast<int64_t>(q + u) * n + j];
#pragma unroll
        for (int u = 0; u < 8; ++u)
            sum += x[u];
    }
    for (; q < end; ++q)
        sum += part[static_cast<int64_t>(q) * n + j];
    C[static_cast<int64_t>(r) * n + j] = sum;
}

} // namespace

int64_t split_piece_bound(int64_t n_long, int64_t long_entries)
{
    // ceil(len / kPiece) <= len / kPiece + 1 per row
    return n_long <= 0 ? 0 : long_entries / kPiece + n_long;
}

cudaError_t launch_split_plan(const int32_t *row_ptr, const int32_t *list, const unsigned long long *count,
                              int64_t list_cap, int32_t *piece_first, int32_t *piece_row, int64_t cap,
                              int32_t *total, cudaStream_t st)
{
    split_plan_kernel<<<1, kPlanThreads, 0, st>>>(row_ptr, list, count, list_cap, piece_first, piece_row, cap,
                                                   total);
    count_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_spdm_split(const Entry *packed, const int32_t *row_ptr, const int32_t *list, int64_t n_long,
                              const int32_t *piece_first, const int32_t *piece_row, const int32_t *total,
                              int64_t pieces_bound, const float *B, int64_t n, float *part, float *C,
                              cudaStream_t st)
{
    if (n_long <= 0 || n <= 0 || pieces_bound <= 0)
        return cudaSuccess;
    const int64_t groups = (n + kPieceCols - 1) / kPieceCols;
    const int64_t warps = pieces_bound * groups;
    const int64_t blocks = (warps + 1) / 2;
    const int64_t ny = (n + 255) / 256;
    if (groups > 0x7fffffffLL || blocks > 0x7fffffffLL || n_long > 0x7fffffffLL || ny > 65535)
        return cudaErrorInvalidConfiguration;
    spdm_piece_kernel<<<static_cast<unsigned>(blocks), 64, 0, st>>>(packed, row_ptr, list, piece_first, piece_row,
                                                                     total, B, n, static_cast<int32_t>(groups), part);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess)
        return e;
    dim3 grid(static_cast<unsigned>(n_long), static_cast<unsigned>(ny));
    split_combine_kernel<<<grid, 256, 0, st>>>(row_ptr, list, piece_first, total, part, n, C);
    count_launches(2);
    return cudaGetLastError();
}

} // namespace gcoo
