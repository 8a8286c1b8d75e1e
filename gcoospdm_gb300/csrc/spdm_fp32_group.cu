// spdm_fp32_group.cu -- FP32 multiply in GCOO order, for groups whose rows
// share columns.
//
// The same product as spdm_fp32_kernel and the reference's
// sparse_dense_groupcoo_mat_mul_kernel (src/gcoo_spdm_kernels.cu:92-158),
// organised like the latter: a warp walks all entries of its group in the
// reference's GCOO order (column, then row) and keeps one accumulator set per
// row of the group (four rows: the reference's c0..c3). Consecutive entries
// with the same column reuse the B values already in registers, so when the
// rows of a group share columns (block-clustered matrices) a B segment is
// fetched once per group instead of once per row. Each row's entries are
// still visited in column order, so every C element is the same fmaf chain as
// the reference's: the same bits.
//
// One CTA per (group, 4 * 32 * V columns); the group's entries are staged
// cooperatively in chunks into shared memory as {col, row in group, value};
// each warp covers 32 * V columns of all four rows, B loaded V columns per lane
// with one vector load per distinct column, the loads of U column runs in
// flight together.
#include "internal.cuh"

namespace gcoo {

namespace {

constexpr int kGroupRows = 4;
constexpr int kGThreads = 128;
constexpr int kGWarps = kGThreads / 32;
constexpr int kGChunk = 1024; // entries staged per pass (16 KB)

template <int V>
__device__ __forceinline__ void ldv(const float *p, float (&o)[V])
{
    if (V == 8) {
        const float4 t = __ldg(reinterpret_cast<const float4 *>(p));
        const float4 w = __ldg(reinterpret_cast<const float4 *>(p) + 1);
        o[0] = t.x;
        o[1] = t.y;
        o[2] = t.z;
        o[3] = t.w;
        o[4 % V] = w.x;
        o[5 % V] = w.y;
        o[6 % V] = w.z;
        o[7 % V] = w.w;
    } else if (V == 4) {
        const float4 t = __ldg(reinterpret_cast<const float4 *>(p));
        o[0] = t.x;
        o[1] = t.y;
        o[2] = t.z;
        o[3] = t.w;
    } else if (V == 2) {
        const float2 t = __ldg(reinterpret_cast<const float2 *>(p));
        o[0] = t.x;
        o[1] = t.y;
    } else {
        o[0] = __ldg(p);
    }
}

template <int V>
__device__ __forceinline__ void stv(float *p, const float (&o)[V])
{
    if (V == 8) {
        reinterpret_cast<float4 *>(p)[0] = make_float4(o[0], o[1], o[2], o[3]);
        reinterpret_cast<float4 *>(p)[1] = make_float4(o[4 % V], o[5 % V], o[6 % V], o[7 % V]);
    } else if (V == 4)
        *reinterpret_cast<float4 *>(p) = make_float4(o[0], o[1], o[2], o[3]);
    else if (V == 2)
        *reinterpret_cast<float2 *>(p) = make_float2(o[0], o[1]);
    else
        *p = o[0];
}

// acc[lr] += a * b, lr warp-uniform in [0, 4): a uniform branch, as in the
// reference's if-chain.
template <int V>
__device__ __forceinline__ void fma_row(float (&acc)[kGroupRows][V], int lr, float a, const float (&b)[V])
{
    if (lr == 0) {
#pragma unroll
        for (int v = 0; v < V; ++v)
            acc[0][v] = fmaf(a, b[v], acc[0][v]);
    } else if (lr == 1) {
#pragma unroll
        for (int v = 0; v < V; ++v)
            acc[1][v] = fmaf(a, b[v], acc[1][v]);
    } else if (lr == 2) {
#pragma unroll
        for (int v = 0; v < V; ++v)
            acc[2][v] = fmaf(a, b[v], acc[2][v]);
    } else {
#pragma unroll
        for (int v = 0; v < V; ++v)
            acc[3][v] = fmaf(a, b[v], acc[3][v]);
    }
}

// Takes the next U run starts (lanes) from `starts`; rs[U] is the start after
// them (or wn), so run u covers lanes [rs[u], rs[u+1]). Missing runs get wn.
template <int U>
__device__ __forceinline__ void take_runs(unsigned &starts, int wn, int (&rs)[U + 1])
{
#pragma unroll
    for (int u = 0; u < U; ++u) {
        rs[u] = starts ? __ffs(starts) - 1 : wn;
        starts &= starts ? starts - 1 : 0u;
    }
    rs[U] = starts ? __ffs(starts) - 1 : wn;
}

template <int U, int V>
__device__ __forceinline__ void load_runs(const int (&rs)[U + 1], int wn, int col_of_lane, bool has_col,
                                          const float *Bj, int64_t n, float (&b)[U][V])
{
#pragma unroll
    for (int u = 0; u < U; ++u) {
        const int c = __shfl_sync(0xffffffffu, col_of_lane, rs[u] < 32 ? rs[u] : 0);
        if (rs[u] < wn && has_col)
            ldv<V>(Bj + static_cast<int64_t>(c) * n, b[u]);
    }
}

// Applies each run's entries (at most one per row, rows ascending) in order.
template <int U, int V>
__device__ __forceinline__ void apply_runs(const int (&rs)[U + 1], int wn, const int4 &mine, const float (&b)[U][V],
                                           float (&acc)[kGroupRows][V], int &prev, float (&pb)[V])
{
#pragma unroll
    for (int u = 0; u < U; ++u) {
        if (rs[u] >= wn)
            break;
        if (rs[u + 1] - rs[u] == kGroupRows) {
            // a full run: rows 0..3 in order (GCOO order is column, then row)
#pragma unroll
            for (int r = 0; r < kGroupRows; ++r) {
                const float a = __int_as_float(__shfl_sync(0xffffffffu, mine.z, rs[u] + r));
#pragma unroll
                for (int v = 0; v < V; ++v)
                    acc[r][v] = fmaf(a, b[u][v], acc[r][v]);
            }
        } else {
            for (int q = rs[u]; q < rs[u + 1]; ++q)
                fma_row<V>(acc, __shfl_sync(0xffffffffu, mine.y, q), __int_as_float(__shfl_sync(0xffffffffu, mine.z, q)),
                           b[u]);
        }
        prev = __shfl_sync(0xffffffffu, mine.x, rs[u]);
#pragma unroll
        for (int v = 0; v < V; ++v)
            pb[v] = b[u][v];
    }
}

template <int V, int U>
__global__ void __launch_bounds__(kGThreads)
spdm_fp32_group_kernel(const float *__restrict__ vals, const int32_t *__restrict__ rows,
                       const int32_t *__restrict__ cols, const int32_t *__restrict__ group_index, int64_t m,
                       const float *__restrict__ B, int64_t n, float *__restrict__ C)
{
    __shared__ int4 s_e[kGChunk]; // {col, row - r0, value bits, 0}
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t g = blockIdx.x;
    const int64_t r0 = g * kGroupRows;
    const int nrows = static_cast<int>(r0 + kGroupRows <= m ? kGroupRows : m - r0);
    const int64_t j = (static_cast<int64_t>(blockIdx.y) * kGWarps + warp) * (32 * V) + static_cast<int64_t>(lane) * V;
    const bool has_col = j < n;
    const float *Bj = B + (has_col ? j : 0);
    const int64_t e0 = group_index[g], e1 = group_index[g + 1];

    float acc[kGroupRows][V];
#pragma unroll
    for (int r = 0; r < kGroupRows; ++r)
#pragma unroll
        for (int v = 0; v < V; ++v)
            acc[r][v] = 0.0f;
    int prev = -1; // column whose B values are in pb
    float pb[V];
#pragma unroll
    for (int v = 0; v < V; ++v)
        pb[v] = 0.0f;

    for (int64_t cs = e0; cs < e1; cs += kGChunk) {
        const int cnt = static_cast<int>(e1 - cs < kGChunk ? e1 - cs : kGChunk);
        __syncthreads(); // the previous chunk has been consumed
        for (int i = threadIdx.x; i < cnt; i += kGThreads)
            s_e[i] = make_int4(cols[cs + i], rows[cs + i] - static_cast<int32_t>(r0), __float_as_int(vals[cs + i]), 0);
        __syncthreads();
        // the window logic below is warp-synchronous: lanes past n take part
        // in it without loading, and a warp skips only when none has columns
        if (!__any_sync(0xffffffffu, has_col))
            continue;
        // 32-entry windows: one ballot finds where column runs start; the B
        // loads of up to U runs are issued together, then each run's entries
        // (at most one per row) are applied in order. A run continuing from
        // the previous window keeps the B values already held in pb.
        for (int base = 0; base < cnt; base += 32) {
            const int wn = cnt - base < 32 ? cnt - base : 32;
            const int4 mine = lane < wn ? s_e[base + lane] : make_int4(-1, 0, 0, 0);
            int before = __shfl_up_sync(0xffffffffu, mine.x, 1);
            if (lane == 0)
                before = prev;
            unsigned starts = __ballot_sync(0xffffffffu, lane < wn && mine.x != before);
            // entries ahead of the first run start continue the previous column
            const int head = starts ? __ffs(starts) - 1 : wn;
            for (int q = 0; q < head; ++q)
                fma_row<V>(acc, __shfl_sync(0xffffffffu, mine.y, q), __int_as_float(__shfl_sync(0xffffffffu, mine.z, q)),
                           pb);
            while (starts) {
                int rs[U + 1];
                float b[U][V];
                take_runs<U>(starts, wn, rs);
                load_runs<U, V>(rs, wn, mine.x, has_col, Bj, n, b);
                apply_runs<U, V>(rs, wn, mine, b, acc, prev, pb);
            }
        }
    }
    if (has_col) {
#pragma unroll
        for (int r = 0; r < kGroupRows; ++r)
            if (r < nrows)
                stv<V>(C + (r0 + r) * n + j, acc[r]);
    }
}

} // namespace

bool group_order_ok(int32_t rows_per_group) { return rows_per_group == kGroupRows; }

cudaError_t launch_spdm_fp32_group(const float *vals, const int32_t *rows, const int32_t *cols,
                                   const int32_t *group_index, int64_t m, int64_t ng, const float *B, int64_t n,
                                   float *C, int vec, cudaStream_t st)
{
    if (ng <= 0 || n <= 0)
        return cudaSuccess;
    const int64_t tile = static_cast<int64_t>(kGWarps) * 32 * vec;
    const int64_t ny = (n + tile - 1) / tile;
    if (ny > 65535 || ng > 0x7fffffffLL)
        return cudaErrorInvalidConfiguration;
    dim3 grid(static_cast<unsigned>(ng), static_cast<unsigned>(ny));
    if (vec == 8)
        spdm_fp32_group_kernel<8, 2><<<grid, kGThreads, 0, st>>>(vals, rows, cols, group_index, m, B, n, C);
    else if (vec == 4)
        spdm_fp32_group_kernel<4, 2><<<grid, kGThreads, 0, st>>>(vals, rows, cols, group_index, m, B, n, C);
    else if (vec == 2)
        spdm_fp32_group_kernel<2, 4><<<grid, kGThreads, 0, st>>>(vals, rows, cols, group_index, m, B, n, C);
    else
        spdm_fp32_group_kernel<1, 4><<<grid, kGThreads, 0, st>>>(vals, rows, cols, group_index, m, B, n, C);
    count_launches(1);
    return cudaGetLastError();
}

} // namespace gcoo
