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
//
// The same walk serves the BF16 and FP8-B forms on the FMA engine (B already
// converted by spdm_lowp.cu: bf16, or E4M3 with per-column scales applied to
// the finished sums): a B segment is decoded once per column run instead of
// once per row. Per element the entries are the same and in the same order as
// in the row walk of those forms, so the results are identical to it.
#include <cuda_bf16.h>
#include <cuda_fp8.h>

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

enum GForm { kGF32 = 0, kGBF16 = 1, kGFP8 = 3 };

__device__ __forceinline__ float gbf_lo(uint32_t w) { return __uint_as_float(w << 16); }
__device__ __forceinline__ float gbf_hi(uint32_t w) { return __uint_as_float(w & 0xffff0000u); }

// V values of B's row c at columns j.. as floats: FP32 as is, BF16 widened,
// FP8 E4M3 decoded (per-column scales are applied at the end).
template <int F, int V>
__device__ __forceinline__ void ldb(const void *B, int64_t off, float (&o)[V])
{
    if constexpr (F == kGF32) {
        ldv<V>(static_cast<const float *>(B) + off, o);
    } else if constexpr (F == kGBF16) {
        static_assert(V == 8, "BF16 B: 8 columns per lane");
        const uint4 w = __ldg(reinterpret_cast<const uint4 *>(static_cast<const uint16_t *>(B) + off));
        const uint32_t x[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            o[(2 * i) % V] = gbf_lo(x[i]);
            o[(2 * i + 1) % V] = gbf_hi(x[i]);
        }
    } else {
        static_assert(V == 8, "FP8 B: 8 columns per lane");
        const uint2 w = __ldg(reinterpret_cast<const uint2 *>(static_cast<const uint8_t *>(B) + off));
        const uint32_t x[2] = {w.x, w.y};
#pragma unroll
        for (int i = 0; i < 2; ++i) {
            const __half2_raw h01 = __nv_cvt_fp8x2_to_halfraw2(static_cast<__nv_fp8x2_storage_t>(x[i] & 0xffffu), __NV_E4M3);
            const __half2_raw h23 = __nv_cvt_fp8x2_to_halfraw2(static_cast<__nv_fp8x2_storage_t>(x[i] >> 16), __NV_E4M3);
            const float2 f01 = __half22float2(*reinterpret_cast<const __half2 *>(&h01));
            const float2 f23 = __half22float2(*reinterpret_cast<const __half2 *>(&h23));
            o[(4 * i + 0) % V] = f01.x;
            o[(4 * i + 1) % V] = f01.y;
            o[(4 * i + 2) % V] = f23.x;
            o[(4 * i + 3) % V] = f23.y;
        }
    }
}

// The value an entry multiplies with: BF16 rounds A's value like the row walk.
template <int F>
__device__ __forceinline__ float entry_val(int bits)
{
    const float a = __int_as_float(bits);
    if constexpr (F == kGBF16)
        return __bfloat162float(__float2bfloat16_rn(a));
    else
        return a;
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

template <int F, int U, int V>
__device__ __forceinline__ void load_runs(const int (&rs)[U + 1], int wn, int col_of_lane, bool has_col,
                                          const void *B, int64_t j, int64_t n, float (&b)[U][V])
{
#pragma unroll
    for (int u = 0; u < U; ++u) {
        const int c = __shfl_sync(0xffffffffu, col_of_lane, rs[u] < 32 ? rs[u] : 0);
        if (rs[u] < wn && has_col)
            ldb<F, V>(B, static_cast<int64_t>(c) * n + j, b[u]);
    }
}

// Applies each run's entries (at most one per row, rows ascending) in order.
template <int F, int U, int V>
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
                const float a = entry_val<F>(__shfl_sync(0xffffffffu, mine.z, rs[u] + r));
#pragma unroll
                for (int v = 0; v < V; ++v)
                    acc[r][v] = fmaf(a, b[u][v], acc[r][v]);
            }
        } else {
            for (int q = rs[u]; q < rs[u + 1]; ++q)
                fma_row<V>(acc, __shfl_sync(0xffffffffu, mine.y, q), entry_val<F>(__shfl_sync(0xffffffffu, mine.z, q)),
                           b[u]);
        }
        prev = __shfl_sync(0xffffffffu, mine.x, rs[u]);
#pragma unroll
        for (int v = 0; v < V; ++v)
            pb[v] = b[u][v];
    }
}

template <int F, int V, int U>
__global__ void __launch_bounds__(kGThreads)
spdm_group_kernel(const float *__restrict__ vals, const int32_t *__restrict__ rows, const int32_t *__restrict__ cols,
                  const int32_t *__restrict__ group_index, int64_t m, const void *__restrict__ B,
                  const float *__restrict__ col_scale, int64_t n, float *__restrict__ C)
{
    __shared__ int4 s_e[kGChunk]; // {col, row - r0, value bits, 0}
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t g = blockIdx.x;
    const int64_t r0 = g * kGroupRows;
    const int nrows = static_cast<int>(r0 + kGroupRows <= m ? kGroupRows : m - r0);
    const int64_t j = (static_cast<int64_t>(blockIdx.y) * kGWarps + warp) * (32 * V) + static_cast<int64_t>(lane) * V;
    const bool has_col = j < n;
    const int64_t jb = has_col ? j : 0;
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
                fma_row<V>(acc, __shfl_sync(0xffffffffu, mine.y, q), entry_val<F>(__shfl_sync(0xffffffffu, mine.z, q)),
                           pb);
            while (starts) {
                int rs[U + 1];
                float b[U][V];
                take_runs<U>(starts, wn, rs);
                load_runs<F, U, V>(rs, wn, mine.x, has_col, B, jb, n, b);
                apply_runs<F, U, V>(rs, wn, mine, b, acc, prev, pb);
            }
        }
    }
    if (has_col) {
        if constexpr (F == kGFP8) {
            // the per-column scales of the FP8 form, once per finished sum
#pragma unroll
            for (int v = 0; v < V; ++v) {
                const float sc = col_scale[j + v];
#pragma unroll
                for (int r = 0; r < kGroupRows; ++r)
                    acc[r][v] *= sc;
            }
        }
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
#define GCOO_GROUP(V, U)                                                                                       \
    spdm_group_kernel<kGF32, V, U><<<grid, kGThreads, 0, st>>>(vals, rows, cols, group_index, m, B, nullptr, n, C)
    if (vec == 8)
        GCOO_GROUP(8, 2);
    else if (vec == 4)
        GCOO_GROUP(4, 2);
    else if (vec == 2)
        GCOO_GROUP(2, 4);
    else
        GCOO_GROUP(1, 4);
#undef GCOO_GROUP
    count_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_spdm_lowp_group(const float *vals, const int32_t *rows, const int32_t *cols,
                                   const int32_t *group_index, int64_t m, int64_t ng, const void *B,
                                   const float *col_scale, int64_t n, float *C, gcoo_precision prec, cudaStream_t st)
{
    if (ng <= 0 || n <= 0)
        return cudaSuccess;
    if (n % 8 != 0 || (prec != GCOO_PREC_BF16 && prec != GCOO_PREC_FP8_B))
        return cudaErrorInvalidValue;
    const int64_t tile = static_cast<int64_t>(kGWarps) * 32 * 8;
    const int64_t ny = (n + tile - 1) / tile;
    if (ny > 65535 || ng > 0x7fffffffLL)
        return cudaErrorInvalidConfiguration;
    dim3 grid(static_cast<unsigned>(ng), static_cast<unsigned>(ny));
    if (prec == GCOO_PREC_BF16)
        spdm_group_kernel<kGBF16, 8, 2><<<grid, kGThreads, 0, st>>>(vals, rows, cols, group_index, m, B, nullptr, n, C);
    else
        spdm_group_kernel<kGFP8, 8, 2><<<grid, kGThreads, 0, st>>>(vals, rows, cols, group_index, m, B, col_scale, n, C);
    count_launches(1);
    return cudaGetLastError();
}

} // namespace gcoo
