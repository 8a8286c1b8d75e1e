// convert_tiled.cu -- dense -> GCOO conversion split into column segments.
//
// Same results as the per-group conversion in convert.cu (the reference's
// order and zero test, src/gcoo_spdm_kernels.cu:4-90), organised so that no
// thread block walks a whole row and no warp waits on another: the unit of
// work is one warp on (group of CPG rows, segment of 128 columns), one
// 128-bit load per lane per row; a CTA holds the 8 warps of 8 consecutive
// segments of one group.
//   1. seg_count_kernel   per-(row, segment) nonzero counts into cnt[r][s];
//   2. seg_prefix_kernel  one warp per row: exclusive prefix of the row's
//                         segment counts (in place) and the row total (the
//                         input of the row scan in convert.cu);
//   3. seg_scatter_kernel each warp writes its entries at
//                           GCOO:   group_index[g] + sum_r prefix[r][s]
//                                   + rank in the segment (column, then row)
//                           packed: row_ptr[r] + prefix[r][s]
//                                   + rank of the entry in row r's segment part.
// Once the counts are scanned every warp is independent: a conversion of a
// few hundred rows takes about one memory round trip, a large one streams A.
#include "internal.cuh"

namespace gcoo {

namespace {

constexpr int kTileThreads = 256;              // 8 warps: 8 consecutive segments of one group
constexpr int kSegCols = 128;                   // one warp, one float4 per lane
constexpr int kSegsPerCta = kTileThreads / 32;
constexpr int kTileCols = kSegsPerCta * kSegCols;

__device__ __forceinline__ uint32_t nzb(float v) { return v != 0.0f ? 1u : 0u; }

__device__ __forceinline__ uint32_t nz_bits(const float4 &v)
{
    return nzb(v.x) | (nzb(v.y) << 1) | (nzb(v.z) << 2) | (nzb(v.w) << 3);
}

// Unit of a warp: group g, segment s (CTA = 8 segments of a group).
struct SegUnit {
    int64_t g, s, r0, c;
    int nrows;
    bool live; // segment starts inside the row
};

template <int CPG>
__device__ __forceinline__ SegUnit seg_unit(int64_t m, int64_t k, int64_t tiles)
{
    SegUnit u;
    const int64_t b = blockIdx.x;
    u.g = b / tiles;
    const int64_t t = b - u.g * tiles;
    u.s = t * kSegsPerCta + (threadIdx.x >> 5);
    u.r0 = u.g * CPG;
    u.nrows = static_cast<int>(u.r0 + CPG <= m ? CPG : m - u.r0);
    u.c = u.s * kSegCols + static_cast<int64_t>(threadIdx.x & 31) * 4;
    u.live = u.s * kSegCols < k;
    return u;
}

// distinct (when not null) accumulates the number of distinct (group,
// column) pairs, i.e. columns with a nonzero in at least one row of the
// group; nnz / distinct tells how many rows of a group share a B row.
template <int CPG>
__global__ void __launch_bounds__(kTileThreads)
seg_count_kernel(const float *__restrict__ A, int64_t m, int64_t k, int64_t tiles, int64_t S,
                 int32_t *__restrict__ cnt, unsigned long long *__restrict__ distinct)
{
    __shared__ int s_dist[kSegsPerCta];
    const SegUnit u = seg_unit<CPG>(m, k, tiles);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    float4 v[CPG];
#pragma unroll
    for (int r = 0; r < CPG; ++r)
        v[r] = (u.live && r < u.nrows && u.c < k)
                   ? __ldg(reinterpret_cast<const float4 *>(A + (u.r0 + r) * k + u.c))
                   : make_float4(0.f, 0.f, 0.f, 0.f);
    uint32_t any = 0;
#pragma unroll
    for (int r = 0; r < CPG; ++r) {
        const uint32_t b = nz_bits(v[r]);
        any |= b;
        const int x = __reduce_add_sync(0xffffffffu, __popc(b));
        if (u.live && lane == r && r < u.nrows)
            cnt[(u.r0 + r) * S + u.s] = x;
    }
    if (distinct) {
        const int d = __reduce_add_sync(0xffffffffu, __popc(any));
        if (lane == 0)
            s_dist[warp] = d;
        __syncthreads(); // every warp of the CTA reaches this (no early exit above)
        if (threadIdx.x == 0) {
            int t = 0;
#pragma unroll
            for (int w = 0; w < kSegsPerCta; ++w)
                t += s_dist[w];
            if (t)
                atomicAdd(distinct, static_cast<unsigned long long>(t));
        }
    }
}

// One warp per row: exclusive prefix of the row's segment counts, in place,
// and the row total into row_cnt[r].
__global__ void seg_prefix_kernel(int32_t *__restrict__ cnt, int64_t m, int64_t S, int32_t *__restrict__ row_cnt)
{
    const int lane = threadIdx.x & 31;
    const int64_t w0 = (static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = (static_cast<int64_t>(gridDim.x) * blockDim.x) >> 5;
    for (int64_t r = w0; r < m; r += nw) {
        int32_t *row = cnt + r * S;
        int32_t carry = 0;
        for (int64_t b = 0; b < S; b += 32) {
            const int32_t x = b + lane < S ? row[b + lane] : 0;
            int32_t incl = x;
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const int32_t y = __shfl_up_sync(0xffffffffu, incl, d);
                if (lane >= d)
                    incl += y;
            }
            if (b + lane < S)
                row[b + lane] = carry + incl - x;
            carry += __shfl_sync(0xffffffffu, incl, 31);
        }
        if (lane == 0)
            row_cnt[r] = carry;
    }
}

// Ranks inside one warp's segment: per row, the nonzeros of the lanes before
// this one. Per-lane counts (0..4) are packed four rows to a word in 8-bit
// fields so one warp scan per word serves four rows at once.
template <int CPG>
// 6 CTAs per SM for up to 4 rows per group: more loads of A in flight
__global__ void __launch_bounds__(kTileThreads, CPG <= 4 ? 6 : 4)
seg_scatter_kernel(const float *__restrict__ A, int64_t m, int64_t k, int64_t tiles, int64_t S,
                   const int32_t *__restrict__ pref, const int32_t *__restrict__ group_index,
                   const int32_t *__restrict__ row_ptr, float *__restrict__ vals, int32_t *__restrict__ rows,
                   int32_t *__restrict__ cols, Entry *__restrict__ packed)
{
    constexpr int NP = (CPG + 3) / 4;
    const SegUnit u = seg_unit<CPG>(m, k, tiles);
    if (!u.live)
        return;
    const int lane = threadIdx.x & 31;
    // the offsets do not depend on A: issue their loads with A's, lane l for row r0 + l
    const int32_t my_pre = lane < u.nrows ? pref[(u.r0 + lane) * S + u.s] : 0;
    const int32_t my_rp = (packed && lane < u.nrows) ? row_ptr[u.r0 + lane] : 0;
    const int64_t g_base = (vals && group_index) ? group_index[u.g] : 0;
    float4 v[CPG];
#pragma unroll
    for (int r = 0; r < CPG; ++r)
        v[r] = (r < u.nrows && u.c < k) ? __ldcs(reinterpret_cast<const float4 *>(A + (u.r0 + r) * k + u.c))
                                        : make_float4(0.f, 0.f, 0.f, 0.f);
    uint32_t bits[CPG];
    uint32_t word[NP];
    uint32_t any = 0;
#pragma unroll
    for (int i = 0; i < NP; ++i)
        word[i] = 0;
#pragma unroll
    for (int r = 0; r < CPG; ++r) {
        bits[r] = nz_bits(v[r]);
        any |= bits[r];
        word[r / 4] |= static_cast<uint32_t>(__popc(bits[r])) << (8 * (r % 4));
    }
    if (!__any_sync(0xffffffffu, any != 0))
        return; // nothing to write in this segment
    uint32_t excl[NP];
#pragma unroll
    for (int i = 0; i < NP; ++i) {
        uint32_t incl = word[i];
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, incl, d);
            if (lane >= d)
                incl += y; // a field's prefix is at most 4 * 32: no carry between fields
        }
        excl[i] = incl - word[i];
    }
    // broadcast the row offsets while the whole warp is here
    int32_t pre[CPG], rp[CPG];
#pragma unroll
    for (int r = 0; r < CPG; ++r) {
        pre[r] = __shfl_sync(0xffffffffu, my_pre, r);
        rp[r] = __shfl_sync(0xffffffffu, my_rp, r);
    }
    if (!any)
        return;
    if (vals) {
        // reference GCOO order: column, then row; the warp's entries start after
        // the group's entries of earlier segments
        int64_t pos = g_base;
#pragma unroll
        for (int r = 0; r < CPG; ++r)
            pos += pre[r] + static_cast<int>((excl[r / 4] >> (8 * (r % 4))) & 0xffu);
#pragma unroll
        for (int q = 0; q < 4; ++q) {
#pragma unroll
            for (int r = 0; r < CPG; ++r) {
                if ((bits[r] >> q) & 1u) {
                    vals[pos] = q == 0 ? v[r].x : q == 1 ? v[r].y : q == 2 ? v[r].z : v[r].w;
                    rows[pos] = static_cast<int32_t>(u.r0 + r);
                    cols[pos] = static_cast<int32_t>(u.c + q);
                    ++pos;
                }
            }
        }
    }
    if (packed) {
        // execution layout: row, then column
#pragma unroll
        for (int r = 0; r < CPG; ++r) {
            if (!bits[r])
                continue;
            int64_t q_pos = static_cast<int64_t>(rp[r]) + pre[r] +
                            static_cast<int>((excl[r / 4] >> (8 * (r % 4))) & 0xffu);
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                if ((bits[r] >> q) & 1u) {
                    Entry e;
                    e.col = static_cast<int32_t>(u.c + q);
                    e.val = q == 0 ? v[r].x : q == 1 ? v[r].y : q == 2 ? v[r].z : v[r].w;
                    packed[q_pos++] = e;
                }
            }
        }
    }
}

} // namespace

int64_t conv_segments(int64_t k) { return (k + kSegCols - 1) / kSegCols; }

static int64_t conv_tiles(int64_t k) { return (k + kTileCols - 1) / kTileCols; }

bool tiled_convert_ok(const float *A, int64_t m, int64_t k, int32_t cpg)
{
    const int64_t units = ((m + cpg - 1) / cpg) * conv_tiles(k);
    return k % 4 == 0 && (reinterpret_cast<uintptr_t>(A) & 15) == 0 && cpg <= 8 && units > 0 &&
           units < 0x7fffffffLL;
}

cudaError_t launch_tile_count(const float *A, int64_t m, int64_t k, int32_t cpg, int32_t *cnt,
                              unsigned long long *distinct, cudaStream_t st)
{
    const int64_t tiles = conv_tiles(k), S = conv_segments(k);
    const int64_t units = ((m + cpg - 1) / cpg) * tiles;
    if (units <= 0)
        return cudaSuccess;
    const unsigned grid = static_cast<unsigned>(units);
    switch (cpg) {
    case 1: seg_count_kernel<1><<<grid, kTileThreads, 0, st>>>(A, m, k, tiles, S, cnt, distinct); break;
    case 2: seg_count_kernel<2><<<grid, kTileThreads, 0, st>>>(A, m, k, tiles, S, cnt, distinct); break;
    case 4: seg_count_kernel<4><<<grid, kTileThreads, 0, st>>>(A, m, k, tiles, S, cnt, distinct); break;
    case 8: seg_count_kernel<8><<<grid, kTileThreads, 0, st>>>(A, m, k, tiles, S, cnt, distinct); break;
    default: return cudaErrorInvalidValue;
    }
    count_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_tile_prefix(int32_t *cnt, int64_t m, int64_t k, int32_t *row_cnt, cudaStream_t st)
{
    if (m <= 0)
        return cudaSuccess;
    int64_t blocks = (m + 7) / 8; // 8 warps per CTA, one row each
    if (blocks > 16384)
        blocks = 16384;
    seg_prefix_kernel<<<static_cast<unsigned>(blocks), 256, 0, st>>>(cnt, m, conv_segments(k), row_cnt);
    count_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_tile_scatter(const float *A, int64_t m, int64_t k, int32_t cpg, const int32_t *pref,
                                const int32_t *group_index, const int32_t *row_ptr, float *vals, int32_t *rows,
                                int32_t *cols, Entry *packed, cudaStream_t st)
{
    const int64_t tiles = conv_tiles(k), S = conv_segments(k);
    const int64_t units = ((m + cpg - 1) / cpg) * tiles;
    if (units <= 0)
        return cudaSuccess;
    const unsigned grid = static_cast<unsigned>(units);
#define GCOO_SEG_SCATTER(C)                                                                                    \
    seg_scatter_kernel<C><<<grid, kTileThreads, 0, st>>>(A, m, k, tiles, S, pref, group_index, row_ptr, vals, \
                                                         rows, cols, packed)
    switch (cpg) {
    case 1: GCOO_SEG_SCATTER(1); break;
    case 2: GCOO_SEG_SCATTER(2); break;
    case 4: GCOO_SEG_SCATTER(4); break;
    case 8: GCOO_SEG_SCATTER(8); break;
    default: return cudaErrorInvalidValue;
    }
#undef GCOO_SEG_SCATTER
    count_launches(1);
    return cudaGetLastError();
}

} // namespace gcoo
