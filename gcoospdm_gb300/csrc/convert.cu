// convert.cu -- dense -> GCOO conversion on sm_103a.
//
// Replaces the reference's three conversion kernels
// (src/gcoo_spdm_kernels.cu:4-90 and :160-168, orchestrated by
// src/ShGCOOSpDM.cu:19-126) with:
//   1. row_count_kernel    one warp per row, 128-bit loads, per-row nonzero
//                          counts (a group count is the sum of its rows);
//   2. scan_*_kernels      a device-wide reduce-then-scan (three small
//                          launches, no single-thread serial scan) giving
//                          row pointers, group_index, nnz_per_group and the
//                          int64 total;
//   3. scatter_kernel      one CTA per group: ballot/popc ranks inside each
//                          warp, a warp-total exchange across the CTA, and
//                          a stable write of every entry twice: in the
//                          reference's GCOO order (column, then row) into
//                          vals/rows/cols, and in row order (row, then
//                          column) into the packed execution layout.
// The zero test is `v != 0.0f` everywhere, as in the reference.
#include "internal.cuh"

namespace gcoo {

namespace {

constexpr int kCountThreads = 256;
constexpr int kScanThreads = 256;
constexpr int kScanItems = 16;
constexpr int kScanTile = kScanThreads * kScanItems;
constexpr int kTopThreads = 1024;
constexpr int kScatterThreads = 256;

__device__ __forceinline__ int nz(float v) { return v != 0.0f ? 1 : 0; }

__global__ void __launch_bounds__(kCountThreads)
row_count_kernel(const float *__restrict__ A, int64_t m, int64_t k, int32_t *__restrict__ row_nnz)
{
    const int lane = threadIdx.x & 31;
    const int64_t warp = (static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = (static_cast<int64_t>(gridDim.x) * blockDim.x) >> 5;
    for (int64_t r = warp; r < m; r += nwarps) {
        const float *row = A + r * k;
        int cnt = 0;
        // scalar head up to the first 16-byte boundary (rows start 4-byte aligned)
        const uintptr_t addr = reinterpret_cast<uintptr_t>(row);
        int64_t head = static_cast<int64_t>(((16u - (addr & 15u)) & 15u) >> 2);
        if (head > k)
            head = k;
        if (lane < head)
            cnt += nz(__ldg(row + lane));
        const float4 *body = reinterpret_cast<const float4 *>(row + head);
        const int64_t nb = (k - head) >> 2;
        int64_t i = lane;
#pragma unroll 1
        for (; i + 96 < nb; i += 128) {
            const float4 v0 = __ldcs(body + i);
            const float4 v1 = __ldcs(body + i + 32);
            const float4 v2 = __ldcs(body + i + 64);
            const float4 v3 = __ldcs(body + i + 96);
            cnt += nz(v0.x) + nz(v0.y) + nz(v0.z) + nz(v0.w);
            cnt += nz(v1.x) + nz(v1.y) + nz(v1.z) + nz(v1.w);
            cnt += nz(v2.x) + nz(v2.y) + nz(v2.z) + nz(v2.w);
            cnt += nz(v3.x) + nz(v3.y) + nz(v3.z) + nz(v3.w);
        }
        for (; i < nb; i += 32) {
            const float4 v = __ldcs(body + i);
            cnt += nz(v.x) + nz(v.y) + nz(v.z) + nz(v.w);
        }
        const int64_t t0 = head + nb * 4;
        if (t0 + lane < k)
            cnt += nz(__ldg(row + t0 + lane));
        cnt = __reduce_add_sync(0xffffffffu, cnt);
        if (lane == 0)
            row_nnz[r] = cnt;
    }
}

// Block-wide exclusive scan of one int64 per thread; returns the exclusive
// prefix and writes the block total to *total (all threads).
template <int THREADS>
__device__ __forceinline__ int64_t block_exclusive_scan(int64_t x, int64_t *s_warp, int64_t *total)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int64_t incl = x;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const int64_t y = __shfl_up_sync(0xffffffffu, incl, d);
        if (lane >= d)
            incl += y;
    }
    if (lane == 31)
        s_warp[warp] = incl;
    __syncthreads();
    constexpr int W = THREADS / 32;
    if (warp == 0) {
        int64_t v = lane < W ? s_warp[lane] : 0;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const int64_t y = __shfl_up_sync(0xffffffffu, v, d);
            if (lane >= d)
                v += y;
        }
        if (lane < W)
            s_warp[lane] = v; // inclusive warp prefix
    }
    __syncthreads();
    const int64_t warp_excl = warp ? s_warp[warp - 1] : 0;
    *total = s_warp[W - 1];
    __syncthreads();
    return warp_excl + incl - x;
}

__global__ void __launch_bounds__(kScanThreads)
scan_reduce_kernel(const int32_t *__restrict__ cnt, int64_t m, int64_t *__restrict__ block_sums)
{
    __shared__ int64_t s_warp[32];
    const int64_t base = static_cast<int64_t>(blockIdx.x) * kScanTile + threadIdx.x * kScanItems;
    int64_t s = 0;
#pragma unroll
    for (int i = 0; i < kScanItems; ++i)
        if (base + i < m)
            s += cnt[base + i];
    int64_t total;
    block_exclusive_scan<kScanThreads>(s, s_warp, &total);
    if (threadIdx.x == 0)
        block_sums[blockIdx.x] = total;
}

// One CTA: exclusive scan of the block sums in place; writes the grand total.
__global__ void __launch_bounds__(kTopThreads)
scan_top_kernel(int64_t *__restrict__ block_sums, int64_t nb, int64_t *__restrict__ d_total,
                int32_t *__restrict__ row_ptr, int64_t m, uint32_t *__restrict__ status)
{
    __shared__ int64_t s_warp[32];
    int64_t carry = 0;
    for (int64_t base = 0; base < nb; base += kTopThreads) {
        const int64_t i = base + threadIdx.x;
        const int64_t x = i < nb ? block_sums[i] : 0;
        int64_t total;
        const int64_t ex = block_exclusive_scan<kTopThreads>(x, s_warp, &total);
        if (i < nb)
            block_sums[i] = carry + ex;
        carry += total;
    }
    if (threadIdx.x == 0) {
        *d_total = carry;
        row_ptr[m] = static_cast<int32_t>(carry);
        if (carry > 0x7fffffffLL && status)
            atomicOr(status, kStatusOverflow);
    }
}

__global__ void __launch_bounds__(kScanThreads)
scan_down_kernel(int32_t *__restrict__ data, int64_t m, const int64_t *__restrict__ block_off)
{
    __shared__ int64_t s_warp[32];
    const int64_t base = static_cast<int64_t>(blockIdx.x) * kScanTile + threadIdx.x * kScanItems;
    int32_t v[kScanItems];
    int64_t s = 0;
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) {
        v[i] = base + i < m ? data[base + i] : 0;
        s += v[i];
    }
    int64_t total;
    int64_t run = block_off[blockIdx.x] + block_exclusive_scan<kScanThreads>(s, s_warp, &total);
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) {
        if (base + i < m)
            data[base + i] = static_cast<int32_t>(run);
        run += v[i];
    }
}

// The whole row scan of a matrix of up to kSmallScanRows rows in one CTA:
// row counts -> row_ptr (in place, row_ptr[m] = total), the total and the
// longest row into d_total[0] / d_total[1], and the group arrays when given.
// Same results as scan_reduce / scan_top / scan_down + group_arrays +
// row_max, in one launch instead of five.
constexpr int kSmallScanItems = 8;
constexpr int64_t kSmallScanRows = 16384; // two chunks; the three-kernel scan is faster beyond

__global__ void __launch_bounds__(kTopThreads)
scan_small_kernel(int32_t *__restrict__ data, int64_t m, int32_t cpg, int32_t *__restrict__ group_index,
                  int32_t *__restrict__ nnz_per_group, int64_t *__restrict__ d_total, uint32_t *__restrict__ status)
{
    __shared__ int64_t s_warp[32];
    __shared__ int s_max[32];
    constexpr int64_t kChunk = static_cast<int64_t>(kTopThreads) * kSmallScanItems;
    int64_t carry = 0;
    int mx = 0;
    for (int64_t c0 = 0; c0 < m; c0 += kChunk) {
        const int64_t base = c0 + static_cast<int64_t>(threadIdx.x) * kSmallScanItems;
        int32_t v[kSmallScanItems];
        int64_t sum = 0;
#pragma unroll
        for (int i = 0; i < kSmallScanItems; ++i) {
            v[i] = base + i < m ? data[base + i] : 0;
            sum += v[i];
            mx = v[i] > mx ? v[i] : mx;
        }
        int64_t total;
        int64_t run = carry + block_exclusive_scan<kTopThreads>(sum, s_warp, &total);
        // whole groups inside the thread's rows (rows_per_group dividing the item count): their
        // arrays straight from the registers
        const bool own_groups = group_index && kSmallScanItems % cpg == 0;
        int32_t gsum = 0;
        int64_t gstart = run;
#pragma unroll
        for (int i = 0; i < kSmallScanItems; ++i) {
            if (base + i < m)
                data[base + i] = static_cast<int32_t>(run);
            run += v[i];
            gsum += v[i];
            if (own_groups && (i + 1) % cpg == 0) {
                const int64_t r0 = base + i + 1 - cpg;
                if (r0 < m) {
                    group_index[r0 / cpg] = static_cast<int32_t>(gstart);
                    nnz_per_group[r0 / cpg] = gsum;
                }
                gsum = 0;
                gstart = run;
            }
        }
        carry += total;
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) {
        const int y = __shfl_xor_sync(0xffffffffu, mx, o);
        mx = y > mx ? y : mx;
    }
    if ((threadIdx.x & 31) == 0)
        s_max[threadIdx.x >> 5] = mx;
    __syncthreads(); // also orders the row_ptr writes above before the group reads below
    if (threadIdx.x == 0) {
        int best = 0;
        for (int w = 0; w < kTopThreads / 32; ++w)
            best = s_max[w] > best ? s_max[w] : best;
        d_total[0] = carry;
        d_total[1] = best;
        data[m] = static_cast<int32_t>(carry);
        if (carry > 0x7fffffffLL && status)
            atomicOr(status, kStatusOverflow);
    }
    if (!group_index)
        return;
    const int64_t ng = (m + cpg - 1) / cpg;
    if (kSmallScanItems % cpg == 0) {
        if (threadIdx.x == 0) {
            group_index[ng] = static_cast<int32_t>(carry);
            nnz_per_group[ng] = 0; // the reference memsets nGroup+1 entries
        }
        return;
    }
    __syncthreads();
    for (int64_t g = threadIdx.x; g <= ng; g += kTopThreads) {
        if (g == ng) {
            group_index[ng] = data[m];
            nnz_per_group[ng] = 0; // the reference memsets nGroup+1 entries
        } else {
            const int64_t r0 = g * cpg;
            const int64_t r1 = r0 + cpg < m ? r0 + cpg : m;
            group_index[g] = data[r0];
            nnz_per_group[g] = data[r1] - data[r0];
        }
    }
}

__global__ void group_arrays_kernel(const int32_t *__restrict__ row_ptr, int64_t m, int32_t cpg,
                                    int64_t ng, int32_t *__restrict__ group_index,
                                    int32_t *__restrict__ nnz_per_group)
{
    for (int64_t g = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; g <= ng;
         g += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        if (g == ng) {
            group_index[ng] = row_ptr[m];
            nnz_per_group[ng] = 0; // the reference memsets nGroup+1 entries
        } else {
            const int64_t r0 = g * cpg;
            const int64_t r1 = r0 + cpg < m ? r0 + cpg : m;
            group_index[g] = row_ptr[r0];
            nnz_per_group[g] = row_ptr[r1] - row_ptr[r0];
        }
    }
}

// One CTA per group of CPG rows; the group is walked in column tiles of
// kScatterThreads columns, one column per thread.
template <int CPG>
__global__ void __launch_bounds__(kScatterThreads)
scatter_kernel(const float *__restrict__ A, int64_t m, int64_t k, const int32_t *__restrict__ group_index,
               const int32_t *__restrict__ row_ptr, float *__restrict__ vals, int32_t *__restrict__ rows,
               int32_t *__restrict__ cols, Entry *__restrict__ packed)
{
    constexpr int W = kScatterThreads / 32;
    __shared__ int s_col[W];
    __shared__ int s_row[W][CPG];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const unsigned lt = (1u << lane) - 1u;
    const int64_t g = blockIdx.x;
    const int64_t r0 = g * CPG;
    const int nrows = static_cast<int>(r0 + CPG <= m ? CPG : m - r0);

    const int64_t gbase = group_index ? group_index[g] : 0;
    int32_t row_base[CPG];
#pragma unroll
    for (int r = 0; r < CPG; ++r)
        row_base[r] = (r < nrows && packed) ? row_ptr[r0 + r] : 0;

    int64_t col_run = 0;
    int row_run[CPG];
#pragma unroll
    for (int r = 0; r < CPG; ++r)
        row_run[r] = 0;

    for (int64_t c0 = 0; c0 < k; c0 += kScatterThreads) {
        const int64_t c = c0 + threadIdx.x;
        float v[CPG];
        unsigned bal[CPG];
        int cc = 0;
#pragma unroll
        for (int r = 0; r < CPG; ++r) {
            v[r] = (r < nrows && c < k) ? __ldcs(A + (r0 + r) * k + c) : 0.0f;
            const int f = nz(v[r]);
            cc += f;
            bal[r] = __ballot_sync(0xffffffffu, f);
        }
        int incl = cc;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, incl, d);
            if (lane >= d)
                incl += y;
        }
        if (lane == 31)
            s_col[warp] = incl;
        if (lane == 0) {
#pragma unroll
            for (int r = 0; r < CPG; ++r)
                s_row[warp][r] = __popc(bal[r]);
        }
        __syncthreads();
        int col_before = 0, col_tile = 0;
#pragma unroll
        for (int w = 0; w < W; ++w) {
            const int x = s_col[w];
            col_before += w < warp ? x : 0;
            col_tile += x;
        }
        // GCOO order: (column, row)
        int64_t pos = gbase + col_run + col_before + (incl - cc);
#pragma unroll
        for (int r = 0; r < CPG; ++r) {
            int before = 0, tile = 0;
#pragma unroll
            for (int w = 0; w < W; ++w) {
                const int x = s_row[w][r];
                before += w < warp ? x : 0;
                tile += x;
            }
            if (v[r] != 0.0f) {
                if (vals) {
                    vals[pos] = v[r];
                    rows[pos] = static_cast<int32_t>(r0 + r);
                    cols[pos] = static_cast<int32_t>(c);
                }
                if (packed) {
                    const int64_t q = static_cast<int64_t>(row_base[r]) + row_run[r] + before + __popc(bal[r] & lt);
                    Entry e;
                    e.col = static_cast<int32_t>(c);
                    e.val = v[r];
                    packed[q] = e;
                }
                ++pos;
            }
            row_run[r] += tile;
        }
        col_run += col_tile;
        __syncthreads();
    }
}

// Vectorised scatter (k % 4 == 0, 16-byte aligned A): each thread owns 4
// consecutive columns of the group's rows (one 128-bit load per row), so a
// CTA covers 1024 columns per step. The per-row counts of a thread (0..4)
// are packed four to a word in 8-bit fields and one warp scan of the packed
// words gives, at once, every row's rank among the lanes (row order) and,
// summed over the rows, the column-major rank (the reference's GCOO order).
template <int CPG>
__global__ void __launch_bounds__(kScatterThreads)
scatter_vec_kernel(const float *__restrict__ A, int64_t m, int64_t k, const int32_t *__restrict__ group_index,
                   const int32_t *__restrict__ row_ptr, float *__restrict__ vals, int32_t *__restrict__ rows,
                   int32_t *__restrict__ cols, Entry *__restrict__ packed)
{
    constexpr int W = kScatterThreads / 32;
    constexpr int NP = (CPG + 3) / 4;
    constexpr int kTileCols = kScatterThreads * 4;
    __shared__ uint32_t s_tot[W][NP];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t g = blockIdx.x;
    const int64_t r0 = g * CPG;
    const int nrows = static_cast<int>(r0 + CPG <= m ? CPG : m - r0);
    const int64_t gbase = group_index ? group_index[g] : 0;
    int32_t row_base[CPG];
    int row_run[CPG];
#pragma unroll
    for (int r = 0; r < CPG; ++r) {
        row_base[r] = (r < nrows && packed) ? row_ptr[r0 + r] : 0;
        row_run[r] = 0;
    }
    int64_t col_run = 0;

    for (int64_t c0 = 0; c0 < k; c0 += kTileCols) {
        const int64_t c = c0 + threadIdx.x * 4;
        float4 v[CPG];
#pragma unroll
        for (int r = 0; r < CPG; ++r)
            v[r] = (r < nrows && c < k) ? __ldcs(reinterpret_cast<const float4 *>(A + (r0 + r) * k + c))
                                        : make_float4(0.f, 0.f, 0.f, 0.f);
        uint32_t bits[CPG];
        uint32_t word[NP];
#pragma unroll
        for (int i = 0; i < NP; ++i)
            word[i] = 0;
#pragma unroll
        for (int r = 0; r < CPG; ++r) {
            bits[r] = nz(v[r].x) | (nz(v[r].y) << 1) | (nz(v[r].z) << 2) | (nz(v[r].w) << 3);
            word[r / 4] |= static_cast<uint32_t>(__popc(bits[r])) << (8 * (r % 4));
        }
        uint32_t incl[NP];
#pragma unroll
        for (int i = 0; i < NP; ++i) {
            incl[i] = word[i];
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const uint32_t y = __shfl_up_sync(0xffffffffu, incl[i], d);
                if (lane >= d)
                    incl[i] += y; // fields never carry: a field's prefix is at most 4 * 32
            }
            if (lane == 31)
                s_tot[warp][i] = incl[i];
        }
        __syncthreads();
        int before[CPG], tile[CPG], lane_ex[CPG];
#pragma unroll
        for (int r = 0; r < CPG; ++r) {
            before[r] = 0;
            tile[r] = 0;
            lane_ex[r] = static_cast<int>(((incl[r / 4] - word[r / 4]) >> (8 * (r % 4))) & 0xffu);
        }
#pragma unroll
        for (int w = 0; w < W; ++w) {
#pragma unroll
            for (int r = 0; r < CPG; ++r) {
                const int x = static_cast<int>((s_tot[w][r / 4] >> (8 * (r % 4))) & 0xffu);
                before[r] += w < warp ? x : 0;
                tile[r] += x;
            }
        }
        int64_t pos = gbase + col_run;
#pragma unroll
        for (int r = 0; r < CPG; ++r)
            pos += before[r] + lane_ex[r];
        // reference GCOO order: column, then row
#pragma unroll
        for (int q = 0; q < 4; ++q) {
#pragma unroll
            for (int r = 0; r < CPG; ++r) {
                if ((bits[r] >> q) & 1u) {
                    if (vals) {
                        const float x = q == 0 ? v[r].x : q == 1 ? v[r].y : q == 2 ? v[r].z : v[r].w;
                        vals[pos] = x;
                        rows[pos] = static_cast<int32_t>(r0 + r);
                        cols[pos] = static_cast<int32_t>(c + q);
                    }
                    ++pos;
                }
            }
        }
        // execution layout: row, then column
        if (packed) {
#pragma unroll
            for (int r = 0; r < CPG; ++r) {
                int64_t q_pos = static_cast<int64_t>(row_base[r]) + row_run[r] + before[r] + lane_ex[r];
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    if ((bits[r] >> q) & 1u) {
                        Entry e;
                        e.col = static_cast<int32_t>(c + q);
                        e.val = q == 0 ? v[r].x : q == 1 ? v[r].y : q == 2 ? v[r].z : v[r].w;
                        packed[q_pos++] = e;
                    }
                }
            }
        }
        int64_t tile_all = 0;
#pragma unroll
        for (int r = 0; r < CPG; ++r) {
            row_run[r] += tile[r];
            tile_all += tile[r];
        }
        col_run += tile_all;
        __syncthreads();
    }
}

int sm_count()
{
    static int sms = 0;
    if (!sms) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (sms <= 0)
            sms = 152;
    }
    return sms;
}

} // namespace

cudaError_t launch_row_count(const float *A, int64_t m, int64_t k, int32_t *row_nnz, cudaStream_t st)
{
    if (m <= 0)
        return cudaSuccess;
    const int64_t warps_needed = m;
    const int64_t per_block = kCountThreads / 32;
    int64_t blocks = (warps_needed + per_block - 1) / per_block;
    const int64_t cap = static_cast<int64_t>(sm_count()) * 16;
    if (blocks > cap)
        blocks = cap;
    row_count_kernel<<<static_cast<unsigned>(blocks), kCountThreads, 0, st>>>(A, m, k, row_nnz);
    count_launches(1);
    return cudaGetLastError();
}

namespace {
__global__ void row_max_kernel(const int32_t *__restrict__ row_ptr, int64_t m, unsigned long long *__restrict__ out)
{
    long long mx = 0;
    for (int64_t r = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; r < m;
         r += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const long long len = row_ptr[r + 1] - row_ptr[r];
        mx = len > mx ? len : mx;
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) {
        const long long y = __shfl_xor_sync(0xffffffffu, mx, o);
        mx = y > mx ? y : mx;
    }
    if ((threadIdx.x & 31) == 0 && mx > 0)
        atomicMax(out, static_cast<unsigned long long>(mx));
}
} // namespace

cudaError_t launch_row_max(const int32_t *row_ptr, int64_t m, int64_t *out, cudaStream_t st)
{
    int64_t blocks = (m + 255) / 256;
    if (blocks > 1024)
        blocks = 1024;
    row_max_kernel<<<static_cast<unsigned>(blocks < 1 ? 1 : blocks), 256, 0, st>>>(
        row_ptr, m, reinterpret_cast<unsigned long long *>(out));
    count_launches(1);
    return cudaGetLastError();
}

size_t scan_scratch_elems(int64_t m)
{
    const int64_t nb = (m + kScanTile - 1) / kScanTile;
    return static_cast<size_t>(nb + 1);
}

cudaError_t launch_row_scan(int32_t *data, int64_t m, int32_t cpg, int32_t *group_index,
                            int32_t *nnz_per_group, int64_t *d_total, int64_t *scratch,
                            uint32_t *status, cudaStream_t st)
{
    const int64_t nb = (m + kScanTile - 1) / kScanTile;
    if (nb > 0) {
        scan_reduce_kernel<<<static_cast<unsigned>(nb), kScanThreads, 0, st>>>(data, m, scratch);
        count_launches(1);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess)
            return e;
    }
    scan_top_kernel<<<1, kTopThreads, 0, st>>>(scratch, nb, d_total, data, m, status);
    count_launches(1);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess)
        return e;
    if (nb > 0) {
        scan_down_kernel<<<static_cast<unsigned>(nb), kScanThreads, 0, st>>>(data, m, scratch);
        count_launches(1);
        e = cudaGetLastError();
        if (e != cudaSuccess)
            return e;
    }
    if (group_index) {
        const int64_t ng = (m + cpg - 1) / cpg;
        int64_t blocks = (ng + 1 + 255) / 256;
        if (blocks > 4096)
            blocks = 4096;
        group_arrays_kernel<<<static_cast<unsigned>(blocks), 256, 0, st>>>(data, m, cpg, ng, group_index,
                                                                           nnz_per_group);
        count_launches(1);
        e = cudaGetLastError();
    }
    return e;
}

cudaError_t launch_row_scan_max(int32_t *data, int64_t m, int32_t cpg, int32_t *group_index,
                                int32_t *nnz_per_group, int64_t *d_total, int64_t *scratch, uint32_t *status,
                                cudaStream_t st)
{
    if (m > 0 && m <= kSmallScanRows) {
        scan_small_kernel<<<1, kTopThreads, 0, st>>>(data, m, cpg, group_index, nnz_per_group, d_total, status);
        count_launches(1);
        return cudaGetLastError();
    }
    cudaError_t e = launch_row_scan(data, m, cpg, group_index, nnz_per_group, d_total, scratch, status, st);
    if (e != cudaSuccess)
        return e;
    return launch_row_max(data, m, d_total + 1, st);
}

cudaError_t launch_scatter(const float *A, int64_t m, int64_t k, int32_t cpg, const int32_t *group_index,
                           const int32_t *row_ptr, float *vals, int32_t *rows, int32_t *cols, Entry *packed,
                           cudaStream_t st)
{
    const int64_t ng = (m + cpg - 1) / cpg;
    if (ng <= 0)
        return cudaSuccess;
    const unsigned grid = static_cast<unsigned>(ng);
    if (k % 4 == 0 && (reinterpret_cast<uintptr_t>(A) & 15) == 0 && cpg <= 8) {
        switch (cpg) {
        case 1: scatter_vec_kernel<1><<<grid, kScatterThreads, 0, st>>>(A, m, k, group_index, row_ptr, vals, rows, cols, packed); break;
        case 2: scatter_vec_kernel<2><<<grid, kScatterThreads, 0, st>>>(A, m, k, group_index, row_ptr, vals, rows, cols, packed); break;
        case 4: scatter_vec_kernel<4><<<grid, kScatterThreads, 0, st>>>(A, m, k, group_index, row_ptr, vals, rows, cols, packed); break;
        case 8: scatter_vec_kernel<8><<<grid, kScatterThreads, 0, st>>>(A, m, k, group_index, row_ptr, vals, rows, cols, packed); break;
        case 16: scatter_vec_kernel<16><<<grid, kScatterThreads, 0, st>>>(A, m, k, group_index, row_ptr, vals, rows, cols, packed); break;
        case 32: scatter_vec_kernel<32><<<grid, kScatterThreads, 0, st>>>(A, m, k, group_index, row_ptr, vals, rows, cols, packed); break;
        default: return cudaErrorInvalidValue;
        }
        count_launches(1);
        return cudaGetLastError();
    }
    switch (cpg) {
    case 1: scatter_kernel<1><<<grid, kScatterThreads, 0, st>>>(A, m, k, group_index, row_ptr, vals, rows, cols, packed); break;
    case 2: scatter_kernel<2><<<grid, kScatterThreads, 0, st>>>(A, m, k, group_index, row_ptr, vals, rows, cols, packed); break;
    case 4: scatter_kernel<4><<<grid, kScatterThreads, 0, st>>>(A, m, k, group_index, row_ptr, vals, rows, cols, packed); break;
    case 8: scatter_kernel<8><<<grid, kScatterThreads, 0, st>>>(A, m, k, group_index, row_ptr, vals, rows, cols, packed); break;
    case 16: scatter_kernel<16><<<grid, kScatterThreads, 0, st>>>(A, m, k, group_index, row_ptr, vals, rows, cols, packed); break;
    case 32: scatter_kernel<32><<<grid, kScatterThreads, 0, st>>>(A, m, k, group_index, row_ptr, vals, rows, cols, packed); break;
    default: return cudaErrorInvalidValue;
    }
    count_launches(1);
    return cudaGetLastError();
}

} // namespace gcoo
