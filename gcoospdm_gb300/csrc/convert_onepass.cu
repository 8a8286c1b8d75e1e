// convert_onepass.cu -- dense -> GCOO conversion reading A once.
//
// Same arrays as convert_tiled.cu (the reference's order and zero test,
// src/gcoo_spdm_kernels.cu:4-90), but the count pass is folded into the
// scatter with a decoupled look-back over the work units:
//   * a unit is (group g of CPG rows, 2 * 1024 columns), units taken
//     in the GCOO order u = g * tiles + t from a ticket counter, so every
//     unit a CTA waits on already belongs to a running CTA;
//   * each CTA counts its tile (warp scans of 8-bit packed per-lane counts),
//     publishes its total, then looks back over its predecessors (32 at a
//     time, one warp) until it finds a published inclusive prefix: that is
//     where its entries start in GCOO order, which it publishes in turn;
//   * it writes its entries (vals, rows, cols), the per-(row, segment)
//     counts (for the row pointers), group_index[g] for the group's first
//     tile, and the grand total for the last unit.
// Every wait is bounded (%globaltimer, kWaitNs); a CTA that gives up sets the
// status word, writes nothing and still publishes, so no CTA waits forever.
// The row-ordered execution layout is then derived from the GCOO arrays by
// pack_kernel (one warp per group, 20 bytes per entry of traffic) instead of a
// second pass over A.
#include "internal.cuh"

namespace gcoo {

namespace {

constexpr int kThreads = 256; // 8 warps: 8 consecutive 128-column segments of one group
constexpr int kSegCols = 128;
constexpr int kSegsPerCta = kThreads / 32;
constexpr int kTileCols = kSegsPerCta * kSegCols;
constexpr int kTPU = 2;                          // 1024-column tiles per unit
constexpr int kUnitCols = kTPU * kTileCols;
constexpr int kSegsPerUnit = kTPU * kSegsPerCta;
static_assert(kSegsPerUnit <= 32, "one warp sums the unit's segment totals");

// unit state word: value << 2 | flag (1: the unit's own total, 2: inclusive prefix)
constexpr unsigned long long kFlagAggregate = 1, kFlagInclusive = 2;

__device__ __forceinline__ uint32_t nzb(float v) { return v != 0.0f ? 1u : 0u; }

__device__ __forceinline__ uint32_t nz_bits(const float4 &v)
{
    return nzb(v.x) | (nzb(v.y) << 1) | (nzb(v.z) << 2) | (nzb(v.w) << 3);
}

__device__ __forceinline__ unsigned long long load_state(const unsigned long long *p)
{
    return *reinterpret_cast<const volatile unsigned long long *>(p);
}

template <int CPG>
__global__ void __launch_bounds__(kThreads)
onepass_kernel(const float *__restrict__ A, int64_t m, int64_t k, int64_t tiles, int64_t S, int64_t units,
               int32_t *__restrict__ cnt, unsigned long long *__restrict__ distinct,
               unsigned long long *__restrict__ state, unsigned int *__restrict__ ticket, float *__restrict__ vals,
               int32_t *__restrict__ rows, int32_t *__restrict__ cols, int64_t cap, int32_t *__restrict__ group_index,
               int64_t ng, int64_t *__restrict__ d_total, uint32_t *__restrict__ status)
{
    constexpr int NP = (CPG + 3) / 4;
    __shared__ long long s_u, s_prefix;
    __shared__ int s_wtot[kSegsPerUnit], s_dist[kSegsPerCta];
    if (threadIdx.x == 0)
        s_u = static_cast<long long>(atomicAdd(ticket, 1u));
    __syncthreads();
    const int64_t u = s_u;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t g = u / tiles, t = u - g * tiles;
    const int64_t r0 = g * CPG;
    const int nrows = static_cast<int>(r0 + CPG <= m ? CPG : m - r0);

    // the unit's kTPU tiles: warp w holds segment w of each
    int64_t seg[kTPU], c[kTPU];
    bool live[kTPU];
    float4 v[kTPU][CPG];
#pragma unroll
    for (int i = 0; i < kTPU; ++i) {
        seg[i] = (t * kTPU + i) * kSegsPerCta + warp;
        c[i] = seg[i] * kSegCols + static_cast<int64_t>(lane) * 4;
        live[i] = seg[i] * kSegCols < k;
#pragma unroll
        for (int r = 0; r < CPG; ++r)
            v[i][r] = (live[i] && r < nrows && c[i] < k)
                          ? __ldcs(reinterpret_cast<const float4 *>(A + (r0 + r) * k + c[i]))
                          : make_float4(0.f, 0.f, 0.f, 0.f);
    }
    uint32_t bits[kTPU][CPG], excl[kTPU][NP];
    uint32_t any = 0;
#pragma unroll
    for (int i = 0; i < kTPU; ++i) {
        uint32_t word[NP];
#pragma unroll
        for (int q = 0; q < NP; ++q)
            word[q] = 0;
#pragma unroll
        for (int r = 0; r < CPG; ++r) {
            bits[i][r] = nz_bits(v[i][r]);
            any |= bits[i][r];
            word[r / 4] |= static_cast<uint32_t>(__popc(bits[i][r])) << (8 * (r % 4));
        }
        int wsum = 0;
#pragma unroll
        for (int q = 0; q < NP; ++q) {
            uint32_t incl = word[q];
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const uint32_t y = __shfl_up_sync(0xffffffffu, incl, d);
                if (lane >= d)
                    incl += y; // a field's prefix is at most 4 * 32: no carry between fields
            }
            excl[i][q] = incl - word[q];
            const uint32_t tot = __shfl_sync(0xffffffffu, incl, 31);
#pragma unroll
            for (int f = 0; f < 4; ++f) {
                const int r = 4 * q + f;
                if (r < CPG) {
                    const int x = static_cast<int>((tot >> (8 * f)) & 0xffu);
                    wsum += x;
                    if (live[i] && lane == r && r < nrows)
                        cnt[(r0 + r) * S + seg[i]] = x;
                }
            }
        }
        if (lane == 0)
            s_wtot[i * kSegsPerCta + warp] = wsum;
    }
    if (lane == 0)
        s_dist[warp] = 0;
    if (distinct) {
        const int d = __reduce_add_sync(0xffffffffu, __popc(any));
        if (lane == 0)
            s_dist[warp] = d;
    }
    __syncthreads();

    if (warp == 0) {
        const long long agg = __reduce_add_sync(0xffffffffu, lane < kSegsPerUnit ? s_wtot[lane] : 0);
        if (lane == 0)
            atomicExch(state + u, (static_cast<unsigned long long>(agg) << 2) |
                                      (u == 0 ? kFlagInclusive : kFlagAggregate));
        long long prefix = 0;
        if (u > 0) {
            int64_t idx = u - 1; // the predecessor lane 0 examines
            uint64_t t0 = 0;
            bool started = false;
            for (;;) {
                const int64_t my = idx - lane;
                // before unit 0 counts as an inclusive prefix of 0
                const unsigned long long w = my >= 0 ? load_state(state + my) : kFlagInclusive;
                const unsigned flag = static_cast<unsigned>(w & 3ull);
                const unsigned inc = __ballot_sync(0xffffffffu, flag == kFlagInclusive);
                const unsigned notready = __ballot_sync(0xffffffffu, flag == 0);
                const int p = inc ? __ffs(inc) - 1 : 32; // nearest published inclusive prefix
                const unsigned need = p < 31 ? ((2u << p) - 1u) : 0xffffffffu;
                if (notready & need) {
                    const uint64_t now = global_ns();
                    if (!started) {
                        t0 = now;
                        started = true;
                    } else if (now - t0 > kWaitNs) {
                        prefix = -1; // gave up: flagged below, nothing written
                        break;
                    }
                    continue;
                }
                long long x = lane <= p ? static_cast<long long>(w >> 2) : 0ll;
#pragma unroll
                for (int o = 16; o; o >>= 1)
                    x += __shfl_xor_sync(0xffffffffu, x, o);
                prefix += x;
                if (p < 32)
                    break;
                idx -= 32;
            }
        }
        if (lane == 0) {
            // publish where the next units start (also after giving up, so no successor waits on this unit)
            const long long incl = (prefix < 0 ? 0 : prefix) + agg;
            atomicExch(state + u, (static_cast<unsigned long long>(incl) << 2) | kFlagInclusive);
            s_prefix = prefix;
            if (prefix < 0)
                atomicOr(status, kStatusWaitTimeout);
            if (t == 0 && prefix >= 0)
                group_index[g] = static_cast<int32_t>(prefix);
            if (u == units - 1 && prefix >= 0) {
                d_total[0] = incl;
                group_index[ng] = static_cast<int32_t>(incl);
                if (incl > 0x7fffffffLL)
                    atomicOr(status, kStatusOverflow);
            }
            if (distinct) {
                int dsum = 0;
#pragma unroll
                for (int w2 = 0; w2 < kSegsPerCta; ++w2)
                    dsum += s_dist[w2];
                if (dsum)
                    atomicAdd(distinct, static_cast<unsigned long long>(dsum));
            }
        }
    }
    __syncthreads();
    const long long prefix = s_prefix;
    if (prefix < 0 || !any)
        return;
    // GCOO order inside the unit: column, then row; segment i * 8 + warp holds this warp's columns of tile i
#pragma unroll
    for (int i = 0; i < kTPU; ++i) {
        long long pos = prefix;
        for (int w2 = 0; w2 < i * kSegsPerCta + warp; ++w2)
            pos += s_wtot[w2];
#pragma unroll
        for (int r = 0; r < CPG; ++r)
            pos += static_cast<int>((excl[i][r / 4] >> (8 * (r % 4))) & 0xffu);
#pragma unroll
        for (int q = 0; q < 4; ++q) {
#pragma unroll
            for (int r = 0; r < CPG; ++r) {
                if ((bits[i][r] >> q) & 1u) {
                    if (pos < cap) {
                        vals[pos] = q == 0 ? v[i][r].x : q == 1 ? v[i][r].y : q == 2 ? v[i][r].z : v[i][r].w;
                        rows[pos] = static_cast<int32_t>(r0 + r);
                        cols[pos] = static_cast<int32_t>(c[i] + q);
                    } else {
                        atomicOr(status, kStatusOverflow);
                    }
                    ++pos;
                }
            }
        }
    }
}

// Row-ordered execution layout from the GCOO arrays: one warp per group walks
// the group's entries (column order) in 32-entry windows; an entry's place is
// row_ptr[its row] + the entries of its row seen before it (ballot ranks).
template <int CPG>
__global__ void pack_kernel(const float *__restrict__ vals, const int32_t *__restrict__ rows,
                            const int32_t *__restrict__ cols, const int32_t *__restrict__ group_index,
                            const int32_t *__restrict__ row_ptr, int64_t m, int64_t ng, Entry *__restrict__ packed)
{
    const int lane = threadIdx.x & 31;
    const int64_t w0 = (static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = (static_cast<int64_t>(gridDim.x) * blockDim.x) >> 5;
    const unsigned lt = (1u << lane) - 1u;
    for (int64_t g = w0; g < ng; g += nw) {
        const int64_t r0 = g * CPG;
        const int64_t e0 = group_index[g], e1 = group_index[g + 1];
        const int32_t my_rp = (lane < CPG && r0 + lane < m) ? row_ptr[r0 + lane] : 0;
        int64_t run[CPG];
#pragma unroll
        for (int r = 0; r < CPG; ++r)
            run[r] = __shfl_sync(0xffffffffu, my_rp, r);
        // four windows' loads in flight, then their ranks in order
        for (int64_t b = e0; b < e1; b += 128) {
            int lr[4], col[4];
            float val[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int64_t e = b + q * 32 + lane;
                lr[q] = -1;
                col[q] = 0;
                val[q] = 0.0f;
                if (e < e1) {
                    lr[q] = rows[e] - static_cast<int32_t>(r0);
                    col[q] = cols[e];
                    val[q] = vals[e];
                }
            }
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                int64_t dst = -1;
#pragma unroll
                for (int r = 0; r < CPG; ++r) {
                    const unsigned mask = __ballot_sync(0xffffffffu, lr[q] == r);
                    if (lr[q] == r)
                        dst = run[r] + __popc(mask & lt);
                    run[r] += __popc(mask);
                }
                if (dst >= 0) {
                    Entry en;
                    en.col = col[q];
                    en.val = val[q];
                    packed[dst] = en;
                }
            }
        }
    }
}

// nnz_per_group[g] = group_index[g + 1] - group_index[g]; the last entry 0.
__global__ void group_counts_kernel(const int32_t *__restrict__ group_index, int64_t ng,
                                    int32_t *__restrict__ nnz_per_group)
{
    for (int64_t g = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; g <= ng;
         g += static_cast<int64_t>(gridDim.x) * blockDim.x)
        nnz_per_group[g] = g < ng ? group_index[g + 1] - group_index[g] : 0;
}

} // namespace

bool onepass_convert_ok(const float *A, int64_t m, int64_t k, int32_t cpg)
{
    const int64_t units = ((m + cpg - 1) / cpg) * ((k + kUnitCols - 1) / kUnitCols);
    return k % 4 == 0 && (reinterpret_cast<uintptr_t>(A) & 15) == 0 && (cpg == 1 || cpg == 2 || cpg == 4 || cpg == 8) &&
           units > 0 && units < 0x7fffffffLL;
}

int64_t onepass_units(int64_t m, int64_t k, int32_t cpg)
{
    return ((m + cpg - 1) / cpg) * ((k + kUnitCols - 1) / kUnitCols);
}

cudaError_t launch_onepass(const float *A, int64_t m, int64_t k, int32_t cpg, int32_t *cnt,
                           unsigned long long *distinct, unsigned long long *state, unsigned int *ticket, float *vals,
                           int32_t *rows, int32_t *cols, int64_t cap, int32_t *group_index, int64_t *d_total,
                           uint32_t *status, cudaStream_t st)
{
    const int64_t tiles = (k + kUnitCols - 1) / kUnitCols, S = (k + kSegCols - 1) / kSegCols;
    const int64_t ng = (m + cpg - 1) / cpg;
    const int64_t units = ng * tiles;
    if (units <= 0)
        return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(state, 0, static_cast<size_t>(units) * sizeof(unsigned long long), st);
    if (e == cudaSuccess)
        e = cudaMemsetAsync(ticket, 0, sizeof(unsigned int), st);
    if (e != cudaSuccess)
        return e;
    const unsigned grid = static_cast<unsigned>(units);
#define GCOO_ONEPASS(C)                                                                                           \
    onepass_kernel<C><<<grid, kThreads, 0, st>>>(A, m, k, tiles, S, units, cnt, distinct, state, ticket, vals, rows, \
                                                 cols, cap, group_index, ng, d_total, status)
    switch (cpg) {
    case 1: GCOO_ONEPASS(1); break;
    case 2: GCOO_ONEPASS(2); break;
    case 4: GCOO_ONEPASS(4); break;
    case 8: GCOO_ONEPASS(8); break;
    default: return cudaErrorInvalidValue;
    }
#undef GCOO_ONEPASS
    count_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_pack(const float *vals, const int32_t *rows, const int32_t *cols, int32_t *group_index,
                        int32_t *nnz_per_group, const int32_t *row_ptr, int64_t m, int32_t cpg, Entry *packed,
                        cudaStream_t st)
{
    const int64_t ng = (m + cpg - 1) / cpg;
    if (ng <= 0)
        return cudaSuccess;
    int64_t blocks = (ng + 7) / 8; // 8 warps per CTA, one group each
    if (blocks > 65535)
        blocks = 65535;
    switch (cpg) {
    case 1: pack_kernel<1><<<static_cast<unsigned>(blocks), 256, 0, st>>>(vals, rows, cols, group_index, row_ptr, m, ng, packed); break;
    case 2: pack_kernel<2><<<static_cast<unsigned>(blocks), 256, 0, st>>>(vals, rows, cols, group_index, row_ptr, m, ng, packed); break;
    case 4: pack_kernel<4><<<static_cast<unsigned>(blocks), 256, 0, st>>>(vals, rows, cols, group_index, row_ptr, m, ng, packed); break;
    case 8: pack_kernel<8><<<static_cast<unsigned>(blocks), 256, 0, st>>>(vals, rows, cols, group_index, row_ptr, m, ng, packed); break;
    default: return cudaErrorInvalidValue;
    }
    count_launches(1);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess || !nnz_per_group)
        return e;
    int64_t gb = (ng + 1 + 255) / 256;
    if (gb > 4096)
        gb = 4096;
    group_counts_kernel<<<static_cast<unsigned>(gb), 256, 0, st>>>(group_index, ng, nnz_per_group);
    count_launches(1);
    return cudaGetLastError();
}

} // namespace gcoo
