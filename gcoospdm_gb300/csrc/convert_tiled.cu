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

// b: the CTA's tile (group-major: b = g * tiles + t)
template <int CPG>
__device__ __forceinline__ SegUnit seg_unit(int64_t m, int64_t k, int64_t tiles, int64_t b)
{
    SegUnit u;
    // tiles and b < 2^31 (tiled_convert_ok): 32-bit division
    u.g = static_cast<int64_t>(static_cast<uint32_t>(b) / static_cast<uint32_t>(tiles));
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
    const SegUnit u = seg_unit<CPG>(m, k, tiles, blockIdx.x);
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
__device__ __forceinline__ void scatter_segment(const float *__restrict__ A, int64_t k, int64_t S, const SegUnit &u,
                                                const int32_t *__restrict__ pref,
                                                const int32_t *__restrict__ group_index,
                                                const int32_t *__restrict__ row_ptr, float *__restrict__ vals,
                                                int32_t *__restrict__ rows, int32_t *__restrict__ cols,
                                                Entry *__restrict__ packed)
{
    constexpr int NP = (CPG + 3) / 4;
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

template <int CPG>
// 6 CTAs per SM for up to 4 rows per group: more loads of A in flight
__global__ void __launch_bounds__(kTileThreads, CPG <= 4 ? 6 : 4)
seg_scatter_kernel(const float *__restrict__ A, int64_t m, int64_t k, int64_t tiles, int64_t S,
                   const int32_t *__restrict__ pref, const int32_t *__restrict__ group_index,
                   const int32_t *__restrict__ row_ptr, float *__restrict__ vals, int32_t *__restrict__ rows,
                   int32_t *__restrict__ cols, Entry *__restrict__ packed)
{
    scatter_segment<CPG>(A, k, S, seg_unit<CPG>(m, k, tiles, blockIdx.x), pref, group_index, row_ptr, vals, rows,
                         cols, packed);
}

// ---- staged rebuild: A read once --------------------------------------------------
// stage_kernel is seg_count_kernel that also keeps each tile's entries (a
// tile: CPG rows x 1024 columns, one CTA, brought into shared memory by bulk
// copies) in a fixed slot of `slot` entries, in the tile's GCOO order
// (column, then row), each as (col << 3 | row in group, value bits).
// tile_tot[b] = the tile's entry count, or -1 when it overflowed its slot;
// an overflowed tile is appended to over_list instead.
// No CTA waits on another. place_kernel then runs after the segment prefix and
// the row scan: one warp per staged tile copies its entries to
//   GCOO:   group_index[g] + sum_r prefix[r][first segment of the tile] + i
//   packed: row_ptr[r] + prefix[r][first segment] + rank of the entry in row r
// and blocks past the staged ones rescan A for the overflowed tiles with the
// two-pass scatter. Same arrays as the two-pass conversion, bit for bit.
// L columns per lane: 8 where the lane's CPG x 8 nonzero bits fit one word
// (CPG <= 4), else 4. A warp then covers L / 4 segments and a tile's CTA has
// 1024 / (32 L) warps: with L = 8 each warp's fixed costs (barriers, ranks,
// the tile's bookkeeping) serve twice the columns and 4-warp CTAs fit 12 per
// SM (192 KB of A in flight per SM against 128 KB with 8-warp CTAs).
template <int CPG, int L>
__global__ void __launch_bounds__(1024 / L, L == 8 ? 12 : (CPG <= 4 ? 8 : 6))
stage_kernel(const float *__restrict__ A, int64_t m, int64_t k, int64_t tiles, int64_t S, int32_t *__restrict__ cnt,
             unsigned long long *__restrict__ distinct, int32_t slot, uint2 *__restrict__ stage,
             int32_t *__restrict__ tile_tot, int32_t *__restrict__ over_list,
             unsigned long long *__restrict__ over_count, uint32_t *__restrict__ status)
{
    constexpr int kWarps = 1024 / L / 32;
    constexpr int kSegPerWarp = L / 4;
    static_assert(CPG * L <= 32, "a lane's nonzeros are one 32-bit mask");
    static_assert(kWarps == 4 || kWarps == 8, "two int4 loads at most read the warp totals");
    // the tile's rows arrive by bulk copies: no registers held while they are in
    // flight, so a full complement of CTAs per SM keeps A streaming
    __shared__ __align__(128) float s_a[CPG][kTileCols];
    __shared__ __align__(8) uint64_t s_bar;
    __shared__ __align__(16) int s_wtot[8];
    __shared__ int s_dist[8];
    __shared__ long long s_g; // the tile's group, computed once
    const int64_t b = blockIdx.x;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) {
        mbar_init(&s_bar, 1);
        fence_mbar_init();
        const SegUnit u0 = seg_unit<CPG>(m, k, tiles, b);
        s_g = u0.g;
        // k % 4 == 0 and a 16-byte aligned A: every row piece starts on 16 bytes and is a multiple of 16 long
        const int64_t c0 = (b - u0.g * tiles) * kTileCols;
        const int64_t w = k - c0 < kTileCols ? k - c0 : kTileCols;
        const uint32_t bytes = static_cast<uint32_t>(w * static_cast<int64_t>(sizeof(float)));
        mbar_arrive_expect_tx(&s_bar, bytes * static_cast<uint32_t>(u0.nrows));
        for (int r = 0; r < u0.nrows; ++r)
            bulk_g2s(s_a[r], A + (u0.r0 + r) * k + c0, bytes, &s_bar);
    }
    __syncthreads();
    const int64_t g = s_g;
    const int64_t t = b - g * tiles;
    const int64_t r0 = g * CPG;
    const int nrows = static_cast<int>(r0 + CPG <= m ? CPG : m - r0);
    const int sc = warp * (32 * L) + lane * L;                        // the lane's first column inside the tile
    const int64_t c = t * kTileCols + sc;                              // ... in A
    const int64_t s0 = t * (kTileCols / kSegCols) + warp * kSegPerWarp; // the warp's first segment
    // one warp polls the barrier, the others wait at the CTA barrier (no issue
    // slots spent); a wait that gives up (it never should) flags the build,
    // which the host then redoes on the two-pass path, once the copies landed
    bool waited = true;
    if (warp == 0)
        waited = mbar_wait_sleep(&s_bar, 0);
    if (!__syncthreads_and(waited)) {
        if (threadIdx.x == 0) {
            atomicOr(status, kStatusWaitTimeout);
            mbar_wait(&s_bar, 0);
        }
        return;
    }
    // the lane's nonzeros as one mask in GCOO order: bit q * CPG + r = (row r, column c + q)
    uint32_t msk = 0;
#pragma unroll
    for (int r = 0; r < CPG; ++r) {
        if (r < nrows) {
#pragma unroll
            for (int h = 0; h < L / 4; ++h) {
                if (c + 4 * h < k) { // k % 4 == 0: a float4 is wholly inside or wholly past the row
                    const float4 x = *reinterpret_cast<const float4 *>(&s_a[r][sc + 4 * h]);
                    const int q0 = 4 * h;
                    msk |= (nzb(x.x) << (q0 * CPG + r)) | (nzb(x.y) << ((q0 + 1) * CPG + r)) |
                           (nzb(x.z) << ((q0 + 2) * CPG + r)) | (nzb(x.w) << ((q0 + 3) * CPG + r));
                }
            }
        }
    }
    constexpr uint32_t kCol = (CPG == 4) ? (L == 8 ? 0x11111111u : 0x1111u)
                            : (CPG == 2) ? (L == 8 ? 0x5555u : 0x55u)
                            : (CPG == 1) ? (L == 8 ? 0xffu : 0xfu) : 0x01010101u;
    // per-row counts of the warp's segment(s): lanes 16..31 cover the second one (L = 8),
    // so one reduction of (first | second << 16) counts both
    const uint32_t hi = (L == 8 && lane >= 16) ? 16u : 0u;
    int wsum = 0, my_a = 0, my_b = 0;
#pragma unroll
    for (int r = 0; r < CPG; ++r) {
        const uint32_t x = __reduce_add_sync(0xffffffffu, static_cast<uint32_t>(__popc(msk & (kCol << r))) << hi);
        const int xa = static_cast<int>(x & 0xffffu), xb = static_cast<int>(x >> 16);
        wsum += xa + xb;
        my_a = lane == r ? xa : my_a;
        my_b = lane == 16 + r ? xb : my_b;
    }
    if (lane < nrows && s0 * kSegCols < k)
        cnt[(r0 + lane) * S + s0] = my_a; // lane r: row r's count
    if (L == 8 && lane >= 16 && lane - 16 < nrows && (s0 + 1) * kSegCols < k)
        cnt[(r0 + lane - 16) * S + s0 + 1] = my_b;
    if (lane == 0) {
        s_wtot[warp] = wsum;
        s_dist[warp] = 0;
    }
    if (distinct) {
        // fold the rows of each column onto its lowest bit: the columns with a nonzero
        uint32_t f = msk;
#pragma unroll
        for (int sh = 1; sh < CPG; sh <<= 1)
            f |= f >> sh;
        const int d = static_cast<int>(__reduce_add_sync(0xffffffffu, static_cast<uint32_t>(__popc(f & kCol))));
        if (lane == 0)
            s_dist[warp] = d;
    }
    // the lane's first entry in the warp's part: exclusive prefix of the lanes'
    // counts, one ballot per count level (a level rarely past 1 or 2 when sparse)
    const int mine = __popc(msk);
    const unsigned lt = (1u << lane) - 1u;
    int before = 0;
    for (int j = 0; __any_sync(0xffffffffu, mine > j); ++j)
        before += __popc(__ballot_sync(0xffffffffu, mine > j) & lt);
    __syncthreads(); // every warp of the CTA reaches this (no early exit above)
    int off = 0, T = 0;
    {
        int wt[8];
        const int4 w0 = *reinterpret_cast<const int4 *>(&s_wtot[0]);
        wt[0] = w0.x; wt[1] = w0.y; wt[2] = w0.z; wt[3] = w0.w;
        if (kWarps == 8) {
            const int4 w1 = *reinterpret_cast<const int4 *>(&s_wtot[4]);
            wt[4] = w1.x; wt[5] = w1.y; wt[6] = w1.z; wt[7] = w1.w;
        }
#pragma unroll
        for (int w = 0; w < kWarps; ++w) {
            off += w < warp ? wt[w] : 0;
            T += wt[w];
        }
    }
    const bool fits = T <= slot;
    if (threadIdx.x == 0) {
        tile_tot[b] = fits ? T : -1;
        if (!fits)
            over_list[atomicAdd(over_count, 1ull)] = static_cast<int32_t>(b);
        if (distinct) {
            int dsum = 0;
#pragma unroll
            for (int w = 0; w < kWarps; ++w)
                dsum += s_dist[w];
            if (dsum)
                atomicAdd(distinct, static_cast<unsigned long long>(dsum));
        }
    }
    if (!fits)
        return;
    int64_t pos = b * static_cast<int64_t>(slot) + off + before;
    while (msk) {
        const int i = __ffs(msk) - 1;
        msk &= msk - 1u;
        const int q = i / CPG, r = i % CPG;
        stage[pos++] = make_uint2((static_cast<uint32_t>(c + q) << 3) | static_cast<uint32_t>(r),
                                  __float_as_uint(s_a[r][sc + q]));
    }
}

template <int CPG>
__global__ void __launch_bounds__(kTileThreads, CPG <= 4 ? 6 : 4)
place_kernel(const float *__restrict__ A, int64_t m, int64_t k, int64_t tiles, int64_t S, int64_t units,
             int32_t slot, const uint2 *__restrict__ stage, const int32_t *__restrict__ tile_tot,
             const int32_t *__restrict__ over_list, const unsigned long long *__restrict__ over_count,
             const int32_t *__restrict__ pref, const int32_t *__restrict__ group_index,
             const int32_t *__restrict__ row_ptr, float *__restrict__ vals, int32_t *__restrict__ rc,
             Entry *__restrict__ packed, const int64_t *__restrict__ d_total, int64_t cap, int64_t packed_cap,
             int64_t staged_blocks)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const bool staged_block = static_cast<int64_t>(blockIdx.x) < staged_blocks;
    const int64_t b = static_cast<int64_t>(blockIdx.x) * kSegsPerCta + warp;
    // the tile's count is loaded alongside the totals (one round trip)
    const int32_t T = staged_block && b < units ? tile_tot[b] : 0;
    const int64_t total = d_total[0];
    if (d_total[3] != 0 || total < 0 || total > 0x7fffffffLL || total > cap || total + 2 > packed_cap)
        return; // staging gave up or the arrays are too small: the host converts again on the two-pass path
    // from here every position is below total < 2^31: 32-bit offsets
    int32_t *rows = rc, *cols = rc + total; // the reference's one rows|cols block
    if (staged_block) {
        if (T <= 0)
            return; // empty, or overflowed and placed by the rescan blocks
        const int64_t g = b / tiles, t = b - g * tiles, r0 = g * CPG, s0 = t * kSegsPerCta;
        const int nrows = static_cast<int>(r0 + CPG <= m ? CPG : m - r0);
        // every load the tile needs goes out at once: offsets and up to 4 windows of entries
        const int32_t my_pre = lane < nrows ? pref[(r0 + lane) * S + s0] : 0;
        const int32_t my_rp = lane < nrows ? row_ptr[r0 + lane] : 0;
        const int32_t gi = group_index[g];
        const uint2 *src = stage + b * static_cast<int64_t>(slot);
        constexpr int kWin = 4;
        uint2 e[kWin];
#pragma unroll
        for (int j = 0; j < kWin; ++j)
            e[j] = 32 * j + lane < T ? src[32 * j + lane] : make_uint2(0u, 0u);
        int32_t gpos = static_cast<int32_t>(gi);
        int32_t base[CPG];
#pragma unroll
        for (int r = 0; r < CPG; ++r) {
            const int32_t pre = __shfl_sync(0xffffffffu, my_pre, r);
            gpos += pre;
            base[r] = __shfl_sync(0xffffffffu, my_rp, r) + pre;
        }
        const unsigned lt = (1u << lane) - 1u;
        for (int w0 = 0; w0 < T; w0 += 32 * kWin) {
            if (w0 > 0) {
#pragma unroll
                for (int j = 0; j < kWin; ++j)
                    e[j] = w0 + 32 * j + lane < T ? src[w0 + 32 * j + lane] : make_uint2(0u, 0u);
            }
#pragma unroll
            for (int j = 0; j < kWin; ++j) {
                const int w = w0 + 32 * j;
                if (w >= T)
                    break;
                const bool ok = w + lane < T;
                const int r = static_cast<int>(e[j].x & 7u);
                const int32_t col = static_cast<int32_t>(e[j].x >> 3);
                if (ok) {
                    vals[gpos + w + lane] = __uint_as_float(e[j].y);
                    rows[gpos + w + lane] = static_cast<int32_t>(r0 + r);
                    cols[gpos + w + lane] = col;
                }
#pragma unroll
                for (int rr = 0; rr < CPG; ++rr) {
                    const unsigned mk = __ballot_sync(0xffffffffu, ok && r == rr);
                    if (ok && r == rr) {
                        Entry en;
                        en.col = col;
                        en.val = __uint_as_float(e[j].y);
                        packed[base[rr] + __popc(mk & lt)] = en;
                    }
                    base[rr] += __popc(mk);
                }
            }
        }
        return;
    }
    // rescan blocks: one overflowed tile at a time, a warp per segment
    const int64_t n_over = static_cast<int64_t>(*over_count);
    const int64_t stride = static_cast<int64_t>(gridDim.x) - staged_blocks;
    for (int64_t i = static_cast<int64_t>(blockIdx.x) - staged_blocks; i < n_over; i += stride)
        scatter_segment<CPG>(A, k, S, seg_unit<CPG>(m, k, tiles, over_list[i]), pref, group_index, row_ptr, vals,
                             rows, cols, packed);
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

bool staged_convert_ok(const float *A, int64_t m, int64_t k, int32_t cpg)
{
    return tiled_convert_ok(A, m, k, cpg) && k < (static_cast<int64_t>(1) << 28);
}

int64_t staged_tiles(int64_t m, int64_t k, int32_t cpg) { return ((m + cpg - 1) / cpg) * conv_tiles(k); }

int32_t staged_slot(int64_t last_nnz, int64_t tiles, int32_t cpg)
{
    const int64_t avg = tiles > 0 && last_nnz > 0 ? (last_nnz + tiles - 1) / tiles : 0;
    const int64_t want = 2 * avg + 32;
    // at most 256 entries per row of the tile: the slots take at most half of A's bytes
    int32_t slot = 32;
    while (slot < want && slot < 256 * cpg)
        slot <<= 1;
    return slot;
}

cudaError_t launch_stage(const float *A, int64_t m, int64_t k, int32_t cpg, int32_t slot, int32_t *cnt,
                         unsigned long long *distinct, uint2 *stage, int32_t *tile_tot, int32_t *over_list,
                         unsigned long long *over_count, uint32_t *status, cudaStream_t st)
{
    const int64_t tiles = conv_tiles(k), S = conv_segments(k);
    const int64_t units = ((m + cpg - 1) / cpg) * tiles;
    if (units <= 0)
        return cudaSuccess;
    const unsigned grid = static_cast<unsigned>(units);
#define GCOO_STAGE(C, L)                                                                                        \
    stage_kernel<C, L><<<grid, 1024 / (L), 0, st>>>(A, m, k, tiles, S, cnt, distinct, slot, stage, tile_tot,   \
                                                    over_list, over_count, status)
    switch (cpg) {
    case 1: GCOO_STAGE(1, 8); break;
    case 2: GCOO_STAGE(2, 8); break;
    case 4: GCOO_STAGE(4, 8); break;
    case 8: GCOO_STAGE(8, 4); break;
    default: return cudaErrorInvalidValue;
    }
#undef GCOO_STAGE
    count_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_place(const float *A, int64_t m, int64_t k, int32_t cpg, int32_t slot, const uint2 *stage,
                         const int32_t *tile_tot, const int32_t *over_list, const unsigned long long *over_count,
                         const int32_t *pref, const int32_t *group_index, const int32_t *row_ptr, float *vals,
                         int32_t *rc, Entry *packed, const int64_t *d_total, int64_t cap, int64_t packed_cap,
                         cudaStream_t st)
{
    const int64_t tiles = conv_tiles(k), S = conv_segments(k);
    const int64_t units = ((m + cpg - 1) / cpg) * tiles;
    if (units <= 0)
        return cudaSuccess;
    const int64_t staged_blocks = (units + kSegsPerCta - 1) / kSegsPerCta;
    // rescan blocks: enough to cover the GPU for matrices whose tiles mostly overflow
    int64_t rescan_blocks = static_cast<int64_t>(device_sms()) * 6;
    if (rescan_blocks > units)
        rescan_blocks = units;
    const unsigned grid = static_cast<unsigned>(staged_blocks + rescan_blocks);
#define GCOO_PLACE(C)                                                                                            \
    place_kernel<C><<<grid, kTileThreads, 0, st>>>(A, m, k, tiles, S, units, slot, stage, tile_tot, over_list,  \
                                                   over_count, pref, group_index, row_ptr, vals, rc, packed,   \
                                                   d_total, cap, packed_cap, staged_blocks)
    switch (cpg) {
    case 1: GCOO_PLACE(1); break;
    case 2: GCOO_PLACE(2); break;
    case 4: GCOO_PLACE(4); break;
    case 8: GCOO_PLACE(8); break;
    default: return cudaErrorInvalidValue;
    }
#undef GCOO_PLACE
    count_launches(1);
    return cudaGetLastError();
}

} // namespace gcoo
