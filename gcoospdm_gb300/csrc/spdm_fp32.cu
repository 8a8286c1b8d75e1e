// spdm_fp32.cu -- the plain FP32 GCOO x dense multiply on sm_103a.
//
// Replaces sparse_dense_groupcoo_mat_mul_kernel (src/gcoo_spdm_kernels.cu:
// 92-158). One CTA per (GCOO group, column tile):
//   * one elected thread stages the group's nonzeros (the contiguous range
//     [row_ptr[g*cpg], row_ptr[(g+1)*cpg]) of the packed row-ordered layout)
//     into shared memory with cp.async.bulk, completing on an mbarrier;
//   * each warp owns one row of the group and 32*V output columns; for every
//     entry of its row (a shared-memory broadcast) each lane loads V
//     consecutive B values with one 128-bit (V=4) coalesced load and updates
//     V register accumulators with fmaf;
//   * rows of the group run side by side, so B rows shared by several rows of
//     a group are served from L1.
// Every C element is a sequential fmaf chain over its row's entries in
// column order starting from 0.0f -- the same chain the reference kernel
// evaluates (its entries of one row are visited in column order too), so
// the FP32 result is bit-identical to the reference's.
#include "internal.cuh"

namespace gcoo {

namespace {

constexpr int kChunk = 2048; // most entries staged per pass (16 KB)

template <int V>
struct Vec;
template <>
struct Vec<4> {
    static __device__ __forceinline__ void load(const float *p, float (&o)[4])
    {
        const float4 t = __ldg(reinterpret_cast<const float4 *>(p));
        o[0] = t.x; o[1] = t.y; o[2] = t.z; o[3] = t.w;
    }
    static __device__ __forceinline__ void store(float *p, const float (&o)[4])
    {
        *reinterpret_cast<float4 *>(p) = make_float4(o[0], o[1], o[2], o[3]);
    }
};
template <>
struct Vec<2> {
    static __device__ __forceinline__ void load(const float *p, float (&o)[2])
    {
        const float2 t = __ldg(reinterpret_cast<const float2 *>(p));
        o[0] = t.x; o[1] = t.y;
    }
    static __device__ __forceinline__ void store(float *p, const float (&o)[2])
    {
        *reinterpret_cast<float2 *>(p) = make_float2(o[0], o[1]);
    }
};
template <>
struct Vec<1> {
    static __device__ __forceinline__ void load(const float *p, float (&o)[1]) { o[0] = __ldg(p); }
    static __device__ __forceinline__ void store(float *p, const float (&o)[1]) { *p = o[0]; }
};

template <int V, int U, bool PIPE>
__device__ __forceinline__ void row_chain(const Entry *__restrict__ s, int cnt, const float *__restrict__ Bj,
                                          int64_t n, float (&acc)[V])
{
    int i = 0;
    if (PIPE && cnt >= 2 * U) {
        // software pipeline: the B loads of batch i+1 are in flight while
        // batch i is accumulated (the fmaf order per element is unchanged)
        float a[U], b[U][V], a2[U], b2[U][V];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const Entry e = s[u];
            a[u] = e.val;
            Vec<V>::load(Bj + static_cast<int64_t>(e.col) * n, b[u]);
        }
#pragma unroll 1
        for (i = U; i + U <= cnt; i += U) {
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const Entry e = s[i + u];
                a2[u] = e.val;
                Vec<V>::load(Bj + static_cast<int64_t>(e.col) * n, b2[u]);
            }
#pragma unroll
            for (int u = 0; u < U; ++u)
#pragma unroll
                for (int v = 0; v < V; ++v)
                    acc[v] = fmaf(a[u], b[u][v], acc[v]);
#pragma unroll
            for (int u = 0; u < U; ++u) {
                a[u] = a2[u];
#pragma unroll
                for (int v = 0; v < V; ++v)
                    b[u][v] = b2[u][v];
            }
        }
#pragma unroll
        for (int u = 0; u < U; ++u)
#pragma unroll
            for (int v = 0; v < V; ++v)
                acc[v] = fmaf(a[u], b[u][v], acc[v]);
    }
#pragma unroll 1
    for (; i + U <= cnt; i += U) {
        Entry e[U];
        float b[U][V];
#pragma unroll
        for (int u = 0; u < U; ++u)
            e[u] = s[i + u];
#pragma unroll
        for (int u = 0; u < U; ++u)
            Vec<V>::load(Bj + static_cast<int64_t>(e[u].col) * n, b[u]);
#pragma unroll
        for (int u = 0; u < U; ++u)
#pragma unroll
            for (int v = 0; v < V; ++v)
                acc[v] = fmaf(e[u].val, b[u][v], acc[v]);
    }
#pragma unroll 1
    for (; i < cnt; ++i) {
        const Entry e = s[i];
        float b[V];
        Vec<V>::load(Bj + static_cast<int64_t>(e.col) * n, b);
#pragma unroll
        for (int v = 0; v < V; ++v)
            acc[v] = fmaf(e.val, b[v], acc[v]);
    }
}

// One row's chain over two column tiles at once (same entries, same fmaf
// order per element as row_chain): U entries per batch, 2U B loads in flight.
template <int V, int U>
__device__ __forceinline__ void row_chain_pair(const Entry *__restrict__ s, int cnt, const float *__restrict__ Ba,
                                               const float *__restrict__ Bb, int64_t n, float (&acc_a)[V],
                                               float (&acc_b)[V])
{
    int i = 0;
#pragma unroll 1
    for (; i + U <= cnt; i += U) {
        Entry e[U];
        float ba[U][V], bb[U][V];
#pragma unroll
        for (int u = 0; u < U; ++u)
            e[u] = s[i + u];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            Vec<V>::load(Ba + static_cast<int64_t>(e[u].col) * n, ba[u]);
            Vec<V>::load(Bb + static_cast<int64_t>(e[u].col) * n, bb[u]);
        }
#pragma unroll
        for (int u = 0; u < U; ++u)
#pragma unroll
            for (int v = 0; v < V; ++v) {
                acc_a[v] = fmaf(e[u].val, ba[u][v], acc_a[v]);
                acc_b[v] = fmaf(e[u].val, bb[u][v], acc_b[v]);
            }
    }
#pragma unroll 1
    for (; i < cnt; ++i) {
        const Entry e = s[i];
        float ba[V], bb[V];
        Vec<V>::load(Ba + static_cast<int64_t>(e.col) * n, ba);
        Vec<V>::load(Bb + static_cast<int64_t>(e.col) * n, bb);
#pragma unroll
        for (int v = 0; v < V; ++v) {
            acc_a[v] = fmaf(e.val, ba[v], acc_a[v]);
            acc_b[v] = fmaf(e.val, bb[v], acc_b[v]);
        }
    }
}

// MAXT bounds the CTA size (rows_per_group * col_warps warps); the 1024-thread
// variant (rows_per_group 32) unrolls less to stay within 64 registers.
// col_iters > 1 (only when every group's entries fit one staging chunk): each
// warp walks col_iters column tiles, col_warps tiles apart, reusing the
// staged entries, so short rows do not pay one staging per tile.
template <int V, int MAXT, bool PIPE, bool MULTI>
__global__ void __launch_bounds__(MAXT)
spdm_fp32_kernel(const Entry *__restrict__ packed, const int32_t *__restrict__ row_ptr, int64_t m,
                 int32_t cpg, const float *__restrict__ B, int64_t n, float *__restrict__ C,
                 int32_t col_warps, int32_t col_iters, int32_t chunk_cap, uint32_t *__restrict__ status)
{
    if (!MULTI)
        col_iters = 1;
    extern __shared__ __align__(128) unsigned char smem[];
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem);
    Entry *s_nz = reinterpret_cast<Entry *>(smem + 128);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int slot = warp / col_warps, sub = warp - slot * col_warps;
    const int64_t r0 = static_cast<int64_t>(blockIdx.x) * cpg;
    const int64_t r_end = r0 + cpg < m ? r0 + cpg : m;
    const int64_t row = r0 + slot;
    const bool has_row = slot < cpg && row < r_end;
    const int64_t tile_stride = static_cast<int64_t>(col_warps) * (32 * V);
    const int64_t j = (static_cast<int64_t>(blockIdx.y) * col_iters * col_warps + sub) * (32 * V) +
                      static_cast<int64_t>(lane) * V;

    const int64_t gs = row_ptr[r0];
    const int64_t ge = row_ptr[r_end];
    int64_t rs = 0, re = 0;
    if (has_row) {
        rs = row_ptr[row];
        re = row_ptr[row + 1];
    }
    if (threadIdx.x == 0) {
        mbar_init(bar, 1);
        fence_mbar_init();
    }
    __syncthreads();

    float acc[V];
    // chunk: entries staged per pass, what the launch's shared memory holds
    const int64_t chunk = chunk_cap < kChunk ? chunk_cap : kChunk;
    const int64_t total = ge - gs;
    const int64_t nchunks = (total + chunk - 1) / chunk;
    // several column tiles per warp from one staging (the group fits one
    // chunk): every tile, the first included, is walked after the staging,
    // two at a time for short rows
    const bool multi_all = MULTI && col_iters > 1 && nchunks == 1;
    // otherwise each of the warp's tiles walks the group chunk by chunk
    const int tiles_staged = multi_all ? 1 : col_iters;
    bool ok = true;
    uint32_t phase = 0;
    for (int it = 0; it < tiles_staged && ok; ++it) {
        const int64_t jt = j + it * tile_stride;
        const float *Bj = B + jt;
#pragma unroll
        for (int v = 0; v < V; ++v)
            acc[v] = 0.0f;
        for (int64_t ch = 0; ch < nchunks; ++ch, ++phase) {
            const int64_t cs = gs + ch * chunk;
            const int64_t ce = cs + chunk < ge ? cs + chunk : ge;
            const int64_t a0 = cs & ~static_cast<int64_t>(1); // 16-byte aligned superset
            const int64_t a1 = (ce + 1) & ~static_cast<int64_t>(1);
            if (threadIdx.x == 0) {
                fence_proxy_async();
                const uint32_t bytes = static_cast<uint32_t>((a1 - a0) * static_cast<int64_t>(sizeof(Entry)));
                mbar_arrive_expect_tx(bar, bytes);
                bulk_g2s(s_nz, packed + a0, bytes, bar);
            }
            const bool waited = mbar_wait(bar, phase & 1);
            ok = __syncthreads_and(waited) != 0;
            if (!ok) {
                if (threadIdx.x == 0)
                    atomicOr(status, kStatusWaitTimeout);
                mbar_wait(bar, phase & 1); // let the copy in flight land
                break;
            }
            const int64_t lo = rs > cs ? rs : cs;
            const int64_t hi = re < ce ? re : ce;
            if (!multi_all && jt < n && lo < hi)
                row_chain<V, (MAXT > 512 ? 4 : 8), PIPE>(s_nz + (lo - a0), static_cast<int>(hi - lo), Bj, n, acc);
            __syncthreads(); // buffer free before the next copy
        }
        if (!multi_all && has_row && jt < n && ok)
            Vec<V>::store(C + row * n + jt, acc);
    }
    // all column tiles of the warp's row from the (single) staged chunk
    if (multi_all && ok && has_row) {
        const int64_t a0 = gs & ~static_cast<int64_t>(1);
        const Entry *s_row = s_nz + (rs - a0);
        const int cnt = static_cast<int>(re - rs);
        int it = 0;
        // very short rows: two tiles at a time, twice the B loads in flight
        // (longer rows already keep a batch of 8 loads in flight per tile)
        for (; cnt < 16 && it + 1 < col_iters; it += 2) {
            const int64_t ja = j + it * tile_stride, jb = ja + tile_stride;
            if (ja >= n)
                break;
            float a2[V], b2[V];
#pragma unroll
            for (int v = 0; v < V; ++v)
                a2[v] = b2[v] = 0.0f;
            if (jb < n)
                row_chain_pair<V, 4>(s_row, cnt, B + ja, B + jb, n, a2, b2);
            else if (cnt > 0)
                row_chain<V, 4, false>(s_row, cnt, B + ja, n, a2);
            Vec<V>::store(C + row * n + ja, a2);
            if (jb < n)
                Vec<V>::store(C + row * n + jb, b2);
        }
        for (; it < col_iters; ++it) {
            const int64_t jt = j + it * tile_stride;
            if (jt >= n)
                break;
#pragma unroll
            for (int v = 0; v < V; ++v)
                acc[v] = 0.0f;
            if (cnt > 0)
                row_chain<V, (MAXT > 512 ? 4 : 8), false>(s_row, cnt, B + jt, n, acc);
            Vec<V>::store(C + row * n + jt, acc);
        }
    }
}

// The short rows of a skewed matrix (its long rows go to spdm_long.cu or
// spdm_split.cu): one warp per (row, 32*V-column tile), nothing staged and no
// CTA barrier -- a row of a dozen entries is all latency, and a staging round
// trip and a group barrier would double it. The row's two pointers come in
// one load (lanes 0 and 1) and are shuffled to the warp. Lane i loads entry i
// of each 32-entry window; the B rows of eight entries at a time are loaded
// with their columns shuffled from the owning lanes; each column's fmaf chain
// runs over the row's entries in column order from 0.0f, as in every other
// FP32 kernel. Measured slower on the Zipf workload (0.148 ms for this
// kernel with the long rows beside it): runs of 2-8 rows per warp with the
// next row's entries requested early (0.158-0.171 ms), bundles of 2-8 rows
// whose batches of eight entries run across row boundaries (0.159-0.211 ms),
// and one warp on both 128-column tiles of a row (0.167 ms): at a dozen
// entries per row, more independent warps in flight beat fewer round trips
// per warp. When B is larger than kShortTileMajorBytes the warps walk
// tile-major (every row's first column tile, then every row's second, ...),
// so one column slab of B is live in L2 instead of all of B: 0.150 -> 0.142
// ms with the long rows beside it (B 65536 x 256, 67 MB, was read from DRAM
// about twice in row-major order).
template <int V>
__device__ __forceinline__ void short_window(const Entry &my, int nw, bool all_cols, bool has_col,
                                             const float *__restrict__ Bj, int64_t n, float (&acc)[V])
{
    int u0 = 0;
    if (all_cols) { // warp-uniform: every lane takes part in the shuffles below
        // whole batches of eight: no per-entry predicates
        for (; u0 + 8 <= nw; u0 += 8) {
            float a[8], b[8][V];
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                const int col = __shfl_sync(0xffffffffu, my.col, u0 + u);
                a[u] = __shfl_sync(0xffffffffu, my.val, u0 + u);
                Vec<V>::load(Bj + static_cast<int64_t>(col) * n, b[u]);
            }
#pragma unroll
            for (int u = 0; u < 8; ++u)
#pragma unroll
                for (int v = 0; v < V; ++v)
                    acc[v] = fmaf(a[u], b[u][v], acc[v]);
        }
    }
    // the tail batch (and lanes past n: shuffles only)
    for (; u0 < nw; u0 += 8) {
        float a[8], b[8][V];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            const int col = __shfl_sync(0xffffffffu, my.col, (u0 + u) & 31);
            a[u] = __shfl_sync(0xffffffffu, my.val, (u0 + u) & 31);
            if (u0 + u < nw && has_col) {
                Vec<V>::load(Bj + static_cast<int64_t>(col) * n, b[u]);
            } else {
#pragma unroll
                for (int v = 0; v < V; ++v)
                    b[u][v] = 0.0f;
            }
        }
#pragma unroll
        for (int u = 0; u < 8; ++u)
            if (u0 + u < nw)
#pragma unroll
                for (int v = 0; v < V; ++v)
                    acc[v] = fmaf(a[u], b[u][v], acc[v]);
    }
}

// B larger than this walks tile-major (see spdm_short_kernel)
constexpr int64_t kShortTileMajorBytes = 32ll << 20;

template <int V>
__global__ void __launch_bounds__(64, 16)
spdm_short_kernel(const Entry *__restrict__ packed, const int32_t *__restrict__ row_ptr, int64_t m,
                  const float *__restrict__ B, int64_t n, float *__restrict__ C, int32_t tiles, int32_t long_min,
                  int32_t tile_major)
{
    const int lane = threadIdx.x & 31;
    const int64_t gw = (static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    int64_t row;
    int t;
    if (tile_major) { // every row's tile 0, then every row's tile 1, ...: one B column slab live in L2 at a time
        t = static_cast<int>(gw / m);
        row = gw - static_cast<int64_t>(t) * m;
        if (t >= tiles)
            return;
    } else {
        row = gw / tiles;
        if (row >= m)
            return;
        t = static_cast<int>(gw - row * tiles);
    }
    const int32_t rp = lane < 2 ? row_ptr[row + lane] : 0;
    const int32_t rs = __shfl_sync(0xffffffffu, rp, 0);
    const int cnt = __shfl_sync(0xffffffffu, rp, 1) - rs;
    if (long_min > 0 && cnt >= long_min)
        return; // the long-row kernel writes this row (warp-uniform)
    const int64_t j = static_cast<int64_t>(t) * (32 * V) + static_cast<int64_t>(lane) * V;
    const bool has_col = j < n;
    const bool all_cols = __all_sync(0xffffffffu, has_col);
    const float *Bj = B + (has_col ? j : 0);
    float acc[V];
#pragma unroll
    for (int v = 0; v < V; ++v)
        acc[v] = 0.0f;
    for (int w0 = 0; w0 < cnt; w0 += 32) {
        const int nw = cnt - w0 < 32 ? cnt - w0 : 32;
        Entry my;
        my.col = 0;
        my.val = 0.0f;
        if (lane < nw)
            my = packed[rs + w0 + lane];
        short_window<V>(my, nw, all_cols, has_col, Bj, n, acc);
    }
    if (has_col)
        Vec<V>::store(C + row * n + j, acc);
}

// Multiply straight from reference-layout arrays (entries of a group in
// column-then-row order, separate vals/rows/cols): one thread per output
// column, one shared-memory accumulator per (group row, column) so any
// rows_per_group works; each accumulator still sees its row's entries in
// column order, hence the same fmaf chain.
constexpr int kViewThreads = 128;
__global__ void __launch_bounds__(kViewThreads)
spdm_view_kernel(const float *__restrict__ vals, const int32_t *__restrict__ rows,
                 const int32_t *__restrict__ cols, const int32_t *__restrict__ group_index,
                 const int32_t *__restrict__ nnz_per_group, int64_t m, int32_t cpg,
                 const float *__restrict__ B, int64_t n, float *__restrict__ C)
{
    extern __shared__ float s_acc[]; // [cpg][kViewThreads]
    const int64_t g = blockIdx.x;
    const int64_t r0 = g * cpg;
    const int64_t j = static_cast<int64_t>(blockIdx.y) * kViewThreads + threadIdx.x;
    for (int r = 0; r < cpg; ++r)
        s_acc[r * kViewThreads + threadIdx.x] = 0.0f;
    const int64_t e0 = group_index[g];
    const int64_t e1 = e0 + nnz_per_group[g];
    if (j < n) {
        for (int64_t e = e0; e < e1; ++e) {
            const int32_t lr = rows[e] - static_cast<int32_t>(r0);
            if (lr < 0 || lr >= cpg)
                continue; // not this group's row: malformed input, skipped
            float *a = s_acc + lr * kViewThreads + threadIdx.x;
            *a = fmaf(vals[e], __ldg(B + static_cast<int64_t>(cols[e]) * n + j), *a);
        }
        for (int r = 0; r < cpg && r0 + r < m; ++r)
            C[(r0 + r) * n + j] = s_acc[r * kViewThreads + threadIdx.x];
    }
}

} // namespace

int device_sms()
{
    static int sms = 0;
    if (!sms) {
        int dev = 0;
        cudaGetDevice(&dev);
        if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0)
            sms = 152;
    }
    return sms;
}

bool row_lengths_skewed(int64_t m, int64_t nnz, int64_t max_row)
{
    const double mean = m > 0 ? static_cast<double>(nnz) / static_cast<double>(m) : 0.0;
    return max_row >= 256 && static_cast<double>(max_row) > 8.0 * (mean > 1.0 ? mean : 1.0);
}

LaunchShape pick_shape(const gcoo_params &p, int64_t m, int64_t n, int64_t nnz, int64_t max_row,
                       uintptr_t b_addr, uintptr_t c_addr)
{
    LaunchShape s;
    // Heavy-tailed row lengths (the longest row far above the mean): one row
    // per CTA, so a long row does not hold its group's other rows back, and
    // the next batch's B loads in flight, since a long row is one long
    // dependent chain. The per-element fmaf order is the same either way.
    const double mean = m > 0 ? static_cast<double>(nnz) / static_cast<double>(m) : 0.0;
    const bool skewed = row_lengths_skewed(m, nnz, max_row);
    s.rows = skewed ? 1 : p.rows_per_group;
    int vmax = 4;
    if (n % 4 != 0 || (b_addr & 15) || (c_addr & 15))
        vmax = 2;
    if (vmax == 2 && (n % 2 != 0 || (b_addr & 7) || (c_addr & 7)))
        vmax = 1;
    int v = p.vec > 0 ? p.vec : (n >= 128 ? 4 : (n >= 64 ? 2 : 1));
    if (v > vmax)
        v = vmax;
    if (v != 1 && v != 2 && v != 4)
        v = 1;
    s.vec = v;
    // Every group fits one staging chunk: one staging of a group's entries
    // can serve several column tiles per warp. With the launch shape left to
    // the library, a CTA takes fewer rows (down to one) where that makes its
    // group fit; rows of up to 2046 entries then stay on the one-warp-per-row
    // path (any rows per CTA gives the same fmaf chains).
    const auto fits = [&](int rows) { return max_row > 0 && max_row * static_cast<int64_t>(rows) + 2 <= kChunk; };
    if (!skewed && p.warps <= 0 && p.col_warps <= 0)
        while (s.rows > 1 && !fits(s.rows) && fits(1))
            s.rows = s.rows / 2 > 0 ? s.rows / 2 : 1;
    const int cpg = s.rows;
    const bool one_chunk = fits(s.rows);
    int cw;
    if (p.col_warps > 0)
        cw = p.col_warps;
    else if (p.warps <= 0 && !skewed && one_chunk)
        // One warp per row, 4-warp CTAs, each warp walking several column
        // tiles of its row: measured on GB300 1.06 against 1.15 ms (8192^2,
        // 1 %) and 0.178 against 0.201 ms (8192^2, 0.1 %) for two warps per
        // row: twice the CTAs resident per SM keep more B loads in flight,
        // and the latency of the loads is what bounds these matrices.
        cw = 1;
    else {
        const int target = p.warps > 0 ? p.warps : 8;
        cw = target / cpg;
        if (cw < 1)
            cw = 1;
        // no wider than the matrix
        while (cw > 1 && static_cast<int64_t>(cw / 2) * 32 * v >= n)
            cw /= 2;
    }
    if (cw * cpg > 32)
        cw = 32 / cpg > 0 ? 32 / cpg : 1;
    s.col_warps = cw;
    s.warps = cw * cpg;
    s.depth = p.depth > 0 ? p.depth : (skewed ? 2 : 1);
    s.col_iters = 1;
    if (one_chunk) {
        const int64_t tile = static_cast<int64_t>(s.col_warps) * 32 * s.vec;
        const int64_t ny = (n + tile - 1) / tile;
        // about 768 columns per CTA (0.5-0.9 K columns measured best from
        // 2048^2 to 16384^2 at 1 % to 0.1 % density), but at least two waves
        // of CTAs (12 four-warp CTAs resident per SM) on small matrices
        int64_t ci = 768 / tile;
        const int64_t groups = (m + s.rows - 1) / s.rows;
        const int64_t resident = static_cast<int64_t>(device_sms()) * (s.warps <= 4 ? 12 : 6);
        const int64_t by_grid = groups * ny / (2 * resident);
        ci = ci > by_grid ? by_grid : ci;
        ci = ci < 1 ? 1 : (ci > ny ? ny : ci);
        s.col_iters = static_cast<int>(ci > 64 ? 64 : ci);
        // shared memory for the largest possible group only, not a full
        // chunk: the rest of the SM's L1 array then holds B loads in flight
        // (measured 2-6 % faster at 0.1-1 % density)
        s.chunk = static_cast<int>(max_row * s.rows);
    }
    return s;
}

cudaError_t launch_spdm_fp32(const Entry *packed, const int32_t *row_ptr, int64_t m, const float *B, int64_t n,
                             float *C, const LaunchShape &s, uint32_t *status, cudaStream_t st)
{
    const int32_t cpg = s.rows; // rows per CTA (any value gives the same fmaf chains)
    const int64_t ng = (m + cpg - 1) / cpg;
    const int64_t tile = static_cast<int64_t>(s.col_warps) * 32 * s.vec * (s.col_iters > 1 ? s.col_iters : 1);
    const int64_t ny = (n + tile - 1) / tile;
    if (ng <= 0 || ny <= 0)
        return cudaSuccess;
    if (ny > 65535)
        return cudaErrorInvalidConfiguration;
    dim3 grid(static_cast<unsigned>(ng), static_cast<unsigned>(ny));
    const int threads = s.warps * 32;
    // entries staged per pass and the shared memory that holds them (the
    // kernel stages any larger group in several passes)
    const int chunk = s.chunk > 0 && s.chunk < kChunk ? s.chunk : kChunk;
    const int smem = 128 + (chunk + 2) * static_cast<int>(sizeof(Entry));
#define GCOO_FP32_LAUNCH(V, T, P)                                                                       \
    do {                                                                                                \
        if (s.col_iters > 1)                                                                            \
            spdm_fp32_kernel<V, T, P, true><<<grid, threads, smem, st>>>(                               \
                packed, row_ptr, m, cpg, B, n, C, s.col_warps, s.col_iters, chunk, status);             \
        else                                                                                            \
            spdm_fp32_kernel<V, T, P, false><<<grid, threads, smem, st>>>(                              \
                packed, row_ptr, m, cpg, B, n, C, s.col_warps, 1, chunk, status);                       \
    } while (0)
#define GCOO_FP32_VEC(T, P)                                                                             \
    do {                                                                                                \
        if (s.vec == 4) GCOO_FP32_LAUNCH(4, T, P);                                                      \
        else if (s.vec == 2) GCOO_FP32_LAUNCH(2, T, P);                                                 \
        else GCOO_FP32_LAUNCH(1, T, P);                                                                 \
    } while (0)
    const bool pipe = s.depth >= 2;
    if (threads <= 512) {
        if (pipe) GCOO_FP32_VEC(512, true);
        else GCOO_FP32_VEC(512, false);
    } else {
        if (pipe) GCOO_FP32_VEC(1024, true);
        else GCOO_FP32_VEC(1024, false);
    }
#undef GCOO_FP32_VEC
#undef GCOO_FP32_LAUNCH
    count_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_spdm_short(const Entry *packed, const int32_t *row_ptr, int64_t m, int64_t k, const float *B,
                              int64_t n, float *C, int32_t long_min, cudaStream_t st)
{
    if (m <= 0 || n <= 0)
        return cudaSuccess;
    const uintptr_t b = reinterpret_cast<uintptr_t>(B), c = reinterpret_cast<uintptr_t>(C);
    int v = 1;
    if (n % 4 == 0 && !(b & 15) && !(c & 15))
        v = 4;
    else if (n % 2 == 0 && !(b & 7) && !(c & 7))
        v = 2;
    const int64_t tiles = (n + 32 * v - 1) / (32 * v);
    const int64_t warps = m * tiles;
    // two-warp CTAs: rows of very different lengths do not hold one another's
    // CTA slot (8-warp CTAs: 145 us on the Zipf workload, 2-warp: 127 us, 1-warp: 134 us)
    const int64_t blocks = (warps + 1) / 2;
    if (tiles > 0x7fffffffLL || blocks > 0x7fffffffLL)
        return cudaErrorInvalidConfiguration;
    const unsigned grid = static_cast<unsigned>(blocks);
    const int32_t nt = static_cast<int32_t>(tiles);
    const int32_t tm = tiles > 1 && k * n * 4 > kShortTileMajorBytes ? 1 : 0;
    if (v == 4)
        spdm_short_kernel<4><<<grid, 64, 0, st>>>(packed, row_ptr, m, B, n, C, nt, long_min, tm);
    else if (v == 2)
        spdm_short_kernel<2><<<grid, 64, 0, st>>>(packed, row_ptr, m, B, n, C, nt, long_min, tm);
    else
        spdm_short_kernel<1><<<grid, 64, 0, st>>>(packed, row_ptr, m, B, n, C, nt, long_min, tm);
    count_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_spdm_view(const gcoo_view &a, const float *B, int64_t n, float *C, cudaStream_t st)
{
    if (a.n_group <= 0 || n <= 0)
        return cudaSuccess;
    const int64_t ny = (n + kViewThreads - 1) / kViewThreads;
    if (ny > 65535)
        return cudaErrorInvalidConfiguration;
    dim3 grid(static_cast<unsigned>(a.n_group), static_cast<unsigned>(ny));
    const size_t smem = sizeof(float) * static_cast<size_t>(a.rows_per_group) * kViewThreads;
    spdm_view_kernel<<<grid, kViewThreads, smem, st>>>(a.vals, a.rows, a.cols, a.group_index, a.nnz_per_group,
                                                       a.m, a.rows_per_group, B, n, C);
    count_launches(1);
    return cudaGetLastError();
}

} // namespace gcoo
