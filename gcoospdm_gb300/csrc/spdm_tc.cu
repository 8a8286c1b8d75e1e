// spdm_tc.cu -- tensor-core (tcgen05) engine for matrices whose nonzeros
// densify into 16-wide blocks.
//
// Plan (built once per handle and form, from the GCOO entries):
//   * A is cut into panels (256 rows for BF16 and FP8-B, 128 for split-BF16);
//     a tile is the panel's 16-column slice at column block cb, active when
//     it holds any entry;
//   * each active tile is stored densely (zeros where A has none) as BF16,
//     each 128-row half in the K-major, 32-byte-swizzled shared-memory layout
//     of tcgen05 (row r at r*32 bytes, 16-byte chunk c at
//     (c ^ ((r >> 2) & 1)) * 16), so a 4 KB copy lands a half ready for the
//     MMA; split-BF16 keeps two more tiles (lo = x - hi and lo2 = x - hi -
//     lo, each rounded to BF16: hi + lo + lo2 is x exactly), stored side by
//     side;
//   * B is converted per call into tiles of N output columns x 16 k (the
//     same layout, N rows of 32 bytes).
// BF16 / FP8-B kernel (spdm_tc_pair_kernel): a cluster of two CTAs on two
// SMs per (256-row panel, 256 or 512 output columns); each CTA streams its
// 128-row half of four tiles and its 128-column halves of their B tiles per
// stage with tensor-map bulk copies (cta_group::2, completing on the first
// CTA's barrier), and the first CTA issues tcgen05.mma.cta_group::2 (M=256,
// N=256, K=16) into both CTAs' tensor memory, one accumulator per 256
// columns. Split-BF16 kernel (spdm_tc_kernel): one CTA per (128-row panel,
// 128 columns), one stage per tile, six MMAs per tile. Every wait is bounded.
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_fp8.h>

#include <cuda.h>

#include <mutex>

#include "handle.hpp"

namespace gcoo {

constexpr int kPanel = 128;   // rows of a tile half (one CTA's MMA rows)
constexpr int kTileK = 16;    // columns per tile (MMA K)
constexpr int kTileBytes = kPanel * kTileK * 2; // one 128-row half

struct TcPlan {
    int64_t panels = 0, kb = 0, tiles = 0;
    int panel_rows = kPanel; // 256 for the pair kernel (two halves per tile), 128 for split-BF16
    bool split = false;
    int64_t nnz = 0;
    DevBuf<int32_t> pf;       // exclusive prefix over (panel, cb) flags, size panels*kb + 1
    DevBuf<int32_t> tile_cb;  // cb of each tile (ascending within a panel)
    DevBuf<uint16_t> a_hi;    // tiles * (panel_rows / 128) * 2048 bf16 (swizzled halves)
    DevBuf<uint16_t> a_lo;    // split only: tiles * 2 * 2048 bf16 (lo, then lo2, per tile)
    DevBuf<int64_t> scratch;
    // B workspace (per call)
    DevBuf<uint16_t> b_hi, b_lo; // b_lo (split only): lo then lo2 per B tile
    int64_t b_n = 0;
    // FP8-B: per-column power-of-two scales (and their absmax scratch)
    DevBuf<float> b_scale;
    DevBuf<unsigned> b_amax;
    // tensor maps of the pair kernel's copies (host copies, passed by value)
    CUtensorMap map_a, map_b;
    const void *map_a_base = nullptr, *map_b_base = nullptr;
    uint64_t map_a_rows = 0, map_b_rows = 0;
};

void destroy_tc_plan(TcPlan *p) { delete p; }

namespace {

// ---- small PTX wrappers for tcgen05 ----------------------------------------------
__device__ __forceinline__ uint64_t smem_desc_sw32(uint32_t saddr)
{
    // start address >> 4 | LBO (unused for swizzled K-major) = 1 | SBO = 256 B (8 rows x 32 B)
    // | version 1 (bits 46-47) | layout SWIZZLE_32B = 6 (bits 61-63)
    return static_cast<uint64_t>((saddr >> 4) & 0x3FFFu) | (static_cast<uint64_t>(1) << 16) |
           (static_cast<uint64_t>(256 >> 4) << 32) | (static_cast<uint64_t>(1) << 46) |
           (static_cast<uint64_t>(6) << 61);
}

__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N)
{
    // D f32 (bits 4-5 = 1), A bf16 (7-9 = 1), B bf16 (10-12 = 1), both K-major,
    // N >> 3 at bits 17-22, M >> 4 at bits 24-28.
    return (1u << 4) | (1u << 7) | (1u << 10) | (static_cast<uint32_t>(N >> 3) << 17) |
           (static_cast<uint32_t>(M >> 4) << 24);
}

__device__ __forceinline__ void tc_mma(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc)
{
    asm volatile("{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                 "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
                 "l"(a), "l"(b), "r"(idesc), "r"(acc)
                 : "memory");
}

__device__ __forceinline__ void tc_commit(uint64_t *bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32])
{
    uint32_t r[32];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x32.b32 "
                 "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
                 "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                   "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
                   "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]),
                   "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]),
                   "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
                 : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; ++i)
        v[i] = __uint_as_float(r[i]);
}

// Byte offset of element (row r, column c) of a 32-byte-row K-major tile in
// the 32B-swizzled layout.
__host__ __device__ __forceinline__ uint32_t sw32_offset(uint32_t r, uint32_t c)
{
    const uint32_t chunk = (c >> 3) ^ ((r >> 2) & 1u);
    return r * 32u + chunk * 16u + (c & 7u) * 2u;
}

// ---- plan building --------------------------------------------------------------------
__global__ void tile_flags_kernel(const Entry *__restrict__ packed, const int32_t *__restrict__ row_ptr, int64_t m,
                                  int64_t kb, int panel_rows, int32_t *__restrict__ flags)
{
    const int lane = threadIdx.x & 31;
    const int64_t warp = (static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = (static_cast<int64_t>(gridDim.x) * blockDim.x) >> 5;
    for (int64_t r = warp; r < m; r += nw) {
        const int64_t base = (r / panel_rows) * kb;
        for (int64_t e = row_ptr[r] + lane; e < row_ptr[r + 1]; e += 32)
            flags[base + packed[e].col / kTileK] = 1;
    }
}

__global__ void tile_list_kernel(const int32_t *__restrict__ pf, int64_t total, int64_t kb, int32_t *__restrict__ tile_cb)
{
    for (int64_t f = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; f < total;
         f += static_cast<int64_t>(gridDim.x) * blockDim.x)
        if (pf[f + 1] != pf[f])
            tile_cb[pf[f]] = static_cast<int32_t>(f % kb);
}

// lo (split-BF16 only) is filled with 128-row panels.
__global__ void tile_fill_kernel(const Entry *__restrict__ packed, const int32_t *__restrict__ row_ptr, int64_t m,
                                 int64_t kb, int panel_rows, const int32_t *__restrict__ pf,
                                 __nv_bfloat16 *__restrict__ hi, __nv_bfloat16 *__restrict__ lo)
{
    const int lane = threadIdx.x & 31;
    const int64_t warp = (static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = (static_cast<int64_t>(gridDim.x) * blockDim.x) >> 5;
    const int64_t tile_elems = static_cast<int64_t>(panel_rows / kPanel) * (kTileBytes / 2);
    for (int64_t r = warp; r < m; r += nw) {
        const int64_t base = (r / panel_rows) * kb;
        const uint32_t lr = static_cast<uint32_t>(r % panel_rows);
        for (int64_t e = row_ptr[r] + lane; e < row_ptr[r + 1]; e += 32) {
            const Entry t = packed[e];
            const int64_t tile = pf[base + t.col / kTileK];
            const uint32_t off = (lr / kPanel) * (kTileBytes / 2) +
                                 sw32_offset(lr % kPanel, static_cast<uint32_t>(t.col % kTileK)) / 2;
            const __nv_bfloat16 h = __float2bfloat16_rn(t.val);
            hi[tile * tile_elems + off] = h;
            if (lo) {
                const float r1 = t.val - __bfloat162float(h); // exact
                const __nv_bfloat16 l1 = __float2bfloat16_rn(r1);
                lo[tile * kTileBytes + off] = l1;
                lo[tile * kTileBytes + kTileBytes / 2 + off] = __float2bfloat16_rn(r1 - __bfloat162float(l1));
            }
        }
    }
}

// B (k x n FP32, row-major) -> tiles [jt][cb] of N rows (output columns) x 16 k, swizzled.
// With fp8_scale (FP8-B): each value is first quantized to E4M3 in units of
// its column's power-of-two scale, then stored as the exact BF16 value of
// E4M3 x scale, so the BF16 MMA multiplies the FP8-B operand exactly.
// One CTA per tile: the 16 x N block of B is staged in shared memory with
// coalesced 16-byte loads (64 lanes per 256 columns of a row), then thread
// jj builds tile row jj (output column jt*N + jj: 16 values read down a
// shared-memory column, conflict-free across the warp) and writes its 32
// bytes with two 16-byte stores, so a warp writes 1 KB contiguous. (Lanes
// loading 4-byte values down B's columns directly: 20 us for B 8192 x 1024.)
__device__ __forceinline__ uint32_t pack_bf16(__nv_bfloat16 lo_half, __nv_bfloat16 hi_half)
{
    return static_cast<uint32_t>(__bfloat16_as_ushort(lo_half)) |
           (static_cast<uint32_t>(__bfloat16_as_ushort(hi_half)) << 16);
}

constexpr int kBTileMaxN = 256;

// Needs n % 4 == 0 and B 16-byte aligned (the tensor engine takes n % 16 == 0).
__global__ void __launch_bounds__(256)
b_tiles_kernel(const float *__restrict__ B, int64_t k, int64_t n, int N, int64_t kb, __nv_bfloat16 *__restrict__ hi,
               __nv_bfloat16 *__restrict__ lo, const float *__restrict__ fp8_scale)
{
    __shared__ __align__(16) float blk[kTileK][kBTileMaxN];
    const int64_t cb = blockIdx.x;
    const int64_t jt = blockIdx.y;
    const int64_t tile = jt * kb + cb;
    const size_t tile_elems = static_cast<size_t>(N) * kTileK;
    const int n4 = N / 4; // float4 columns per block row
    for (int i = threadIdx.x; i < kTileK * n4; i += blockDim.x) {
        const int r = i / n4, c4 = i - r * n4;
        const int64_t c = cb * kTileK + r;
        const int64_t j = jt * N + c4 * 4;
        float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
        if (c < k && j < n)
            v = __ldg(reinterpret_cast<const float4 *>(B + c * n + j));
        *reinterpret_cast<float4 *>(&blk[r][c4 * 4]) = v;
    }
    __syncthreads();
    for (int jj = threadIdx.x; jj < N; jj += blockDim.x) {
        const int64_t j = jt * N + jj;
        float sc = 1.0f;
        if (fp8_scale && j < n)
            sc = fp8_scale[j];
        // a power of two in the normal range has an exact reciprocal, so
        // v * inv is v / sc exactly; otherwise divide
        const bool by_inv = sc >= 1.17549435e-38f && sc <= 8.50705917e37f;
        const float inv = by_inv ? 1.0f / sc : 0.0f;
        uint32_t wh[8], wl[8], wl2[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            __nv_bfloat16 h2[2], l2[2], m2[2];
#pragma unroll
            for (int e = 0; e < 2; ++e) {
                float v = blk[q * 2 + e][jj];
                if (fp8_scale && j < n) {
                    const __nv_fp8_storage_t f8 =
                        __nv_cvt_float_to_fp8(by_inv ? v * inv : v / sc, __NV_SATFINITE, __NV_E4M3);
                    v = __half2float(__half(__nv_cvt_fp8_to_halfraw(f8, __NV_E4M3))) * sc;
                }
                h2[e] = __float2bfloat16_rn(v);
                const float r1 = v - __bfloat162float(h2[e]); // exact
                l2[e] = __float2bfloat16_rn(r1);
                m2[e] = __float2bfloat16_rn(r1 - __bfloat162float(l2[e]));
            }
            wh[q] = pack_bf16(h2[0], h2[1]);
            wl[q] = pack_bf16(l2[0], l2[1]);
            wl2[q] = pack_bf16(m2[0], m2[1]);
        }
#pragma unroll
        for (int half = 0; half < 2; ++half) {
            const uint32_t off = sw32_offset(static_cast<uint32_t>(jj), static_cast<uint32_t>(half * 8)) / 2;
            const int w0 = half * 4;
            *reinterpret_cast<uint4 *>(hi + tile * tile_elems + off) = make_uint4(wh[w0], wh[w0 + 1], wh[w0 + 2], wh[w0 + 3]);
            if (lo) {
                *reinterpret_cast<uint4 *>(lo + 2 * tile * tile_elems + off) =
                    make_uint4(wl[w0], wl[w0 + 1], wl[w0 + 2], wl[w0 + 3]);
                *reinterpret_cast<uint4 *>(lo + (2 * tile + 1) * tile_elems + off) =
                    make_uint4(wl2[w0], wl2[w0 + 1], wl2[w0 + 2], wl2[w0 + 3]);
            }
        }
    }
}

// ---- the MMA kernel ---------------------------------------------------------------------
template <int N, int S, bool SPLIT>
struct TcCfg {
    static constexpr int kABytes = kTileBytes * (SPLIT ? 3 : 1); // hi (, lo, lo2)
    static constexpr int kBBytes = N * 32 * (SPLIT ? 3 : 1);
    static constexpr int kStage = kABytes + kBBytes;
    static constexpr int kBanks = SPLIT ? 2 : 1;       // accumulators of N columns each
    static constexpr int kTmemCols = N * kBanks;       // a power of two in [32, 512]
    static constexpr int kSmem = 1024 /* barriers, tmem slot */ + S * kStage + 1024 /* alignment slack */;
    static_assert(kTmemCols >= 32 && kTmemCols <= 512 && (kTmemCols & (kTmemCols - 1)) == 0,
                  "tensor memory is allocated in powers of two of at most 512 columns");
    static_assert(kSmem <= 227 * 1024, "the ring must fit one CTA's shared memory");
};

template <int N, int S, bool SPLIT>
__global__ void __launch_bounds__(128, 1)
spdm_tc_kernel(const int32_t *__restrict__ pf, const int32_t *__restrict__ tile_cb, const uint16_t *__restrict__ a_hi,
               const uint16_t *__restrict__ a_lo, const uint16_t *__restrict__ b_hi, const uint16_t *__restrict__ b_lo,
               int64_t m, int64_t n, int64_t kb, float *__restrict__ C, uint32_t *__restrict__ status)
{
    using Cfg = TcCfg<N, S, SPLIT>;
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    // carve: [0,1024) control, then 1024-aligned stages
    unsigned char *base = reinterpret_cast<unsigned char *>(
        (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~static_cast<uintptr_t>(1023));
    uint64_t *full = reinterpret_cast<uint64_t *>(base);
    uint64_t *empty = full + S;
    uint64_t *done = empty + S;
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(done + 1);
    volatile int *abort_flag = reinterpret_cast<volatile int *>(tmem_slot + 1);
    unsigned char *stages = base + 1024;

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t panel = blockIdx.x;
    const int64_t jt = blockIdx.y;
    const int64_t t0 = pf[panel * kb];
    const int64_t t1 = pf[(panel + 1) * kb];
    const int64_t ntiles = t1 - t0;

    if (threadIdx.x == 0) {
        for (int s = 0; s < S; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        mbar_init(done, 1);
        *abort_flag = 0;
        fence_mbar_init();
    }
    if (warp == 2) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(Cfg::kTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;
    // split-BF16 keeps the leading products (ah * bh) in bank 0 and the five
    // correction products in bank 1, so each correction is rounded at its
    // own (2^-8 smaller) magnitude, not at the running total's; the epilogue
    // adds bank 1 to bank 0
    constexpr int BANKS = Cfg::kBanks;
    const int banks_used = BANKS;

    if (ntiles > 0) {
        if (warp == 0 && lane == 0) {
            // producer
            for (int64_t i = 0; i < ntiles; ++i) {
                const int s = static_cast<int>(i % S);
                if (i >= S && !mbar_wait(&empty[s], static_cast<uint32_t>(((i / S) - 1) & 1))) {
                    atomicOr(status, kStatusWaitTimeout);
                    *abort_flag = 1;
                    break;
                }
                if (*abort_flag)
                    break;
                unsigned char *st = stages + static_cast<size_t>(s) * Cfg::kStage;
                const int64_t tile = t0 + i;
                const int64_t btile = jt * kb + tile_cb[tile];
                mbar_arrive_expect_tx(&full[s], Cfg::kStage);
                bulk_g2s(st, a_hi + tile * (kTileBytes / 2), kTileBytes, &full[s]);
                bulk_g2s(st + Cfg::kABytes, b_hi + btile * (N * 16), N * 32, &full[s]);
                if (SPLIT) { // lo and lo2 of A, then of B: one contiguous copy each
                    bulk_g2s(st + kTileBytes, a_lo + tile * kTileBytes, 2 * kTileBytes, &full[s]);
                    bulk_g2s(st + Cfg::kABytes + N * 32, b_lo + btile * (N * 32), 2 * N * 32, &full[s]);
                }
            }
        } else if (warp == 1 && lane == 0) {
            // MMA issuer
            const uint32_t idesc = idesc_bf16(kPanel, N);
            int64_t i = 0;
            for (; i < ntiles; ++i) {
                const int s = static_cast<int>(i % S);
                if (!mbar_wait(&full[s], static_cast<uint32_t>((i / S) & 1))) {
                    atomicOr(status, kStatusWaitTimeout);
                    *abort_flag = 1;
                    break;
                }
                tc_fence_after();
                const uint32_t st = smem_u32(stages + static_cast<size_t>(s) * Cfg::kStage);
                const uint64_t ah = smem_desc_sw32(st);
                const uint64_t bh = smem_desc_sw32(st + Cfg::kABytes);
                tc_mma(tmem, ah, bh, idesc, i > 0 ? 1u : 0u);
                if (SPLIT) {
                    // (ah + al + al2)(bh + bl + bl2): every product above 2^-24
                    // of the leading one (al * bl2, al2 * bl, al2 * bl2 dropped),
                    // into the correction bank
                    const uint32_t dx = tmem + static_cast<uint32_t>(N);
                    const uint64_t al = smem_desc_sw32(st + kTileBytes);
                    const uint64_t al2 = smem_desc_sw32(st + 2 * kTileBytes);
                    const uint64_t bl = smem_desc_sw32(st + Cfg::kABytes + N * 32);
                    const uint64_t bl2 = smem_desc_sw32(st + Cfg::kABytes + 2 * N * 32);
                    tc_mma(dx, ah, bl, idesc, i > 0 ? 1u : 0u);
                    tc_mma(dx, al, bh, idesc, 1u);
                    tc_mma(dx, al, bl, idesc, 1u);
                    tc_mma(dx, ah, bl2, idesc, 1u);
                    tc_mma(dx, al2, bh, idesc, 1u);
                }
                tc_commit(&empty[s]); // slot reusable once these MMAs have read it
            }
            tc_commit(done); // arrives when every MMA issued above has completed
        }
        __syncwarp();
        // epilogue: all four warps (warp w owns TMEM lanes 32w..32w+31 = panel rows)
        const bool ok = mbar_wait(done, 0);
        if (!ok && lane == 0)
            atomicOr(status, kStatusWaitTimeout);
        tc_fence_after();
        const int64_t row = panel * kPanel + warp * 32 + lane;
        if (__all_sync(0xffffffffu, ok ? 1 : 0) && !*abort_flag) {
#pragma unroll 1
            for (int c = 0; c < N; c += 32) {
                float v[32];
                tmem_ld32(tmem + (static_cast<uint32_t>(warp * 32) << 16) + static_cast<uint32_t>(c), v);
                for (int bank = 1; bank < banks_used; ++bank) {
                    float w[32];
                    tmem_ld32(tmem + (static_cast<uint32_t>(warp * 32) << 16) + static_cast<uint32_t>(bank * N + c), w);
#pragma unroll
                    for (int q = 0; q < 32; ++q)
                        v[q] += w[q];
                }
                const int64_t j = jt * N + c;
                if (row < m && j < n) {
                    float *out = C + row * n + j;
                    if (j + 32 <= n) {
#pragma unroll
                        for (int q = 0; q < 32; q += 4)
                            *reinterpret_cast<float4 *>(out + q) = make_float4(v[q], v[q + 1], v[q + 2], v[q + 3]);
                    } else {
#pragma unroll
                        for (int q = 0; q < 32; ++q)
                            if (j + q < n)
                                out[q] = v[q];
                    }
                }
            }
        }
        // the producer's copies in flight must land before the CTA exits
        if (*abort_flag && threadIdx.x == 0) {
            for (int s = 0; s < S; ++s)
                mbar_wait(&full[s], 0);
        }
    } else {
        // panel without entries: C rows are zero
        const int64_t row = panel * kPanel + warp * 32 + lane;
        if (row < m)
            for (int64_t j = jt * N; j < (jt + 1) * N && j < n; ++j)
                C[row * n + j] = 0.0f;
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 2) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(Cfg::kTmemCols)
                     : "memory");
    }
}

// ---- the pair kernel (BF16, FP8-B) ----------------------------------------------------
__device__ __forceinline__ uint32_t cluster_rank()
{
    uint32_t r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}

// The shared::cluster address of `saddr` (a shared::cta address) in CTA `rank` of the cluster.
__device__ __forceinline__ uint32_t mapa_rank(uint32_t saddr, uint32_t rank)
{
    uint32_t r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(saddr), "r"(rank));
    return r;
}

__device__ __forceinline__ void cluster_sync_all()
{
    asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}

// One box of a 2-D tensor map into this CTA's shared memory, completing on an
// mbarrier in either CTA of the pair.
__device__ __forceinline__ void tma_2d_pair(uint32_t dst, const CUtensorMap *map, int32_t x, int32_t y, uint32_t mbar)
{
    asm volatile("cp.async.bulk.tensor.2d.cta_group::2.shared::cluster.global.mbarrier::complete_tx::bytes"
                 " [%0], [%1, {%2, %3}], [%4];" ::"r"(dst),
                 "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(mbar)
                 : "memory");
}

__device__ __forceinline__ void tc_mma_pair(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc)
{
    asm volatile("{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                 "tcgen05.mma.cta_group::2.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
                 "l"(a), "l"(b), "r"(idesc), "r"(acc)
                 : "memory");
}

// Arrives on the mbarrier at the same offset in both CTAs once the MMAs issued so far have completed.
__device__ __forceinline__ void tc_commit_pair(uint64_t *bar)
{
    asm volatile("tcgen05.commit.cta_group::2.mbarrier::arrive::one.shared::cluster.multicast::cluster.b64 [%0], %1;"
                 ::"r"(smem_u32(bar)), "h"(static_cast<uint16_t>(3))
                 : "memory");
}

constexpr int kPairN = 256;                // output columns per accumulator (MMA N)
constexpr int kPairMaxNT = 2;              // accumulators per CTA: all 512 tensor-memory columns
constexpr int kPairK = 8;                  // tiles per stage (4 x 4 stages: 3 % slower; 2 x 8: 12 %)
constexpr int kPairHalf = kTileBytes;      // 4 KB: a tile's 128-row half, or a B tile's 128-column half
constexpr int kPairStage = (1 + kPairMaxNT) * kPairK * kPairHalf; // [A halves][B halves, accumulator 0][... 1]
constexpr int kPairS = 2;                  // stages of 96 KB: 194 KB, so one CTA per SM
constexpr int kPairSmem = 1024 + kPairS * kPairStage + 1024;
constexpr uint64_t kPairDrainNs = 2000000; // after a wait gives up: time for copies in flight to land
static_assert(kPairSmem <= 227 * 1024 && 2 * kPairSmem > 228 * 1024,
              "one pair CTA per SM: its tensor-memory allocation never waits for another");

// One cluster of two CTAs per (256-row panel, nt * 256 output columns). CTA
// `rank` holds rows [128 rank, 128 rank + 128) of the panel: per stage its
// halves of up to kPairK of the panel's tiles and the matching 128-column
// halves of the B tiles, copied by its warp 0 with tensor-map bulk copies
// that complete on the first CTA's `full` barrier (which expects both CTAs'
// bytes). Warp 1 of the first CTA issues, per tile and accumulator, one
// tcgen05.mma.cta_group::2 (M=256, N=256, K=16) reading both CTAs' shared
// memory, and tcgen05.commit frees the slot in both CTAs. Each CTA drains
// its 128 rows of the accumulators from its own tensor memory.
__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(128, 1)
spdm_tc_pair_kernel(const __grid_constant__ CUtensorMap tm_a, const __grid_constant__ CUtensorMap tm_b,
                    const int32_t *__restrict__ pf, const int32_t *__restrict__ tile_cb, int64_t m, int64_t n,
                    int64_t kb, int nt_cta, float *__restrict__ C, uint32_t *__restrict__ status)
{
    constexpr int N = kPairN, S = kPairS;
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    // the same carve in both CTAs: the MMA reads the second CTA's operands at the first's offsets
    unsigned char *base = reinterpret_cast<unsigned char *>(
        (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~static_cast<uintptr_t>(1023));
    uint64_t *full = reinterpret_cast<uint64_t *>(base);
    uint64_t *empty = full + S;
    uint64_t *done = empty + S;
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(done + 1);
    unsigned char *stages = base + 1024;

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t rank = cluster_rank();
    const int64_t panel = blockIdx.x >> 1;
    const int64_t jt = blockIdx.y; // nt_cta accumulators of 256 columns
    const int64_t t0 = pf[panel * kb];
    const int64_t ntiles = pf[(panel + 1) * kb] - t0;
    const int64_t nstages = (ntiles + kPairK - 1) / kPairK;
    const int64_t ntn = (n + N - 1) / N;
    const int nt = static_cast<int>(ntn - jt * nt_cta < nt_cta ? ntn - jt * nt_cta : nt_cta);
    bool gave_up = false;

    if (threadIdx.x == 0) {
        for (int s = 0; s < S; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        mbar_init(done, 1);
        fence_mbar_init();
    }
    if (warp == 2) {
        asm volatile("tcgen05.alloc.cta_group::2.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(kPairMaxNT * N)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::2.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    cluster_sync_all(); // both CTAs' barriers initialised and tensor memory allocated
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    if (ntiles > 0) {
        if (warp == 0 && lane == 0) {
            // producer (both CTAs)
            for (int64_t i = 0; i < nstages; ++i) {
                const int s = static_cast<int>(i % S);
                if (i >= S && !mbar_wait(&empty[s], static_cast<uint32_t>(((i / S) - 1) & 1))) {
                    atomicOr(status, kStatusWaitTimeout);
                    gave_up = true;
                    break;
                }
                const int64_t q0 = i * kPairK;
                const int nq = ntiles - q0 < kPairK ? static_cast<int>(ntiles - q0) : kPairK;
                if (rank == 0) // both CTAs' bytes
                    mbar_arrive_expect_tx(&full[s], static_cast<uint32_t>(2 * (1 + nt) * nq * kPairHalf));
                const uint32_t st = smem_u32(stages + static_cast<size_t>(s) * kPairStage);
                const uint32_t leader_full = mapa_rank(smem_u32(&full[s]), 0);
                for (int q = 0; q < nq; ++q) {
                    const int64_t tile = t0 + q0 + q;
                    const int64_t cb = tile_cb[tile];
                    // maps in rows of 512 B: a tile is 16 rows, a half 8
                    tma_2d_pair(st + q * kPairHalf, &tm_a, 0, static_cast<int32_t>(tile * 16 + rank * 8), leader_full);
                    for (int t = 0; t < nt; ++t)
                        tma_2d_pair(st + ((1 + t) * kPairK + q) * kPairHalf, &tm_b, 0,
                                    static_cast<int32_t>(((jt * nt_cta + t) * kb + cb) * 16 + rank * 8), leader_full);
                }
            }
        } else if (warp == 1 && lane == 0 && rank == 0) {
            // MMA issuer (first CTA only)
            const uint32_t idesc = idesc_bf16(2 * kPanel, N);
            for (int64_t i = 0; i < nstages; ++i) {
                const int s = static_cast<int>(i % S);
                if (!mbar_wait(&full[s], static_cast<uint32_t>((i / S) & 1))) {
                    atomicOr(status, kStatusWaitTimeout);
                    gave_up = true;
                    break;
                }
                tc_fence_after();
                const uint32_t st = smem_u32(stages + static_cast<size_t>(s) * kPairStage);
                const int64_t q0 = i * kPairK;
                const int nq = ntiles - q0 < kPairK ? static_cast<int>(ntiles - q0) : kPairK;
                for (int q = 0; q < nq; ++q)
                    for (int t = 0; t < nt; ++t)
                        tc_mma_pair(tmem + static_cast<uint32_t>(t * N), smem_desc_sw32(st + q * kPairHalf),
                                    smem_desc_sw32(st + ((1 + t) * kPairK + q) * kPairHalf), idesc,
                                    (i > 0 || q > 0) ? 1u : 0u);
                tc_commit_pair(&empty[s]); // the slot is free in both CTAs once these MMAs have read it
            }
            tc_commit_pair(done); // arrives in both CTAs when every MMA issued above has completed
        }
        __syncwarp();
        const bool ok = mbar_wait(done, 0);
        if (!ok && lane == 0)
            atomicOr(status, kStatusWaitTimeout);
        tc_fence_after();
        const int64_t row = panel * (2 * kPanel) + rank * kPanel + warp * 32 + lane;
        if (__all_sync(0xffffffffu, ok ? 1 : 0)) {
#pragma unroll 1
            for (int c = 0; c < nt * N; c += 32) {
                float v[32];
                tmem_ld32(tmem + (static_cast<uint32_t>(warp * 32) << 16) + static_cast<uint32_t>(c), v);
                const int64_t j = jt * nt_cta * N + c;
                if (row < m && j < n) {
                    float *out = C + row * n + j;
                    if (j + 32 <= n) {
#pragma unroll
                        for (int q = 0; q < 32; q += 4)
                            *reinterpret_cast<float4 *>(out + q) = make_float4(v[q], v[q + 1], v[q + 2], v[q + 3]);
                    } else {
#pragma unroll
                        for (int q = 0; q < 32; ++q)
                            if (j + q < n)
                                out[q] = v[q];
                    }
                }
            }
        }
    } else {
        // panel without entries: its C rows are zero
        const int64_t row = panel * (2 * kPanel) + rank * kPanel + warp * 32 + lane;
        if (row < m)
            for (int64_t j = jt * nt_cta * N; j < (jt + 1) * nt_cta * N && j < n; ++j)
                C[row * n + j] = 0.0f;
    }
    // after a wait gave up (in either CTA: the status word), copies already
    // issued may still be landing in this CTA or signalling the first CTA's
    // barriers: give them a bounded time before the pair leaves
    if (threadIdx.x == 0 && (gave_up || (*reinterpret_cast<volatile uint32_t *>(status) & kStatusWaitTimeout))) {
        const uint64_t t_end = global_ns() + kPairDrainNs;
        while (global_ns() < t_end)
            __nanosleep(10000);
    }
    tc_fence_before();
    cluster_sync_all(); // neither CTA leaves while the pair's MMAs or copies may touch it
    if (warp == 2) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::2.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kPairMaxNT * N)
                     : "memory");
    }
}

// Columns of a B tile: 256 for the pair kernel, 128 for split-BF16, whose
// two accumulator banks stay within half of the 512 tensor-memory columns so
// that two of its CTAs (~98 KB rings) share an SM. (Four banks in all 512
// columns, one CTA per SM with a 12-stage ring, measured 1.8x slower.)
int tile_n_for(bool split) { return split ? 128 : kPairN; }

// cuTensorMapEncodeTiled through the runtime's driver entry-point query (no
// driver library linked).
typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                   const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
EncodeTiledFn encode_tiled_fn()
{
    static EncodeTiledFn fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        cudaDriverEntryPointQueryResult q;
        void *f = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiledFn>(f);
    });
    return fn;
}

// A buffer of swizzled tiles as a 2-D map of 512-byte rows (256 bf16),
// boxes of 8 rows: one box is one contiguous 4 KB half. The bytes are
// already in the MMA's shared-memory layout, so the copy is unswizzled.
// `halves` counts the buffer's 4 KB halves.
bool encode_halves_map(CUtensorMap *map, const void *base, uint64_t halves)
{
    EncodeTiledFn fn = encode_tiled_fn();
    if (!fn || halves == 0)
        return false;
    const cuuint64_t dims[2] = {256, halves * 8};
    const cuuint64_t strides[1] = {512};
    const cuuint32_t box[2] = {256, 8};
    const cuuint32_t elem_strides[2] = {1, 1};
    return fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void *>(base), dims, strides, box, elem_strides,
              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// Accumulators per CTA: two (each A half then feeds two MMAs) unless one per
// CTA still leaves the grid within one wave of one CTA per SM.
int pair_accumulators(int64_t panels, int64_t ntn)
{
    const int64_t pairs = static_cast<int64_t>(device_sms()) / 2;
    return panels * ntn <= pairs ? 1 : kPairMaxNT;
}

cudaError_t launch_pair(TcPlan &p, int64_t m, int64_t n, float *C, uint32_t *status, cudaStream_t st)
{
    const int64_t ntn = (n + kPairN - 1) / kPairN;
    const uint64_t a_halves = static_cast<uint64_t>(p.tiles) * 2, b_halves = static_cast<uint64_t>(ntn * p.kb) * 2;
    if (p.map_a_base != p.a_hi.ptr || p.map_a_rows != a_halves) {
        if (!encode_halves_map(&p.map_a, p.a_hi.ptr, a_halves))
            return cudaErrorInvalidValue;
        p.map_a_base = p.a_hi.ptr;
        p.map_a_rows = a_halves;
    }
    if (p.map_b_base != p.b_hi.ptr || p.map_b_rows != b_halves) {
        if (!encode_halves_map(&p.map_b, p.b_hi.ptr, b_halves))
            return cudaErrorInvalidValue;
        p.map_b_base = p.b_hi.ptr;
        p.map_b_rows = b_halves;
    }
    // y coordinates of the maps are int32
    if (static_cast<int64_t>(a_halves * 8) > 0x7fffffffLL || static_cast<int64_t>(b_halves * 8) > 0x7fffffffLL)
        return cudaErrorInvalidValue;
    cudaError_t e = cudaFuncSetAttribute(spdm_tc_pair_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kPairSmem);
    if (e != cudaSuccess)
        return e;
    const int nt_cta = pair_accumulators(p.panels, ntn);
    const int64_t gy = (ntn + nt_cta - 1) / nt_cta;
    if (2 * p.panels > 0x7fffffffLL || gy > 65535)
        return cudaErrorInvalidConfiguration;
    dim3 grid(static_cast<unsigned>(2 * p.panels), static_cast<unsigned>(gy));
    spdm_tc_pair_kernel<<<grid, 128, kPairSmem, st>>>(p.map_a, p.map_b, p.pf.ptr, p.tile_cb.ptr, m, n, p.kb, nt_cta, C,
                                                      status);
    count_launches(1);
    return cudaGetLastError();
}

template <int N, int S, bool SPLIT>
cudaError_t launch_tc(const TcPlan &p, int64_t m, int64_t n, float *C, uint32_t *status, cudaStream_t st)
{
    using Cfg = TcCfg<N, S, SPLIT>;
    auto kern = spdm_tc_kernel<N, S, SPLIT>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, Cfg::kSmem);
    if (e != cudaSuccess)
        return e;
    dim3 grid(static_cast<unsigned>(p.panels), static_cast<unsigned>((n + N - 1) / N));
    kern<<<grid, 128, Cfg::kSmem, st>>>(p.pf.ptr, p.tile_cb.ptr, p.a_hi.ptr, p.a_lo.ptr, p.b_hi.ptr, p.b_lo.ptr, m, n,
                                        p.kb, C, status);
    count_launches(1);
    return cudaGetLastError();
}

} // namespace

// Builds the densified tile plan (one synchronisation to size the tiles).
gcoo_status tc_build_plan(gcoo_handle *h, bool split, cudaStream_t st)
{
    if (h->tc && h->tc->split == split && h->tc->nnz == h->nnz)
        return GCOO_SUCCESS; // the same entries: built for this form already
    destroy_tc_plan(h->tc);
    h->tc = new (std::nothrow) TcPlan();
    if (!h->tc)
        return fail(GCOO_ERROR_ALLOC, "host allocation failed");
    TcPlan &p = *h->tc;
    p.split = split;
    p.nnz = h->nnz;
    p.panel_rows = split ? kPanel : 2 * kPanel;
    p.panels = (h->m + p.panel_rows - 1) / p.panel_rows;
    p.kb = (h->k + kTileK - 1) / kTileK;
    const int64_t L = p.panels * p.kb;
    const size_t sc = scan_scratch_elems(L);
    if (!p.pf.ensure(L + 1) || !p.scratch.ensure(sc + 1))
        return fail(GCOO_ERROR_ALLOC, "device allocation of the tile plan failed");
    GCOO_CUDA(cudaMemsetAsync(p.pf.ptr, 0, sizeof(int32_t) * (L + 1), st));
    unsigned blocks = static_cast<unsigned>(std::min<int64_t>((h->m + 7) / 8, 152 * 16));
    tile_flags_kernel<<<blocks, 256, 0, st>>>(h->packed.ptr, h->row_ptr.ptr, h->m, p.kb, p.panel_rows, p.pf.ptr);
    count_launches(1);
    GCOO_LAUNCH("tile_flags_kernel");
    GCOO_CUDA(launch_row_scan(p.pf.ptr, L, 1, nullptr, nullptr, p.scratch.ptr + sc, p.scratch.ptr, nullptr, st));
    int64_t total = 0;
    GCOO_CUDA(cudaMemcpyAsync(&total, p.scratch.ptr + sc, sizeof(total), cudaMemcpyDeviceToHost, st));
    GCOO_CUDA(cudaStreamSynchronize(st));
    p.tiles = total;
    const size_t tile_elems = static_cast<size_t>(p.panel_rows / kPanel) * (kTileBytes / 2);
    if (!p.tile_cb.ensure(total + 1) || !p.a_hi.ensure(total * tile_elems + 1) ||
        (split && !p.a_lo.ensure(2 * total * tile_elems + 1)))
        return fail(GCOO_ERROR_ALLOC, "device allocation of the dense tiles failed");
    if (total > 0) {
        tile_list_kernel<<<static_cast<unsigned>(std::min<int64_t>((L + 255) / 256, 4096)), 256, 0, st>>>(p.pf.ptr, L,
                                                                                                          p.kb, p.tile_cb.ptr);
        GCOO_CUDA(cudaMemsetAsync(p.a_hi.ptr, 0, total * tile_elems * 2, st));
        if (split)
            GCOO_CUDA(cudaMemsetAsync(p.a_lo.ptr, 0, 2 * total * kTileBytes, st));
        tile_fill_kernel<<<blocks, 256, 0, st>>>(h->packed.ptr, h->row_ptr.ptr, h->m, p.kb, p.panel_rows, p.pf.ptr,
                                                 reinterpret_cast<__nv_bfloat16 *>(p.a_hi.ptr),
                                                 split ? reinterpret_cast<__nv_bfloat16 *>(p.a_lo.ptr) : nullptr);
        count_launches(2);
        GCOO_LAUNCH("tile plan kernels");
    }
    return GCOO_SUCCESS;
}

// Density of the stored tiles (entries / tile slots); 0 before a plan exists.
double tc_density(const gcoo_handle *h)
{
    if (!h->tc || h->tc->tiles == 0)
        return 0.0;
    return static_cast<double>(h->nnz) / (static_cast<double>(h->tc->tiles) * h->tc->panel_rows * kTileK);
}

gcoo_status tc_prepare_b(gcoo_handle *h, int64_t n, bool fp8)
{
    TcPlan &p = *h->tc;
    const int N = tile_n_for(p.split);
    const int64_t nt = (n + N - 1) / N;
    const size_t elems = static_cast<size_t>(nt) * p.kb * N * kTileK;
    if (!p.b_hi.ensure(elems) || (p.split && !p.b_lo.ensure(2 * elems)) ||
        (fp8 && (!p.b_scale.ensure(static_cast<size_t>(n)) || !p.b_amax.ensure(static_cast<size_t>(n)))))
        return fail(GCOO_ERROR_ALLOC, "device allocation of the B tiles failed");
    p.b_n = n;
    return GCOO_SUCCESS;
}

gcoo_status tc_spdm(gcoo_handle *h, const float *dB, int64_t n, float *dC, bool fp8, cudaStream_t st)
{
    TcPlan &p = *h->tc;
    const int N = tile_n_for(p.split);
    if (fp8)
        GCOO_CUDA(launch_fp8_scales(dB, h->k, n, p.b_amax.ptr, p.b_scale.ptr, st));
    dim3 g(static_cast<unsigned>(p.kb), static_cast<unsigned>((n + N - 1) / N));
    b_tiles_kernel<<<g, 256, 0, st>>>(dB, h->k, n, N, p.kb, reinterpret_cast<__nv_bfloat16 *>(p.b_hi.ptr),
                                      p.split ? reinterpret_cast<__nv_bfloat16 *>(p.b_lo.ptr) : nullptr,
                                      fp8 ? p.b_scale.ptr : nullptr);
    count_launches(1);
    GCOO_LAUNCH("b_tiles_kernel");
    if (p.split) {
        const cudaError_t e = launch_tc<128, 4, true>(p, h->m, n, dC, h->status.ptr, st);
        if (e != cudaSuccess)
            return cuda_fail(e, "spdm_tc_kernel launch");
        return GCOO_SUCCESS;
    }
    const cudaError_t e = launch_pair(p, h->m, n, dC, h->status.ptr, st);
    if (e != cudaSuccess)
        return cuda_fail(e, "spdm_tc_pair_kernel launch (or its tensor maps)");
    return GCOO_SUCCESS;
}

} // namespace gcoo
