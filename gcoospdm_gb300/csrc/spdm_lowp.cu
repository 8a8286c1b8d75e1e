// spdm_lowp.cu -- the reduced-precision forms of the multiply on the FMA
// pipes (the tensor-core engine for block-structured matrices is in
// spdm_tc.cu). Same CTA/warp mapping as the FP32 kernel (one CTA per GCOO
// group and column tile, the group's entries staged to shared memory with
// cp.async.bulk, one warp per row), with B read in a narrower format:
//   BF16        B as bf16 (8 columns per 128-bit load), A values rounded to
//               bf16, FP32 accumulation (the mixed-precision bf16 FMA of
//               sm_100+: no widening of the B values);
//   SPLIT_BF16  B = Bh + Bl and a = ah + al as bf16 pairs; acc += ah*Bh +
//               ah*Bl + al*Bh (three products, FP32 accumulation) -- FP32-level
//               accuracy from bf16 operands;
//   FP8_B       B as FP8 E4M3 scaled per column (s_j = the smallest power of
//               two with max_c |B[c][j]| / s_j <= 448), 16 columns per 128-bit
//               load, A kept FP32; the scale is applied once to the
//               accumulated column.
// B is converted into the handle's workspace by a pre-pass kernel per call.
#include <cuda_bf16.h>
#include <cuda_fp8.h>

#include "handle.hpp"

namespace gcoo {

struct LowpWork {
    DevBuf<uint16_t> bf;     // k*n bf16
    DevBuf<uint32_t> split;  // k*n (hi | lo << 16) bf16 pairs
    DevBuf<uint8_t> f8;      // k*n e4m3
    DevBuf<float> scale;     // n column scales
    DevBuf<unsigned> amax;   // n column absmax (float bits)
};

void destroy_lowp_work(LowpWork *w) { delete w; }

namespace {

constexpr int kChunk = 2048;
constexpr int kSmemBytes = 128 + (kChunk + 2) * static_cast<int>(sizeof(Entry));

__device__ __forceinline__ float bf_lo(uint32_t w) { return __uint_as_float(w << 16); }
__device__ __forceinline__ float bf_hi(uint32_t w) { return __uint_as_float(w & 0xffff0000u); }
__device__ __forceinline__ float round_bf16(float x) { return __bfloat162float(__float2bfloat16_rn(x)); }

enum Form { kBF16 = 1, kSplit = 2, kFP8 = 3 };

// Columns per lane for each form (one 128-bit load per entry).
template <int F> struct FormTraits;
template <> struct FormTraits<kBF16> { static constexpr int V = 8; using T = uint16_t; };
template <> struct FormTraits<kSplit> { static constexpr int V = 4; using T = uint32_t; };
template <> struct FormTraits<kFP8> { static constexpr int V = 16; using T = uint8_t; };

// acc + a * b with bf16 a and b, one rounding (the mixed-precision FMA of
// sm_100+): the same result as fmaf on the widened values, since a product of
// two bf16 values is exact in FP32 -- without widening each B value first.
__device__ __forceinline__ float fma_bf16(uint16_t a, uint16_t b, float c)
{
    float d;
    asm("fma.rn.f32.bf16 %0, %1, %2, %3;" : "=f"(d) : "h"(a), "h"(b), "f"(c));
    return d;
}

template <int F>
__device__ __forceinline__ void fma_entry(float a, const uint4 &w, float (&acc)[FormTraits<F>::V])
{
    if constexpr (F == kBF16) {
        // a is already a bf16 value: its top 16 bits are exact
        const uint16_t ab = static_cast<uint16_t>(__float_as_uint(a) >> 16);
        const uint32_t x[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            acc[2 * i] = fma_bf16(ab, static_cast<uint16_t>(x[i] & 0xffffu), acc[2 * i]);
            acc[2 * i + 1] = fma_bf16(ab, static_cast<uint16_t>(x[i] >> 16), acc[2 * i + 1]);
        }
    } else if constexpr (F == kFP8) {
        const uint32_t x[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const __half2_raw h01 = __nv_cvt_fp8x2_to_halfraw2(static_cast<__nv_fp8x2_storage_t>(x[i] & 0xffffu), __NV_E4M3);
            const __half2_raw h23 = __nv_cvt_fp8x2_to_halfraw2(static_cast<__nv_fp8x2_storage_t>(x[i] >> 16), __NV_E4M3);
            const float2 f01 = __half22float2(*reinterpret_cast<const __half2 *>(&h01));
            const float2 f23 = __half22float2(*reinterpret_cast<const __half2 *>(&h23));
            acc[4 * i + 0] = fmaf(a, f01.x, acc[4 * i + 0]);
            acc[4 * i + 1] = fmaf(a, f01.y, acc[4 * i + 1]);
            acc[4 * i + 2] = fmaf(a, f23.x, acc[4 * i + 2]);
            acc[4 * i + 3] = fmaf(a, f23.y, acc[4 * i + 3]);
        }
    }
}

template <int F, int U>
__device__ __forceinline__ void row_chain_lowp(const Entry *__restrict__ s, int cnt, const typename FormTraits<F>::T *__restrict__ Bj,
                                               int64_t n, float (&acc)[FormTraits<F>::V])
{
    int i = 0;
#pragma unroll 1
    for (; i + U <= cnt; i += U) {
        Entry e[U];
        uint4 w[U];
#pragma unroll
        for (int u = 0; u < U; ++u)
            e[u] = s[i + u];
#pragma unroll
        for (int u = 0; u < U; ++u)
            w[u] = __ldg(reinterpret_cast<const uint4 *>(Bj + static_cast<int64_t>(e[u].col) * n));
#pragma unroll
        for (int u = 0; u < U; ++u) {
            if constexpr (F == kSplit) {
                const float ah = round_bf16(e[u].val);
                const float al = round_bf16(e[u].val - ah);
                const uint32_t x[4] = {w[u].x, w[u].y, w[u].z, w[u].w};
#pragma unroll
                for (int v = 0; v < 4; ++v) {
                    const float bh = bf_lo(x[v]), bl = bf_hi(x[v]);
                    acc[v] = fmaf(al, bh, fmaf(ah, bl, fmaf(ah, bh, acc[v])));
                }
            } else {
                fma_entry<F>(F == kBF16 ? round_bf16(e[u].val) : e[u].val, w[u], acc);
            }
        }
    }
#pragma unroll 1
    for (; i < cnt; ++i) {
        const Entry e = s[i];
        const uint4 w = __ldg(reinterpret_cast<const uint4 *>(Bj + static_cast<int64_t>(e.col) * n));
        if constexpr (F == kSplit) {
            const float ah = round_bf16(e.val);
            const float al = round_bf16(e.val - ah);
            const uint32_t x[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
            for (int v = 0; v < 4; ++v) {
                const float bh = bf_lo(x[v]), bl = bf_hi(x[v]);
                acc[v] = fmaf(al, bh, fmaf(ah, bl, fmaf(ah, bh, acc[v])));
            }
        } else {
            fma_entry<F>(F == kBF16 ? round_bf16(e.val) : e.val, w, acc);
        }
    }
}

// One CTA per (group, column tile); warps = rows_per_group * col_warps.
// n must be a multiple of the form's V and B/C suitably aligned (host checks).
template <int F>
__global__ void __launch_bounds__(512)
spdm_lowp_kernel(const Entry *__restrict__ packed, const int32_t *__restrict__ row_ptr, int64_t m, int32_t cpg,
                 const typename FormTraits<F>::T *__restrict__ B, const float *__restrict__ col_scale, int64_t n,
                 float *__restrict__ C, int32_t col_warps, uint32_t *__restrict__ status)
{
    constexpr int V = FormTraits<F>::V;
    extern __shared__ __align__(128) unsigned char smem[];
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem);
    Entry *s_nz = reinterpret_cast<Entry *>(smem + 128);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int slot = warp / col_warps, sub = warp - slot * col_warps;
    const int64_t r0 = static_cast<int64_t>(blockIdx.x) * cpg;
    const int64_t r_end = r0 + cpg < m ? r0 + cpg : m;
    const int64_t row = r0 + slot;
    const bool has_row = slot < cpg && row < r_end;
    const int64_t j = (static_cast<int64_t>(blockIdx.y) * col_warps + sub) * (32 * V) + static_cast<int64_t>(lane) * V;
    const bool has_col = j < n;
    const int64_t gs = row_ptr[r0], ge = row_ptr[r_end];
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
#pragma unroll
    for (int v = 0; v < V; ++v)
        acc[v] = 0.0f;
    const typename FormTraits<F>::T *Bj = B + j;
    const int64_t nchunks = (ge - gs + kChunk - 1) / kChunk;
    bool ok = true;
    for (int64_t ch = 0; ch < nchunks && ok; ++ch) {
        const int64_t cs = gs + ch * kChunk;
        const int64_t ce = cs + kChunk < ge ? cs + kChunk : ge;
        const int64_t a0 = cs & ~static_cast<int64_t>(1);
        const int64_t a1 = (ce + 1) & ~static_cast<int64_t>(1);
        if (threadIdx.x == 0) {
            fence_proxy_async();
            const uint32_t bytes = static_cast<uint32_t>((a1 - a0) * static_cast<int64_t>(sizeof(Entry)));
            mbar_arrive_expect_tx(bar, bytes);
            bulk_g2s(s_nz, packed + a0, bytes, bar);
        }
        const bool waited = mbar_wait(bar, static_cast<uint32_t>(ch & 1));
        ok = __syncthreads_and(waited) != 0;
        if (!ok) {
            if (threadIdx.x == 0)
                atomicOr(status, kStatusWaitTimeout);
            mbar_wait(bar, static_cast<uint32_t>(ch & 1));
            break;
        }
        const int64_t lo = rs > cs ? rs : cs, hi = re < ce ? re : ce;
        if (has_col && lo < hi)
            row_chain_lowp<F, 4>(s_nz + (lo - a0), static_cast<int>(hi - lo), Bj, n, acc);
        __syncthreads();
    }
    if (has_row && has_col && ok) {
        float *out = C + row * n + j;
#pragma unroll
        for (int v = 0; v < V; v += 4) {
            float4 o = make_float4(acc[v], acc[v + 1], acc[v + 2], acc[v + 3]);
            if constexpr (F == kFP8) {
                const float4 s = *reinterpret_cast<const float4 *>(col_scale + j + v);
                o.x *= s.x; o.y *= s.y; o.z *= s.z; o.w *= s.w;
            }
            *reinterpret_cast<float4 *>(out + v) = o;
        }
    }
}

// ---- B pre-pass kernels (grid-stride over k*n / 4) ----------------------------------
__global__ void prep_bf16_kernel(const float4 *__restrict__ B, uint2 *__restrict__ out, int64_t n4)
{
    for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n4;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const float4 v = __ldcs(B + i);
        const __nv_bfloat162 a = __floats2bfloat162_rn(v.x, v.y);
        const __nv_bfloat162 b = __floats2bfloat162_rn(v.z, v.w);
        out[i] = make_uint2(*reinterpret_cast<const uint32_t *>(&a), *reinterpret_cast<const uint32_t *>(&b));
    }
}

__global__ void prep_split_kernel(const float4 *__restrict__ B, uint4 *__restrict__ out, int64_t n4)
{
    for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n4;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const float4 v = __ldcs(B + i);
        const float x[4] = {v.x, v.y, v.z, v.w};
        uint32_t w[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const __nv_bfloat16 h = __float2bfloat16_rn(x[q]);
            const __nv_bfloat16 l = __float2bfloat16_rn(x[q] - __bfloat162float(h));
            w[q] = static_cast<uint32_t>(*reinterpret_cast<const uint16_t *>(&h)) |
                   (static_cast<uint32_t>(*reinterpret_cast<const uint16_t *>(&l)) << 16);
        }
        out[i] = make_uint4(w[0], w[1], w[2], w[3]);
    }
}

// Column absmax: each thread owns 4 columns and a slice of rows.
__global__ void colmax_kernel(const float *__restrict__ B, int64_t k, int64_t n, unsigned *__restrict__ amax,
                              int rows_per_cta)
{
    const int64_t j = (static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x) * 4;
    if (j >= n)
        return;
    const int64_t c0 = static_cast<int64_t>(blockIdx.y) * rows_per_cta;
    const int64_t c1 = c0 + rows_per_cta < k ? c0 + rows_per_cta : k;
    float m0 = 0.f, m1 = 0.f, m2 = 0.f, m3 = 0.f;
#pragma unroll 8
    for (int64_t c = c0; c < c1; ++c) {
        const float4 v = __ldg(reinterpret_cast<const float4 *>(B + c * n + j));
        m0 = fmaxf(m0, fabsf(v.x)); m1 = fmaxf(m1, fabsf(v.y));
        m2 = fmaxf(m2, fabsf(v.z)); m3 = fmaxf(m3, fabsf(v.w));
    }
    atomicMax(amax + j, __float_as_uint(m0));
    atomicMax(amax + j + 1, __float_as_uint(m1));
    atomicMax(amax + j + 2, __float_as_uint(m2));
    atomicMax(amax + j + 3, __float_as_uint(m3));
}

// Per-column scale: the smallest power of two s with absmax / s <= 448 (the
// largest E4M3 value). A power of two divides exactly, so both engines see
// the same E4M3 values, and the tensor engine can fold s into its BF16 tiles
// without a rounding (an E4M3 value times a power of two is a BF16 value).
__global__ void scale_kernel(const unsigned *__restrict__ amax, float *__restrict__ scale, int64_t n)
{
    const int64_t j = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (j < n) {
        const float a = __uint_as_float(amax[j]);
        float s = 1.0f;
        if (a > 0.0f && a < INFINITY) {
            int e = 0;
            const float mant = frexpf(a / 448.0f, &e); // a / 448 = mant * 2^e, mant in [0.5, 1)
            s = ldexpf(1.0f, mant == 0.5f ? e - 1 : e);
        }
        scale[j] = s;
    }
}

__global__ void prep_fp8_kernel(const float4 *__restrict__ B, const float *__restrict__ scale, uint32_t *__restrict__ out,
                                int64_t n4, int64_t n)
{
    for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n4;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const float4 v = __ldcs(B + i);
        const int64_t j = (i * 4) % n;
        const float x[4] = {v.x / scale[j], v.y / scale[j + 1], v.z / scale[j + 2], v.w / scale[j + 3]};
        uint32_t w = 0;
#pragma unroll
        for (int q = 0; q < 4; ++q)
            w |= static_cast<uint32_t>(__nv_cvt_float_to_fp8(x[q], __NV_SATFINITE, __NV_E4M3)) << (8 * q);
        out[i] = w;
    }
}

unsigned grid_for(int64_t items, int threads)
{
    int64_t b = (items + threads - 1) / threads;
    if (b > 152 * 32)
        b = 152 * 32;
    return static_cast<unsigned>(b < 1 ? 1 : b);
}

} // namespace

cudaError_t launch_fp8_scales(const float *B, int64_t k, int64_t n, unsigned *amax, float *scale, cudaStream_t st)
{
    cudaError_t e = cudaMemsetAsync(amax, 0, sizeof(unsigned) * static_cast<size_t>(n), st);
    if (e != cudaSuccess)
        return e;
    // 32 rows per CTA: k / 32 CTAs per column strip, enough loads in flight
    // to stream B (256 rows per CTA left the pass latency-bound: 64 CTAs at
    // B 8192 x 1024)
    const int rows_per_cta = 32;
    dim3 g(static_cast<unsigned>((n / 4 + 127) / 128), static_cast<unsigned>((k + rows_per_cta - 1) / rows_per_cta));
    colmax_kernel<<<g, 128, 0, st>>>(B, k, n, amax, rows_per_cta);
    scale_kernel<<<static_cast<unsigned>((n + 255) / 256), 256, 0, st>>>(amax, scale, n);
    count_launches(2);
    return cudaGetLastError();
}

// Width constraint of each form on the FMA engine.
int lowp_vec(gcoo_precision prec) { return prec == GCOO_PREC_BF16 ? 8 : prec == GCOO_PREC_SPLIT_BF16 ? 4 : 16; }

gcoo_status lowp_prepare(gcoo_handle *h, int64_t n, gcoo_precision prec)
{
    if (!h->lowp)
        h->lowp = new (std::nothrow) LowpWork();
    if (!h->lowp)
        return fail(GCOO_ERROR_ALLOC, "host allocation failed");
    const size_t kn = static_cast<size_t>(h->k) * static_cast<size_t>(n);
    bool ok = true;
    if (prec == GCOO_PREC_BF16)
        ok = h->lowp->bf.ensure(kn);
    else if (prec == GCOO_PREC_SPLIT_BF16)
        ok = h->lowp->split.ensure(kn);
    else
        ok = h->lowp->f8.ensure(kn) && h->lowp->scale.ensure(n) && h->lowp->amax.ensure(n);
    return ok ? GCOO_SUCCESS : fail(GCOO_ERROR_ALLOC, "device allocation of the form workspace failed");
}

// Converts B into the form's workspace (also used by the tensor engine for FP8 scales).
gcoo_status lowp_convert_b(gcoo_handle *h, const float *dB, int64_t n, gcoo_precision prec, cudaStream_t st)
{
    const int64_t n4 = h->k * n / 4;
    LowpWork *w = h->lowp;
    if (prec == GCOO_PREC_BF16) {
        prep_bf16_kernel<<<grid_for(n4, 256), 256, 0, st>>>(reinterpret_cast<const float4 *>(dB),
                                                            reinterpret_cast<uint2 *>(w->bf.ptr), n4);
        count_launches(1);
    } else if (prec == GCOO_PREC_SPLIT_BF16) {
        prep_split_kernel<<<grid_for(n4, 256), 256, 0, st>>>(reinterpret_cast<const float4 *>(dB),
                                                             reinterpret_cast<uint4 *>(w->split.ptr), n4);
        count_launches(1);
    } else {
        GCOO_CUDA(launch_fp8_scales(dB, h->k, n, w->amax.ptr, w->scale.ptr, st));
        prep_fp8_kernel<<<grid_for(n4, 256), 256, 0, st>>>(reinterpret_cast<const float4 *>(dB), w->scale.ptr,
                                                           reinterpret_cast<uint32_t *>(w->f8.ptr), n4, n);
        count_launches(1);
    }
    GCOO_LAUNCH("B conversion kernel");
    return GCOO_SUCCESS;
}

gcoo_status lowp_spdm(gcoo_handle *h, int64_t n, float *dC, gcoo_precision prec, cudaStream_t st)
{
    const int V = lowp_vec(prec);
    const int cpg = h->p.rows_per_group;
    int cw = 8 / cpg;
    if (cw < 1)
        cw = 1;
    while (cw > 1 && static_cast<int64_t>(cw / 2) * 32 * V >= n)
        cw /= 2;
    if (cw * cpg > 16)
        cw = 16 / cpg > 0 ? 16 / cpg : 1;
    if (cpg > 16)
        return fail(GCOO_ERROR_UNSUPPORTED, "reduced-precision forms on the FMA engine support rows_per_group <= 16");
    LowpWork *w = h->lowp;
    if (prec != GCOO_PREC_SPLIT_BF16 && n % 8 == 0 && group_order_chosen(h)) {
        // rows of a group share columns: decode each B segment once per group
        cudaError_t e = launch_spdm_lowp_group(
            h->vals.ptr, h->rc.ptr, h->rc.ptr + h->nnz, h->group_index(), h->m, h->ng,
            prec == GCOO_PREC_BF16 ? static_cast<const void *>(w->bf.ptr) : static_cast<const void *>(w->f8.ptr),
            w->scale.ptr, n, dC, prec, st);
        if (e != cudaSuccess)
            return cuda_fail(e, "spdm_group_kernel launch (reduced precision)");
        return GCOO_SUCCESS;
    }
    const int64_t tile = static_cast<int64_t>(cw) * 32 * V;
    const int64_t ny = (n + tile - 1) / tile;
    dim3 grid(static_cast<unsigned>(h->ng), static_cast<unsigned>(ny));
    const int threads = cw * cpg * 32;
    if (prec == GCOO_PREC_BF16)
        spdm_lowp_kernel<kBF16><<<grid, threads, kSmemBytes, st>>>(h->packed.ptr, h->row_ptr.ptr, h->m, cpg, w->bf.ptr,
                                                                  nullptr, n, dC, cw, h->status.ptr);
    else if (prec == GCOO_PREC_SPLIT_BF16)
        spdm_lowp_kernel<kSplit><<<grid, threads, kSmemBytes, st>>>(h->packed.ptr, h->row_ptr.ptr, h->m, cpg,
                                                                   w->split.ptr, nullptr, n, dC, cw, h->status.ptr);
    else
        spdm_lowp_kernel<kFP8><<<grid, threads, kSmemBytes, st>>>(h->packed.ptr, h->row_ptr.ptr, h->m, cpg, w->f8.ptr,
                                                                 w->scale.ptr, n, dC, cw, h->status.ptr);
    count_launches(1);
    GCOO_LAUNCH("spdm_lowp_kernel");
    return GCOO_SUCCESS;
}

} // namespace gcoo
