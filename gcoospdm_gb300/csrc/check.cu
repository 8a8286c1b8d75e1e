// check.cu -- gcoo_check_arrays: structural validation of a built handle's
// arrays on the GPU, the library's stand-in for sanitizer runs (which this
// build cannot rely on): every invariant the multiply kernels assume is
// checked, and a violation is reported through the status word instead of
// being discovered as a wrong product or a bad address.
//
// Per group (one warp each): group_index / nnz_per_group consistent; entries
// in the reference's order (column, then row), rows inside the group, columns
// in [0, k), values nonzero (the `v != 0` test: NaN passes, -0.0 does not);
// row pointers consistent with the group bounds; each row's packed entries in
// strictly ascending column order; and the packed entries the same multiset
// as the GCOO entries (order-independent hash of (row, col, value bits)).
// Every index read from the arrays is clamped to the arrays' bounds before it
// is used, so a corrupted handle is reported, never dereferenced out of
// bounds.
#include "handle.hpp"

namespace gcoo {
namespace {

__device__ __forceinline__ unsigned long long mix(uint32_t row, uint32_t col, uint32_t bits)
{
    unsigned long long x = (static_cast<unsigned long long>(row) << 32) ^ col;
    x ^= static_cast<unsigned long long>(bits) * 0x9E3779B97F4A7C15ull;
    x ^= x >> 31;
    x *= 0xBF58476D1CE4E5B9ull;
    x ^= x >> 29;
    return x;
}

__device__ __forceinline__ int64_t clamp64(int64_t v, int64_t lo, int64_t hi) { return v < lo ? lo : (v > hi ? hi : v); }

__global__ void check_kernel(const int32_t *__restrict__ gi, const int32_t *__restrict__ npg,
                             const int32_t *__restrict__ rp, const float *__restrict__ vals,
                             const int32_t *__restrict__ rows, const int32_t *__restrict__ cols,
                             const Entry *__restrict__ packed, int64_t m, int64_t k, int32_t cpg, int64_t ng,
                             int64_t nnz, uint32_t *__restrict__ status, unsigned long long *__restrict__ bad_groups)
{
    const int lane = threadIdx.x & 31;
    const int64_t w0 = (static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = (static_cast<int64_t>(gridDim.x) * blockDim.x) >> 5;
    if (w0 == 0 && lane == 0) {
        const bool ends = gi[0] == 0 && gi[ng] == nnz && npg[ng] == 0 && rp[0] == 0 && rp[m] == nnz;
        if (!ends) {
            atomicOr(status, kStatusIndex);
            atomicAdd(bad_groups, 1ull);
        }
    }
    for (int64_t g = w0; g < ng; g += nw) {
        bool bad = false;
        const int64_t g0 = gi[g], g1 = gi[g + 1];
        bad |= g0 < 0 || g1 < g0 || g1 > nnz || npg[g] != g1 - g0;
        const int64_t e0 = clamp64(g0, 0, nnz), e1 = clamp64(g1, e0, nnz);
        const int64_t r0 = g * cpg, r1 = r0 + cpg < m ? r0 + cpg : m;
        bad |= rp[r0] != g0 || rp[r1] != g1;
        unsigned long long h_gcoo = 0, h_packed = 0;
        for (int64_t e = e0 + lane; e < e1; e += 32) {
            const int32_t row = rows[e], col = cols[e];
            const float v = vals[e];
            bad |= row < r0 || row >= r1 || col < 0 || col >= k || !(v != 0.0f);
            if (e > e0) {
                const int32_t pr = rows[e - 1], pc = cols[e - 1];
                bad |= !(pc < col || (pc == col && pr < row)); // (column, row) strictly ascending
            }
            h_gcoo += mix(static_cast<uint32_t>(row), static_cast<uint32_t>(col), __float_as_uint(v));
        }
        for (int64_t r = r0; r < r1; ++r) {
            const int64_t q0 = clamp64(rp[r], 0, nnz), q1 = clamp64(rp[r + 1], q0, nnz);
            bad |= rp[r] > rp[r + 1];
            for (int64_t q = q0 + lane; q < q1; q += 32) {
                const Entry en = packed[q];
                bad |= en.col < 0 || en.col >= k || !(en.val != 0.0f);
                if (q > q0)
                    bad |= !(packed[q - 1].col < en.col);
                h_packed += mix(static_cast<uint32_t>(r), static_cast<uint32_t>(en.col), __float_as_uint(en.val));
            }
        }
#pragma unroll
        for (int o = 16; o; o >>= 1) {
            h_gcoo += __shfl_xor_sync(0xffffffffu, h_gcoo, o);
            h_packed += __shfl_xor_sync(0xffffffffu, h_packed, o);
        }
        bad |= h_gcoo != h_packed;
        if (__any_sync(0xffffffffu, bad) && lane == 0) {
            atomicOr(status, kStatusIndex);
            atomicAdd(bad_groups, 1ull);
        }
    }
}

} // namespace
} // namespace gcoo

using namespace gcoo;

extern "C" gcoo_status gcoo_check_arrays(gcoo_handle *h, void *stream, int64_t *bad_groups)
{
    if (!h)
        return fail(GCOO_ERROR_INVALID_VALUE, "handle is NULL");
    if (!h->built)
        return fail(GCOO_ERROR_NOT_BUILT, "gcoo_build has not run");
    NvtxRange nvtx("gcoo_check_arrays");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    DevBuf<uint32_t> status;
    DevBuf<unsigned long long> bad;
    if (!status.ensure(1) || !bad.ensure(1))
        return fail(GCOO_ERROR_ALLOC, "device allocation failed");
    GCOO_CUDA(cudaMemsetAsync(status.ptr, 0, sizeof(uint32_t), st));
    GCOO_CUDA(cudaMemsetAsync(bad.ptr, 0, sizeof(unsigned long long), st));
    int64_t blocks = (h->ng + 7) / 8;
    blocks = blocks < 1 ? 1 : (blocks > 65535 ? 65535 : blocks);
    check_kernel<<<static_cast<unsigned>(blocks), 256, 0, st>>>(
        h->group_index(), h->nnz_per_group(), h->row_ptr.ptr, h->vals.ptr, h->rc.ptr, h->rc.ptr + h->nnz,
        h->packed.ptr, h->m, h->k, h->p.rows_per_group, h->ng, h->nnz, status.ptr, bad.ptr);
    count_launches(1);
    GCOO_LAUNCH("check_kernel");
    unsigned long long nbad = 0;
    GCOO_CUDA(cudaMemcpyAsync(&nbad, bad.ptr, sizeof(nbad), cudaMemcpyDeviceToHost, st));
    GCOO_CUDA(cudaStreamSynchronize(st));
    if (bad_groups)
        *bad_groups = static_cast<int64_t>(nbad);
    if (nbad)
        return fail(GCOO_ERROR_FORMAT, std::to_string(nbad) + " group(s) of the GCOO arrays violate the format");
    return GCOO_SUCCESS;
}
