// left.cu -- the other orientation, C = D x A (D dense p x m, A the handle's
// sparse m x k, C p x k, row-major): the plugin's mutiply(), which the
// reference's GCOO plugin leaves empty (src/ShGCOOSpDM.h:21; the interface
// is src/ShGemm.h:16).
//
// C^T = A^T x D^T, so it runs on the FP32 row kernel with A^T in the packed
// row layout (A's entries ordered by column, then row: built once per handle
// with a stable radix sort and kept), D^T as the dense operand and C^T as the
// output, with tiled shared-memory transposes on either side. Each C element
// is a sequential fmaf chain over A's rows in ascending order.
#include <cub/device/device_radix_sort.cuh>

#include "handle.hpp"

namespace gcoo {

struct LeftPlan {
    int64_t nnz = -1;
    int64_t max_col = 0;
    DevBuf<int32_t> col_ptr;   // k + 1
    DevBuf<Entry> packed_t;    // {row, value}, column order, nnz + 2
    DevBuf<float> dt, ct;      // D^T (m x p), C^T (k x p)
    int64_t p_cap = 0;
};

void destroy_left_plan(LeftPlan *p) { delete p; }

namespace {

__global__ void left_keys_kernel(const Entry *__restrict__ packed, const int32_t *__restrict__ row_ptr, int64_t m,
                                 uint64_t *__restrict__ keys, float *__restrict__ vals)
{
    const int lane = threadIdx.x & 31;
    const int64_t warp = (static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = (static_cast<int64_t>(gridDim.x) * blockDim.x) >> 5;
    for (int64_t r = warp; r < m; r += nw)
        for (int64_t e = row_ptr[r] + lane; e < row_ptr[r + 1]; e += 32) {
            const Entry t = packed[e];
            keys[e] = static_cast<uint64_t>(t.col) * static_cast<uint64_t>(m) + static_cast<uint64_t>(r);
            vals[e] = t.val;
        }
}

__global__ void left_fill_kernel(const uint64_t *__restrict__ keys, const float *__restrict__ vals, int64_t nnz,
                                 int64_t m, Entry *__restrict__ packed_t, int32_t *__restrict__ col_cnt)
{
    for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < nnz;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        Entry e;
        e.col = static_cast<int32_t>(keys[i] % static_cast<uint64_t>(m)); // the row of A
        e.val = vals[i];
        packed_t[i] = e;
        atomicAdd(&col_cnt[keys[i] / static_cast<uint64_t>(m)], 1);
    }
}

// out[c][r] = in[r][c] for an R x Cc row-major input.
__global__ void transpose_kernel(const float *__restrict__ in, float *__restrict__ out, int64_t R, int64_t Cc)
{
    __shared__ float tile[32][33];
    const int64_t c0 = static_cast<int64_t>(blockIdx.x) * 32, r0 = static_cast<int64_t>(blockIdx.y) * 32;
    for (int i = threadIdx.y; i < 32; i += blockDim.y) {
        const int64_t r = r0 + i, c = c0 + threadIdx.x;
        if (r < R && c < Cc)
            tile[i][threadIdx.x] = in[r * Cc + c];
    }
    __syncthreads();
    for (int i = threadIdx.y; i < 32; i += blockDim.y) {
        const int64_t c = c0 + i, r = r0 + threadIdx.x;
        if (r < R && c < Cc)
            out[c * R + r] = tile[threadIdx.x][i];
    }
}

cudaError_t transpose(const float *in, float *out, int64_t R, int64_t Cc, cudaStream_t st)
{
    const int64_t gx = (Cc + 31) / 32, gy = (R + 31) / 32;
    if (gy > 65535)
        return cudaErrorInvalidConfiguration;
    transpose_kernel<<<dim3(static_cast<unsigned>(gx), static_cast<unsigned>(gy)), dim3(32, 8), 0, st>>>(in, out, R, Cc);
    count_launches(1);
    return cudaGetLastError();
}

int bits_for_left(uint64_t maxkey)
{
    int b = 1;
    while (b < 64 && (maxkey >> b))
        ++b;
    return b;
}

} // namespace

gcoo_status left_prepare(gcoo_handle *h, LeftPlan *&plan, int64_t p, cudaStream_t st)
{
    if (!plan)
        plan = new (std::nothrow) LeftPlan();
    if (!plan)
        return fail(GCOO_ERROR_ALLOC, "host allocation failed");
    LeftPlan &L = *plan;
    if (L.nnz != h->nnz) {
        const size_t nnz = static_cast<size_t>(h->nnz);
        DevBuf<uint64_t> keys, keys2;
        DevBuf<float> vals, vals2;
        DevBuf<unsigned char> tmp;
        DevBuf<int64_t> sc;
        const size_t scn = scan_scratch_elems(h->k);
        if (!keys.ensure(nnz + 1) || !keys2.ensure(nnz + 1) || !vals.ensure(nnz + 1) || !vals2.ensure(nnz + 1) ||
            !L.col_ptr.ensure(static_cast<size_t>(h->k) + 1) || !L.packed_t.ensure(nnz + 2) || !sc.ensure(scn + 2))
            return fail(GCOO_ERROR_ALLOC, "device allocation of the column layout failed");
        GCOO_CUDA(cudaMemsetAsync(L.col_ptr.ptr, 0, sizeof(int32_t) * (h->k + 1), st));
        if (nnz > 0) {
            unsigned blocks = static_cast<unsigned>(std::min<int64_t>((h->m + 7) / 8, 152 * 16));
            left_keys_kernel<<<blocks, 256, 0, st>>>(h->packed.ptr, h->row_ptr.ptr, h->m, keys.ptr, vals.ptr);
            count_launches(1);
            GCOO_LAUNCH("left_keys_kernel");
            const int nbits = bits_for_left(static_cast<uint64_t>(h->k) * static_cast<uint64_t>(h->m));
            size_t tmp_bytes = 0;
            GCOO_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, tmp_bytes, keys.ptr, keys2.ptr, vals.ptr, vals2.ptr,
                                                      static_cast<int64_t>(nnz), 0, nbits, st));
            if (!tmp.ensure(tmp_bytes))
                return fail(GCOO_ERROR_ALLOC, "device allocation of sort scratch failed");
            GCOO_CUDA(cub::DeviceRadixSort::SortPairs(tmp.ptr, tmp_bytes, keys.ptr, keys2.ptr, vals.ptr, vals2.ptr,
                                                      static_cast<int64_t>(nnz), 0, nbits, st));
            const int64_t nb = (static_cast<int64_t>(nnz) + 255) / 256;
            left_fill_kernel<<<static_cast<unsigned>(std::min<int64_t>(nb, 152 * 16)), 256, 0, st>>>(
                keys2.ptr, vals2.ptr, static_cast<int64_t>(nnz), h->m, L.packed_t.ptr, L.col_ptr.ptr);
            count_launches(1);
            GCOO_LAUNCH("left_fill_kernel");
        }
        int64_t *d_tot = sc.ptr + scn;
        GCOO_CUDA(cudaMemsetAsync(d_tot + 1, 0, sizeof(int64_t), st));
        GCOO_CUDA(launch_row_scan_max(L.col_ptr.ptr, h->k, 1, nullptr, nullptr, d_tot, sc.ptr, nullptr, st));
        int64_t t2[2] = {0, 0};
        GCOO_CUDA(cudaMemcpyAsync(t2, d_tot, sizeof(t2), cudaMemcpyDeviceToHost, st));
        GCOO_CUDA(cudaStreamSynchronize(st)); // temporaries are released on return
        L.max_col = t2[1];
        L.nnz = h->nnz;
    }
    if (p > L.p_cap) {
        if (!L.dt.ensure(static_cast<size_t>(h->m) * p) || !L.ct.ensure(static_cast<size_t>(h->k) * p))
            return fail(GCOO_ERROR_ALLOC, "device allocation of the transposed operands failed");
        L.p_cap = p;
    }
    return GCOO_SUCCESS;
}

gcoo_status left_spdm(gcoo_handle *h, const LeftPlan &L, const float *dD, int64_t p, float *dC, cudaStream_t st)
{
    GCOO_CUDA(transpose(dD, L.dt.ptr, p, h->m, st)); // D (p x m) -> D^T (m x p)
    gcoo_params prm = h->p;
    const LaunchShape s = pick_shape(prm, h->k, p, h->nnz, L.max_col, reinterpret_cast<uintptr_t>(L.dt.ptr),
                                     reinterpret_cast<uintptr_t>(L.ct.ptr));
    GCOO_CUDA(launch_spdm_fp32(L.packed_t.ptr, L.col_ptr.ptr, h->k, L.dt.ptr, p, L.ct.ptr, s, h->status.ptr, st));
    GCOO_CUDA(transpose(L.ct.ptr, dC, h->k, p, st)); // C^T (k x p) -> C (p x k)
    return GCOO_SUCCESS;
}

} // namespace gcoo
