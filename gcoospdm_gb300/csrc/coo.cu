// coo.cu -- sparse-input ingestion: COO triplets on the device -> the
// handle's GCOO arrays, without an m x k dense buffer.
//
// The reference only reaches GCOO through a dense matrix: its Matrix Market
// reader writes every triplet into a zeroed dense buffer in file order (a
// later duplicate overwrites an earlier one; src/MatrixReader.cpp:11-84) and
// the conversion then keeps the entries with v != 0. gcoo_create_coo gives the
// same arrays as that densify-then-convert, directly from the triplets:
//   1. keys row * k + col, stably radix-sorted with the triplet index, so the
//      last triplet of a run of equal keys is the one the dense write kept;
//   2. keep that one if its value passes v != 0, compact in (row, col) order:
//      the packed execution layout, row counts -> row pointers, group arrays;
//   3. a second stable sort by (group, column, row) gives the reference's
//      GCOO order for vals / rows / cols.
// The sorts use CUB's device radix sort from the CUDA toolkit, at build time
// only; nothing on the multiply path depends on it.
#include <cub/device/device_radix_sort.cuh>

#include "handle.hpp"

namespace gcoo {

namespace {

__global__ void coo_keys_kernel(const int32_t *__restrict__ rows, const int32_t *__restrict__ cols, int64_t nnz,
                                int64_t m, int64_t k, uint64_t *__restrict__ keys, int64_t *__restrict__ idx,
                                uint32_t *__restrict__ status)
{
    for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < nnz;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const int64_t r = rows[i], c = cols[i];
        if (r < 0 || r >= m || c < 0 || c >= k) {
            atomicOr(status, kStatusIndex);
            keys[i] = static_cast<uint64_t>(m) * static_cast<uint64_t>(k); // sorts last, never kept
        } else {
            keys[i] = static_cast<uint64_t>(r) * static_cast<uint64_t>(k) + static_cast<uint64_t>(c);
        }
        idx[i] = i;
    }
}

// keep[i] = 1 for the last triplet of each key run whose value is nonzero.
__global__ void coo_keep_kernel(const uint64_t *__restrict__ keys, const int64_t *__restrict__ idx,
                                const float *__restrict__ vals, int64_t nnz, uint64_t mk, int32_t *__restrict__ keep)
{
    for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < nnz;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const bool last = (i + 1 == nnz) || keys[i + 1] != keys[i];
        keep[i] = (last && keys[i] < mk && vals[idx[i]] != 0.0f) ? 1 : 0;
    }
}

// Scatter the kept triplets (positions = exclusive prefix of keep) into the
// packed row-order layout; count entries per row.
__global__ void coo_compact_kernel(const uint64_t *__restrict__ keys, const int64_t *__restrict__ idx,
                                   const float *__restrict__ vals, const int32_t *__restrict__ keep,
                                   const int32_t *__restrict__ pos, int64_t nnz, int64_t k, Entry *__restrict__ packed,
                                   int32_t *__restrict__ row_cnt, uint64_t *__restrict__ gkeys,
                                   int64_t *__restrict__ gidx, int32_t cpg)
{
    for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < nnz;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        if (!keep[i])
            continue;
        const int64_t p = pos[i];
        const int64_t r = static_cast<int64_t>(keys[i] / static_cast<uint64_t>(k));
        const int64_t c = static_cast<int64_t>(keys[i] % static_cast<uint64_t>(k));
        Entry e;
        e.col = static_cast<int32_t>(c);
        e.val = vals[idx[i]];
        packed[p] = e;
        atomicAdd(&row_cnt[r], 1);
        // reference GCOO order: group, then column, then row inside the group
        const uint64_t g = static_cast<uint64_t>(r / cpg);
        gkeys[p] = (g * static_cast<uint64_t>(k) + static_cast<uint64_t>(c)) * static_cast<uint64_t>(cpg) +
                   static_cast<uint64_t>(r % cpg);
        gidx[p] = p;
    }
}

__global__ void coo_gcoo_kernel(const uint64_t *__restrict__ gkeys, const int64_t *__restrict__ gidx,
                                const Entry *__restrict__ packed, int64_t total, int64_t k, int32_t cpg,
                                float *__restrict__ vals, int32_t *__restrict__ rows, int32_t *__restrict__ cols)
{
    for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < total;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const uint64_t key = gkeys[i];
        const uint64_t lr = key % static_cast<uint64_t>(cpg);
        const uint64_t gc = key / static_cast<uint64_t>(cpg);
        const uint64_t g = gc / static_cast<uint64_t>(k);
        const Entry e = packed[gidx[i]];
        vals[i] = e.val;
        rows[i] = static_cast<int32_t>(g * cpg + lr);
        cols[i] = e.col;
    }
}

unsigned blocks_for(int64_t n)
{
    int64_t b = (n + 255) / 256;
    if (b > 152 * 16)
        b = 152 * 16;
    return static_cast<unsigned>(b < 1 ? 1 : b);
}

int bits_for(uint64_t maxkey)
{
    int b = 1;
    while (b < 64 && (maxkey >> b))
        ++b;
    return b;
}

} // namespace

// Ingests the handle's COO triplets into its GCOO arrays (gcoo_build of a
// handle made by gcoo_create_coo). Synchronises once to size the arrays.
gcoo_status coo_build(gcoo_handle *h, cudaStream_t st)
{
    const int64_t nnz_in = h->coo_nnz;
    const int32_t cpg = h->p.rows_per_group;
    const size_t n = static_cast<size_t>(nnz_in > 0 ? nnz_in : 1);
    DevBuf<uint64_t> keys, keys2;
    DevBuf<int64_t> idx, idx2;
    DevBuf<int32_t> keep;
    DevBuf<unsigned char> tmp1, tmp2; // sort scratch, released after the final synchronisation
    const uint64_t mk = static_cast<uint64_t>(h->m) * static_cast<uint64_t>(h->k);
    const size_t sc_n = scan_scratch_elems(static_cast<int64_t>(n));
    DevBuf<int64_t> sc;
    if (!keys.ensure(n) || !keys2.ensure(n) || !idx.ensure(n) || !idx2.ensure(n) || !keep.ensure(n + 1) ||
        !sc.ensure(sc_n + 1) || !h->row_ptr.ensure(static_cast<size_t>(h->m) + 1) ||
        !h->groups.ensure(2 * static_cast<size_t>(h->ng + 1)) || !h->scratch.ensure(scan_scratch_elems(h->m) + 2) ||
        !h->status.ensure(1))
        return fail(GCOO_ERROR_ALLOC, "device allocation for COO ingestion failed");
    GCOO_CUDA(cudaMemsetAsync(h->status.ptr, 0, sizeof(uint32_t), st));
    GCOO_CUDA(cudaMemsetAsync(h->row_ptr.ptr, 0, sizeof(int32_t) * (h->m + 1), st));
    if (nnz_in > 0) {
        coo_keys_kernel<<<blocks_for(nnz_in), 256, 0, st>>>(h->coo_rows, h->coo_cols, nnz_in, h->m, h->k, keys.ptr,
                                                             idx.ptr, h->status.ptr);
        count_launches(1);
        GCOO_LAUNCH("coo_keys_kernel");
        // stable radix sort of (key, triplet index) over the bits the keys need
        // (invalid triplets carry the key m*k)
        size_t tmp_bytes = 0;
        const int nbits = bits_for(mk);
        GCOO_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, tmp_bytes, keys.ptr, keys2.ptr, idx.ptr, idx2.ptr,
                                                  static_cast<int64_t>(nnz_in), 0, nbits, st));
        if (!tmp1.ensure(tmp_bytes))
            return fail(GCOO_ERROR_ALLOC, "device allocation of sort scratch failed");
        GCOO_CUDA(cub::DeviceRadixSort::SortPairs(tmp1.ptr, tmp_bytes, keys.ptr, keys2.ptr, idx.ptr, idx2.ptr,
                                                  static_cast<int64_t>(nnz_in), 0, nbits, st));
        coo_keep_kernel<<<blocks_for(nnz_in), 256, 0, st>>>(keys2.ptr, idx2.ptr, h->coo_vals, nnz_in, mk, keep.ptr);
        count_launches(1);
        GCOO_LAUNCH("coo_keep_kernel");
    }
    // positions of the kept triplets (in place: keep -> exclusive prefix), total at sc[sc_n]
    DevBuf<int32_t> pos;
    if (!pos.ensure(n + 1))
        return fail(GCOO_ERROR_ALLOC, "device allocation failed");
    if (nnz_in > 0) {
        GCOO_CUDA(cudaMemcpyAsync(pos.ptr, keep.ptr, sizeof(int32_t) * nnz_in, cudaMemcpyDeviceToDevice, st));
        GCOO_CUDA(launch_row_scan(pos.ptr, nnz_in, 1, nullptr, nullptr, sc.ptr + sc_n, sc.ptr, nullptr, st));
    } else {
        GCOO_CUDA(cudaMemsetAsync(sc.ptr + sc_n, 0, sizeof(int64_t), st));
    }
    int64_t total = 0;
    uint32_t status = 0;
    GCOO_CUDA(cudaMemcpyAsync(&total, sc.ptr + sc_n, sizeof(total), cudaMemcpyDeviceToHost, st));
    GCOO_CUDA(cudaMemcpyAsync(&status, h->status.ptr, sizeof(status), cudaMemcpyDeviceToHost, st));
    GCOO_CUDA(cudaStreamSynchronize(st));
    if (status & kStatusIndex)
        return fail(GCOO_ERROR_INVALID_VALUE, "a COO row or column index is out of range");
    if (total > 0x7fffffffLL)
        return fail(GCOO_ERROR_FORMAT, "nnz exceeds the int32 GCOO format");
    const size_t tot = static_cast<size_t>(total);
    DevBuf<uint64_t> gkeys, gkeys2;
    DevBuf<int64_t> gidx, gidx2;
    if (!h->vals.ensure(tot) || !h->rc.ensure(2 * tot) || !h->packed.ensure(tot + 2) || !gkeys.ensure(tot + 1) ||
        !gkeys2.ensure(tot + 1) || !gidx.ensure(tot + 1) || !gidx2.ensure(tot + 1))
        return fail(GCOO_ERROR_ALLOC, "device allocation of the GCOO arrays failed");
    if (nnz_in > 0) {
        coo_compact_kernel<<<blocks_for(nnz_in), 256, 0, st>>>(keys2.ptr, idx2.ptr, h->coo_vals, keep.ptr, pos.ptr,
                                                                nnz_in, h->k, h->packed.ptr, h->row_ptr.ptr, gkeys.ptr,
                                                                gidx.ptr, cpg);
        count_launches(1);
        GCOO_LAUNCH("coo_compact_kernel");
    }
    // row counts -> row pointers and the group arrays; longest row
    int64_t *d_total = h->scratch.ptr + scan_scratch_elems(h->m);
    GCOO_CUDA(cudaMemsetAsync(d_total + 1, 0, sizeof(int64_t), st));
    GCOO_CUDA(launch_row_scan_max(h->row_ptr.ptr, h->m, cpg, h->group_index(), h->nnz_per_group(), d_total,
                                  h->scratch.ptr, h->status.ptr, st));
    if (total > 0) {
        size_t tmp_bytes = 0;
        const uint64_t maxkey = (static_cast<uint64_t>(h->ng) * static_cast<uint64_t>(h->k)) * static_cast<uint64_t>(cpg);
        const int nbits = bits_for(maxkey);
        GCOO_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, tmp_bytes, gkeys.ptr, gkeys2.ptr, gidx.ptr, gidx2.ptr,
                                                  total, 0, nbits, st));
        if (!tmp2.ensure(tmp_bytes))
            return fail(GCOO_ERROR_ALLOC, "device allocation of sort scratch failed");
        GCOO_CUDA(cub::DeviceRadixSort::SortPairs(tmp2.ptr, tmp_bytes, gkeys.ptr, gkeys2.ptr, gidx.ptr, gidx2.ptr, total,
                                                  0, nbits, st));
        coo_gcoo_kernel<<<blocks_for(total), 256, 0, st>>>(gkeys2.ptr, gidx2.ptr, h->packed.ptr, total, h->k, cpg,
                                                            h->vals.ptr, h->rc.ptr, h->rc.ptr + tot);
        count_launches(1);
        GCOO_LAUNCH("coo_gcoo_kernel");
    }
    int64_t tot2[2] = {0, 0};
    GCOO_CUDA(cudaMemcpyAsync(tot2, d_total, sizeof(tot2), cudaMemcpyDeviceToHost, st));
    GCOO_CUDA(cudaStreamSynchronize(st)); // the temporaries above are freed on return
    h->nnz = total;
    h->max_row_nnz = tot2[1];
    return GCOO_SUCCESS;
}

} // namespace gcoo
