// internal.cuh -- shared definitions of the GB300 GCOO library (not installed).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "gcoo.h"

namespace gcoo {

// ---- status word bits written by kernels -------------------------------------
enum : uint32_t {
    kStatusWaitTimeout = 1u << 1, // a bounded mbarrier / flag wait gave up
    kStatusIndex = 1u << 2,       // an index check failed (entry skipped)
    kStatusOverflow = 1u << 3     // a count did not fit the int32 format
};

// Bounds of one mbarrier wait before a kernel gives up and reports
// kStatusWaitTimeout: a wall-clock limit read from %globaltimer, and a poll
// count (each try_wait suspends the thread for a hardware-chosen interval).
constexpr uint64_t kWaitNs = 2000000000ull; // 2 s: no legitimate copy or MMA takes this long
constexpr uint32_t kWaitLimit = 1u << 26;

// ---- error reporting -------------------------------------------------------------
void set_error(const std::string &msg);
gcoo_status fail(gcoo_status s, const std::string &msg);
gcoo_status cuda_fail(cudaError_t e, const char *what);

#define GCOO_CUDA(call)                                                     \
    do {                                                                    \
        cudaError_t e_ = (call);                                            \
        if (e_ != cudaSuccess)                                              \
            return ::gcoo::cuda_fail(e_, #call);                            \
    } while (0)

#define GCOO_LAUNCH(what)                                                   \
    do {                                                                    \
        cudaError_t e_ = cudaGetLastError();                                \
        if (e_ != cudaSuccess)                                              \
            return ::gcoo::cuda_fail(e_, what);                             \
    } while (0)

// Adds n to the process-wide launch counter (gcoo_kernel_launches).
void count_launches(int n);

// NVTX range over a scope (entry points and the session's phases): visible in
// profilers that attach an NVTX tool, a no-op otherwise (NVTX3 is header-only).
struct NvtxRange {
    explicit NvtxRange(const char *name);
    ~NvtxRange();
    NvtxRange(const NvtxRange &) = delete;
    NvtxRange &operator=(const NvtxRange &) = delete;
};

// ---- device allocation through the pluggable allocator -----------------------------
void *dev_alloc(size_t bytes);
void dev_free(void *p);

template <class T>
struct DevBuf {
    T *ptr = nullptr;
    size_t count = 0; // capacity in elements
    ~DevBuf() { reset(); }
    void reset()
    {
        if (ptr)
            dev_free(ptr);
        ptr = nullptr;
        count = 0;
    }
    // Grow (never shrink) to at least n elements; contents are not kept.
    bool ensure(size_t n)
    {
        if (n <= count && ptr)
            return true;
        reset();
        size_t bytes = (n ? n : 1) * sizeof(T);
        ptr = static_cast<T *>(dev_alloc(bytes));
        if (!ptr)
            return false;
        count = n ? n : 1;
        return true;
    }
};

// One packed entry of the execution layout: column and FP32 value bits.
struct __align__(8) Entry {
    int32_t col;
    float val;
};

// ---- kernel launchers (convert.cu) ----------------------------------------------------
// Per-row nonzero counts (row_nnz[0..m)).
cudaError_t launch_row_count(const float *A, int64_t m, int64_t k, int32_t *row_nnz,
                             cudaStream_t st);
// Exclusive scan of row counts into row_ptr[0..m] (in place allowed) and the
// derived group arrays; *d_total receives the int64 total. scratch needs
// scan_scratch_elems(m) int64 elements.
size_t scan_scratch_elems(int64_t m);
cudaError_t launch_row_scan(int32_t *row_counts_then_ptr, int64_t m, int32_t rows_per_group,
                            int32_t *group_index, int32_t *nnz_per_group, int64_t *d_total,
                            int64_t *scratch, uint32_t *status, cudaStream_t st);
// launch_row_scan followed by the longest row into d_total[1] (zeroed by the
// caller): one single-CTA kernel for up to 16384 rows, else the two launches.
cudaError_t launch_row_scan_max(int32_t *row_counts_then_ptr, int64_t m, int32_t rows_per_group,
                                int32_t *group_index, int32_t *nnz_per_group, int64_t *d_total,
                                int64_t *scratch, uint32_t *status, cudaStream_t st);
// Group arrays only (count entry point without row pointers): from row counts.
cudaError_t launch_scatter(const float *A, int64_t m, int64_t k, int32_t rows_per_group,
                           const int32_t *group_index, const int32_t *row_ptr, float *vals,
                           int32_t *rows, int32_t *cols, Entry *packed, cudaStream_t st);

// ---- tiled conversion (convert_tiled.cu): a warp per (group, 128-column segment)
int64_t conv_segments(int64_t k); // segments per row: the count array is m x conv_segments(k)
// The tiled kernels need k % 4 == 0, a 16-byte aligned A and rows_per_group <= 8.
bool tiled_convert_ok(const float *A, int64_t m, int64_t k, int32_t cpg);
// cnt[r * S + s] = nonzeros of row r in column segment s (S = conv_segments(k)).
// distinct (may be null; zeroed by the caller) += columns with a nonzero in
// at least one row of their group, summed over groups.
cudaError_t launch_tile_count(const float *A, int64_t m, int64_t k, int32_t cpg, int32_t *cnt,
                              unsigned long long *distinct, cudaStream_t st);
// cnt rows -> exclusive prefix over segments (in place); row totals -> row_cnt[0..m).
cudaError_t launch_tile_prefix(int32_t *cnt, int64_t m, int64_t k, int32_t *row_cnt, cudaStream_t st);
// Same outputs as launch_scatter, from the segment prefixes.
cudaError_t launch_tile_scatter(const float *A, int64_t m, int64_t k, int32_t cpg, const int32_t *pref,
                                const int32_t *group_index, const int32_t *row_ptr, float *vals,
                                int32_t *rows, int32_t *cols, Entry *packed, cudaStream_t st);

// ---- staged rebuild conversion (convert_tiled.cu): A read once -----------------------
// Needs tiled_convert_ok and k < 2^28 (a staged entry keeps col << 3 | row in group).
bool staged_convert_ok(const float *A, int64_t m, int64_t k, int32_t cpg);
int64_t staged_tiles(int64_t m, int64_t k, int32_t cpg); // CPG rows x 1024 columns each
// Entries kept per tile: a power of two >= 2 x the mean of the last build + 32.
int32_t staged_slot(int64_t last_nnz, int64_t tiles, int32_t cpg);
// Segment counts (as launch_tile_count, distinct included), tile_tot[t] (-1
// for a tile that overflowed its slot, listed in over_list[0..*over_count));
// *status gets kStatusWaitTimeout if a bulk copy wait gave up.
cudaError_t launch_stage(const float *A, int64_t m, int64_t k, int32_t cpg, int32_t slot, int32_t *cnt,
                         unsigned long long *distinct, uint2 *stage, int32_t *tile_tot, int32_t *over_list,
                         unsigned long long *over_count, uint32_t *status, cudaStream_t st);
// After launch_tile_prefix and launch_row_scan: the GCOO arrays (vals, rc =
// rows | cols at rc + total) and the packed row order, total = d_total[0] read
// on the device; writes nothing unless the stage status (d_total[3]) is 0,
// total <= cap and total + 2 <= packed_cap.
cudaError_t launch_place(const float *A, int64_t m, int64_t k, int32_t cpg, int32_t slot, const uint2 *stage,
                         const int32_t *tile_tot, const int32_t *over_list, const unsigned long long *over_count,
                         const int32_t *pref, const int32_t *group_index, const int32_t *row_ptr, float *vals,
                         int32_t *rc, Entry *packed, const int64_t *d_total, int64_t cap, int64_t packed_cap,
                         cudaStream_t st);

// ---- FP32 multiply (spdm_fp32.cu) ------------------------------------------------------
int device_sms(); // SMs of the current device (152 on a GB300)
struct LaunchShape {
    int vec;       // columns per thread (1, 2, 4)
    int warps;     // warps per CTA
    int col_warps; // warps side by side on one row
    int depth;     // 1: plain batches, 2: B loads of the next batch in flight
    int rows;      // rows per CTA
    int col_iters = 1; // column tiles each warp walks with one staging of its group's entries
    int chunk = 0;     // entries staged per pass (shared memory), 0: the full 2048
};
// Heavy-tailed row lengths: the longest row at least 256 entries and above 8x the mean.
bool row_lengths_skewed(int64_t m, int64_t nnz, int64_t max_row);
LaunchShape pick_shape(const gcoo_params &p, int64_t m, int64_t n, int64_t nnz, int64_t max_row,
                       uintptr_t b_addr, uintptr_t c_addr);
cudaError_t launch_spdm_fp32(const Entry *packed, const int32_t *row_ptr, int64_t m, const float *B,
                             int64_t n, float *C, const LaunchShape &s, uint32_t *status,
                             cudaStream_t st);
// The rows shorter than long_min, one warp per (row, column tile), nothing
// staged (skewed matrices, whose long rows go to launch_spdm_long); k is
// B's row count, which sets the walk order.
cudaError_t launch_spdm_short(const Entry *packed, const int32_t *row_ptr, int64_t m, int64_t k, const float *B,
                              int64_t n, float *C, int32_t long_min, cudaStream_t st);
// ---- FP8-B scales (spdm_lowp.cu) -----------------------------------------------------------
// scale[j] = the smallest power of two with absmax(B[:, j]) / scale[j] <= 448;
// n % 4 == 0, B 16-byte aligned; amax: n words of scratch.
cudaError_t launch_fp8_scales(const float *B, int64_t k, int64_t n, unsigned *amax, float *scale, cudaStream_t st);
// ---- long rows of skewed matrices (spdm_long.cu) -----------------------------------------
int32_t long_row_min(); // 256 entries
// n % 4 == 0 and a 16-byte aligned B (16-byte copies of B row pieces)
bool long_rows_ok(int64_t n, const float *B);
// list[0..min(*count, cap)) = the rows of at least long_row_min() entries (any order)
cudaError_t launch_collect_long(const int32_t *row_ptr, int64_t m, int32_t *list, int64_t cap,
                                unsigned long long *count, cudaStream_t st);
// ---- long rows summed in pieces (spdm_split.cu, gcoo_params.fp32_sum = split) --------------
// Pieces of a long-row list whose rows hold long_entries entries in total:
// at most this many (also a bound for any list of n_long rows over nnz
// entries with long_entries = nnz).
int64_t split_piece_bound(int64_t n_long, int64_t long_entries);
// The piece plan of the listed rows (count[0] of them, at most list_cap):
// piece_first[row index], piece_row[piece] (at most cap pieces), *total.
cudaError_t launch_split_plan(const int32_t *row_ptr, const int32_t *list, const unsigned long long *count,
                              int64_t list_cap, int32_t *piece_first, int32_t *piece_row, int64_t cap,
                              int32_t *total, cudaStream_t st);
// C rows of the listed rows: partial sums per piece into part (pieces_bound
// x n floats), then added in piece order. n % 4 == 0, B 16-byte aligned.
cudaError_t launch_spdm_split(const Entry *packed, const int32_t *row_ptr, const int32_t *list, int64_t n_long,
                              const int32_t *piece_first, const int32_t *piece_row, const int32_t *total,
                              int64_t pieces_bound, const float *B, int64_t n, float *part, float *C,
                              cudaStream_t st);
// C rows of the listed rows, the same fmaf chains as launch_spdm_fp32
cudaError_t launch_spdm_long(const Entry *packed, const int32_t *row_ptr, const int32_t *list, int64_t n_long,
                             const float *B, int64_t n, float *C, cudaStream_t st);
// FP32 multiply in GCOO order (spdm_fp32_group.cu): one B load per column
// shared by a group's rows; groups of 4 rows; vec 1, 2, 4 or 8.
bool group_order_ok(int32_t rows_per_group);
cudaError_t launch_spdm_fp32_group(const float *vals, const int32_t *rows, const int32_t *cols,
                                   const int32_t *group_index, int64_t m, int64_t ng, const float *B,
                                   int64_t n, float *C, int vec, cudaStream_t st);
// The same walk for the BF16 / FP8-B forms on the FMA engine, from B already
// converted to bf16 or E4M3 (+ per-column scales); n % 8 == 0.
cudaError_t launch_spdm_lowp_group(const float *vals, const int32_t *rows, const int32_t *cols,
                                   const int32_t *group_index, int64_t m, int64_t ng, const void *B,
                                   const float *col_scale, int64_t n, float *C, gcoo_precision prec,
                                   cudaStream_t st);
// Longest row (row_ptr[r+1] - row_ptr[r]) into *out (an int64 zeroed by the caller).
cudaError_t launch_row_max(const int32_t *row_ptr, int64_t m, int64_t *out, cudaStream_t st);
// Multiply straight from reference-layout GCOO arrays (column-major order
// inside a group): one thread per column per group row.
cudaError_t launch_spdm_view(const gcoo_view &a, const float *B, int64_t n, float *C,
                             cudaStream_t st);

// ---- autotune table (autotune.cu) ------------------------------------------------------
struct TuneEntry {
    int vec = 0, warps = 0, col_warps = 0, depth = 0, rows_per_item = 0;
    double us = 0.0;
};
std::string bucket_key(int64_t m, int64_t k, int64_t nnz, int64_t n);
bool tune_lookup(const std::string &key, TuneEntry *out);
void tune_store(const std::string &key, const TuneEntry &e);

// ---- FP64 check (errnorm.cu) -----------------------------------------------------------
cudaError_t launch_error_norm(const Entry *packed, const int32_t *row_ptr, int64_t m,
                              const float *B, int64_t n, const float *C, double *acc2,
                              cudaStream_t st);

// ---- inline PTX helpers -----------------------------------------------------------------
#if defined(__CUDACC__)
__device__ __forceinline__ uint32_t smem_u32(const void *p)
{
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
                 : "memory");
}

__device__ __forceinline__ void fence_mbar_init()
{
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void fence_proxy_async()
{
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
                 "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t *bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ uint64_t global_ns()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ bool mbar_wait_ns(uint64_t *bar, uint32_t parity, uint64_t limit_ns);

// Returns true once the phase with the given parity has completed, false if
// it has not completed within kWaitNs nanoseconds (or kWaitLimit polls).
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity) { return mbar_wait_ns(bar, parity, kWaitNs); }

__device__ __forceinline__ bool mbar_wait_ns(uint64_t *bar, uint32_t parity, uint64_t limit_ns)
{
    const uint32_t addr = smem_u32(bar);
    uint64_t t0 = 0;
    for (uint32_t it = 0; it < kWaitLimit; ++it) {
        uint32_t done;
        asm volatile("{\n\t.reg .pred p;\n\t"
                     "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                     "selp.u32 %0, 1, 0, p;\n\t}"
                     : "=r"(done)
                     : "r"(addr), "r"(parity)
                     : "memory");
        if (done)
            return true;
        const uint64_t now = global_ns();
        if (it == 0)
            t0 = now;
        else if (now - t0 > limit_ns)
            return false;
    }
    return false;
}

// mbar_wait for a waiter with nothing else to do: each poll lets the hardware
// suspend the thread for up to 20 us (it resumes as soon as the phase
// completes), so a waiting warp takes almost no issue slots from the warps
// that compute. Same limits and result as mbar_wait.
__device__ __forceinline__ bool mbar_wait_sleep(uint64_t *bar, uint32_t parity)
{
    const uint32_t addr = smem_u32(bar);
    constexpr uint32_t kSuspendNs = 20000;
    uint64_t t0 = 0;
    for (uint32_t it = 0; it < kWaitLimit; ++it) {
        uint32_t done;
        asm volatile("{\n\t.reg .pred p;\n\t"
                     "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
                     "selp.u32 %0, 1, 0, p;\n\t}"
                     : "=r"(done)
                     : "r"(addr), "r"(parity), "r"(kSuspendNs)
                     : "memory");
        if (done)
            return true;
        const uint64_t now = global_ns();
        if (it == 0)
            t0 = now;
        else if (now - t0 > kWaitNs)
            return false;
    }
    return false;
}

// Bulk (non-tensor) async copy global -> shared, completing on `bar`.
// dst, src 16-byte aligned; bytes a multiple of 16.
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes,
                                         uint64_t *bar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes "
                 "[%0], [%1], %2, [%3];" ::"r"(smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ float4 ldg_f4(const float4 *p) { return __ldg(p); }
#endif

} // namespace gcoo
