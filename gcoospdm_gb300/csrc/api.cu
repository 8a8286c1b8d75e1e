// api.cu -- the C ABI (include/gcoo.h): validation, handle lifecycle, the
// conversion orchestration and dispatch to the kernels. Every entry point
// returns a status; CUDA errors are captured after each launch.
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <mutex>
#include <string>

#include <nvtx3/nvToolsExt.h>

#include "handle.hpp"

namespace gcoo {

NvtxRange::NvtxRange(const char *name) { nvtxRangePushA(name); }
NvtxRange::~NvtxRange() { nvtxRangePop(); }

// ---- errors --------------------------------------------------------------------
static thread_local std::string t_last_error;

void set_error(const std::string &msg) { t_last_error = msg; }

gcoo_status fail(gcoo_status s, const std::string &msg)
{
    t_last_error = std::string(gcoo_status_string(s)) + ": " + msg;
    return s;
}

gcoo_status cuda_fail(cudaError_t e, const char *what)
{
    t_last_error = std::string("CUDA error in ") + what + ": " + cudaGetErrorName(e) + " (" +
                   cudaGetErrorString(e) + ")";
    return e == cudaErrorMemoryAllocation ? GCOO_ERROR_ALLOC : GCOO_ERROR_CUDA;
}

// ---- launch counter ------------------------------------------------------------------
static std::atomic<uint64_t> g_launches{0};
void count_launches(int n) { g_launches.fetch_add(static_cast<uint64_t>(n), std::memory_order_relaxed); }

// ---- allocator ---------------------------------------------------------------------
static gcoo_alloc_fn g_alloc = nullptr;
static gcoo_free_fn g_free = nullptr;
static void *g_alloc_ctx = nullptr;

void *dev_alloc(size_t bytes)
{
    if (g_alloc)
        return g_alloc(bytes, g_alloc_ctx);
    void *p = nullptr;
    if (cudaMalloc(&p, bytes) != cudaSuccess) {
        cudaGetLastError(); // clear the sticky-free error state of this call
        return nullptr;
    }
    return p;
}

void dev_free(void *p)
{
    if (!p)
        return;
    if (g_free)
        g_free(p, g_alloc_ctx);
    else
        cudaFree(p);
}

// coo.cu
gcoo_status coo_build(gcoo_handle *h, cudaStream_t st);
// left.cu
gcoo_status left_prepare(gcoo_handle *h, LeftPlan *&plan, int64_t p, cudaStream_t st);
gcoo_status left_spdm(gcoo_handle *h, const LeftPlan &L, const float *dD, int64_t p, float *dC, cudaStream_t st);

// Implemented in forms.cu / autotune.cpp.
gcoo_status run_form(gcoo_handle *h, const float *dB, int64_t n, float *dC, gcoo_precision prec,
                     cudaStream_t st, bool prepare_only);
bool form_uses_tensor(gcoo_handle *h, gcoo_precision prec);
bool tuned_params(int64_t m, int64_t k, int64_t nnz, int64_t n, gcoo_params *out);

static bool valid_cpg(int32_t c) { return c == 1 || c == 2 || c == 4 || c == 8 || c == 16 || c == 32; }

static gcoo_status check_dims(int64_t m, int64_t k)
{
    if (m <= 0 || k <= 0)
        return fail(GCOO_ERROR_INVALID_VALUE, "m and k must be positive");
    if (m >= (int64_t(1) << 31) || k >= (int64_t(1) << 31))
        return fail(GCOO_ERROR_INVALID_VALUE, "m and k must fit int32 indices");
    return GCOO_SUCCESS;
}

static gcoo_status check_n(int64_t n)
{
    if (n <= 0 || n >= (int64_t(1) << 31))
        return fail(GCOO_ERROR_INVALID_VALUE, "n must be in [1, 2^31)");
    return GCOO_SUCCESS;
}

// Whether the FP32 multiply (and the BF16 / FP8-B forms on the FMA engine)
// walks groups in GCOO order (one B load per column shared by a group's rows)
// instead of rows: forced by fp32_order, else when the conversion saw at
// least 1.5 entries per distinct (group, column) pair.
bool group_order_chosen(const gcoo_handle *h)
{
    if (h->coo || !group_order_ok(h->p.rows_per_group) || h->p.fp32_order == 1)
        return false;
    if (h->p.fp32_order == 2)
        return true;
    return h->distinct_cols > 0 && 2 * h->nnz >= 3 * h->distinct_cols;
}

// The split summation's partial sums for B of n columns (grown, never
// shrunk: allocated by the first multiply of a width, or by gcoo_prepare).
gcoo_status ensure_split_work(gcoo_handle *h, int64_t n)
{
    if (h->pieces_bound <= 0)
        return GCOO_SUCCESS;
    if (!h->split_part.ensure(static_cast<size_t>(h->pieces_bound) * static_cast<size_t>(n)))
        return fail(GCOO_ERROR_ALLOC, "device allocation of the long rows' partial sums failed");
    return GCOO_SUCCESS;
}

gcoo_status spdm_fp32(gcoo_handle *h, const float *dB, int64_t n, float *dC, cudaStream_t st,
                      const gcoo_params *override_params)
{
    if (!override_params && group_order_chosen(h)) {
        // 8 columns per lane (two 16-byte loads: more FMAs per shuffled entry) where n allows
        int v = n % 8 == 0 ? 8 : 4;
        const uintptr_t b = reinterpret_cast<uintptr_t>(dB), c = reinterpret_cast<uintptr_t>(dC);
        if (n % 4 != 0 || (b & 15) || (c & 15))
            v = (n % 2 != 0 || (b & 7) || (c & 7)) ? 1 : 2;
        if (h->p.vec > 0 && h->p.vec < v)
            v = h->p.vec;
        cudaError_t e = launch_spdm_fp32_group(h->vals.ptr, h->rc.ptr, h->rc.ptr + h->nnz, h->group_index(), h->m,
                                               h->ng, dB, n, dC, v, st);
        if (e != cudaSuccess)
            return cuda_fail(e, "spdm_fp32_group_kernel launch");
        return GCOO_SUCCESS;
    }
    gcoo_params p = h->p;
    if (override_params) {
        p = *override_params;
        p.rows_per_group = h->p.rows_per_group;
    } else {
        gcoo_params t;
        if (tuned_params(h->m, h->k, h->nnz, n, &t)) {
            p.vec = t.vec;
            p.warps = t.warps;
            p.col_warps = t.col_warps;
            p.depth = t.depth;
        }
    }
    // a skewed matrix (explicit launch-shape overrides aside): its long rows go
    // to their own kernel, the short rest to a kernel without staging
    if (!override_params && h->n_long > 0 && h->side && h->ev_fork && h->ev_join && long_rows_ok(n, dB)) {
        const bool split = h->p.fp32_sum == GCOO_SUM_SPLIT && h->pieces_bound > 0;
        if (split) {
            gcoo_status ws = ensure_split_work(h, n);
            if (ws != GCOO_SUCCESS)
                return ws;
        }
        // the two kernels write disjoint rows of C: the long rows run on the
        // side stream, forked from and joined back into the caller's stream
        GCOO_CUDA(cudaEventRecord(h->ev_fork, st));
        GCOO_CUDA(cudaStreamWaitEvent(h->side, h->ev_fork, 0));
        const cudaError_t el =
            split ? launch_spdm_split(h->packed.ptr, h->row_ptr.ptr, h->long_rows.ptr, h->n_long, h->piece_first.ptr,
                                      h->piece_row.ptr, h->piece_total.ptr, h->pieces_bound, dB, n,
                                      h->split_part.ptr, dC, h->side)
                  : launch_spdm_long(h->packed.ptr, h->row_ptr.ptr, h->long_rows.ptr, h->n_long, dB, n, dC, h->side);
        const cudaError_t es = el == cudaSuccess
                                   ? launch_spdm_short(h->packed.ptr, h->row_ptr.ptr, h->m, h->k, dB, n, dC, long_row_min(), st)
                                   : cudaSuccess;
        // joined whatever happened: nothing of this call runs past it on the side stream
        GCOO_CUDA(cudaEventRecord(h->ev_join, h->side));
        GCOO_CUDA(cudaStreamWaitEvent(st, h->ev_join, 0));
        if (el != cudaSuccess)
            return cuda_fail(el, split ? "spdm_piece_kernel launch" : "spdm_long_kernel launch");
        if (es != cudaSuccess)
            return cuda_fail(es, "spdm_short_kernel launch");
        return GCOO_SUCCESS;
    }
    const LaunchShape s = pick_shape(p, h->m, n, h->nnz, h->max_row_nnz, reinterpret_cast<uintptr_t>(dB),
                                     reinterpret_cast<uintptr_t>(dC));
    cudaError_t e = launch_spdm_fp32(h->packed.ptr, h->row_ptr.ptr, h->m, dB, n, dC, s, h->status.ptr, st);
    if (e != cudaSuccess)
        return cuda_fail(e, "spdm_fp32_kernel launch");
    return GCOO_SUCCESS;
}

} // namespace gcoo

using namespace gcoo;

extern "C" {

int gcoo_abi_version(void) { return GCOO_ABI_VERSION; }

uint64_t gcoo_kernel_launches(void) { return g_launches.load(std::memory_order_relaxed); }

const char *gcoo_status_string(gcoo_status s)
{
    switch (s) {
    case GCOO_SUCCESS: return "GCOO_SUCCESS";
    case GCOO_ERROR_INVALID_VALUE: return "GCOO_ERROR_INVALID_VALUE";
    case GCOO_ERROR_ALLOC: return "GCOO_ERROR_ALLOC";
    case GCOO_ERROR_CUDA: return "GCOO_ERROR_CUDA";
    case GCOO_ERROR_NOT_BUILT: return "GCOO_ERROR_NOT_BUILT";
    case GCOO_ERROR_UNSUPPORTED: return "GCOO_ERROR_UNSUPPORTED";
    case GCOO_ERROR_FORMAT: return "GCOO_ERROR_FORMAT";
    case GCOO_ERROR_TIMEOUT: return "GCOO_ERROR_TIMEOUT";
    case GCOO_ERROR_CAPACITY: return "GCOO_ERROR_CAPACITY";
    }
    return "GCOO_ERROR_UNKNOWN";
}

const char *gcoo_last_error(void) { return t_last_error.c_str(); }

gcoo_status gcoo_params_default(gcoo_params *p)
{
    if (!p)
        return fail(GCOO_ERROR_INVALID_VALUE, "params is NULL");
    memset(p, 0, sizeof(*p));
    p->rows_per_group = 4; // src/constants.h:4 COLUMN_PER_GROUP
    p->engine = GCOO_ENGINE_AUTO;
    return GCOO_SUCCESS;
}

gcoo_status gcoo_set_allocator(gcoo_alloc_fn alloc, gcoo_free_fn release, void *ctx)
{
    if ((alloc == nullptr) != (release == nullptr))
        return fail(GCOO_ERROR_INVALID_VALUE, "allocator and free function must be given together");
    g_alloc = alloc;
    g_free = release;
    g_alloc_ctx = ctx;
    return GCOO_SUCCESS;
}

gcoo_status gcoo_create(gcoo_handle **out, const float *dA, int64_t m, int64_t k, const gcoo_params *params)
{
    if (!out)
        return fail(GCOO_ERROR_INVALID_VALUE, "out is NULL");
    *out = nullptr;
    if (!dA)
        return fail(GCOO_ERROR_INVALID_VALUE, "dense matrix pointer is NULL");
    gcoo_status s = check_dims(m, k);
    if (s != GCOO_SUCCESS)
        return s;
    gcoo_params p;
    gcoo_params_default(&p);
    if (params)
        p = *params;
    if (!valid_cpg(p.rows_per_group))
        return fail(GCOO_ERROR_INVALID_VALUE, "rows_per_group must be a power of two in [1, 32]");
    if (p.vec != 0 && p.vec != 1 && p.vec != 2 && p.vec != 4)
        return fail(GCOO_ERROR_INVALID_VALUE, "vec must be 0, 1, 2 or 4");
    if (p.warps < 0 || p.warps > 32 || p.col_warps < 0 || p.col_warps > 32)
        return fail(GCOO_ERROR_INVALID_VALUE, "warps / col_warps out of range");
    if (p.engine < GCOO_ENGINE_AUTO || p.engine > GCOO_ENGINE_TENSOR)
        return fail(GCOO_ERROR_INVALID_VALUE, "unknown engine");
    if (p.depth < 0 || p.depth > 2)
        return fail(GCOO_ERROR_INVALID_VALUE, "depth must be 0, 1 or 2");
    if (p.fp32_order < 0 || p.fp32_order > 2)
        return fail(GCOO_ERROR_INVALID_VALUE, "fp32_order must be 0, 1 or 2");
    if (p.fp32_order == 2 && !group_order_ok(p.rows_per_group))
        return fail(GCOO_ERROR_UNSUPPORTED, "the group-order FP32 multiply needs rows_per_group 4");
    if (p.fp32_sum != GCOO_SUM_CHAIN && p.fp32_sum != GCOO_SUM_SPLIT)
        return fail(GCOO_ERROR_INVALID_VALUE, "fp32_sum must be GCOO_SUM_CHAIN (0) or GCOO_SUM_SPLIT (1)");
    gcoo_handle *h = new (std::nothrow) gcoo_handle();
    if (!h)
        return fail(GCOO_ERROR_ALLOC, "host allocation of the handle failed");
    h->dA = dA;
    h->m = m;
    h->k = k;
    h->p = p;
    h->ng = (m + p.rows_per_group - 1) / p.rows_per_group;
    *out = h;
    return GCOO_SUCCESS;
}

namespace {

// The end of every successful build: plans derived from the old arrays go,
// and for a skewed matrix the list of its long rows (multiplied by their own
// kernel) is collected, one readback of its length.
gcoo_status finish_build(gcoo_handle *h, cudaStream_t st)
{
    if (h->tc)
        destroy_tc_plan(h->tc);
    h->tc = nullptr;
    destroy_left_plan(h->left);
    h->left = nullptr;
    h->n_long = 0;
    h->long_entries = 0;
    h->pieces_bound = 0;
    if (row_lengths_skewed(h->m, h->nnz, h->max_row_nnz) && h->packed.count >= static_cast<size_t>(h->nnz) + 2) {
        const int64_t cap = h->nnz / long_row_min() + 1;
        if (!h->long_rows.ensure(static_cast<size_t>(cap)) || !h->long_count.ensure(2))
            return fail(GCOO_ERROR_ALLOC, "device allocation of the long-row list failed");
        unsigned long long *d_cnt = h->long_count.ptr;
        GCOO_CUDA(cudaMemsetAsync(d_cnt, 0, 2 * sizeof(*d_cnt), st));
        GCOO_CUDA(launch_collect_long(h->row_ptr.ptr, h->m, h->long_rows.ptr, cap, d_cnt, st));
        const bool split = h->p.fp32_sum == GCOO_SUM_SPLIT;
        if (split) {
            // the piece plan, before the readback (its tables bounded without it)
            const int64_t pcap = split_piece_bound(cap, h->nnz);
            if (!h->piece_first.ensure(static_cast<size_t>(cap)) || !h->piece_row.ensure(static_cast<size_t>(pcap)) ||
                !h->piece_total.ensure(1))
                return fail(GCOO_ERROR_ALLOC, "device allocation of the long rows' piece plan failed");
            GCOO_CUDA(launch_split_plan(h->row_ptr.ptr, h->long_rows.ptr, d_cnt, cap, h->piece_first.ptr,
                                        h->piece_row.ptr, pcap, h->piece_total.ptr, st));
        }
        if (!h->readback && cudaMallocHost(&h->readback, 4 * sizeof(int64_t)) != cudaSuccess) {
            h->readback = nullptr;
            return fail(GCOO_ERROR_ALLOC, "page-locked allocation of the readback words failed");
        }
        GCOO_CUDA(cudaMemcpyAsync(h->readback, d_cnt, 2 * sizeof(int64_t), cudaMemcpyDeviceToHost, st));
        GCOO_CUDA(cudaStreamSynchronize(st));
        h->n_long = std::min<int64_t>(h->readback[0], cap);
        h->long_entries = h->readback[1];
        h->pieces_bound = split ? split_piece_bound(h->n_long, h->long_entries) : 0;
        if (h->n_long > 0) {
            // the long rows are the multiply's critical path: their CTAs go first
            // (each object made once; one that failed is retried by the next build)
            if (!h->side) {
                int lo = 0, hi = 0;
                cudaStream_t side = nullptr;
                GCOO_CUDA(cudaDeviceGetStreamPriorityRange(&lo, &hi));
                GCOO_CUDA(cudaStreamCreateWithPriority(&side, cudaStreamNonBlocking, hi));
                h->side = side;
            }
            for (cudaEvent_t *ev : {&h->ev_fork, &h->ev_join}) {
                if (*ev)
                    continue;
                cudaEvent_t made = nullptr;
                GCOO_CUDA(cudaEventCreateWithFlags(&made, cudaEventDisableTiming));
                *ev = made;
            }
        }
    }
    h->built = true;
    return GCOO_SUCCESS;
}

} // namespace

gcoo_status gcoo_build(gcoo_handle *h, void *stream)
{
    NvtxRange nvtx("gcoo_build");
    if (!h)
        return fail(GCOO_ERROR_INVALID_VALUE, "handle is NULL");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    h->built = false;
    if (h->coo) {
        gcoo_status s = coo_build(h, st);
        if (s != GCOO_SUCCESS)
            return s;
        return finish_build(h, st);
    }
    const size_t sc = scan_scratch_elems(h->m);
    if (!h->row_ptr.ensure(static_cast<size_t>(h->m) + 1) || !h->groups.ensure(2 * static_cast<size_t>(h->ng + 1)) ||
        !h->scratch.ensure(sc + 8) || !h->status.ensure(1))
        return fail(GCOO_ERROR_ALLOC, "device allocation of the GCOO index arrays failed");
    GCOO_CUDA(cudaMemsetAsync(h->status.ptr, 0, sizeof(uint32_t), st));
    // [0] total nnz, [1] longest row, [2] distinct group columns, [3] staging status, [4] overflowed tiles
    int64_t *d_total = h->scratch.ptr + sc;
    GCOO_CUDA(cudaMemsetAsync(d_total + 1, 0, 7 * sizeof(int64_t), st));
    const int32_t cpg = h->p.rows_per_group;
    const bool tiled = tiled_convert_ok(h->dA, h->m, h->k, cpg);
    // One read of A when the entry arrays of an earlier build have room (a
    // steady loop of mutiplyBy / build); otherwise, or if they turn out too
    // small, the two-pass path below converts and sizes them exactly.
    const int64_t cap = std::min<int64_t>(static_cast<int64_t>(h->vals.count), static_cast<int64_t>(h->rc.count / 2));
    if (tiled && h->vals.ptr && h->rc.ptr && cap > 0 && staged_convert_ok(h->dA, h->m, h->k, cpg)) {
        const int64_t tiles = staged_tiles(h->m, h->k, cpg);
        const int32_t slot = staged_slot(h->nnz, tiles, cpg);
        if (!h->tile_cnt.ensure(static_cast<size_t>(h->m * conv_segments(h->k))) ||
            !h->stage.ensure(static_cast<size_t>(tiles) * static_cast<size_t>(slot)) ||
            !h->tile_tot.ensure(static_cast<size_t>(tiles)) || !h->over_list.ensure(static_cast<size_t>(tiles)))
            return fail(GCOO_ERROR_ALLOC, "device allocation of the staged conversion state failed");
        unsigned long long *over_count = reinterpret_cast<unsigned long long *>(d_total + 4);
        GCOO_CUDA(launch_stage(h->dA, h->m, h->k, cpg, slot, h->tile_cnt.ptr,
                               reinterpret_cast<unsigned long long *>(d_total + 2), h->stage.ptr, h->tile_tot.ptr,
                               h->over_list.ptr, over_count, reinterpret_cast<uint32_t *>(d_total + 3), st));
        GCOO_CUDA(launch_tile_prefix(h->tile_cnt.ptr, h->m, h->k, h->row_ptr.ptr, st));
        GCOO_CUDA(launch_row_scan_max(h->row_ptr.ptr, h->m, cpg, h->group_index(), h->nnz_per_group(), d_total,
                                      h->scratch.ptr, h->status.ptr, st));
        // placed on the device before the one readback (the kernel checks the fit itself)
        const int64_t packed_cap = static_cast<int64_t>(h->packed.count);
        GCOO_CUDA(launch_place(h->dA, h->m, h->k, cpg, slot, h->stage.ptr, h->tile_tot.ptr, h->over_list.ptr,
                               over_count, h->tile_cnt.ptr, h->group_index(), h->row_ptr.ptr, h->vals.ptr, h->rc.ptr,
                               h->packed.ptr, d_total, cap, packed_cap, st));
        if (!h->readback && cudaMallocHost(&h->readback, 4 * sizeof(int64_t)) != cudaSuccess) {
            h->readback = nullptr;
            return fail(GCOO_ERROR_ALLOC, "page-locked allocation of the readback words failed");
        }
        int64_t *t3 = h->readback;
        GCOO_CUDA(cudaMemcpyAsync(t3, d_total, 4 * sizeof(int64_t), cudaMemcpyDeviceToHost, st));
        GCOO_CUDA(cudaStreamSynchronize(st));
        const int64_t total = t3[0];
        if (t3[3] == 0 && (total < 0 || total > 0x7fffffffLL))
            return fail(GCOO_ERROR_FORMAT, "nnz = " + std::to_string(total) + " exceeds the int32 GCOO format");
        if (t3[3] == 0 && total <= cap && total + 2 <= packed_cap) {
            h->max_row_nnz = t3[1];
            h->distinct_cols = t3[2];
            h->nnz = total;
            return finish_build(h, st);
        }
        GCOO_CUDA(cudaMemsetAsync(d_total + 1, 0, 7 * sizeof(int64_t), st));
    }
    if (tiled) {
        if (!h->tile_cnt.ensure(static_cast<size_t>(h->m * conv_segments(h->k))))
            return fail(GCOO_ERROR_ALLOC, "device allocation of the tile counts failed");
        GCOO_CUDA(launch_tile_count(h->dA, h->m, h->k, cpg, h->tile_cnt.ptr,
                                    reinterpret_cast<unsigned long long *>(d_total + 2), st));
        GCOO_CUDA(launch_tile_prefix(h->tile_cnt.ptr, h->m, h->k, h->row_ptr.ptr, st));
    } else {
        GCOO_CUDA(launch_row_count(h->dA, h->m, h->k, h->row_ptr.ptr, st));
    }
    GCOO_CUDA(launch_row_scan_max(h->row_ptr.ptr, h->m, h->p.rows_per_group, h->group_index(), h->nnz_per_group(),
                                  d_total, h->scratch.ptr, h->status.ptr, st));
    int64_t tot2[3] = {0, 0, 0};
    GCOO_CUDA(cudaMemcpyAsync(tot2, d_total, sizeof(tot2), cudaMemcpyDeviceToHost, st));
    GCOO_CUDA(cudaStreamSynchronize(st));
    const int64_t total = tot2[0];
    h->max_row_nnz = tot2[1];
    h->distinct_cols = tiled ? tot2[2] : 0; // 0: not counted
    if (total < 0 || total > 0x7fffffffLL)
        return fail(GCOO_ERROR_FORMAT, "nnz = " + std::to_string(total) + " exceeds the int32 GCOO format");
    const size_t nnz = static_cast<size_t>(total);
    // a little room beyond nnz lets later builds of a similar matrix take the one-pass path
    const size_t room = tiled ? nnz + nnz / 16 + 1024 : nnz;
    if (!h->vals.ensure(room) || !h->rc.ensure(2 * room) || !h->packed.ensure(room + 2))
        return fail(GCOO_ERROR_ALLOC, "device allocation of the GCOO entry arrays failed");
    // rows and cols live in one block, as in the reference (src/ShGCOOSpDM.cu:95-97)
    int32_t *rows = h->rc.ptr;
    int32_t *cols = h->rc.ptr + nnz;
    if (tiled)
        GCOO_CUDA(launch_tile_scatter(h->dA, h->m, h->k, cpg, h->tile_cnt.ptr, h->group_index(), h->row_ptr.ptr,
                                      h->vals.ptr, rows, cols, h->packed.ptr, st));
    else
        GCOO_CUDA(launch_scatter(h->dA, h->m, h->k, cpg, h->group_index(), h->row_ptr.ptr, h->vals.ptr, rows,
                                 cols, h->packed.ptr, st));
    h->nnz = total;
    return finish_build(h, st);
}

gcoo_status gcoo_spdm_left(gcoo_handle *h, const float *dD, int64_t p, float *dC, void *stream)
{
    NvtxRange nvtx("gcoo_spdm_left");
    if (!h || !dD || !dC)
        return fail(GCOO_ERROR_INVALID_VALUE, "NULL handle or matrix pointer");
    if (!h->built)
        return fail(GCOO_ERROR_NOT_BUILT, "gcoo_build has not run");
    gcoo_status s = check_n(p);
    if (s != GCOO_SUCCESS)
        return s;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    s = left_prepare(h, h->left, p, st);
    if (s != GCOO_SUCCESS)
        return s;
    return left_spdm(h, *h->left, dD, p, dC, st);
}

gcoo_status gcoo_create_coo(gcoo_handle **out, int64_t m, int64_t k, const int32_t *d_rows, const int32_t *d_cols,
                            const float *d_vals, int64_t nnz, const gcoo_params *params)
{
    if (!out)
        return fail(GCOO_ERROR_INVALID_VALUE, "out is NULL");
    *out = nullptr;
    if (nnz < 0 || (nnz > 0 && (!d_rows || !d_cols || !d_vals)))
        return fail(GCOO_ERROR_INVALID_VALUE, "NULL triplet arrays or negative nnz");
    if (nnz > 0x7fffffffLL)
        return fail(GCOO_ERROR_FORMAT, "more triplets than the int32 GCOO format holds");
    // reuse the dense constructor's validation with a placeholder operand
    static const float placeholder = 0.0f;
    gcoo_status s = gcoo_create(out, &placeholder, m, k, params);
    if (s != GCOO_SUCCESS)
        return s;
    gcoo_handle *h = *out;
    h->dA = nullptr;
    h->coo = true;
    h->coo_rows = d_rows;
    h->coo_cols = d_cols;
    h->coo_vals = d_vals;
    h->coo_nnz = nnz;
    return GCOO_SUCCESS;
}

gcoo_status gcoo_export(const gcoo_handle *h, gcoo_view *out)
{
    if (!h || !out)
        return fail(GCOO_ERROR_INVALID_VALUE, "handle or view is NULL");
    if (!h->built)
        return fail(GCOO_ERROR_NOT_BUILT, "gcoo_build has not run");
    out->m = h->m;
    out->k = h->k;
    out->nnz = h->nnz;
    out->n_group = h->ng;
    out->rows_per_group = h->p.rows_per_group;
    out->group_index = h->groups.ptr;
    out->nnz_per_group = h->groups.ptr + (h->ng + 1);
    out->vals = h->vals.ptr;
    out->rows = h->rc.ptr;
    out->cols = h->rc.ptr + h->nnz;
    return GCOO_SUCCESS;
}

gcoo_status gcoo_spdm(gcoo_handle *h, const float *dB, int64_t n, float *dC, void *stream)
{
    NvtxRange nvtx("gcoo_spdm");
    if (!h || !dB || !dC)
        return fail(GCOO_ERROR_INVALID_VALUE, "NULL handle or matrix pointer");
    if (!h->built)
        return fail(GCOO_ERROR_NOT_BUILT, "gcoo_build has not run");
    gcoo_status s = check_n(n);
    if (s != GCOO_SUCCESS)
        return s;
    return spdm_fp32(h, dB, n, dC, static_cast<cudaStream_t>(stream), nullptr);
}

gcoo_status gcoo_spdm_ex(gcoo_handle *h, const float *dB, int64_t n, float *dC, gcoo_precision prec, void *stream)
{
    NvtxRange nvtx("gcoo_spdm_ex");
    if (!h || !dB || !dC)
        return fail(GCOO_ERROR_INVALID_VALUE, "NULL handle or matrix pointer");
    if (!h->built)
        return fail(GCOO_ERROR_NOT_BUILT, "gcoo_build has not run");
    gcoo_status s = check_n(n);
    if (s != GCOO_SUCCESS)
        return s;
    if (prec == GCOO_PREC_FP32)
        return spdm_fp32(h, dB, n, dC, static_cast<cudaStream_t>(stream), nullptr);
    if (prec < GCOO_PREC_FP32 || prec > GCOO_PREC_FP8_B)
        return fail(GCOO_ERROR_INVALID_VALUE, "unknown precision");
    return run_form(h, dB, n, dC, prec, static_cast<cudaStream_t>(stream), false);
}

gcoo_status gcoo_prepare(gcoo_handle *h, int64_t n, gcoo_precision prec, void *stream)
{
    if (!h)
        return fail(GCOO_ERROR_INVALID_VALUE, "handle is NULL");
    if (!h->built)
        return fail(GCOO_ERROR_NOT_BUILT, "gcoo_build has not run");
    gcoo_status s = check_n(n);
    if (s != GCOO_SUCCESS)
        return s;
    if (prec == GCOO_PREC_FP32) // the split summation's partial sums, if this handle sums in pieces
        return h->p.fp32_sum == GCOO_SUM_SPLIT && h->n_long > 0 ? ensure_split_work(h, n) : GCOO_SUCCESS;
    if (prec < GCOO_PREC_FP32 || prec > GCOO_PREC_FP8_B)
        return fail(GCOO_ERROR_INVALID_VALUE, "unknown precision");
    return run_form(h, nullptr, n, nullptr, prec, static_cast<cudaStream_t>(stream), true);
}

gcoo_status gcoo_multiply_by(gcoo_handle *h, const float *dB, int64_t n, float *dC, void *stream)
{
    NvtxRange nvtx("gcoo_multiply_by");
    if (!h || !dB || !dC)
        return fail(GCOO_ERROR_INVALID_VALUE, "NULL handle or matrix pointer");
    gcoo_status s = check_n(n);
    if (s != GCOO_SUCCESS)
        return s;
    s = gcoo_build(h, stream);
    if (s != GCOO_SUCCESS)
        return s;
    return spdm_fp32(h, dB, n, dC, static_cast<cudaStream_t>(stream), nullptr);
}

gcoo_status gcoo_destroy(gcoo_handle *h)
{
    delete h; // DevBuf members release through the allocator
    return GCOO_SUCCESS;
}

gcoo_status gcoo_query_engine(gcoo_handle *h, gcoo_precision prec, int32_t *tensor)
{
    if (!h || !tensor)
        return fail(GCOO_ERROR_INVALID_VALUE, "NULL argument");
    if (!h->built)
        return fail(GCOO_ERROR_NOT_BUILT, "gcoo_build has not run");
    *tensor = (prec != GCOO_PREC_FP32 && form_uses_tensor(h, prec)) ? 1 : 0;
    return GCOO_SUCCESS;
}

gcoo_status gcoo_device_status(gcoo_handle *h, void *stream, uint32_t *status)
{
    if (!h || !status)
        return fail(GCOO_ERROR_INVALID_VALUE, "NULL argument");
    *status = 0;
    if (!h->status.ptr)
        return GCOO_SUCCESS;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    GCOO_CUDA(cudaMemcpyAsync(status, h->status.ptr, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    GCOO_CUDA(cudaStreamSynchronize(st));
    if (*status & kStatusWaitTimeout)
        return fail(GCOO_ERROR_TIMEOUT, "a bounded device wait gave up");
    return GCOO_SUCCESS;
}

gcoo_status gcoo_convert_count(const float *dA, int64_t m, int64_t k, int32_t rows_per_group, int32_t *d_group_index,
                               int32_t *d_nnz_per_group, int64_t *nnz, void *stream)
{
    if (!dA || !d_group_index || !d_nnz_per_group || !nnz)
        return fail(GCOO_ERROR_INVALID_VALUE, "NULL argument");
    gcoo_status s = check_dims(m, k);
    if (s != GCOO_SUCCESS)
        return s;
    if (!valid_cpg(rows_per_group))
        return fail(GCOO_ERROR_INVALID_VALUE, "rows_per_group must be a power of two in [1, 32]");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    DevBuf<int32_t> counts;
    DevBuf<int64_t> scratch;
    const size_t sc = scan_scratch_elems(m);
    if (!counts.ensure(static_cast<size_t>(m) + 1) || !scratch.ensure(sc + 1))
        return fail(GCOO_ERROR_ALLOC, "device allocation of conversion scratch failed");
    GCOO_CUDA(launch_row_count(dA, m, k, counts.ptr, st));
    GCOO_CUDA(launch_row_scan(counts.ptr, m, rows_per_group, d_group_index, d_nnz_per_group, scratch.ptr + sc,
                              scratch.ptr, nullptr, st));
    int64_t total = 0;
    GCOO_CUDA(cudaMemcpyAsync(&total, scratch.ptr + sc, sizeof(total), cudaMemcpyDeviceToHost, st));
    GCOO_CUDA(cudaStreamSynchronize(st));
    *nnz = total;
    if (total > 0x7fffffffLL)
        return fail(GCOO_ERROR_FORMAT, "nnz exceeds the int32 GCOO format");
    return GCOO_SUCCESS;
}

gcoo_status gcoo_convert_scatter(const float *dA, int64_t m, int64_t k, int32_t rows_per_group,
                                 const int32_t *d_group_index, float *d_vals, int32_t *d_rows, int32_t *d_cols,
                                 void *stream)
{
    if (!dA || !d_group_index || !d_vals || !d_rows || !d_cols)
        return fail(GCOO_ERROR_INVALID_VALUE, "NULL argument");
    gcoo_status s = check_dims(m, k);
    if (s != GCOO_SUCCESS)
        return s;
    if (!valid_cpg(rows_per_group))
        return fail(GCOO_ERROR_INVALID_VALUE, "rows_per_group must be a power of two in [1, 32]");
    GCOO_CUDA(launch_scatter(dA, m, k, rows_per_group, d_group_index, nullptr, d_vals, d_rows, d_cols, nullptr,
                             static_cast<cudaStream_t>(stream)));
    return GCOO_SUCCESS;
}

gcoo_status gcoo_spdm_view(const gcoo_view *a, const float *dB, int64_t n, float *dC, void *stream)
{
    if (!a || !dB || !dC || !a->group_index || !a->nnz_per_group)
        return fail(GCOO_ERROR_INVALID_VALUE, "NULL argument");
    if (a->nnz > 0 && (!a->vals || !a->rows || !a->cols))
        return fail(GCOO_ERROR_INVALID_VALUE, "NULL entry arrays");
    gcoo_status s = check_dims(a->m, a->k);
    if (s != GCOO_SUCCESS)
        return s;
    s = check_n(n);
    if (s != GCOO_SUCCESS)
        return s;
    if (a->rows_per_group < 1 || a->rows_per_group > 32 ||
        a->n_group != (a->m + a->rows_per_group - 1) / a->rows_per_group)
        return fail(GCOO_ERROR_INVALID_VALUE, "inconsistent rows_per_group / n_group");
    GCOO_CUDA(launch_spdm_view(*a, dB, n, dC, static_cast<cudaStream_t>(stream)));
    return GCOO_SUCCESS;
}

gcoo_status gcoo_error_norm(gcoo_handle *h, const float *dB, int64_t n, const float *dC, double *rel_fro,
                            void *stream)
{
    if (!h || !dB || !dC || !rel_fro)
        return fail(GCOO_ERROR_INVALID_VALUE, "NULL argument");
    if (!h->built)
        return fail(GCOO_ERROR_NOT_BUILT, "gcoo_build has not run");
    gcoo_status s = check_n(n);
    if (s != GCOO_SUCCESS)
        return s;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (!h->norm.ensure(2))
        return fail(GCOO_ERROR_ALLOC, "device allocation failed");
    GCOO_CUDA(cudaMemsetAsync(h->norm.ptr, 0, 2 * sizeof(double), st));
    GCOO_CUDA(launch_error_norm(h->packed.ptr, h->row_ptr.ptr, h->m, dB, n, dC, h->norm.ptr, st));
    double acc[2] = {0.0, 0.0};
    GCOO_CUDA(cudaMemcpyAsync(acc, h->norm.ptr, sizeof(acc), cudaMemcpyDeviceToHost, st));
    GCOO_CUDA(cudaStreamSynchronize(st));
    if (acc[1] == 0.0)
        *rel_fro = acc[0] == 0.0 ? 0.0 : INFINITY;
    else
        *rel_fro = sqrt(acc[0]) / sqrt(acc[1]);
    return GCOO_SUCCESS;
}

} // extern "C"
