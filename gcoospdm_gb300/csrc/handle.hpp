// handle.hpp -- the gcoo_handle object behind the C ABI (not installed).
#pragma once

#include "internal.cuh"

namespace gcoo {
struct TcPlan;    // tensor-core tiles (spdm_tc.cu)
struct LowpWork;  // low-precision workspaces (spdm_lowp.cu)
struct LeftPlan;  // column-order layout for C = D x A (left.cu)
void destroy_tc_plan(TcPlan *p);
void destroy_lowp_work(LowpWork *w);
void destroy_left_plan(LeftPlan *p);
} // namespace gcoo

struct gcoo_handle;
namespace gcoo {
// Whether multiplies walk groups in GCOO order (api.cu): forced by
// fp32_order, else when the rows of a group share columns.
bool group_order_chosen(const gcoo_handle *h);
} // namespace gcoo

struct gcoo_handle {
    const float *dA = nullptr;
    // COO source (gcoo_create_coo): device triplets, not owned
    bool coo = false;
    const int32_t *coo_rows = nullptr, *coo_cols = nullptr;
    const float *coo_vals = nullptr;
    int64_t coo_nnz = 0;
    int64_t m = 0, k = 0;
    gcoo_params p{};
    int64_t ng = 0;
    bool built = false;
    int64_t nnz = 0;
    int64_t max_row_nnz = 0;
    int64_t distinct_cols = 0; // (group, column) pairs with a nonzero; 0 when not counted

    gcoo::DevBuf<int32_t> row_ptr;   // m + 1 (row counts, then exclusive prefix)
    gcoo::DevBuf<int32_t> groups;    // group_index[ng+1] | nnz_per_group[ng+1]
    gcoo::DevBuf<float> vals;        // reference GCOO order
    gcoo::DevBuf<int32_t> rc;        // rows[nnz] | cols[nnz]
    gcoo::DevBuf<gcoo::Entry> packed; // row order, nnz + 2 (16-byte padded)
    gcoo::DevBuf<int32_t> tile_cnt;  // per-(row, column segment) counts of the tiled conversion
    gcoo::DevBuf<uint2> stage;       // staged rebuild: each tile's entries in a fixed slot
    gcoo::DevBuf<int32_t> tile_tot;  // staged rebuild: entries per tile, -1 when it overflowed
    gcoo::DevBuf<int32_t> over_list; // staged rebuild: the overflowed tiles
    int64_t *readback = nullptr;     // page-locked: the staged build's readback
    gcoo::DevBuf<int32_t> long_rows; // skewed matrices: rows multiplied by the long-row kernel
    gcoo::DevBuf<unsigned long long> long_count; // [0] long rows, [1] their entries
    int64_t n_long = 0;
    int64_t long_entries = 0;
    // fp32_sum = split: the piece plan of the long rows and the partial sums
    gcoo::DevBuf<int32_t> piece_first;  // per long row: its first piece
    gcoo::DevBuf<int32_t> piece_row;    // per piece: its long row (index into long_rows)
    gcoo::DevBuf<int32_t> piece_total;  // pieces planned
    gcoo::DevBuf<float> split_part;     // pieces x n partial sums (grown to the widest B)
    int64_t pieces_bound = 0;
    // the long-row kernel runs beside the short-row one: a side stream joined by events
    cudaStream_t side = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    gcoo::DevBuf<int64_t> scratch;   // scan block sums (+1) and the total
    gcoo::DevBuf<uint32_t> status;   // device status word
    gcoo::DevBuf<double> norm;       // error-norm accumulators

    gcoo::TcPlan *tc = nullptr;
    gcoo::LowpWork *lowp = nullptr;
    gcoo::LeftPlan *left = nullptr;

    int32_t *group_index() { return groups.ptr; }
    int32_t *nnz_per_group() { return groups.ptr + (ng + 1); }

    ~gcoo_handle()
    {
        if (readback)
            cudaFreeHost(readback);
        if (ev_fork)
            cudaEventDestroy(ev_fork);
        if (ev_join)
            cudaEventDestroy(ev_join);
        if (side)
            cudaStreamDestroy(side);
        gcoo::destroy_tc_plan(tc);
        gcoo::destroy_lowp_work(lowp);
        gcoo::destroy_left_plan(left);
    }
};
