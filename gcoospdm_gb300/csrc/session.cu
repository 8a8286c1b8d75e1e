// session.cu -- mutiplyBy from host buffers, pipelined over row panels.
//
// The reference's driver copies A and B to the device, runs the plugin and
// copies C back, one step after another (src/main.cu:23-40,86-89 around
// src/ShGCOOSpDM.cu:131-180). On GB300 the host link (about 210 GB/s in,
// 190 GB/s out) is the slowest part of that sequence, so a session keeps it
// busy instead:
//   copy-in stream  : A panel 0, B, A panel 1, A panel 2, ...
//   compute lanes   : two streams taking alternate panels, each with its own
//                     workspace; per panel p (once A panel p, and for the
//                     multiply B, are in): counts -> row scan -> packed
//                     scatter -> FP32 multiply into C rows of panel p. One
//                     lane's conversion and launch gaps overlap the other
//                     lane's multiply.
//   copy-out stream : C panel p as soon as its multiply is done
// Panel conversion needs no host round trip: the packed workspace holds a
// dense panel's worth of entries (panel_rows * k), so nothing depends on the
// nnz before the multiply. Conversion and multiply are the library's own
// kernels on panel-local row pointers, so every C element is the same fmaf
// chain as in gcoo_multiply_by: the same bits.
#include <string.h>

#include <algorithm>
#include <vector>

#include "internal.cuh"

namespace gcoo {
// One compute lane: a stream and the per-panel conversion workspace.
struct SessionLane {
    cudaStream_t s = nullptr;
    DevBuf<int32_t> row_ptr;  // panel rows + 1
    DevBuf<int32_t> tile_cnt; // panel rows x column tiles
    DevBuf<Entry> packed;     // a dense panel's entries + 2
    DevBuf<int64_t> scratch;  // scan block sums + total
};
constexpr int kLanes = 2;
} // namespace gcoo

struct gcoo_session {
    gcoo_params p{};
    int64_t panel_rows_req = 0;
    gcoo::DevBuf<float> dA, dB, dC; // grown to the largest call
    gcoo::DevBuf<uint32_t> status;
    gcoo::SessionLane lane[gcoo::kLanes];
    cudaStream_t s_in = nullptr, s_out = nullptr;
    cudaEvent_t ev_start = nullptr, ev_b = nullptr;
    std::vector<cudaEvent_t> ev_a, ev_mul;
    int32_t last_launches = 0, last_panels = 0;

    ~gcoo_session()
    {
        for (cudaEvent_t e : ev_a)
            cudaEventDestroy(e);
        for (cudaEvent_t e : ev_mul)
            cudaEventDestroy(e);
        if (ev_start)
            cudaEventDestroy(ev_start);
        if (ev_b)
            cudaEventDestroy(ev_b);
        for (gcoo::SessionLane &l : lane)
            if (l.s)
                cudaStreamDestroy(l.s);
        if (s_in)
            cudaStreamDestroy(s_in);
        if (s_out)
            cudaStreamDestroy(s_out);
    }
};

namespace gcoo {

namespace {

// Largest panel: the request, or an eighth of A; capped so a dense panel's
// entries stay within 1 GiB and the panel-local row pointers within int32.
int64_t pick_panel_rows(int64_t m, int64_t k, int32_t cpg, int64_t requested)
{
    int64_t rows = requested > 0 ? requested : (m + 7) / 8;
    const int64_t by_bytes = (int64_t(1) << 30) / (k * static_cast<int64_t>(sizeof(Entry)));
    const int64_t by_int32 = 0x7fffffffLL / k;
    rows = std::min(rows, std::min(by_bytes, by_int32));
    rows = (rows + cpg - 1) / cpg * cpg;
    if (rows < cpg)
        rows = cpg;
    return std::min(rows, (m + cpg - 1) / cpg * cpg);
}

// Panel boundaries. With an explicit panel height: uniform panels. Otherwise
// a quarter panel first (converted while B moves, without delaying B much),
// full panels while the copy-in of A is the bottleneck, then halving panels
// down to a quarter panel over the last two full panels' worth of rows, so
// that the multiply and copy-out left once the last A bytes arrive are short.
// (Smaller panels do not pay: every panel's multiply reads all of B.) Every
// panel starts on a rows_per_group boundary.
std::vector<int64_t> panel_starts(int64_t m, int32_t cpg, int64_t P, bool taper)
{
    std::vector<int64_t> st{0};
    const int64_t smallest = std::max<int64_t>(cpg, (P / 4) / cpg * cpg);
    int64_t r = 0;
    while (r < m) {
        const int64_t rem = m - r;
        int64_t size = P;
        if (taper && r == 0)
            size = smallest;
        else if (taper && rem <= 2 * P)
            size = std::max(smallest, (rem / 2) / cpg * cpg);
        size = std::min(size, rem);
        r += size;
        st.push_back(r);
    }
    return st;
}

gcoo_status ensure_events(gcoo_session *s, size_t panels)
{
    while (s->ev_a.size() < panels) {
        cudaEvent_t a, b;
        GCOO_CUDA(cudaEventCreateWithFlags(&a, cudaEventDisableTiming));
        if (cudaEventCreateWithFlags(&b, cudaEventDisableTiming) != cudaSuccess) {
            cudaEventDestroy(a);
            return fail(GCOO_ERROR_CUDA, "event creation failed");
        }
        s->ev_a.push_back(a);
        s->ev_mul.push_back(b);
    }
    return GCOO_SUCCESS;
}

// The copies and launches of one session multiply, in stream order (no waits
// on the host); an error returns at once and the caller drains the streams.
gcoo_status session_enqueue(gcoo_session *s, const float *hA, int64_t k, const float *hB, int64_t n, float *hC,
                            cudaStream_t user, const std::vector<int64_t> &starts, int64_t P, int lanes)
{
    const int32_t cpg = s->p.rows_per_group;
    const int64_t panels = static_cast<int64_t>(starts.size()) - 1;
    GCOO_CUDA(cudaEventRecord(s->ev_start, user));
    GCOO_CUDA(cudaStreamWaitEvent(s->s_in, s->ev_start, 0));
    GCOO_CUDA(cudaMemsetAsync(s->status.ptr, 0, sizeof(uint32_t), s->s_in));

    // copy-in: A panel 0 (converted while B moves), B (every multiply needs
    // all of it), then the other A panels; a second early panel would delay
    // B by more than its conversion saves
    float *dA = s->dA.ptr, *dB = s->dB.ptr, *dC = s->dC.ptr;
    auto copy_a = [&](int64_t q) -> cudaError_t {
        const int64_t r0 = starts[q], rows = starts[q + 1] - r0;
        cudaError_t e = cudaMemcpyAsync(dA + r0 * k, hA + r0 * k, static_cast<size_t>(rows * k) * sizeof(float),
                                        cudaMemcpyHostToDevice, s->s_in);
        if (e == cudaSuccess)
            e = cudaEventRecord(s->ev_a[q], s->s_in);
        return e;
    };
    GCOO_CUDA(copy_a(0));
    GCOO_CUDA(cudaMemcpyAsync(dB, hB, static_cast<size_t>(k * n) * sizeof(float), cudaMemcpyHostToDevice, s->s_in));
    GCOO_CUDA(cudaEventRecord(s->ev_b, s->s_in));
    for (int64_t q = 1; q < panels; ++q)
        GCOO_CUDA(copy_a(q));

    // uniform-row launch shape: the nnz is never read back, so the heavy-tail
    // heuristic (which needs the longest row) is not applied here
    const LaunchShape shape = pick_shape(s->p, P, n, 0, 0, reinterpret_cast<uintptr_t>(dB),
                                         reinterpret_cast<uintptr_t>(dC));
    for (int64_t q = 0; q < panels; ++q) {
        SessionLane &L = s->lane[q % lanes];
        const int64_t r0 = starts[q], rows = starts[q + 1] - r0;
        const float *Ap = dA + r0 * k;
        int64_t *d_total = L.scratch.ptr + scan_scratch_elems(P);
        GCOO_CUDA(cudaStreamWaitEvent(L.s, s->ev_a[q], 0)); // also orders after the status reset
        // panels start on rows_per_group boundaries, so A + r0 * k keeps A's alignment when k % 4 == 0
        const bool tiled = tiled_convert_ok(Ap, rows, k, cpg);
        if (tiled) {
            GCOO_CUDA(launch_tile_count(Ap, rows, k, cpg, L.tile_cnt.ptr, nullptr, L.s));
            GCOO_CUDA(launch_tile_prefix(L.tile_cnt.ptr, rows, k, L.row_ptr.ptr, L.s));
        } else {
            GCOO_CUDA(launch_row_count(Ap, rows, k, L.row_ptr.ptr, L.s));
        }
        GCOO_CUDA(launch_row_scan_max(L.row_ptr.ptr, rows, cpg, nullptr, nullptr, d_total, L.scratch.ptr,
                                      s->status.ptr, L.s));
        if (tiled)
            GCOO_CUDA(launch_tile_scatter(Ap, rows, k, cpg, L.tile_cnt.ptr, nullptr, L.row_ptr.ptr, nullptr, nullptr,
                                          nullptr, L.packed.ptr, L.s));
        else
            GCOO_CUDA(launch_scatter(Ap, rows, k, cpg, nullptr, L.row_ptr.ptr, nullptr, nullptr, nullptr,
                                     L.packed.ptr, L.s));
        if (q < lanes)
            GCOO_CUDA(cudaStreamWaitEvent(L.s, s->ev_b, 0));
        GCOO_CUDA(launch_spdm_fp32(L.packed.ptr, L.row_ptr.ptr, rows, dB, n, dC + r0 * n, shape, s->status.ptr, L.s));
        GCOO_CUDA(cudaEventRecord(s->ev_mul[q], L.s));
        // copy-out of this panel overlaps the next panels' copy-in and compute
        GCOO_CUDA(cudaStreamWaitEvent(s->s_out, s->ev_mul[q], 0));
        GCOO_CUDA(cudaMemcpyAsync(hC + r0 * n, dC + r0 * n, static_cast<size_t>(rows * n) * sizeof(float),
                                  cudaMemcpyDeviceToHost, s->s_out));
    }
    return GCOO_SUCCESS;
}

} // namespace

} // namespace gcoo

using namespace gcoo;

extern "C" {

gcoo_status gcoo_session_create(gcoo_session **out, const gcoo_params *params, int64_t panel_rows)
{
    if (!out)
        return fail(GCOO_ERROR_INVALID_VALUE, "out is NULL");
    *out = nullptr;
    if (panel_rows < 0)
        return fail(GCOO_ERROR_INVALID_VALUE, "panel_rows must be >= 0");
    gcoo_params p;
    gcoo_params_default(&p);
    if (params)
        p = *params;
    const int32_t c = p.rows_per_group;
    if (!(c == 1 || c == 2 || c == 4 || c == 8 || c == 16 || c == 32))
        return fail(GCOO_ERROR_INVALID_VALUE, "rows_per_group must be 1, 2, 4, 8, 16 or 32");
    gcoo_session *s = new gcoo_session();
    s->p = p;
    s->panel_rows_req = panel_rows;
    if (cudaStreamCreateWithFlags(&s->s_in, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&s->lane[0].s, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&s->lane[1].s, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&s->s_out, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&s->ev_start, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&s->ev_b, cudaEventDisableTiming) != cudaSuccess) {
        delete s;
        return fail(GCOO_ERROR_CUDA, "stream or event creation failed");
    }
    *out = s;
    return GCOO_SUCCESS;
}

gcoo_status gcoo_session_multiply(gcoo_session *s, const float *hA, int64_t m, int64_t k, const float *hB,
                                  int64_t n, float *hC, void *stream)
{
    NvtxRange nvtx("gcoo_session_multiply");
    if (!s || !hA || !hB || !hC)
        return fail(GCOO_ERROR_INVALID_VALUE, "NULL session or matrix pointer");
    if (m <= 0 || k <= 0 || m >= (int64_t(1) << 31) || k >= (int64_t(1) << 31))
        return fail(GCOO_ERROR_INVALID_VALUE, "m and k must be in [1, 2^31)");
    if (n <= 0 || n >= (int64_t(1) << 31))
        return fail(GCOO_ERROR_INVALID_VALUE, "n must be in [1, 2^31)");
    const int32_t cpg = s->p.rows_per_group;
    const int64_t P = pick_panel_rows(m, k, cpg, s->panel_rows_req);
    const std::vector<int64_t> starts = panel_starts(m, cpg, P, s->panel_rows_req == 0);
    const int64_t panels = static_cast<int64_t>(starts.size()) - 1;
    int64_t tallest = 0;
    for (int64_t q = 0; q < panels; ++q)
        tallest = std::max(tallest, starts[q + 1] - starts[q]);
    const int64_t cap = tallest * k; // dense panel: the most entries a panel can have
    // A panel is scattered without a readback of its total, so even a dense
    // panel must fit the int32 offsets. Only k of about 2^31 / rows_per_group
    // columns or more, where a panel is one group high, can break this;
    // gcoo_build checks the total before it scatters and takes such matrices.
    if (cap > 0x7fffffffLL - 2)
        return fail(GCOO_ERROR_UNSUPPORTED, "k too large for a host-buffer panel within the int32 format: "
                                            "use gcoo_create + gcoo_build");

    if (!s->dA.ensure(static_cast<size_t>(m * k)) || !s->dB.ensure(static_cast<size_t>(k * n)) ||
        !s->dC.ensure(static_cast<size_t>(m * n)) || !s->status.ensure(1))
        return fail(GCOO_ERROR_ALLOC, "device allocation of the session buffers failed");
    const int lanes = panels > 1 ? kLanes : 1;
    for (int l = 0; l < lanes; ++l) {
        SessionLane &L = s->lane[l];
        if (!L.row_ptr.ensure(static_cast<size_t>(P) + 1) || !L.packed.ensure(static_cast<size_t>(cap) + 2) ||
            !L.scratch.ensure(scan_scratch_elems(P) + 2) ||
            !L.tile_cnt.ensure(static_cast<size_t>(P * conv_segments(k))))
            return fail(GCOO_ERROR_ALLOC, "device allocation of the session workspace failed");
    }
    gcoo_status st = ensure_events(s, static_cast<size_t>(panels));
    if (st != GCOO_SUCCESS)
        return st;

    const uint64_t launches0 = gcoo_kernel_launches();
    cudaStream_t user = static_cast<cudaStream_t>(stream);
    const gcoo_status enq = session_enqueue(s, hA, k, hB, n, hC, user, starts, P, lanes);
    // whatever was enqueued has finished before the call returns, also after
    // an error: nothing of it may still read hA / hB or write hC afterwards
    cudaError_t drained = cudaSuccess;
    for (cudaStream_t q : {s->lane[0].s, s->lane[1].s, s->s_out, s->s_in}) {
        const cudaError_t e = cudaStreamSynchronize(q);
        if (drained == cudaSuccess)
            drained = e;
    }
    if (enq != GCOO_SUCCESS)
        return enq;
    if (drained != cudaSuccess)
        return cuda_fail(drained, "session stream synchronisation");
    uint32_t status = 0;
    GCOO_CUDA(cudaMemcpy(&status, s->status.ptr, sizeof(uint32_t), cudaMemcpyDeviceToHost));
    s->last_launches = static_cast<int32_t>(gcoo_kernel_launches() - launches0);
    s->last_panels = static_cast<int32_t>(panels);
    if (status & kStatusOverflow)
        return fail(GCOO_ERROR_FORMAT, "a panel's nnz exceeds the int32 format");
    if (status & kStatusWaitTimeout)
        return fail(GCOO_ERROR_TIMEOUT, "a bounded device wait gave up");
    return GCOO_SUCCESS;
}


gcoo_status gcoo_session_stats(const gcoo_session *s, int32_t *launches, int32_t *panels)
{
    if (!s)
        return fail(GCOO_ERROR_INVALID_VALUE, "session is NULL");
    if (launches)
        *launches = s->last_launches;
    if (panels)
        *panels = s->last_panels;
    return GCOO_SUCCESS;
}

gcoo_status gcoo_session_destroy(gcoo_session *s)
{
    if (s) {
        cudaStreamSynchronize(s->s_in);
        for (gcoo::SessionLane &l : s->lane)
            if (l.s)
                cudaStreamSynchronize(l.s);
        cudaStreamSynchronize(s->s_out);
    }
    delete s;
    return GCOO_SUCCESS;
}

} // extern "C"
