// batched.cu -- many independent multiplies in one persistent launch.
//
// gcoo_batch_create turns each problem (a built handle, its B, its C) into
// work items of `rows_per_item` consecutive rows at full width, sorts all
// items by their entry count (descending, so the longest items start first)
// into a device queue, and captures [queue reset, (B -> BF16), persistent
// kernel] into a CUDA graph on a private stream. gcoo_batch_run replays that
// graph on the caller's stream: one kernel launch (two for BF16) whatever the
// number of problems. Warps of the persistent kernel pull items with an
// atomic counter (no waits on other warps); each warp computes whole rows of an item
// with the same sequential fmaf chain as the single-problem kernels, so FP32
// results are bit-identical to gcoo_spdm per problem and BF16 results to
// gcoo_spdm_ex(BF16) on the FMA engine.
//
// The item shape -- rows_per_item and the per-lane vector width (FP32 up to
// 4 floats, BF16 up to 8 values: one 16-byte load per entry), which sets the
// lanes per row (n / width, 4 to 32: several narrow rows share a warp) -- is
// chosen per shape bucket (n and density class) by timing the candidates on
// that bucket's items (the autotune table, persisted with
// gcoo_autotune_save); a loaded table skips the timing.
#include <cuda_bf16.h>
#include <math.h>

#include <algorithm>
#include <map>
#include <string>
#include <vector>

#include "handle.hpp"

namespace gcoo {

struct BatchProb {
    const Entry *packed;
    const int32_t *row_ptr;
    const float *B;
    const uint16_t *Bbf;
    float *C;
    int64_t n;
};

struct BatchItem {
    int32_t prob, row0, row1;
    int16_t vec; // values of B per lane and load
    int16_t lpr; // lanes per row: a warp runs 32 / lpr rows side by side
};

struct ConvSeg {
    const float *src;
    uint16_t *dst;
    int64_t count4;
};

} // namespace gcoo

struct gcoo_batch {
    gcoo_precision prec = GCOO_PREC_FP32;
    int32_t count = 0;
    std::vector<gcoo_problem> probs;
    std::vector<std::vector<int32_t>> row_ptr_h;
    std::vector<std::string> bucket;
    std::vector<int> vec;
    gcoo::DevBuf<gcoo::BatchProb> d_probs;
    gcoo::DevBuf<gcoo::BatchItem> d_items;
    gcoo::DevBuf<unsigned> counter;
    gcoo::DevBuf<uint16_t> bf_ws;
    gcoo::DevBuf<gcoo::ConvSeg> d_segs;
    int nitems = 0;
    int grid = 0;
    cudaStream_t cap = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    ~gcoo_batch()
    {
        if (exec)
            cudaGraphExecDestroy(exec);
        if (graph)
            cudaGraphDestroy(graph);
        if (cap)
            cudaStreamDestroy(cap);
    }
};

namespace gcoo {

namespace {

constexpr int kBatchThreads = 256;

// B loads of V floats per lane (FP32 items).
template <int V, bool BF16>
struct RowLoad;
template <int V>
struct RowLoad<V, false> {
    static __device__ __forceinline__ void load(const BatchProb &p, int64_t off, float (&b)[V])
    {
        if constexpr (V == 4) {
            const float4 t = __ldg(reinterpret_cast<const float4 *>(p.B + off));
            b[0] = t.x; b[1] = t.y; b[2] = t.z; b[3] = t.w;
        } else if constexpr (V == 2) {
            const float2 t = __ldg(reinterpret_cast<const float2 *>(p.B + off));
            b[0] = t.x; b[1] = t.y;
        } else {
            b[0] = __ldg(p.B + off);
        }
    }
};
// V bf16 values of the BF16 copy of B as raw words (value i in the low
// (even i) or high (odd i) half of word i / 2).
template <int V>
__device__ __forceinline__ void load_bf16_words(const uint16_t *q, uint32_t (&w)[(V + 1) / 2])
{
    if constexpr (V == 8) {
        const uint4 t = __ldg(reinterpret_cast<const uint4 *>(q));
        w[0] = t.x; w[1] = t.y; w[2] = t.z; w[3] = t.w;
    } else if constexpr (V == 4) {
        const uint2 t = __ldg(reinterpret_cast<const uint2 *>(q));
        w[0] = t.x; w[1] = t.y;
    } else if constexpr (V == 2) {
        w[0] = __ldg(reinterpret_cast<const unsigned int *>(q));
    } else {
        w[0] = __ldg(reinterpret_cast<const unsigned short *>(q));
    }
}

// acc + a * b with bf16 a and b and one rounding (the mixed-precision FMA of
// sm_100+): a product of two bf16 values is exact in FP32, so this is fmaf on
// the widened values, without widening b first.
__device__ __forceinline__ float fma_bf16(uint16_t a, uint16_t b, float c)
{
    float d;
    asm("fma.rn.f32.bf16 %0, %1, %2, %3;" : "=f"(d) : "h"(a), "h"(b), "f"(c));
    return d;
}

template <int V>
__device__ __forceinline__ void store_row(float *out, const float (&acc)[V])
{
    if constexpr (V == 8) {
        reinterpret_cast<float4 *>(out)[0] = make_float4(acc[0], acc[1], acc[2], acc[3]);
        reinterpret_cast<float4 *>(out)[1] = make_float4(acc[4], acc[5], acc[6], acc[7]);
    } else if constexpr (V == 4) {
        *reinterpret_cast<float4 *>(out) = make_float4(acc[0], acc[1], acc[2], acc[3]);
    } else if constexpr (V == 2) {
        *reinterpret_cast<float2 *>(out) = make_float2(acc[0], acc[1]);
    } else {
        out[0] = acc[0];
    }
}

// The rows of an item, LPR lanes per row (32 / LPR rows per warp side by
// side), V values of B per lane and load; each lane runs its columns' fmaf
// chains over the row's entries in order, batches of four entries' loads in
// flight; a = the entry (BF16: rounded to bf16). The same chains for every
// (V, LPR), so results do not depend on the shape.
template <int V, int LPR, bool BF16>
__device__ __forceinline__ void item_rows(const BatchProb &p, int row0, int row1, int warp, int lane)
{
    constexpr int W = 1; // one warp per item
    constexpr int RPW = 32 / LPR;
    const int sub = lane / LPR, sl = lane % LPR;
    for (int rb = row0 + RPW * warp; rb < row1; rb += RPW * W) {
        const int row = rb + sub;
        if (row >= row1)
            continue; // no row for this lane group (nothing warp-wide below)
        const int64_t e0 = p.row_ptr[row], e1 = p.row_ptr[row + 1];
        for (int64_t j = static_cast<int64_t>(sl) * V; j < p.n; j += LPR * V) {
            float acc[V];
#pragma unroll
            for (int v = 0; v < V; ++v)
                acc[v] = 0.0f;
            int64_t e = e0;
            if constexpr (BF16) {
                // raw bf16 words of B and the mixed-precision FMA: the same
                // results as widening both to FP32 and fmaf
#pragma unroll 1
                for (; e + 4 <= e1; e += 4) {
                    Entry t[4];
                    uint32_t w[4][(V + 1) / 2];
#pragma unroll
                    for (int u = 0; u < 4; ++u)
                        t[u] = p.packed[e + u];
#pragma unroll
                    for (int u = 0; u < 4; ++u)
                        load_bf16_words<V>(p.Bbf + static_cast<int64_t>(t[u].col) * p.n + j, w[u]);
#pragma unroll
                    for (int u = 0; u < 4; ++u) {
                        const __nv_bfloat16 ab = __float2bfloat16_rn(t[u].val);
                        const uint16_t a = __bfloat16_as_ushort(ab);
#pragma unroll
                        for (int v = 0; v < V; ++v)
                            acc[v] = fma_bf16(a, static_cast<uint16_t>((v & 1) ? (w[u][v >> 1] >> 16) : w[u][v >> 1]),
                                              acc[v]);
                    }
                }
#pragma unroll 1
                for (; e < e1; ++e) {
                    const Entry t = p.packed[e];
                    uint32_t w[(V + 1) / 2];
                    load_bf16_words<V>(p.Bbf + static_cast<int64_t>(t.col) * p.n + j, w);
                    const uint16_t a = __bfloat16_as_ushort(__float2bfloat16_rn(t.val));
#pragma unroll
                    for (int v = 0; v < V; ++v)
                        acc[v] = fma_bf16(a, static_cast<uint16_t>((v & 1) ? (w[v >> 1] >> 16) : w[v >> 1]), acc[v]);
                }
            } else {
#pragma unroll 1
                for (; e + 4 <= e1; e += 4) {
                    Entry t[4];
                    float b[4][V];
#pragma unroll
                    for (int u = 0; u < 4; ++u)
                        t[u] = p.packed[e + u];
#pragma unroll
                    for (int u = 0; u < 4; ++u)
                        RowLoad<V, false>::load(p, static_cast<int64_t>(t[u].col) * p.n + j, b[u]);
#pragma unroll
                    for (int u = 0; u < 4; ++u)
#pragma unroll
                        for (int v = 0; v < V; ++v)
                            acc[v] = fmaf(t[u].val, b[u][v], acc[v]);
                }
#pragma unroll 1
                for (; e < e1; ++e) {
                    const Entry t = p.packed[e];
                    float b[V];
                    RowLoad<V, false>::load(p, static_cast<int64_t>(t.col) * p.n + j, b);
#pragma unroll
                    for (int v = 0; v < V; ++v)
                        acc[v] = fmaf(t.val, b[v], acc[v]);
                }
            }
            store_row<V>(p.C + static_cast<int64_t>(row) * p.n + j, acc);
        }
    }
}

// The (V, LPR) shapes an item may take.
template <bool BF16>
__device__ __forceinline__ void run_item(const BatchProb &p, const BatchItem &w, int warp, int lane)
{
#define GCOO_ITEM(V, L)                                                                                 \
    if (w.vec == V && w.lpr == L) {                                                                     \
        item_rows<V, L, BF16>(p, w.row0, w.row1, warp, lane);                                           \
        return;                                                                                         \
    }
    if constexpr (BF16) {
        GCOO_ITEM(8, 4) GCOO_ITEM(8, 8) GCOO_ITEM(8, 16)
    }
    GCOO_ITEM(4, 8) GCOO_ITEM(4, 16) GCOO_ITEM(4, 32) GCOO_ITEM(2, 16) GCOO_ITEM(2, 32)
#undef GCOO_ITEM
    item_rows<1, 32, BF16>(p, w.row0, w.row1, warp, lane); // any n, any alignment
}

// Persistent: every warp pulls work items from the queue with an atomic
// counter (no CTA barrier between items: a warp that finishes early takes
// the next item; the queue is sorted by work, longest first).
template <bool BF16>
__global__ void __launch_bounds__(kBatchThreads)
batch_kernel(const BatchProb *__restrict__ probs, const BatchItem *__restrict__ items, int nitems,
             unsigned *__restrict__ counter)
{
    const int lane = threadIdx.x & 31;
    for (;;) {
        unsigned it = 0;
        if (lane == 0)
            it = atomicAdd(counter, 1u);
        it = __shfl_sync(0xffffffffu, it, 0);
        if (it >= static_cast<unsigned>(nitems))
            break; // warp-uniform
        const BatchItem w = items[it];
        const BatchProb p = probs[w.prob];
        run_item<BF16>(p, w, 0, lane);
    }
}

__global__ void batch_bf16_kernel(const ConvSeg *__restrict__ segs)
{
    const ConvSeg s = segs[blockIdx.y];
    for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < s.count4;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const float4 v = __ldcs(reinterpret_cast<const float4 *>(s.src) + i);
        const __nv_bfloat162 a = __floats2bfloat162_rn(v.x, v.y);
        const __nv_bfloat162 b = __floats2bfloat162_rn(v.z, v.w);
        reinterpret_cast<uint2 *>(s.dst)[i] =
            make_uint2(*reinterpret_cast<const uint32_t *>(&a), *reinterpret_cast<const uint32_t *>(&b));
    }
}

// Widest load per lane (values of B) for a problem: 16-byte loads where n and
// the alignment of B and C allow (the BF16 copy of B is 32-byte aligned per
// problem, so there n and C decide).
int pick_vec_bf16(int64_t n, const float *C)
{
    const uintptr_t c = reinterpret_cast<uintptr_t>(C);
    if (n % 8 == 0 && (c & 15) == 0)
        return 8;
    if (n % 4 == 0 && (c & 15) == 0)
        return 4;
    if (n % 2 == 0 && (c & 7) == 0)
        return 2;
    return 1;
}

int pick_vec(int64_t n, const float *B, const float *C)
{
    const uintptr_t a = reinterpret_cast<uintptr_t>(B) | reinterpret_cast<uintptr_t>(C);
    if (n % 4 == 0 && (a & 15) == 0)
        return 4;
    if (n % 2 == 0 && (a & 7) == 0)
        return 2;
    return 1;
}

// Lanes per row for V values per lane: enough to cover n in one pass, a power
// of two between the narrowest shape the kernel has for V and 32.
int lanes_per_row(int64_t n, int vec)
{
    const int lo = vec == 8 ? 4 : vec == 4 ? 8 : vec == 2 ? 16 : 32;
    int l = 32;
    while (l > lo && static_cast<int64_t>(l / 2) * vec >= n)
        l /= 2;
    return l;
}

std::string batch_bucket(const gcoo_problem &p)
{
    const gcoo_handle *h = p.a;
    const double density = static_cast<double>(h->nnz) / (static_cast<double>(h->m) * h->k);
    const int d = density > 0.0 ? static_cast<int>(floor(-log2(density))) : 99;
    int ln = 0;
    while ((int64_t(1) << ln) < p.n)
        ++ln;
    return "batch_n" + std::to_string(ln) + "_d" + std::to_string(d);
}

// A bucket's tuned shape: rows per work item and the widest per-lane vector
// (a cap on each problem's widest valid width).
struct ItemShape {
    int rows = 16;
    int vec_cap = 8;
};

void make_items(const gcoo_batch &b, const std::vector<int> &probs, const std::map<std::string, ItemShape> &shape,
                std::vector<BatchItem> &items)
{
    std::vector<std::pair<int64_t, BatchItem>> tmp;
    for (int i : probs) {
        const ItemShape &sh = shape.at(b.bucket[i]);
        const int r = sh.rows;
        const int vec = std::min(b.vec[i], std::max(1, sh.vec_cap));
        const int lpr = lanes_per_row(b.probs[i].n, vec);
        const std::vector<int32_t> &rp = b.row_ptr_h[i];
        const int m = static_cast<int>(rp.size()) - 1;
        for (int r0 = 0; r0 < m; r0 += r) {
            const int r1 = std::min(m, r0 + r);
            BatchItem it{i, r0, r1, static_cast<int16_t>(vec), static_cast<int16_t>(lpr)};
            tmp.push_back({static_cast<int64_t>(rp[r1] - rp[r0]) * b.probs[i].n + (r1 - r0), it});
        }
    }
    std::stable_sort(tmp.begin(), tmp.end(), [](const auto &x, const auto &y) { return x.first > y.first; });
    items.clear();
    for (auto &t : tmp)
        items.push_back(t.second);
}

gcoo_status upload_items(gcoo_batch &b, const std::vector<BatchItem> &items, cudaStream_t st)
{
    if (!b.d_items.ensure(items.size() + 1))
        return fail(GCOO_ERROR_ALLOC, "device allocation of the work queue failed");
    if (!items.empty())
        GCOO_CUDA(cudaMemcpyAsync(b.d_items.ptr, items.data(), items.size() * sizeof(BatchItem), cudaMemcpyHostToDevice, st));
    b.nitems = static_cast<int>(items.size());
    return GCOO_SUCCESS;
}

void launch_batch(const gcoo_batch &b, cudaStream_t st)
{
    if (b.prec == GCOO_PREC_BF16)
        batch_kernel<true><<<b.grid, kBatchThreads, 0, st>>>(b.d_probs.ptr, b.d_items.ptr, b.nitems, b.counter.ptr);
    else
        batch_kernel<false><<<b.grid, kBatchThreads, 0, st>>>(b.d_probs.ptr, b.d_items.ptr, b.nitems, b.counter.ptr);
    count_launches(1);
}

} // namespace
} // namespace gcoo

using namespace gcoo;

extern "C" {

gcoo_status gcoo_batch_create(gcoo_batch **out, const gcoo_problem *problems, int32_t count, gcoo_precision prec,
                              void *stream)
{
    if (!out || !problems || count <= 0)
        return fail(GCOO_ERROR_INVALID_VALUE, "NULL argument or empty batch");
    *out = nullptr;
    if (prec != GCOO_PREC_FP32 && prec != GCOO_PREC_BF16)
        return fail(GCOO_ERROR_UNSUPPORTED, "batched forms: GCOO_PREC_FP32 or GCOO_PREC_BF16");
    for (int32_t i = 0; i < count; ++i) {
        const gcoo_problem &p = problems[i];
        if (!p.a || !p.dB || !p.dC || p.n <= 0 || p.n >= (int64_t(1) << 31))
            return fail(GCOO_ERROR_INVALID_VALUE, "problem " + std::to_string(i) + " is incomplete");
        if (!p.a->built)
            return fail(GCOO_ERROR_NOT_BUILT, "problem " + std::to_string(i) + " is not built");
        if (prec == GCOO_PREC_BF16 && ((p.a->k * p.n) % 4 != 0 || (reinterpret_cast<uintptr_t>(p.dB) & 15)))
            return fail(GCOO_ERROR_UNSUPPORTED, "BF16 batch needs k*n % 4 == 0 and 16-byte aligned B");
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    gcoo_batch *b = new (std::nothrow) gcoo_batch();
    if (!b)
        return fail(GCOO_ERROR_ALLOC, "host allocation failed");
    b->prec = prec;
    b->count = count;
    b->probs.assign(problems, problems + count);
    b->row_ptr_h.resize(count);
    b->bucket.resize(count);
    b->vec.resize(count);
    auto bail = [&](gcoo_status s) {
        delete b;
        return s;
    };
    // device problem table, BF16 workspace
    std::vector<BatchProb> hp(count);
    std::vector<ConvSeg> segs;
    std::vector<int64_t> bf_off(count, 0);
    int64_t bf_total = 0;
    for (int32_t i = 0; i < count; ++i) {
        const gcoo_problem &p = problems[i];
        b->vec[i] = prec == GCOO_PREC_BF16 ? pick_vec_bf16(p.n, p.dC) : pick_vec(p.n, p.dB, p.dC);
        b->bucket[i] = batch_bucket(p);
        if (prec == GCOO_PREC_BF16) {
            bf_off[i] = bf_total;
            bf_total += (p.a->k * p.n + 15) / 16 * 16;
        }
    }
    if (prec == GCOO_PREC_BF16 && !b->bf_ws.ensure(static_cast<size_t>(bf_total)))
        return bail(fail(GCOO_ERROR_ALLOC, "device allocation of the BF16 workspace failed"));
    for (int32_t i = 0; i < count; ++i) {
        const gcoo_problem &p = problems[i];
        hp[i] = BatchProb{p.a->packed.ptr, p.a->row_ptr.ptr, p.dB, prec == GCOO_PREC_BF16 ? b->bf_ws.ptr + bf_off[i] : nullptr,
                          p.dC, p.n};
        if (prec == GCOO_PREC_BF16)
            segs.push_back(ConvSeg{p.dB, b->bf_ws.ptr + bf_off[i], p.a->k * p.n / 4});
        b->row_ptr_h[i].resize(p.a->m + 1);
    }
    if (!b->d_probs.ensure(count) || !b->counter.ensure(1) || (prec == GCOO_PREC_BF16 && !b->d_segs.ensure(segs.size())))
        return bail(fail(GCOO_ERROR_ALLOC, "device allocation of the batch tables failed"));
    cudaError_t e = cudaMemcpyAsync(b->d_probs.ptr, hp.data(), sizeof(BatchProb) * count, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess && !segs.empty())
        e = cudaMemcpyAsync(b->d_segs.ptr, segs.data(), sizeof(ConvSeg) * segs.size(), cudaMemcpyHostToDevice, st);
    for (int32_t i = 0; i < count && e == cudaSuccess; ++i)
        e = cudaMemcpyAsync(b->row_ptr_h[i].data(), problems[i].a->row_ptr.ptr, sizeof(int32_t) * (problems[i].a->m + 1),
                            cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(st);
    if (e != cudaSuccess)
        return bail(cuda_fail(e, "batch table upload"));
    int per_sm = 0, dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (prec == GCOO_PREC_BF16)
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, batch_kernel<true>, kBatchThreads, 0);
    else
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, batch_kernel<false>, kBatchThreads, 0);
    b->grid = std::max(1, sms) * std::max(1, per_sm);

    if (prec == GCOO_PREC_BF16) { // the tuning runs below read the BF16 copy of B
        batch_bf16_kernel<<<dim3(64, static_cast<unsigned>(segs.size())), 256, 0, st>>>(b->d_segs.ptr);
        count_launches(1);
    }
    // rows_per_item per shape bucket: from the table, else timed on the bucket's items
    std::map<std::string, std::vector<int>> by_bucket;
    for (int32_t i = 0; i < count; ++i)
        by_bucket[b->bucket[i]].push_back(i);
    std::map<std::string, ItemShape> shapes;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
        if (e0)
            cudaEventDestroy(e0);
        return bail(fail(GCOO_ERROR_CUDA, "event creation for batch tuning failed"));
    }
    for (auto &kv : by_bucket) {
        const std::string key = kv.first + (prec == GCOO_PREC_BF16 ? "_bf16" : "_fp32");
        TuneEntry te;
        if (tune_lookup(key, &te) && te.rows_per_item > 0) {
            shapes[kv.first] = ItemShape{te.rows_per_item, te.vec > 0 ? te.vec : 8};
            continue;
        }
        int vmax = 1;
        for (int i : kv.second)
            vmax = std::max(vmax, b->vec[i]);
        float best = 1e30f;
        ItemShape best_sh{16, vmax};
        for (int vc : {vmax, vmax / 2})
            for (int r : {4, 8, 16, 32, 64}) {
            if (vc < 1 || (vc == vmax / 2 && vmax == 1))
                continue;
            const ItemShape sh{r, vc};
            std::map<std::string, ItemShape> one = {{kv.first, sh}};
            std::vector<BatchItem> items;
            make_items(*b, kv.second, one, items);
            const gcoo_status us = upload_items(*b, items, st);
            if (us != GCOO_SUCCESS) {
                cudaEventDestroy(e0);
                cudaEventDestroy(e1);
                return bail(us);
            }
            float ms_min = 1e30f;
            for (int rep = 0; rep < 3; ++rep) {
                cudaMemsetAsync(b->counter.ptr, 0, sizeof(unsigned), st);
                cudaEventRecord(e0, st);
                launch_batch(*b, st);
                cudaEventRecord(e1, st);
                cudaEventSynchronize(e1);
                float ms = 0.f;
                cudaEventElapsedTime(&ms, e0, e1);
                ms_min = std::min(ms_min, ms);
            }
            if (ms_min < best) {
                best = ms_min;
                best_sh = sh;
            }
        }
        shapes[kv.first] = best_sh;
        te = TuneEntry();
        te.rows_per_item = best_sh.rows;
        te.vec = best_sh.vec_cap;
        te.us = best * 1e3;
        tune_store(key, te);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    e = cudaGetLastError();
    if (e != cudaSuccess)
        return bail(cuda_fail(e, "batch tuning"));
    std::vector<int> all(count);
    for (int32_t i = 0; i < count; ++i)
        all[i] = i;
    std::vector<BatchItem> items;
    make_items(*b, all, shapes, items);
    gcoo_status s = upload_items(*b, items, st);
    if (s != GCOO_SUCCESS)
        return bail(s);
    e = cudaStreamSynchronize(st);
    if (e != cudaSuccess)
        return bail(cuda_fail(e, "batch queue upload"));

    // capture [reset counter, (B -> BF16), persistent kernel] once
    e = cudaStreamCreateWithFlags(&b->cap, cudaStreamNonBlocking);
    if (e == cudaSuccess)
        e = cudaStreamBeginCapture(b->cap, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
        cudaMemsetAsync(b->counter.ptr, 0, sizeof(unsigned), b->cap);
        if (prec == GCOO_PREC_BF16)
            batch_bf16_kernel<<<dim3(64, static_cast<unsigned>(segs.size())), 256, 0, b->cap>>>(b->d_segs.ptr);
        if (prec == GCOO_PREC_BF16)
            batch_kernel<true><<<b->grid, kBatchThreads, 0, b->cap>>>(b->d_probs.ptr, b->d_items.ptr, b->nitems, b->counter.ptr);
        else
            batch_kernel<false><<<b->grid, kBatchThreads, 0, b->cap>>>(b->d_probs.ptr, b->d_items.ptr, b->nitems, b->counter.ptr);
        e = cudaStreamEndCapture(b->cap, &b->graph);
    }
    if (e == cudaSuccess)
        e = cudaGraphInstantiate(&b->exec, b->graph, 0);
    if (e != cudaSuccess)
        return bail(cuda_fail(e, "batch graph capture"));
    *out = b;
    return GCOO_SUCCESS;
}

gcoo_status gcoo_batch_run(gcoo_batch *b, void *stream)
{
    NvtxRange nvtx("gcoo_batch_run");
    if (!b || !b->exec)
        return fail(GCOO_ERROR_INVALID_VALUE, "batch is NULL or not created");
    GCOO_CUDA(cudaGraphLaunch(b->exec, static_cast<cudaStream_t>(stream)));
    count_launches(b->prec == GCOO_PREC_BF16 ? 2 : 1);
    return GCOO_SUCCESS;
}

gcoo_status gcoo_batch_launches(const gcoo_batch *b, int32_t *launches)
{
    if (!b || !launches)
        return fail(GCOO_ERROR_INVALID_VALUE, "NULL argument");
    *launches = b->prec == GCOO_PREC_BF16 ? 2 : 1;
    return GCOO_SUCCESS;
}

gcoo_status gcoo_batch_destroy(gcoo_batch *b)
{
    delete b;
    return GCOO_SUCCESS;
}

} // extern "C"
