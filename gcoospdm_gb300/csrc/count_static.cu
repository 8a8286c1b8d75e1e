// count_static.cu -- gcoo_convert_count_static: the count + exclusive scan of
// the conversion (what gcoo_convert_count does) without allocating anything.
//
// Who needs it: callers that may not allocate device memory at the moment
// they convert -- for example a host whose device memory is handed out
// entirely by another runtime's pool (a stray cudaMalloc there fails or
// fragments the pool), a latency-bound serving loop that must not pay the
// implicit device-wide synchronisation cudaMalloc / cudaFree can cause, or a
// foreign-language caller whose binding exposes no allocator to this
// library. They pass the input and the two output arrays; the per-row counts
// and the scan's block sums live in a fixed array compiled into the library.
//
// The array is a file-scope __device__ object of kStaticScratchBytes
// (about 4.2 MB): every GPU that loads the library holds it until the process
// exits. It bounds the problem to m <= kStaticMaxRows rows (2^20); larger m
// is rejected with GCOO_ERROR_INVALID_VALUE before anything is launched.
//
// Set-up: host code cannot use the array's name as a device address (on the
// host it names a host-side shadow), so the first call on each device, with
// that device current, looks the address up once with cudaGetSymbolAddress
// and caches it per device, together with the id of the CUDA context it was
// found in. A later call in another context on that device (after
// cudaDeviceReset, or once the primary context was released and created
// again, when the module is loaded anew and the array may move) looks it up
// again. Make the first call on a device, and the first after such a reset,
// outside any stream capture.
//
// Sharing: all calls on a device use the same array, and it keeps whatever
// the previous call left. Nothing in it has to start at zero -- each call
// writes every count and every block sum before reading it -- but calls
// whose kernels overlap on the GPU (different streams, no ordering) race on
// the array: order them, or use gcoo_convert_count.
#include <cuda.h>

#include <mutex>

#include "internal.cuh"

namespace gcoo {

namespace {

constexpr int64_t kStaticMaxRows = int64_t(1) << 20;
constexpr size_t kCountsBytes = ((sizeof(int32_t) * (kStaticMaxRows + 1)) + 255) / 256 * 256;
constexpr size_t kSumsElems = (kStaticMaxRows + 4095) / 4096 + 2; // block sums, one spare, the total
constexpr size_t kStaticScratchBytes = kCountsBytes + sizeof(int64_t) * kSumsElems;

static __device__ __align__(256) unsigned char g_count_scratch[kStaticScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
struct ScratchAddr {
    unsigned char *ptr = nullptr;
    unsigned long long ctx_id = 0; // context the address was looked up in (0: unknown)
};
ScratchAddr g_scratch[kMaxDevices];

// Unique id of the calling thread's current CUDA context, 0 when there is none
// or the driver cannot say (the address is then looked up on every call).
// The driver functions come through the runtime's entry-point query, so the
// library links no driver library.
unsigned long long current_context_id()
{
    using GetCurrent = CUresult (*)(CUcontext *);
    using GetId = CUresult (*)(CUcontext, unsigned long long *);
    static GetCurrent get_current = nullptr;
    static GetId get_id = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        cudaDriverEntryPointQueryResult q;
        void *f = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_current = reinterpret_cast<GetCurrent>(f);
        f = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_id = reinterpret_cast<GetId>(f);
    });
    CUcontext ctx = nullptr;
    unsigned long long id = 0;
    if (!get_current || !get_id || get_current(&ctx) != CUDA_SUCCESS || !ctx || get_id(ctx, &id) != CUDA_SUCCESS)
        return 0;
    return id;
}

gcoo_status scratch_for_current_device(unsigned char **out)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess)
        return cuda_fail(e, "cudaGetDevice");
    if (dev < 0 || dev >= kMaxDevices)
        return fail(GCOO_ERROR_UNSUPPORTED, "device ordinal beyond the static scratch table");
    std::lock_guard<std::mutex> lock(g_mu);
    ScratchAddr &c = g_scratch[dev];
    const unsigned long long id = current_context_id();
    if (!c.ptr || id == 0 || id != c.ctx_id) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_count_scratch); // loads the module into the current context if needed
        if (e != cudaSuccess || !p)
            return cuda_fail(e != cudaSuccess ? e : cudaErrorInvalidSymbol, "cudaGetSymbolAddress(g_count_scratch)");
        c.ptr = static_cast<unsigned char *>(p);
        c.ctx_id = current_context_id(); // the context exists now, if it did not before
    }
    *out = c.ptr;
    return GCOO_SUCCESS;
}

} // namespace

} // namespace gcoo

using namespace gcoo;

extern "C" gcoo_status gcoo_convert_count_static(const float *dA, int64_t m, int64_t k, int32_t rows_per_group,
                                                 int32_t *d_group_index, int32_t *d_nnz_per_group, int64_t *nnz,
                                                 void *stream)
{
    if (!dA || !d_group_index || !d_nnz_per_group || !nnz)
        return fail(GCOO_ERROR_INVALID_VALUE, "NULL argument");
    if (m <= 0 || k <= 0 || k >= (int64_t(1) << 31))
        return fail(GCOO_ERROR_INVALID_VALUE, "m and k must be positive and k must fit int32 indices");
    if (m > kStaticMaxRows)
        return fail(GCOO_ERROR_INVALID_VALUE, "m = " + std::to_string(m) + " exceeds the static scratch limit of " +
                                                  std::to_string(kStaticMaxRows) + " rows; use gcoo_convert_count");
    if (rows_per_group != 1 && rows_per_group != 2 && rows_per_group != 4 && rows_per_group != 8 &&
        rows_per_group != 16 && rows_per_group != 32)
        return fail(GCOO_ERROR_INVALID_VALUE, "rows_per_group must be a power of two in [1, 32]");
    unsigned char *scratch = nullptr;
    gcoo_status s = scratch_for_current_device(&scratch);
    if (s != GCOO_SUCCESS)
        return s;
    int32_t *counts = reinterpret_cast<int32_t *>(scratch);
    int64_t *sums = reinterpret_cast<int64_t *>(scratch + kCountsBytes);
    const size_t sc = scan_scratch_elems(m); // <= kSumsElems - 1
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    GCOO_CUDA(launch_row_count(dA, m, k, counts, st));
    GCOO_CUDA(launch_row_scan(counts, m, rows_per_group, d_group_index, d_nnz_per_group, sums + sc, sums, nullptr, st));
    int64_t total = 0;
    GCOO_CUDA(cudaMemcpyAsync(&total, sums + sc, sizeof(total), cudaMemcpyDeviceToHost, st));
    GCOO_CUDA(cudaStreamSynchronize(st));
    *nnz = total;
    if (total > 0x7fffffffLL)
        return fail(GCOO_ERROR_FORMAT, "nnz exceeds the int32 GCOO format");
    return GCOO_SUCCESS;
}
