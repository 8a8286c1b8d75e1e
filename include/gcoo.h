/*
 * gcoo.h -- C ABI of the GB300 (sm_103a) GCOO sparse x dense multiply.
 *
 * Drop-in boundary for the reference's -algo=gcoospdm path (hclhkbu/gcoospdm):
 * the C++ plugin classes in ShGemm.h / ShGCOOSpDM.h / SpGemmBuilder.h are thin
 * shims over these entry points, and any FFI (ctypes, cgo, JNI) can bind them
 * directly. Plain pointers and sizes only; every device pointer is a CUDA
 * device address on the current device; `stream` is a cudaStream_t (NULL =
 * legacy default stream).
 *
 * Orientation (row-major, as the reference kernel indexes its operands):
 *   A  m x k sparse operand, given as a dense FP32 buffer holding zeros
 *      (the reference ctor's `denseMatrix`, src/ShGCOOSpDM.cu:13-17)
 *   B  k x n dense FP32 (the `A` argument of mutiplyBy, src/ShGCOOSpDM.cu:131)
 *   C  m x n FP32, C[r*n+j] = sum_c A[r*k+c] * B[c*n+j]
 *
 * GCOO format (src/ShGCOOSpDM.h:25-32, src/gcoo_spdm_kernels.cu:30-90): rows
 * are grouped `rows_per_group` at a time (the reference's COLUMN_PER_GROUP,
 * 4); nGroup = ceil(m / rows_per_group); group_index[nGroup+1] is the
 * exclusive prefix of nnz_per_group[nGroup+1] (whose last entry is 0); inside
 * a group the entries are ordered by column, then row; rows are absolute.
 * A value is an entry iff `v != 0` (-0.0 is dropped, NaN is kept).
 *
 * Errors: every call returns a gcoo_status; nothing exits or throws.
 * gcoo_last_error() gives a message for the last failure on this thread.
 * Threading: a handle is not thread-safe; distinct handles may be used
 * concurrently from different threads and streams.
 */
#ifndef GCOO_H
#define GCOO_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GCOO_ABI_VERSION 1

typedef enum gcoo_status {
    GCOO_SUCCESS = 0,
    GCOO_ERROR_INVALID_VALUE = 1, /* null pointer, bad size, overflow     */
    GCOO_ERROR_ALLOC = 2,         /* device allocation failed             */
    GCOO_ERROR_CUDA = 3,          /* a CUDA call or kernel launch failed  */
    GCOO_ERROR_NOT_BUILT = 4,     /* multiply before gcoo_build           */
    GCOO_ERROR_UNSUPPORTED = 5,   /* request this library cannot serve    */
    GCOO_ERROR_FORMAT = 6,        /* nnz does not fit the int32 format    */
    GCOO_ERROR_TIMEOUT = 7,       /* a bounded device wait gave up        */
    GCOO_ERROR_CAPACITY = 8       /* caller-provided buffer too small     */
} gcoo_status;

/* Arithmetic forms of the multiply. All accumulate in FP32 and write FP32 C. */
typedef enum gcoo_precision {
    GCOO_PREC_FP32 = 0,       /* plain form; bit-identical to the reference  */
    GCOO_PREC_BF16 = 1,       /* A values and B rounded to BF16              */
    GCOO_PREC_SPLIT_BF16 = 2, /* hi+lo BF16 split, three products            */
    GCOO_PREC_FP8_B = 3       /* B as FP8 E4M3 with per-column scales        */
} gcoo_precision;

/* Which execution engine a non-FP32 form may use. */
typedef enum gcoo_engine {
    GCOO_ENGINE_AUTO = 0,      /* tensor cores where 16-wide blocks densify */
    GCOO_ENGINE_CUDA_CORE = 1, /* FMA pipes only                             */
    GCOO_ENGINE_TENSOR = 2     /* tcgen05 tensor cores                       */
} gcoo_engine;

/* Runtime replacement of the reference's compile-time tile constants
 * (src/constants.h:4-5, filled by src/autotune.py from constants.h.t). */
typedef struct gcoo_params {
    int32_t rows_per_group; /* GCOO group height (reference: 4), 1..32     */
    int32_t vec;            /* output columns per thread: 0 auto, 1, 2, 4   */
    int32_t warps;          /* warps per CTA: 0 auto, 1..32                 */
    int32_t col_warps;      /* warps side by side on one row: 0 auto        */
    int32_t engine;         /* gcoo_engine for non-FP32 forms               */
    int32_t depth;          /* B-load pipelining: 0 auto, 1 off, 2 on        */
    int32_t fp32_order;     /* walk of the FP32 multiply and of the BF16 /
                               FP8-B forms on the FMA engine: 0 auto, 1 rows
                               (packed row order), 2 groups (GCOO order, one
                               B load per column shared by a group's rows;
                               groups of 4 rows). Both give the same bits. */
    int32_t fp32_sum;       /* gcoo_fp32_sum: summation of the FP32
                               multiply's long rows (at least 256 entries,
                               skewed matrices only)                      */
} gcoo_params;

/* FP32 summation order. CHAIN (the default): every output element is one
 * sequential fmaf chain over its row's entries in column order from 0.0f,
 * the reference kernel's order (src/gcoo_spdm_kernels.cu:129-139), so results
 * are bit-identical to the reference's. SPLIT: in a skewed matrix (longest
 * row >= 256 entries and above 8x the mean) the rows of >= 256 entries are
 * summed as chains over pieces of 32 consecutive entries whose partial sums
 * are then added in piece order: deterministic (the same bits on every run),
 * not bit-identical to CHAIN, within FP32 rounding of the exact product
 * (relative Frobenius error against FP64 of the order of 1e-7). Shorter rows
 * and matrices that are not skewed keep the chain. */
typedef enum gcoo_fp32_sum { GCOO_SUM_CHAIN = 0, GCOO_SUM_SPLIT = 1 } gcoo_fp32_sum;

typedef struct gcoo_handle gcoo_handle;

/* Device views of a handle's GCOO arrays (owned by the handle). */
typedef struct gcoo_view {
    int64_t m, k, nnz, n_group;
    int32_t rows_per_group;
    const int32_t *group_index;   /* [n_group + 1]                         */
    const int32_t *nnz_per_group; /* [n_group + 1], last entry 0           */
    const float *vals;            /* [nnz]                                 */
    const int32_t *rows;          /* [nnz]                                 */
    const int32_t *cols;          /* [nnz]                                 */
} gcoo_view;

/* ---- status, version ---------------------------------------------------- */
int gcoo_abi_version(void);
const char *gcoo_status_string(gcoo_status s);
const char *gcoo_last_error(void);

/* Defaults: rows_per_group 4 (the reference's COLUMN_PER_GROUP), the rest
 * chosen per shape at launch. */
gcoo_status gcoo_params_default(gcoo_params *p);

/* Device allocator used for every buffer a handle owns (NULL, NULL restores
 * cudaMalloc/cudaFree). Lets a host framework pool memory, and lets tests
 * inject allocation failures. Not thread-safe; set it before creating
 * handles. */
typedef void *(*gcoo_alloc_fn)(size_t bytes, void *ctx);
typedef void (*gcoo_free_fn)(void *ptr, void *ctx);
gcoo_status gcoo_set_allocator(gcoo_alloc_fn alloc, gcoo_free_fn release, void *ctx);

/* ---- the plugin path ----------------------------------------------------- */

/* ShGCOOSpDM(denseMatrix, nRows, nCols) (src/ShGCOOSpDM.cu:13-17): records
 * the dense sparse operand; nothing runs on the GPU. The handle does not own
 * dA, which must stay valid while the handle builds from it. */
gcoo_status gcoo_create(gcoo_handle **out, const float *dA, int64_t m, int64_t k,
                        const gcoo_params *params);

/* Sparse-input ingestion. The reference reaches GCOO only through a dense
 * buffer (its Matrix Market reader densifies in file order,
 * src/MatrixReader.cpp:11-84); this handle instead takes nnz COO triplets on
 * the device (0-based, any order, not owned: they must stay valid while the
 * handle builds from them). gcoo_build then yields exactly the arrays that
 * writing the triplets into a zero m x k buffer in order (a later duplicate
 * overwrites an earlier one) and converting it would give, without that
 * buffer. An out-of-range index makes gcoo_build fail with
 * GCOO_ERROR_INVALID_VALUE. */
gcoo_status gcoo_create_coo(gcoo_handle **out, int64_t m, int64_t k, const int32_t *d_rows,
                            const int32_t *d_cols, const float *d_vals, int64_t nnz,
                            const gcoo_params *params);

/* The reference driver's -file= input (src/MatrixReader.cpp:11-84): a
 * Matrix Market file read on the host into COO triplets for
 * gcoo_create_coo (copied to the device by the caller), without a dense
 * m x k buffer. Coordinate format; real, integer or pattern values;
 * general, symmetric or skew-symmetric. Indices become 0-based; triplets
 * keep the file's order with each mirror right after its entry, so a later
 * duplicate wins as in the reference's dense buffer. Pattern entries are
 * 1.0 (the reference draws unseeded rand() values) and a skew-symmetric
 * mirror is negated (the reference copies it unchanged). The three arrays
 * are allocated here; release each with gcoo_free_host. Errors:
 * GCOO_ERROR_INVALID_VALUE for a missing, malformed or truncated file or an
 * index out of range, GCOO_ERROR_UNSUPPORTED for the array format, complex
 * values or hermitian symmetry, GCOO_ERROR_FORMAT beyond int32. */
gcoo_status gcoo_read_matrix_market(const char *path, int64_t *m, int64_t *k, int64_t *count,
                                    int32_t **rows, int32_t **cols, float **vals);
void gcoo_free_host(void *p);

/* build() (src/ShGCOOSpDM.cu:182-193): dense -> GCOO conversion into
 * handle-owned arrays (count, device exclusive scan, stable scatter). Reads
 * the total nnz back to size the arrays, so it synchronises `stream` once
 * (twice for a matrix with skewed row lengths, whose long rows it lists).
 * Calling it again re-converts (dA may have changed); a rebuild whose arrays
 * have room reads dA once. A matrix of more than 2^31 - 1 nonzeros does not
 * fit the format's int32 offsets: refused with GCOO_ERROR_FORMAT before any
 * entry is written, leaving the handle unbuilt. */
gcoo_status gcoo_build(gcoo_handle *h, void *stream);

gcoo_status gcoo_export(const gcoo_handle *h, gcoo_view *out);

/* runKernelTest() (src/ShGCOOSpDM.cu:195-213): C = A * B with the GCOO
 * built by gcoo_build, FP32 form. No allocation, no synchronisation; safe
 * to capture in a CUDA graph. dB is k x n, dC is m x n, row-major. For a
 * matrix with skewed row lengths the long rows run on a handle-owned stream
 * forked from `stream` and joined back into it before the call returns.
 * Column tiles lie along the grid's y dimension, as in the reference's
 * launch (src/ShGCOOSpDM.cu:153): n up to 65535 tiles of the chosen shape
 * (16.7 M columns at the default shape when n % 4 == 0, more where short
 * rows walk several tiles per CTA); wider B fails with GCOO_ERROR_CUDA
 * before any launch. */
gcoo_status gcoo_spdm(gcoo_handle *h, const float *dB, int64_t n, float *dC, void *stream);

/* The same multiply in another arithmetic form. The first call for a form
 * (or a larger n) sizes that form's workspace and, for the tensor-core
 * engine, builds the densified block tiles: allocation and one
 * synchronisation happen then, never on later calls of the same shape. */
gcoo_status gcoo_spdm_ex(gcoo_handle *h, const float *dB, int64_t n, float *dC,
                         gcoo_precision prec, void *stream);

/* Prepares a form's workspace and tiles for width n without multiplying, so
 * that later gcoo_spdm_ex calls can be captured in a CUDA graph. */
gcoo_status gcoo_prepare(gcoo_handle *h, int64_t n, gcoo_precision prec, void *stream);

/* mutiplyBy() (src/ShGCOOSpDM.cu:131-180): conversion + multiply in one call
 * (FP32). Reuses the handle's arrays when they are large enough, so a steady
 * loop allocates nothing; it synchronises once to read the nnz, as the
 * reference does. */
gcoo_status gcoo_multiply_by(gcoo_handle *h, const float *dB, int64_t n, float *dC, void *stream);

gcoo_status gcoo_destroy(gcoo_handle *h);

/* mutiply() (src/ShGemm.h:16; the reference's GCOO plugin leaves it empty,
 * src/ShGCOOSpDM.h:21): the other orientation, C = D x A with D dense p x m
 * and C p x k (row-major), FP32, each C element a sequential fmaf chain over
 * A's rows in ascending order. The first call (or a larger p) builds A's
 * column-order layout and sizes the transposed operands: allocation and one
 * synchronisation then, none on later calls of the same width. */
gcoo_status gcoo_spdm_left(gcoo_handle *h, const float *dD, int64_t p, float *dC, void *stream);

/* Form the handle would use for `prec` at width n: writes 1 to *tensor when
 * the tcgen05 block path is taken. Builds nothing. */
gcoo_status gcoo_query_engine(gcoo_handle *h, gcoo_precision prec, int32_t *tensor);

/* No counterpart in the reference (it has no bounded waits). Runs the
 * library's bounded mbarrier wait on a barrier nothing arrives on, with a
 * limit of limit_ns (<= 2e9): returns GCOO_ERROR_TIMEOUT when the wait gave
 * up and reported it, as it must; the context stays usable. */
gcoo_status gcoo_check_bounded_wait(uint64_t limit_ns, void *stream);

/* No counterpart in the reference (it has no checks). Validates a built
 * handle's arrays on the GPU: group_index / nnz_per_group / row pointers
 * consistent, entries in (column, row) order inside their group, columns in
 * [0, k), values nonzero, each row's execution-layout entries in ascending
 * columns and the same entries as the GCOO arrays. Reads only in bounds,
 * whatever the arrays hold. Returns GCOO_ERROR_FORMAT and the number of
 * offending groups in *bad_groups (may be NULL) when any check fails.
 * Synchronises `stream`. */
gcoo_status gcoo_check_arrays(gcoo_handle *h, void *stream, int64_t *bad_groups);

/* Number of kernels this library has launched in this process (all
 * handles, all entry points); lets a caller count launches in a region. */
uint64_t gcoo_kernel_launches(void);

/* Device status word of the handle's kernels (0 = fine; bit 1: a bounded
 * wait gave up; bit 2: an index check failed). Synchronises `stream`. */
gcoo_status gcoo_device_status(gcoo_handle *h, void *stream, uint32_t *status);

/* ---- conversion and multiply on caller-owned arrays ------------------------ */

/* Count + exclusive scan of convertToGroupCOOFormat (src/ShGCOOSpDM.cu:
 * 33-84): fills group_index and nnz_per_group ([n_group+1] each) and returns
 * the total in *nnz (synchronises `stream`). */
gcoo_status gcoo_convert_count(const float *dA, int64_t m, int64_t k, int32_t rows_per_group,
                               int32_t *d_group_index, int32_t *d_nnz_per_group, int64_t *nnz,
                               void *stream);

/* No counterpart in the reference. Same count + scan and same results as
 * gcoo_convert_count, for callers that cannot allocate device memory when
 * they convert (memory owned by another runtime's pool, loops that must not
 * pay cudaMalloc's implicit synchronisation, bindings without an allocator):
 * it allocates nothing and keeps its per-row counts and block sums in a
 * fixed ~4.2 MB __device__ array held by every GPU that loads the library.
 * Limit: m <= 2^20 rows (larger m -> GCOO_ERROR_INVALID_VALUE). The first
 * call on a device looks up that array's address and caches it with the
 * current context's id; the first call after cudaDeviceReset (or in a new
 * primary context) looks it up again. Make those calls before any stream
 * capture. All calls share the array, so calls that overlap on the GPU race.
 * Synchronises `stream` to return *nnz. */
gcoo_status gcoo_convert_count_static(const float *dA, int64_t m, int64_t k, int32_t rows_per_group,
                                      int32_t *d_group_index, int32_t *d_nnz_per_group, int64_t *nnz,
                                      void *stream);

/* Stable scatter of convertToGroupCOOFormat (src/ShGCOOSpDM.cu:94-111,
 * src/gcoo_spdm_kernels.cu:30-90) into caller arrays of at least nnz
 * entries, using a group_index produced by gcoo_convert_count. */
gcoo_status gcoo_convert_scatter(const float *dA, int64_t m, int64_t k, int32_t rows_per_group,
                                 const int32_t *d_group_index, float *d_vals, int32_t *d_rows,
                                 int32_t *d_cols, void *stream);

/* sparse_dense_groupcoo_mat_mul_kernel (src/gcoo_spdm_kernels.cu:92-158) on
 * caller-owned GCOO arrays in the reference layout, FP32, any
 * rows_per_group; result bit-identical to gcoo_spdm. */
gcoo_status gcoo_spdm_view(const gcoo_view *a, const float *dB, int64_t n, float *dC, void *stream);

/* ---- checks ---------------------------------------------------------------- */

/* Relative Frobenius error ||C - A*B||_F / ||A*B||_F with A*B accumulated in
 * FP64 on the GPU (the only FP64 work in the library). Synchronises. */
gcoo_status gcoo_error_norm(gcoo_handle *h, const float *dB, int64_t n, const float *dC,
                            double *rel_fro, void *stream);

/* ---- batched, persistent ---------------------------------------------------- */

typedef struct gcoo_problem {
    gcoo_handle *a; /* built handle */
    const float *dB;
    int64_t n;
    float *dC;
} gcoo_problem;

typedef struct gcoo_batch gcoo_batch;

/* Plans many independent multiplies for one persistent launch: work items
 * (problem, group range, column tile) sorted by nnz, descending, in a device
 * queue; tile parameters per shape bucket from the autotune table when one is
 * loaded, else timed here by running the batch's items (which writes the
 * problems' C) and stored in the table. prec: GCOO_PREC_FP32 or
 * GCOO_PREC_BF16. Allocates; synchronises. */
gcoo_status gcoo_batch_create(gcoo_batch **out, const gcoo_problem *problems, int32_t count,
                              gcoo_precision prec, void *stream);

/* One persistent launch over the whole queue (replayed from a CUDA graph
 * after the first call). No allocation. */
gcoo_status gcoo_batch_run(gcoo_batch *b, void *stream);

/* Number of kernel launches one gcoo_batch_run performs. */
gcoo_status gcoo_batch_launches(const gcoo_batch *b, int32_t *launches);

gcoo_status gcoo_batch_destroy(gcoo_batch *b);

/* ---- multiply from host buffers, pipelined ------------------------------------ */

/* No counterpart in the reference, whose plugin takes device buffers
 * (src/ShGemm.h:11-14) and whose driver copies A and B in and C out around it
 * (src/main.cu:23-40,86-89). A session is mutiplyBy for operands that live in
 * host memory: A is moved in row panels, each panel converted and multiplied
 * as soon as it and B are on the device, and each panel of C copied back while
 * the next panels are in flight (copy-in, compute and copy-out on their own
 * streams). The FP32 results are the same bits as gcoo_multiply_by. */
typedef struct gcoo_session gcoo_session;

/* panel_rows: rows of A per panel (rounded up to rows_per_group); 0 picks
 * eighth-of-A panels, with a quarter-size panel first and halving ones at
 * the end (about a dozen in all). Allocates nothing until the first
 * multiply. */
gcoo_status gcoo_session_create(gcoo_session **out, const gcoo_params *params, int64_t panel_rows);

/* C = A x B, A m x k, B k x n, C m x n, all row-major FP32 in HOST memory
 * (page-locked memory moves at full link speed; pageable memory works, more
 * slowly). Device buffers grow to the largest call and are reused, so a
 * steady loop allocates nothing. Work is ordered after what was queued on
 * `stream` before the call; returns once C is complete on the host, and on
 * an error only once nothing of the call is still running. A panel is
 * scattered without a readback, so k of about 2^31 / rows_per_group
 * columns or more, where one panel could exceed the int32 format, is
 * refused with GCOO_ERROR_UNSUPPORTED (gcoo_build takes such matrices). */
gcoo_status gcoo_session_multiply(gcoo_session *s, const float *hA, int64_t m, int64_t k, const float *hB,
                                  int64_t n, float *hC, void *stream);

/* Kernel launches and panels of the last gcoo_session_multiply. */
gcoo_status gcoo_session_stats(const gcoo_session *s, int32_t *launches, int32_t *panels);

gcoo_status gcoo_session_destroy(gcoo_session *s);

/* ---- autotuner ---------------------------------------------------------------- */

/* Times the candidate (vec, warps, col_warps) settings for this handle at
 * width n (FP32 form) on `stream` and stores the fastest in the in-process
 * table under the shape bucket of (m, k, nnz, n). Writes the winner to
 * *best when not NULL. Synchronises. */
gcoo_status gcoo_autotune(gcoo_handle *h, const float *dB, int64_t n, float *dC, void *stream,
                          gcoo_params *best);

/* Persist / load the table as JSON (one object per bucket). */
gcoo_status gcoo_autotune_save(const char *path);
gcoo_status gcoo_autotune_load(const char *path);
gcoo_status gcoo_autotune_clear(void);

#ifdef __cplusplus
}
#endif
#endif
