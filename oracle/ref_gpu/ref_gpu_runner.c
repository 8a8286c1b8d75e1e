/*
 * ref_gpu_runner.c -- TEST INFRASTRUCTURE ONLY.
 *
 * Loads the cubin that oracle/Makefile compiles from the reference's own
 * kernel file (oracle/_ref/ref_gcoo_sm103a.cubin) through the CUDA driver API
 * and drives it with the reference plugin's host orchestration, so that tests
 * can compare this library against the reference's GPU code bit for bit on the
 * same device buffers. Plain C; built on the machine that runs it (it needs
 * only cuda.h and libcuda), while the cubin is built where the reference
 * tree is.
 *
 * Orchestration restated from src/ShGCOOSpDM.cu:
 *   conversion (:19-126): memset nnzPerGroup[0..nGroup] to 0; count kernel
 *     <512, CPG> on grid nGroup x 512 threads; device sync; prefix_sum_kernel2
 *     <<<1,1>>> over nGroup+1 entries; device sync; read groupIndex[nGroup]
 *     back (the nnz); scatter kernel <512, CPG> on the same grid; device sync;
 *   multiply (:153-167): grid (nGroup, ceil(n / BS)) x BS threads, arguments
 *     (vals, cols, rows, groupIndex, nnzPerGroup, wA = k, hA = m, B, wB = n,
 *     hB = k, C); device sync.
 * Everything runs on the legacy default stream of the current context, like
 * the reference. Device pointers come from the caller.
 */
#include <cuda.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

static CUmodule g_mod;
static CUfunction g_count[5], g_scatter[5], g_prefix, g_mul, g_const;
static int g_cpg_ref, g_bs_ref;
static char g_err[512];

static int fail(const char *what, CUresult r)
{
    const char *s = NULL;
    cuGetErrorString(r, &s);
    snprintf(g_err, sizeof g_err, "%s: %s (%d)", what, s ? s : "?", (int)r);
    return (int)r ? (int)r : -1;
}

const char *refgpu_error(void) { return g_err; }

static int cpg_slot(int cpg)
{
    switch (cpg) {
    case 1: return 0;
    case 2: return 1;
    case 4: return 2;
    case 8: return 3;
    case 16: return 4;
    default: return -1;
    }
}

/* Find a kernel whose (mangled) name contains `needle`. */
static CUfunction find(const CUfunction *fns, unsigned n, const char *needle)
{
    for (unsigned i = 0; i < n; ++i) {
        const char *name = NULL;
        if (cuFuncGetName(&name, fns[i]) == CUDA_SUCCESS && name && strstr(name, needle))
            return fns[i];
    }
    return NULL;
}

/* Load the cubin into the current context (the caller's runtime context, or
 * the primary context of device 0 if none is current). */
int refgpu_load(const char *cubin_path)
{
    CUresult r;
    CUcontext ctx = NULL;
    if ((r = cuInit(0)) != CUDA_SUCCESS)
        return fail("cuInit", r);
    if ((r = cuCtxGetCurrent(&ctx)) != CUDA_SUCCESS)
        return fail("cuCtxGetCurrent", r);
    if (!ctx) {
        CUdevice dev;
        if ((r = cuDeviceGet(&dev, 0)) != CUDA_SUCCESS || (r = cuDevicePrimaryCtxRetain(&ctx, dev)) != CUDA_SUCCESS ||
            (r = cuCtxSetCurrent(ctx)) != CUDA_SUCCESS)
            return fail("primary context", r);
    }
    if (g_mod)
        return 0;
    if ((r = cuModuleLoad(&g_mod, cubin_path)) != CUDA_SUCCESS)
        return fail("cuModuleLoad", r);
    unsigned n = 0;
    if ((r = cuModuleGetFunctionCount(&n, g_mod)) != CUDA_SUCCESS)
        return fail("cuModuleGetFunctionCount", r);
    CUfunction fns[64];
    if (n > 64)
        n = 64;
    if ((r = cuModuleEnumerateFunctions(fns, n, g_mod)) != CUDA_SUCCESS)
        return fail("cuModuleEnumerateFunctions", r);
    static const char *cpgs[5] = {"Li1E", "Li2E", "Li4E", "Li8E", "Li16E"};
    for (int i = 0; i < 5; ++i) {
        char a[128], b[128];
        snprintf(a, sizeof a, "cal_group_coo_format_nnz_kernel_cmILi512E%sE", cpgs[i]);
        snprintf(b, sizeof b, "convert_to_group_coo_format_kernel_cmILi512E%sE", cpgs[i]);
        g_count[i] = find(fns, n, a);
        g_scatter[i] = find(fns, n, b);
        if (!g_count[i] || !g_scatter[i]) {
            snprintf(g_err, sizeof g_err, "conversion kernels for CPG slot %d not in the cubin", i);
            return -1;
        }
    }
    g_prefix = find(fns, n, "prefix_sum_kernel2");
    g_mul = find(fns, n, "sparse_dense_groupcoo_mat_mul_kernel");
    g_const = find(fns, n, "ref_gcoo_constants");
    if (!g_prefix || !g_mul || !g_const) {
        snprintf(g_err, sizeof g_err, "reference kernels missing from the cubin");
        return -1;
    }
    /* the multiply instance's constants, read once */
    CUdeviceptr d = 0;
    int h[2] = {0, 0};
    if ((r = cuMemAlloc(&d, sizeof h)) != CUDA_SUCCESS)
        return fail("cuMemAlloc", r);
    void *args[] = {&d};
    r = cuLaunchKernel(g_const, 1, 1, 1, 1, 1, 1, 0, NULL, args, NULL);
    if (r == CUDA_SUCCESS)
        r = cuMemcpyDtoH(h, d, sizeof h);
    cuMemFree(d);
    if (r != CUDA_SUCCESS)
        return fail("constants", r);
    g_cpg_ref = h[0];
    g_bs_ref = h[1];
    return 0;
}

int refgpu_column_per_group(void) { return g_cpg_ref; }
int refgpu_bs(void) { return g_bs_ref; }

/* Conversion count + scan: fills groupIndex[0..nGroup] and
 * nnzPerGroup[0..nGroup] and returns nnz through *nnz. */
int refgpu_count_scan(int cpg, uint64_t dA, int m, int k, uint64_t dGroupIndex, uint64_t dNnzPerGroup,
                      long long *nnz)
{
    const int s = cpg_slot(cpg);
    if (s < 0 || !g_mod) {
        snprintf(g_err, sizeof g_err, "bad CPG %d or module not loaded", cpg);
        return -1;
    }
    const int nGroup = (m + cpg - 1) / cpg;
    CUresult r;
    CUdeviceptr A = (CUdeviceptr)dA, gi = (CUdeviceptr)dGroupIndex, npg = (CUdeviceptr)dNnzPerGroup;
    if ((r = cuMemsetD32(npg, 0, (size_t)nGroup + 1)) != CUDA_SUCCESS)
        return fail("memset", r);
    void *a1[] = {&A, &m, &k, &npg};
    if ((r = cuLaunchKernel(g_count[s], (unsigned)nGroup, 1, 1, 512, 1, 1, 0, NULL, a1, NULL)) != CUDA_SUCCESS)
        return fail("count launch", r);
    if ((r = cuCtxSynchronize()) != CUDA_SUCCESS)
        return fail("count", r);
    int np1 = nGroup + 1;
    void *a2[] = {&npg, &gi, &np1};
    if ((r = cuLaunchKernel(g_prefix, 1, 1, 1, 1, 1, 1, 0, NULL, a2, NULL)) != CUDA_SUCCESS)
        return fail("prefix launch", r);
    if ((r = cuCtxSynchronize()) != CUDA_SUCCESS)
        return fail("prefix", r);
    int total = 0;
    if ((r = cuMemcpyDtoH(&total, gi + (CUdeviceptr)nGroup * sizeof(int), sizeof(int))) != CUDA_SUCCESS)
        return fail("readback", r);
    *nnz = total;
    return 0;
}

/* Conversion scatter into vals[nnz], rows[nnz], cols[nnz] (after count_scan). */
int refgpu_scatter(int cpg, uint64_t dA, int m, int k, uint64_t dGroupIndex, uint64_t dNnzPerGroup, uint64_t dVals,
                   uint64_t dRows, uint64_t dCols)
{
    const int s = cpg_slot(cpg);
    if (s < 0 || !g_mod) {
        snprintf(g_err, sizeof g_err, "bad CPG %d or module not loaded", cpg);
        return -1;
    }
    const int nGroup = (m + cpg - 1) / cpg;
    CUresult r;
    CUdeviceptr A = (CUdeviceptr)dA, gi = (CUdeviceptr)dGroupIndex, npg = (CUdeviceptr)dNnzPerGroup;
    CUdeviceptr v = (CUdeviceptr)dVals, ro = (CUdeviceptr)dRows, co = (CUdeviceptr)dCols;
    void *a[] = {&A, &m, &k, &v, &ro, &co, &gi, &npg};
    if ((r = cuLaunchKernel(g_scatter[s], (unsigned)nGroup, 1, 1, 512, 1, 1, 0, NULL, a, NULL)) != CUDA_SUCCESS)
        return fail("scatter launch", r);
    if ((r = cuCtxSynchronize()) != CUDA_SUCCESS)
        return fail("scatter", r);
    return 0;
}

/* Multiply C = A_gcoo x B with the reference's compiled CPG and BS. */
int refgpu_spdm(uint64_t dVals, uint64_t dCols, uint64_t dRows, uint64_t dGroupIndex, uint64_t dNnzPerGroup, int m,
                int k, uint64_t dB, int n, uint64_t dC)
{
    if (!g_mod) {
        snprintf(g_err, sizeof g_err, "module not loaded");
        return -1;
    }
    const int nGroup = (m + g_cpg_ref - 1) / g_cpg_ref;
    const unsigned gy = (unsigned)((n + g_bs_ref - 1) / g_bs_ref);
    CUresult r;
    CUdeviceptr v = (CUdeviceptr)dVals, co = (CUdeviceptr)dCols, ro = (CUdeviceptr)dRows;
    CUdeviceptr gi = (CUdeviceptr)dGroupIndex, npg = (CUdeviceptr)dNnzPerGroup, B = (CUdeviceptr)dB,
                Cm = (CUdeviceptr)dC;
    int wA = k, hA = m, wB = n, hB = k;
    void *a[] = {&v, &co, &ro, &gi, &npg, &wA, &hA, &B, &wB, &hB, &Cm};
    if ((r = cuLaunchKernel(g_mul, (unsigned)nGroup, gy, 1, (unsigned)g_bs_ref, 1, 1, 0, NULL, a, NULL)) !=
        CUDA_SUCCESS)
        return fail("multiply launch", r);
    if ((r = cuCtxSynchronize()) != CUDA_SUCCESS)
        return fail("multiply", r);
    return 0;
}
