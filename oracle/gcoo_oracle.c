/*
 * gcoo_oracle.c -- TEST INFRASTRUCTURE ONLY (the checker and the CPU baseline).
 *
 * CPU restatement of the reference's GCOO conversion and GCOO x dense multiply
 * (hclhkbu/gcoospdm, src/gcoo_spdm_kernels.cu and src/ShGCOOSpDM.cu). See
 * gcoo_oracle.h for the contract of each function and the reference lines it
 * follows. Built with -ffp-contract=off so that the only fused multiply-adds
 * are the explicit fmaf calls that mirror the reference kernel's fmaf.
 */
#include "gcoo_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

static int64_t n_groups(int64_t m, int cpg) { return (m + cpg - 1) / cpg; }

int orc_max_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 0;
#endif
}

static int pick_threads(int nthreads)
{
#ifdef _OPENMP
    return nthreads > 0 ? nthreads : omp_get_max_threads();
#else
    (void)nthreads;
    return 1;
#endif
}

/* src/gcoo_spdm_kernels.cu:4-28: each group counts the entries of its rows
 * with v != 0.0 (so -0.0 is not counted and NaN is). */
int64_t orc_group_count(const float *A, int64_t m, int64_t k, int cpg,
                        int32_t *nnzPerGroup, int nthreads)
{
    const int64_t ng = n_groups(m, cpg);
    int64_t total = 0;
    int nt = pick_threads(nthreads);
    (void)nt;
#pragma omp parallel for schedule(static) reduction(+ : total) num_threads(nt)
    for (int64_t g = 0; g < ng; ++g) {
        int64_t cnt = 0;
        const int64_t r0 = g * cpg;
        const int64_t r1 = r0 + cpg < m ? r0 + cpg : m;
        for (int64_t r = r0; r < r1; ++r) {
            const float *row = A + r * k;
            for (int64_t c = 0; c < k; ++c)
                cnt += (row[c] != 0.0f);
        }
        nnzPerGroup[g] = (int32_t)cnt;
        total += cnt;
    }
    nnzPerGroup[ng] = 0; /* the reference memsets nGroup+1 entries */
    if (total > INT32_MAX)
        return -1;
    return total;
}

/* src/gcoo_spdm_kernels.cu:160-168 */
void orc_exclusive_scan(const int32_t *in, int64_t n, int32_t *out)
{
    if (n <= 0)
        return;
    out[0] = 0;
    for (int64_t i = 1; i < n; ++i)
        out[i] = out[i - 1] + in[i - 1];
}

/* src/gcoo_spdm_kernels.cu:30-90: the reference walks the group in column
 * tiles; inside a tile each thread owns one column and emits that column's
 * nonzeros for rows r0..r0+cpg-1 in row order at its block-scan offset, so
 * the resulting order is (column ascending, row ascending). */
void orc_scatter(const float *A, int64_t m, int64_t k, int cpg,
                 const int32_t *groupIndex, float *vals, int32_t *rows,
                 int32_t *cols, int nthreads)
{
    const int64_t ng = n_groups(m, cpg);
    int nt = pick_threads(nthreads);
    (void)nt;
#pragma omp parallel for schedule(static) num_threads(nt)
    for (int64_t g = 0; g < ng; ++g) {
        int64_t off = groupIndex[g];
        const int64_t r0 = g * cpg;
        const int64_t r1 = r0 + cpg < m ? r0 + cpg : m;
        for (int64_t c = 0; c < k; ++c) {
            for (int64_t r = r0; r < r1; ++r) {
                const float v = A[r * k + c];
                if (v != 0.0f) {
                    vals[off] = v;
                    rows[off] = (int32_t)r;
                    cols[off] = (int32_t)c;
                    ++off;
                }
            }
        }
    }
}

/* src/gcoo_spdm_kernels.cu:92-158: one accumulator per (row of the group,
 * output column), starting at 0.0f, updated with fmaf(a, b, acc) in the
 * group's storage order. */
void orc_spdm(int64_t m, int64_t k, int cpg, const int32_t *groupIndex,
              const int32_t *nnzPerGroup, const float *vals,
              const int32_t *rows, const int32_t *cols, const float *B,
              int64_t n, float *C, int nthreads)
{
    (void)k;
    const int64_t ng = n_groups(m, cpg);
    int nt = pick_threads(nthreads);
    (void)nt;
#pragma omp parallel num_threads(nt)
    {
        float *acc = (float *)malloc(sizeof(float) * (size_t)cpg * (size_t)(n > 0 ? n : 1));
#pragma omp for schedule(dynamic, 1)
        for (int64_t g = 0; g < ng; ++g) {
            const int64_t r0 = g * cpg;
            const int64_t r1 = r0 + cpg < m ? r0 + cpg : m;
            memset(acc, 0, sizeof(float) * (size_t)cpg * (size_t)n);
            const int64_t e0 = groupIndex[g];
            const int64_t e1 = e0 + nnzPerGroup[g];
            for (int64_t e = e0; e < e1; ++e) {
                const float a = vals[e];
                float *dst = acc + (int64_t)(rows[e] - r0) * n;
                const float *b = B + (int64_t)cols[e] * n;
                for (int64_t j = 0; j < n; ++j)
                    dst[j] = fmaf(a, b[j], dst[j]);
            }
            for (int64_t r = r0; r < r1; ++r)
                memcpy(C + r * n, acc + (r - r0) * n, sizeof(float) * (size_t)n);
        }
        free(acc);
    }
}

void orc_spdm_f64(int64_t m, int64_t k, int cpg, const int32_t *groupIndex,
                  const int32_t *nnzPerGroup, const float *vals,
                  const int32_t *rows, const int32_t *cols, const float *B,
                  int64_t n, double *C64, int nthreads)
{
    (void)k;
    const int64_t ng = n_groups(m, cpg);
    int nt = pick_threads(nthreads);
    (void)nt;
#pragma omp parallel for schedule(dynamic, 1) num_threads(nt)
    for (int64_t g = 0; g < ng; ++g) {
        const int64_t r0 = g * cpg;
        const int64_t r1 = r0 + cpg < m ? r0 + cpg : m;
        for (int64_t r = r0; r < r1; ++r)
            memset(C64 + r * n, 0, sizeof(double) * (size_t)n);
        const int64_t e0 = groupIndex[g];
        const int64_t e1 = e0 + nnzPerGroup[g];
        for (int64_t e = e0; e < e1; ++e) {
            const double a = (double)vals[e];
            double *dst = C64 + (int64_t)rows[e] * n;
            const float *b = B + (int64_t)cols[e] * n;
            for (int64_t j = 0; j < n; ++j)
                dst[j] = dst[j] + a * (double)b[j];
        }
    }
}

/* src/utils.cpp:30-46, kept in double: sum over kk ascending of A*B. */
void orc_dense_gemm_f64(const float *A, const float *B, int64_t m, int64_t k,
                        int64_t n, double *C64, int nthreads)
{
    int nt = pick_threads(nthreads);
    (void)nt;
#pragma omp parallel for schedule(static) num_threads(nt)
    for (int64_t i = 0; i < m; ++i) {
        double *dst = C64 + i * n;
        for (int64_t j = 0; j < n; ++j)
            dst[j] = 0.0;
        for (int64_t kk = 0; kk < k; ++kk) {
            const double a = (double)A[i * k + kk];
            const float *b = B + kk * n;
            for (int64_t j = 0; j < n; ++j)
                dst[j] = dst[j] + a * (double)b[j];
        }
    }
}

double orc_rel_fro(const float *C, const double *C64, int64_t len)
{
    double num = 0.0, den = 0.0;
    for (int64_t i = 0; i < len; ++i) {
        const double d = (double)C[i] - C64[i];
        num += d * d;
        den += C64[i] * C64[i];
    }
    if (den == 0.0)
        return num == 0.0 ? 0.0 : INFINITY;
    return sqrt(num) / sqrt(den);
}

/* src/ShGCOOSpDM.cu:131-180 (convert, multiply, free) on the host. */
int64_t orc_multiply_by(const float *A, int64_t m, int64_t k, int cpg,
                        const float *B, int64_t n, float *C, int nthreads)
{
    const int64_t ng = n_groups(m, cpg);
    int32_t *gi = (int32_t *)malloc(sizeof(int32_t) * (size_t)(ng + 1) * 2);
    if (!gi)
        return -1;
    int32_t *npg = gi + (ng + 1);
    int64_t nnz = orc_group_count(A, m, k, cpg, npg, nthreads);
    if (nnz < 0) {
        free(gi);
        return -1;
    }
    orc_exclusive_scan(npg, ng + 1, gi);
    float *vals = (float *)malloc(sizeof(float) * (size_t)(nnz > 0 ? nnz : 1));
    int32_t *rc = (int32_t *)malloc(sizeof(int32_t) * (size_t)(nnz > 0 ? nnz : 1) * 2);
    if (!vals || !rc) {
        free(vals);
        free(rc);
        free(gi);
        return -1;
    }
    orc_scatter(A, m, k, cpg, gi, vals, rc, rc + nnz, nthreads);
    orc_spdm(m, k, cpg, gi, npg, vals, rc, rc + nnz, B, n, C, nthreads);
    free(vals);
    free(rc);
    free(gi);
    return nnz;
}
