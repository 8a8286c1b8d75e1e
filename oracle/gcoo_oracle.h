/*
 * gcoo_oracle.h -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C CPU restatement of the reference's GCOO path (hclhkbu/gcoospdm):
 * dense->GCOO conversion (count, exclusive scan, stable scatter) and the GCOO
 * sparse x dense multiply, plus FP64 checks. It is the checker for the CUDA
 * library and the timed CPU baseline; nothing in the product links or calls it.
 *
 * Parity pin: its outputs are compared bit-for-bit with the reference's own
 * kernel source (src/gcoo_spdm_kernels.cu) executed under a CUDA-semantics
 * emulator (oracle/ref_emu), whose results are committed as fixtures under
 * tests/golden/.
 *
 * Conventions (row-major, as the reference kernel indexes them):
 *   A  m x k sparse operand stored dense (zeros kept), FP32
 *   B  k x n dense, FP32
 *   C  m x n, C[r*n+j] = sum_c A[r*k+c] * B[c*n+j]
 *   a group = cpg consecutive rows of A; nGroup = ceil(m / cpg)
 */
#ifndef GCOO_ORACLE_H
#define GCOO_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Per-group nonzero counts. nnzPerGroup has nGroup+1 entries; the last one is
 * 0 (the reference memsets the array, src/ShGCOOSpDM.cu:37).
 * Follows src/gcoo_spdm_kernels.cu:4-28 (zero test `v != 0.0`).
 * Returns the total nnz, or -1 when it does not fit the int32 format. */
int64_t orc_group_count(const float *A, int64_t m, int64_t k, int cpg,
                        int32_t *nnzPerGroup, int nthreads);

/* Exclusive scan over n = nGroup+1 entries: out[0]=0, out[i]=out[i-1]+in[i-1].
 * Follows src/gcoo_spdm_kernels.cu:160-168 (prefix_sum_kernel2). */
void orc_exclusive_scan(const int32_t *in, int64_t n, int32_t *out);

/* Stable scatter into GCOO: within group g the entries are ordered by column
 * ascending, then row ascending; rows are absolute row indices.
 * Follows src/gcoo_spdm_kernels.cu:30-90. */
void orc_scatter(const float *A, int64_t m, int64_t k, int cpg,
                 const int32_t *groupIndex, float *vals, int32_t *rows,
                 int32_t *cols, int nthreads);

/* GCOO x dense in FP32: each C element is a sequential fmaf chain, starting
 * from 0.0f, over the group's entries of that row in storage order.
 * Follows src/gcoo_spdm_kernels.cu:92-158 (for cpg==4 identical to the
 * reference's c0..c3 accumulators; for other cpg the per-row accumulator the
 * kernel intends). Every C element is written (zeros for empty rows). */
void orc_spdm(int64_t m, int64_t k, int cpg, const int32_t *groupIndex,
              const int32_t *nnzPerGroup, const float *vals,
              const int32_t *rows, const int32_t *cols, const float *B,
              int64_t n, float *C, int nthreads);

/* Same product accumulated in FP64 (the error-norm reference). */
void orc_spdm_f64(int64_t m, int64_t k, int cpg, const int32_t *groupIndex,
                  const int32_t *nnzPerGroup, const float *vals,
                  const int32_t *rows, const int32_t *cols, const float *B,
                  int64_t n, double *C64, int nthreads);

/* Dense FP64 product with the semantics of src/utils.cpp:30-46 (matrixMulCPU:
 * double accumulation), kept in double. */
void orc_dense_gemm_f64(const float *A, const float *B, int64_t m, int64_t k,
                        int64_t n, double *C64, int nthreads);

/* ||C - C64||_F / ||C64||_F (0 when both are zero). */
double orc_rel_fro(const float *C, const double *C64, int64_t len);

/* Convert + multiply, as the reference's ShGCOOSpDM::mutiplyBy does
 * (src/ShGCOOSpDM.cu:131-180), on the host. Scratch is malloc'd per call.
 * Returns nnz or -1 on failure. */
int64_t orc_multiply_by(const float *A, int64_t m, int64_t k, int cpg,
                        const float *B, int64_t n, float *C, int nthreads);

/* Threads the OpenMP runtime would use (0 when built without OpenMP). */
int orc_max_threads(void);

#ifdef __cplusplus
}
#endif
#endif
