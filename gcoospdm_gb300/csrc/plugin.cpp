// plugin.cpp -- ShGCOOSpDM, the reference's plugin class, as a thin shim over
// the C ABI (include/gcoo.h). Mirrors src/ShGCOOSpDM.cu of the reference:
// the constructor records the dense sparse operand, build() converts once,
// mutiplyBy() converts and multiplies, runKernelTest() multiplies only.
#include "ShGCOOSpDM.h"

#include <cuda_runtime.h>
#include <stdio.h>

ShGCOOSpDM::ShGCOOSpDM(float *denseMatrix, int nRows, int nCols)
    : ShGemm(nRows, nCols), m_pVals(0), m_pCols(0), m_pRows(0), m_pGroupIndex(0), m_pNnzPerGroup(0),
      m_nGroup(0), m_handle(0), m_stream(0), m_sync(true), m_status(GCOO_SUCCESS), m_nnz(0)
{
    m_pDenseMatrix = denseMatrix;
    m_status = gcoo_create(&m_handle, denseMatrix, nRows, nCols, 0);
}

ShGCOOSpDM::ShGCOOSpDM(float *denseMatrix, int nRows, int nCols, const gcoo_params &params)
    : ShGemm(nRows, nCols), m_pVals(0), m_pCols(0), m_pRows(0), m_pGroupIndex(0), m_pNnzPerGroup(0),
      m_nGroup(0), m_handle(0), m_stream(0), m_sync(true), m_status(GCOO_SUCCESS), m_nnz(0)
{
    m_pDenseMatrix = denseMatrix;
    m_status = gcoo_create(&m_handle, denseMatrix, nRows, nCols, &params);
}

ShGCOOSpDM::~ShGCOOSpDM(void) { gcoo_destroy(m_handle); }

double ShGCOOSpDM::finish(gcoo_status s)
{
    if (s == GCOO_SUCCESS && m_sync) {
        if (cudaStreamSynchronize(static_cast<cudaStream_t>(m_stream)) != cudaSuccess)
            s = GCOO_ERROR_CUDA;
    }
    m_status = s;
    if (s != GCOO_SUCCESS) {
        fprintf(stderr, "ShGCOOSpDM: %s\n", gcoo_last_error());
        return -static_cast<double>(s);
    }
    return 0.0;
}

void ShGCOOSpDM::refreshView()
{
    gcoo_view v;
    if (gcoo_export(m_handle, &v) != GCOO_SUCCESS)
        return;
    m_pVals = const_cast<float *>(v.vals);
    m_pRows = const_cast<int *>(v.rows);
    m_pCols = const_cast<int *>(v.cols);
    m_pGroupIndex = const_cast<int *>(v.group_index);
    m_pNnzPerGroup = const_cast<int *>(v.nnz_per_group);
    m_nGroup = static_cast<int>(v.n_group);
    m_nnz = v.nnz;
}

double ShGCOOSpDM::mutiplyBy(float *A, int nRows, int nCols, float *C)
{
    (void)nRows; // k, implied by the sparse operand (the reference ignores it too)
    if (!m_handle)
        return finish(m_status != GCOO_SUCCESS ? m_status : GCOO_ERROR_INVALID_VALUE);
    gcoo_status s = gcoo_multiply_by(m_handle, A, nCols, C, m_stream);
    if (s == GCOO_SUCCESS)
        refreshView();
    return finish(s);
}

// C = B x self: B is nRows x nCols (nCols == the sparse operand's rows), C is
// nRows x the sparse operand's columns. The reference leaves this empty.
double ShGCOOSpDM::mutiply(float *B, int nRows, int nCols, float *C)
{
    if (!m_handle)
        return finish(m_status != GCOO_SUCCESS ? m_status : GCOO_ERROR_INVALID_VALUE);
    if (nCols != m_nRows)
        return finish(GCOO_ERROR_INVALID_VALUE);
    gcoo_status s = GCOO_SUCCESS;
    gcoo_view v;
    if (gcoo_export(m_handle, &v) != GCOO_SUCCESS) { // not built yet: convert first
        s = gcoo_build(m_handle, m_stream);
        if (s == GCOO_SUCCESS)
            refreshView();
    }
    if (s == GCOO_SUCCESS)
        s = gcoo_spdm_left(m_handle, B, nRows, C, m_stream);
    return finish(s);
}

void ShGCOOSpDM::build()
{
    if (!m_handle)
        return;
    gcoo_status s = gcoo_build(m_handle, m_stream);
    if (s == GCOO_SUCCESS)
        refreshView();
    finish(s);
}

double ShGCOOSpDM::runKernelTest(float *A, int nRows, int nCols, float *C)
{
    (void)nRows;
    if (!m_handle)
        return finish(m_status != GCOO_SUCCESS ? m_status : GCOO_ERROR_INVALID_VALUE);
    return finish(gcoo_spdm(m_handle, A, nCols, C, m_stream));
}

double ShGCOOSpDM::runKernelTest(float *A, int nRows, int nCols, float *C, gcoo_precision prec)
{
    (void)nRows;
    if (!m_handle)
        return finish(m_status != GCOO_SUCCESS ? m_status : GCOO_ERROR_INVALID_VALUE);
    return finish(gcoo_spdm_ex(m_handle, A, nCols, C, prec, m_stream));
}
