// baselines.cpp -- the library baselines the reference benchmarks against
// (src/ShCublasGemm.cpp, src/ShCusparseGemm.cpp), rewritten on current
// cuBLAS and the generic cuSPARSE API (the reference's cusparseSdense2csr /
// cusparseScsrmm2 were removed in CUDA 13). Both compute the same row-major
// C = self x A as ShGCOOSpDM so that results are elementwise comparable.
// Baselines only: nothing of the GCOO path calls them.
#include <cublas_v2.h>
#include <cuda_runtime.h>
#include <cusparse.h>
#include <stdio.h>
#include <string.h>

#include "ShGemm.h"

namespace {

bool ok_cuda(cudaError_t e, const char *what)
{
    if (e != cudaSuccess) {
        fprintf(stderr, "%s: %s\n", what, cudaGetErrorString(e));
        return false;
    }
    return true;
}

bool ok_sp(cusparseStatus_t s, const char *what)
{
    if (s != CUSPARSE_STATUS_SUCCESS) {
        fprintf(stderr, "%s: %s\n", what, cusparseGetErrorString(s));
        return false;
    }
    return true;
}

class CublasGemm : public ShGemm
{
  public:
    CublasGemm(float *dense, int nRows, int nCols) : ShGemm(nRows, nCols)
    {
        m_pDenseMatrix = dense;
        if (cublasCreate(&h_) != CUBLAS_STATUS_SUCCESS)
            h_ = 0;
    }
    ~CublasGemm() { if (h_) cublasDestroy(h_); }
    // row-major C[m x n] = S[m x k] A[k x n]  <=>  column-major C^T = A^T S^T
    double mutiplyBy(float *A, int nRows, int nCols, float *C)
    {
        (void)nRows;
        if (!h_)
            return -3.0;
        const float one = 1.0f, zero = 0.0f;
        cublasStatus_t s = cublasSgemm(h_, CUBLAS_OP_N, CUBLAS_OP_N, nCols, m_nRows, m_nCols, &one, A, nCols,
                                       m_pDenseMatrix, m_nCols, &zero, C, nCols);
        if (s != CUBLAS_STATUS_SUCCESS)
            return -3.0;
        return ok_cuda(cudaDeviceSynchronize(), "cublasSgemm") ? 0.0 : -3.0;
    }
    double mutiply(float *, int, int, float *) { return -5.0; }
    void build() {}
    double runKernelTest(float *A, int nRows, int nCols, float *C) { return mutiplyBy(A, nRows, nCols, C); }

  private:
    cublasHandle_t h_ = 0;
};

class CusparseGemm : public ShGemm
{
  public:
    CusparseGemm(float *dense, int nRows, int nCols) : ShGemm(nRows, nCols)
    {
        m_pDenseMatrix = dense;
        if (cusparseCreate(&h_) != CUSPARSE_STATUS_SUCCESS)
            h_ = 0;
    }
    ~CusparseGemm()
    {
        release();
        if (spmm_buf_)
            cudaFree(spmm_buf_);
        if (h_)
            cusparseDestroy(h_);
    }
    // conversion + multiply, like the reference's mutiplyBy (src/ShCusparseGemm.cpp:251-331)
    double mutiplyBy(float *A, int nRows, int nCols, float *C)
    {
        if (!convert())
            return -3.0;
        double r = multiply(A, nRows, nCols, C);
        release();
        return r;
    }
    double mutiply(float *, int, int, float *) { return -5.0; }
    void build() { convert(); }
    double runKernelTest(float *A, int nRows, int nCols, float *C) { return multiply(A, nRows, nCols, C); }

  private:
    bool convert()
    {
        release();
        if (!h_)
            return false;
        cusparseDnMatDescr_t dense;
        if (!ok_sp(cusparseCreateDnMat(&dense, m_nRows, m_nCols, m_nCols, m_pDenseMatrix, CUDA_R_32F,
                                       CUSPARSE_ORDER_ROW), "CreateDnMat"))
            return false;
        if (!ok_cuda(cudaMalloc(&rowptr_, sizeof(int) * (m_nRows + 1)), "cudaMalloc rowptr"))
            return false;
        ok_sp(cusparseCreateCsr(&sp_, m_nRows, m_nCols, 0, rowptr_, 0, 0, CUSPARSE_INDEX_32I, CUSPARSE_INDEX_32I,
                                CUSPARSE_INDEX_BASE_ZERO, CUDA_R_32F), "CreateCsr");
        size_t bytes = 0;
        void *buf = 0;
        bool ok = ok_sp(cusparseDenseToSparse_bufferSize(h_, dense, sp_, CUSPARSE_DENSETOSPARSE_ALG_DEFAULT, &bytes),
                        "DenseToSparse_bufferSize") &&
                  ok_cuda(cudaMalloc(&buf, bytes ? bytes : 16), "cudaMalloc d2s") &&
                  ok_sp(cusparseDenseToSparse_analysis(h_, dense, sp_, CUSPARSE_DENSETOSPARSE_ALG_DEFAULT, buf),
                        "DenseToSparse_analysis");
        int64_t r = 0, c = 0, nnz = 0;
        if (ok)
            ok = ok_sp(cusparseSpMatGetSize(sp_, &r, &c, &nnz), "SpMatGetSize") &&
                 ok_cuda(cudaMalloc(&cols_, sizeof(int) * (nnz ? nnz : 1)), "cudaMalloc cols") &&
                 ok_cuda(cudaMalloc(&vals_, sizeof(float) * (nnz ? nnz : 1)), "cudaMalloc vals") &&
                 ok_sp(cusparseCsrSetPointers(sp_, rowptr_, cols_, vals_), "CsrSetPointers") &&
                 ok_sp(cusparseDenseToSparse_convert(h_, dense, sp_, CUSPARSE_DENSETOSPARSE_ALG_DEFAULT, buf),
                       "DenseToSparse_convert");
        cusparseDestroyDnMat(dense);
        if (buf)
            cudaFree(buf);
        return ok;
    }
    double multiply(float *A, int nRows, int nCols, float *C)
    {
        if (!sp_)
            return -4.0;
        cusparseDnMatDescr_t b, c;
        const float one = 1.0f, zero = 0.0f;
        cusparseCreateDnMat(&b, nRows, nCols, nCols, A, CUDA_R_32F, CUSPARSE_ORDER_ROW);
        cusparseCreateDnMat(&c, m_nRows, nCols, nCols, C, CUDA_R_32F, CUSPARSE_ORDER_ROW);
        size_t bytes = 0;
        bool ok = ok_sp(cusparseSpMM_bufferSize(h_, CUSPARSE_OPERATION_NON_TRANSPOSE, CUSPARSE_OPERATION_NON_TRANSPOSE,
                                                &one, sp_, b, &zero, c, CUDA_R_32F, CUSPARSE_SPMM_ALG_DEFAULT, &bytes),
                        "SpMM_bufferSize");
        if (ok && bytes > spmm_bytes_) {
            if (spmm_buf_)
                cudaFree(spmm_buf_);
            spmm_buf_ = 0;
            ok = ok_cuda(cudaMalloc(&spmm_buf_, bytes), "cudaMalloc spmm");
            spmm_bytes_ = ok ? bytes : 0;
        }
        if (ok)
            ok = ok_sp(cusparseSpMM(h_, CUSPARSE_OPERATION_NON_TRANSPOSE, CUSPARSE_OPERATION_NON_TRANSPOSE, &one, sp_,
                                    b, &zero, c, CUDA_R_32F, CUSPARSE_SPMM_ALG_DEFAULT, spmm_buf_),
                       "SpMM");
        cusparseDestroyDnMat(b);
        cusparseDestroyDnMat(c);
        if (ok)
            ok = ok_cuda(cudaDeviceSynchronize(), "SpMM sync");
        return ok ? 0.0 : -3.0;
    }
    void release()
    {
        if (sp_)
            cusparseDestroySpMat(sp_);
        sp_ = 0;
        if (rowptr_)
            cudaFree(rowptr_);
        if (cols_)
            cudaFree(cols_);
        if (vals_)
            cudaFree(vals_);
        rowptr_ = cols_ = 0;
        vals_ = 0;
    }
    cusparseHandle_t h_ = 0;
    cusparseSpMatDescr_t sp_ = 0;
    int *rowptr_ = 0, *cols_ = 0;
    float *vals_ = 0;
    void *spmm_buf_ = 0;
    size_t spmm_bytes_ = 0;
};

} // namespace

ShGemm *gcoo_make_cublas_gemm(float *denseMatrix, int nRows, int nCols)
{
    return new CublasGemm(denseMatrix, nRows, nCols);
}

ShGemm *gcoo_make_cusparse_gemm(float *denseMatrix, int nRows, int nCols)
{
    return new CusparseGemm(denseMatrix, nRows, nCols);
}

// baseline_csr.cu: the reference's auxiliary "-algo=csr" plugin
ShGemm *gcoo_make_csr_gemm(float *denseMatrix, int nRows, int nCols);

extern "C" {
// C entry points for FFI callers that want the baselines (benchmarks).
void *gcoo_baseline_create(const char *algo, float *denseMatrix, int nRows, int nCols)
{
    const char *a = algo ? algo : "";
    if (!strcmp(a, "cublas"))
        return gcoo_make_cublas_gemm(denseMatrix, nRows, nCols);
    if (!strcmp(a, "cusparse"))
        return gcoo_make_cusparse_gemm(denseMatrix, nRows, nCols);
    if (!strcmp(a, "csr"))
        return gcoo_make_csr_gemm(denseMatrix, nRows, nCols);
    return 0;
}
double gcoo_baseline_multiply_by(void *g, float *A, int nRows, int nCols, float *C)
{
    return static_cast<ShGemm *>(g)->mutiplyBy(A, nRows, nCols, C);
}
void gcoo_baseline_build(void *g) { static_cast<ShGemm *>(g)->build(); }
double gcoo_baseline_run_kernel(void *g, float *A, int nRows, int nCols, float *C)
{
    return static_cast<ShGemm *>(g)->runKernelTest(A, nRows, nCols, C);
}
void gcoo_baseline_destroy(void *g) { delete static_cast<ShGemm *>(g); }
}
