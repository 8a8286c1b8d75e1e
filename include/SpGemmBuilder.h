/*
 * SpGemmBuilder.h -- the reference's string factory
 * (hclhkbu/gcoospdm src/SpGemmBuilder.h:10-24): same class and method.
 *   "gcoospdm"  -> ShGCOOSpDM (this library, libgcoo.so)
 *   "cublas"    -> ShCublasGemm   (cublasSgemm on the dense-with-zeros
 *                                  operand; libgcoo_baselines.so)
 *   "cusparse"  -> ShCusparseGemm (CSR + generic cusparseSpMM; the
 *                                  reference's csrmm2/dense2csr calls no
 *                                  longer exist in CUDA 13;
 *                                  libgcoo_baselines.so)
 *   "csr"       -> the reference's auxiliary CSR plugin (src/ShCsrSpGemm.cu:
 *                                  per-call CSR conversion, one CTA per
 *                                  row; restated, libgcoo_baselines.so)
 *   anything else -> NULL
 * All four compute the same C = self x A (row-major), unlike the reference
 * whose cuSPARSE/cuBLAS plugins computed the transposed orientation.
 */
#ifndef GCOO_SPGEMMBUILDER_H
#define GCOO_SPGEMMBUILDER_H

#include <string>

#include "ShGCOOSpDM.h"
#include "ShGemm.h"

class ShCublasGemm;
class ShCusparseGemm;
ShGemm *gcoo_make_cublas_gemm(float *denseMatrix, int nRows, int nCols);
ShGemm *gcoo_make_cusparse_gemm(float *denseMatrix, int nRows, int nCols);
ShGemm *gcoo_make_csr_gemm(float *denseMatrix, int nRows, int nCols);

class SpGemmBuilder
{
  public:
    static ShGemm *getShGemmAlgo(float *denseMatrix, int nRows, int nCols, const std::string &desc)
    {
        if (desc == "gcoospdm")
            return new ShGCOOSpDM(denseMatrix, nRows, nCols);
        if (desc == "cublas")
            return gcoo_make_cublas_gemm(denseMatrix, nRows, nCols);
        if (desc == "cusparse")
            return gcoo_make_cusparse_gemm(denseMatrix, nRows, nCols);
        if (desc == "csr")
            return gcoo_make_csr_gemm(denseMatrix, nRows, nCols);
        return 0;
    }
};

#endif
