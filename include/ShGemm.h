/*
 * ShGemm.h -- the reference's plugin interface (hclhkbu/gcoospdm
 * src/ShGemm.h:7-24), same class shape and member names, so that code written
 * against the reference's ShGemm compiles unchanged against this library.
 *
 * Naming follows the reference: the object is constructed from the SPARSE
 * operand given as a dense device buffer (denseMatrix, m x k = nRows x
 * nCols); mutiplyBy / runKernelTest take the DENSE operand (k x n, row-major,
 * their nRows x nCols) and write C (m x n, row-major). The spelling
 * "mutiply" is the reference's.
 *
 * Differences from the reference, all compatible with its callers: the
 * destructor is virtual (the reference deletes through the base pointer);
 * the double return is 0.0 on success and -(gcoo_status) on failure (the
 * reference always returned 0.0 and exited the process on errors).
 */
#ifndef GCOO_SHGEMM_H
#define GCOO_SHGEMM_H

class ShGemm
{
  public:
    ShGemm() : m_nRows(0), m_nCols(0), m_pDenseMatrix(0) {}
    ShGemm(int nRows, int nCols) : m_nRows(nRows), m_nCols(nCols), m_pDenseMatrix(0) {}
    virtual ~ShGemm(void) {}
    // C = self x A in the reference kernel's row-major reading (self is m x k).
    virtual double mutiplyBy(float *A, int nRows, int nCols, float *C) = 0;
    // The other orientation; the reference's GCOO plugin leaves it empty.
    virtual double mutiply(float *B, int nRows, int nCols, float *C) = 0;
    // Converts self once so that runKernelTest times the multiply alone.
    virtual void build() = 0;
    virtual double runKernelTest(float *A, int nRows, int nCols, float *C) = 0;

  public:
    int m_nRows;
    int m_nCols;
    float *m_pDenseMatrix;
};

#endif
