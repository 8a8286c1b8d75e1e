/*
 * ShGCOOSpDM.h -- drop-in for the reference's GCOO plugin
 * (hclhkbu/gcoospdm src/ShGCOOSpDM.h:6-33), implemented over the C ABI in
 * gcoo.h. The public members the reference exposes (m_pVals, m_pCols,
 * m_pRows, m_pGroupIndex, m_pNnzPerGroup, m_nGroup) are device pointers into
 * the handle's GCOO arrays, valid after build() until the next build() or
 * destruction.
 *
 * Semantics kept from the reference: the calls run on the legacy default
 * stream and return after the GPU work completes (the reference synchronises
 * after every step). setStream() / setSynchronous(false) opt out of both.
 */
#ifndef GCOO_SHGCOOSPDM_H
#define GCOO_SHGCOOSPDM_H

#include "ShGemm.h"
#include "gcoo.h"

class ShGCOOSpDM : public ShGemm
{
  public:
    ShGCOOSpDM(float *denseMatrix, int nRows, int nCols);
    ShGCOOSpDM(float *denseMatrix, int nRows, int nCols, const gcoo_params &params);
    ~ShGCOOSpDM(void);

    // convert + multiply (src/ShGCOOSpDM.cu:131-180); A is k x n, C is m x n
    double mutiplyBy(float *A, int nRows, int nCols, float *C);
    // the other orientation, C = B x self (empty in the reference, src/ShGCOOSpDM.h:21)
    double mutiply(float *B, int nRows, int nCols, float *C);
    // conversion into members (src/ShGCOOSpDM.cu:182-193)
    void build();
    // multiply only (src/ShGCOOSpDM.cu:195-213)
    double runKernelTest(float *A, int nRows, int nCols, float *C);

    // Extensions.
    double runKernelTest(float *A, int nRows, int nCols, float *C, gcoo_precision prec);
    void setStream(void *stream) { m_stream = stream; }
    void setSynchronous(bool sync) { m_sync = sync; }
    gcoo_handle *handle() { return m_handle; }
    gcoo_status lastStatus() const { return m_status; }
    long long nnz() const { return m_nnz; }

  public:
    float *m_pVals;
    int *m_pCols;
    int *m_pRows;
    int *m_pGroupIndex;
    int *m_pNnzPerGroup;
    int m_nGroup;

  private:
    double finish(gcoo_status s);
    void refreshView();
    gcoo_handle *m_handle;
    void *m_stream;
    bool m_sync;
    gcoo_status m_status;
    long long m_nnz;
};

#endif
