// Test-only helper: runs the cuSPARSE calls the reference makes --
// cusparseXcsr2bsrNnz + cusparseScsr2bsr (csr2bsr_batch_bsrbmv.cu:302-311,
// row-major blocks, values forced to 1.0) and cusparseSpMM on column-major
// B / C with alpha = 1, beta = 0, CUSPARSE_SPMM_ALG_DEFAULT
// (test_spmm_full.cu:279-307) -- so the GPU tests can compare the library
// against the reference's own dependency on the same inputs.
#include <cuda_runtime.h>
#include <cusparse.h>

extern "C" int ref_csr2bsr_nnz(int nrows, int ncols, const int *rowptr, const int *colind, int bs,
                               int *bsr_rowptr, int *h_nnzb) {
  cusparseHandle_t h;
  if (cusparseCreate(&h) != CUSPARSE_STATUS_SUCCESS) return 1;
  cusparseMatDescr_t a, b;
  cusparseCreateMatDescr(&a);
  cusparseCreateMatDescr(&b);
  cusparseSetMatIndexBase(a, CUSPARSE_INDEX_BASE_ZERO);
  cusparseSetMatIndexBase(b, CUSPARSE_INDEX_BASE_ZERO);
  int st = (int)cusparseXcsr2bsrNnz(h, CUSPARSE_DIRECTION_ROW, nrows, ncols, a, rowptr, colind, bs, b,
                                    bsr_rowptr, h_nnzb);
  cudaDeviceSynchronize();
  cusparseDestroyMatDescr(a);
  cusparseDestroyMatDescr(b);
  cusparseDestroy(h);
  return st;
}

extern "C" int ref_csr2bsr_fill(int nrows, int ncols, const float *vals, const int *rowptr,
                                const int *colind, int bs, float *bsr_val, int *bsr_rowptr,
                                int *bsr_colind) {
  cusparseHandle_t h;
  if (cusparseCreate(&h) != CUSPARSE_STATUS_SUCCESS) return 1;
  cusparseMatDescr_t a, b;
  cusparseCreateMatDescr(&a);
  cusparseCreateMatDescr(&b);
  cusparseSetMatIndexBase(a, CUSPARSE_INDEX_BASE_ZERO);
  cusparseSetMatIndexBase(b, CUSPARSE_INDEX_BASE_ZERO);
  int st = (int)cusparseScsr2bsr(h, CUSPARSE_DIRECTION_ROW, nrows, ncols, a, vals, rowptr, colind, bs,
                                 b, bsr_val, bsr_rowptr, bsr_colind);
  cudaDeviceSynchronize();
  cusparseDestroyMatDescr(a);
  cusparseDestroyMatDescr(b);
  cusparseDestroy(h);
  return st;
}

extern "C" int ref_spmm_colmajor(int nrows, int ncols, int nnz, const int *rowptr, const int *colind,
                                 const float *vals, const float *Bcol, int F, float *Ccol) {
  cusparseHandle_t h;
  if (cusparseCreate(&h) != CUSPARSE_STATUS_SUCCESS) return 1;
  cusparseSpMatDescr_t A;
  cusparseDnMatDescr_t B, C;
  float alpha = 1.f, beta = 0.f;
  cusparseCreateCsr(&A, nrows, ncols, nnz, (void *)rowptr, (void *)colind, (void *)vals,
                    CUSPARSE_INDEX_32I, CUSPARSE_INDEX_32I, CUSPARSE_INDEX_BASE_ZERO, CUDA_R_32F);
  cusparseCreateDnMat(&B, ncols, F, ncols, (void *)Bcol, CUDA_R_32F, CUSPARSE_ORDER_COL);
  cusparseCreateDnMat(&C, nrows, F, nrows, (void *)Ccol, CUDA_R_32F, CUSPARSE_ORDER_COL);
  size_t sz = 0;
  int st = (int)cusparseSpMM_bufferSize(h, CUSPARSE_OPERATION_NON_TRANSPOSE, CUSPARSE_OPERATION_NON_TRANSPOSE,
                                        &alpha, A, B, &beta, C, CUDA_R_32F, CUSPARSE_SPMM_ALG_DEFAULT, &sz);
  void *buf = nullptr;
  if (st == 0 && sz) cudaMalloc(&buf, sz);
  if (st == 0)
    st = (int)cusparseSpMM(h, CUSPARSE_OPERATION_NON_TRANSPOSE, CUSPARSE_OPERATION_NON_TRANSPOSE, &alpha, A, B,
                           &beta, C, CUDA_R_32F, CUSPARSE_SPMM_ALG_DEFAULT, buf);
  cudaDeviceSynchronize();
  if (buf) cudaFree(buf);
  cusparseDestroySpMat(A);
  cusparseDestroyDnMat(B);
  cusparseDestroyDnMat(C);
  cusparseDestroy(h);
  return st;
}

// Timing handle for the comparison script: the SpMM of ref_spmm_colmajor
// (or with row-major B / C, order = 1) set up once -- handle, descriptors,
// work buffer, preprocessing -- so that ref_spmm_handle_run issues only the
// cusparseSpMM call, on the legacy default stream.
struct RefSpmm {
  cusparseHandle_t h;
  cusparseSpMatDescr_t A;
  cusparseDnMatDescr_t B, C;
  void *buf;
};

extern "C" void *ref_spmm_handle_create(int nrows, int ncols, int nnz, const int *rowptr, const int *colind,
                                        const float *vals, const float *B, int F, float *C, int order) {
  RefSpmm *r = new RefSpmm();
  float alpha = 1.f, beta = 0.f;
  if (cusparseCreate(&r->h) != CUSPARSE_STATUS_SUCCESS) { delete r; return nullptr; }
  cusparseCreateCsr(&r->A, nrows, ncols, nnz, (void *)rowptr, (void *)colind, (void *)vals, CUSPARSE_INDEX_32I,
                    CUSPARSE_INDEX_32I, CUSPARSE_INDEX_BASE_ZERO, CUDA_R_32F);
  if (order == 0) {
    cusparseCreateDnMat(&r->B, ncols, F, ncols, (void *)B, CUDA_R_32F, CUSPARSE_ORDER_COL);
    cusparseCreateDnMat(&r->C, nrows, F, nrows, (void *)C, CUDA_R_32F, CUSPARSE_ORDER_COL);
  } else {
    cusparseCreateDnMat(&r->B, ncols, F, F, (void *)B, CUDA_R_32F, CUSPARSE_ORDER_ROW);
    cusparseCreateDnMat(&r->C, nrows, F, F, (void *)C, CUDA_R_32F, CUSPARSE_ORDER_ROW);
  }
  size_t sz = 0;
  cusparseSpMM_bufferSize(r->h, CUSPARSE_OPERATION_NON_TRANSPOSE, CUSPARSE_OPERATION_NON_TRANSPOSE, &alpha, r->A,
                          r->B, &beta, r->C, CUDA_R_32F, CUSPARSE_SPMM_ALG_DEFAULT, &sz);
  r->buf = nullptr;
  if (sz) cudaMalloc(&r->buf, sz);
  cusparseSpMM_preprocess(r->h, CUSPARSE_OPERATION_NON_TRANSPOSE, CUSPARSE_OPERATION_NON_TRANSPOSE, &alpha, r->A,
                          r->B, &beta, r->C, CUDA_R_32F, CUSPARSE_SPMM_ALG_DEFAULT, r->buf);
  cudaDeviceSynchronize();
  return r;
}

extern "C" int ref_spmm_handle_run(void *p) {
  RefSpmm *r = static_cast<RefSpmm *>(p);
  float alpha = 1.f, beta = 0.f;
  return (int)cusparseSpMM(r->h, CUSPARSE_OPERATION_NON_TRANSPOSE, CUSPARSE_OPERATION_NON_TRANSPOSE, &alpha, r->A,
                           r->B, &beta, r->C, CUDA_R_32F, CUSPARSE_SPMM_ALG_DEFAULT, r->buf);
}

extern "C" void ref_spmm_handle_destroy(void *p) {
  RefSpmm *r = static_cast<RefSpmm *>(p);
  if (!r) return;
  cudaDeviceSynchronize();
  if (r->buf) cudaFree(r->buf);
  cusparseDestroySpMat(r->A);
  cusparseDestroyDnMat(r->B);
  cusparseDestroyDnMat(r->C);
  cusparseDestroy(r->h);
  delete r;
}
