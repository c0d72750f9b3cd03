// Internal interface of the merge-path CSR SpMM (shared by the C ABI entry
// points that reuse the kernel: forward, backward dB = A^T dC).
#pragma once

#include "common.cuh"

namespace gbs {

struct SpmmVariant {
  const void *fn;
  int vec, lpr, ch;
};

gbs_status spmm_select(int dt, int F, bool aligned16, SpmmVariant *out);
gbs_status spmm_warps(const SpmmVariant &v, int nrows, int nnz, int *P_out);
size_t spmm_workspace_bytes(int P, int F);
gbs_status spmm_check_args(int nrows, int ncols, int nnz, const int *rowptr, const int *colind,
                           const void *B, int F, const float *C);
gbs_status spmm_prepare(int dt, int nrows, int nnz, int F, const void *B, const float *C,
                        SpmmVariant *v, int *P);
gbs_status spmm_launch(const SpmmVariant &v, int P, int nrows, int nnz, const int *rowptr,
                       const int *colind, const float *vals, const void *B, int F, float *C,
                       void *ws, cudaStream_t stream);

}  // namespace gbs
