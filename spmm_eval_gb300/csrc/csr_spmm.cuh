// Internal interface of the merge-path CSR SpMM (shared by the C ABI entry
// points that reuse the kernel: forward, backward dB = A^T dC).
#pragma once

#include "common.cuh"

namespace gbs {

struct SpmmVariant {
  const void *fn;
  int vec, lpr, ch;
};

struct SpmmPlan {
  SpmmVariant v;
  bool vec16;
  int Fw;    // column-block width
  int nblk;  // F / Fw launches
  int P;     // warps per launch
  int esize; // bytes per B element
  size_t ws_bytes;
};

gbs_status spmm_select(int dt, int Fw, bool vec16, SpmmVariant *out);
gbs_status spmm_warps(const SpmmVariant &v, int nrows, int nnz, int *P_out);
size_t spmm_counter_bytes();
size_t spmm_workspace_bytes(int P, int Fw);
gbs_status spmm_workspace_upper(int dt, int nrows, int nnz, int F, size_t *bytes);
gbs_status spmm_check_args(int nrows, int ncols, int nnz, const int *rowptr, const int *colind,
                           const void *B, int F, const float *C);
gbs_status spmm_plan(int dt, int nrows, int ncols, int nnz, int F, const void *B, const float *C,
                     int col_block, SpmmPlan *p);
gbs_status spmm_launch(const SpmmVariant &v, int P, int nrows, int nnz, const int *rowptr,
                       const int *colind, const float *vals, const void *B, long long ldb, int Fw,
                       float *C, long long ldc, void *ws, cudaStream_t stream, int rp_base = 0,
                       int accumulate = 0);
gbs_status spmm_run(const SpmmPlan &p, int nrows, int nnz, const int *rowptr, const int *colind,
                    const float *vals, const void *B, int F, float *C, void *ws,
                    cudaStream_t stream, int rp_base = 0, int accumulate = 0);

}  // namespace gbs
