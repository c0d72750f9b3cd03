// Internal interface of the merge-path CSR SpMM (shared by the C ABI entry
// points that reuse the kernel: forward, backward dB = A^T dC).
#pragma once

#include <vector>

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

// halfwarp: the gathered rows of B fit in half of L2 (enables the half-warp
// variants for F = 136..256).
// scaled: the degree-normalised kernels (rowscale / colscale, binary A).
gbs_status spmm_select(int dt, int Fw, bool vec16, bool halfwarp, SpmmVariant *out, bool scaled = false);
gbs_status spmm_select_scaled(int dt, int Fw, bool vec16, bool halfwarp, SpmmVariant *out);
gbs_status spmm_warps(const SpmmVariant &v, int nrows, int nnz, int *P_out);
size_t spmm_counter_bytes();
size_t spmm_workspace_bytes(int P, int Fw);
// Largest workspace any forward column block or the fused backward (on a
// matrix of nrows rows) can ask for at this shape.
gbs_status spmm_workspace_upper(int dt, int nrows, int nnz, int F, size_t *bytes);
gbs_status bwd_workspace_bytes(int dt, int nrows, int nnz, int F, size_t *bytes);
gbs_status spmm_check_args(int nrows, int ncols, int nnz, const int *rowptr, const int *colind,
                           const void *B, int F, const float *C);
// gathered_rows: rows of B the launch actually reads (a column part of the
// planned form reads ~ncols / K of them; -1 = ncols).
gbs_status spmm_plan(int dt, int nrows, int ncols, int nnz, int F, const void *B, const float *C,
                     int col_block, SpmmPlan *p, int gathered_rows = -1, bool scaled = false);
// rowscale / colscale (optional, vals null): the degree-normalised product
// C[r] = rowscale[r] * sum_c colscale[c] B[c] over the stored entries of row r.
gbs_status spmm_launch(const SpmmVariant &v, int P, int nrows, int nnz, const int *rowptr,
                       const int *colind, const float *vals, const void *B, long long ldb, int Fw,
                       float *C, long long ldc, void *ws, cudaStream_t stream, int rp_base = 0,
                       int accumulate = 0, const float *rowscale = nullptr, const float *colscale = nullptr);
gbs_status spmm_run(const SpmmPlan &p, int nrows, int nnz, const int *rowptr, const int *colind,
                    const float *vals, const void *B, int F, float *C, void *ws,
                    cudaStream_t stream, int rp_base = 0, int accumulate = 0,
                    const float *rowscale = nullptr, const float *colscale = nullptr);

// Column partition of a CSR matrix (csr_spmm_plan.cu): part p holds, for
// every row, the entries whose column lies in [p S, (p + 1) S), S =
// ceil(ncols / K), in their original order; `extra` (optional) is an int
// array carried along with the entries (the transpose permutation for the
// fused backward).  K = 1 records the caller's arrays without copying.
struct ColumnParts {
  int K = 0;
  bool owned = false;
  int device = 0;
  std::vector<int *> rowptr, colind, extra;
  std::vector<float *> vals;
  std::vector<int> nnz;
  void release();
};
gbs_status partition_columns(int nrows, int ncols, int nnz, const int *rowptr, const int *colind,
                             const float *vals, const int *extra, int K, cudaStream_t s, ColumnParts *out);
// Parts for a gathered operand of `bbytes` bytes: 1 while it fits in half of
// L2 or the matrix is too sparse to amortise re-reading C, else the smallest
// power of two (<= 8) whose slices fit in half of L2.
gbs_status auto_parts(double bbytes, long long nnz, int ncols, int *K);
// Column parts of a forward plan: 1 under the same two conditions, else the
// smallest power of two (2..8) whose slices fit in L2.
gbs_status auto_parts_forward(double bbytes, long long nnz, int ncols, int *K);

}  // namespace gbs
