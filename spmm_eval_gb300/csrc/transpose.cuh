// Layout of the opaque gbs_csr_transpose handle (shared by transpose.cu and
// the fused backward in csr_spmm_bwd.cu).
#pragma once

struct gbs_csr_transpose {
  int nrows, ncols, nnz;  // of A
  int device;
  int *t_rowptr;  // ncols + 1
  int *t_colind;  // nnz
  int *perm;      // nnz: entry i of A^T is entry perm[i] of A
};
