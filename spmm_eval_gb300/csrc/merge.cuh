// Merge-path coordinate search shared by the CSR kernels.
#pragma once

namespace gbs {

// Largest i in [0, n] with rowptr[i] + i <= d: the number of rows finished
// at diagonal d of the merge of the row-end list rowptr[1..n] with the
// nonzero indices 0..nnz-1.
// base: value of rowptr[0] (row pointers of a row range of a larger matrix).
__device__ __forceinline__ int merge_search(const int *__restrict__ rowptr, int n, int nnz, long long d,
                                            int base = 0) {
  long long lo = d - nnz;
  if (lo < 0) lo = 0;
  long long hi = d < n ? d : n;
  while (lo < hi) {
    long long mid = (lo + hi + 1) >> 1;
    if ((long long)(__ldg(rowptr + mid) - base) + mid <= d) lo = mid;
    else hi = mid - 1;
  }
  return (int)lo;
}

}  // namespace gbs
