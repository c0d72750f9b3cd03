"""GB300 (sm_103a) SpMM library: a drop-in for the SpMM evaluation path of
spmm_eval (CSR SpMM, CSR->B2SR packing, B2SR SpMM / BMM, binary GEMM) plus
backward kernels.  Compute runs only in lib/libgbspmm.so (C ABI in
include/gbspmm.h); this package is the host-side mirror."""

__all__ = ["ops", "graphs", "build"]
