// TEST INFRASTRUCTURE ONLY.  Device-only harness around the reference's own
// CUDA kernels, compiled from the reference sources where they lie (the
// include path points at the reference's backend/ folder; no source is
// copied here) into oracle/_ref/ref_kernels.fatbin for sm_103a by
// `make -C oracle REF=<reference checkout> refkern`.  The GPU tests load the
// fatbin with the CUDA driver API (oracle/refkern.py) and run these kernels
// beside the library's, as bit-exact checkers:
//   spmm4_full_full_new2        backend/spmm.cu:877-956 (FBF B2SR-4 SpMM)
//   ToBit{4,8,16,32}Col<float>  backend/spmm.cu:165-194, 226-246, 272-291,
//                               318-335 (tile packers of csr2bsr_batch_*)
//   ToBit32ColUd<float>,        backend/spmm.cu:93-111, 75-91 (sign packers)
//   ToBit32RowDenseSign<float>
//   packUchar2AlignedUnsigned,  backend/csr2bsr_batch_bsrbmv.cu:608-648,
//   packUshort2AlignedUnsigned  :859-888 (aligned B2SR-8/16)
//   BMM32_Arow_Brow<float>, BMM32_MT_M_S, BMM32_BIN, BMM32S_BIN
//                               backend/mm.cu:17-125 (binary GEMM)
// backend/mm.cu uses the pre-CUDA-9 warp intrinsics __shfl / __ballot,
// which no longer exist; they are mapped to their full-warp *_sync forms
// (every call site runs with all 32 lanes active).
#define __shfl(v, l) __shfl_sync(0xffffffffu, (v), (l))
#define __ballot(p) __ballot_sync(0xffffffffu, (p))

#include "csr2bsr_batch_bsrbmv.cu"  // includes spmm.cu and utility.cu
#include "mm.cu"

template __global__ void BMM32_Arow_Brow<float>(const unsigned *__restrict__, const unsigned *__restrict__,
                                                float *, const int, const int, const int);
template __global__ void ToBit4Col<float>(const float *__restrict__, uchar *, const int);
template __global__ void ToBit8Col<float>(const float *__restrict__, uchar *, const int);
template __global__ void ToBit16Col<float>(const float *__restrict__, ushort *, const int);
template __global__ void ToBit32Col<float>(const float *__restrict__, unsigned *, const int, const int);
template __global__ void ToBit32ColUd<float>(const float *__restrict__, unsigned *, const int, const int);
template __global__ void ToBit32RowDenseSign<float>(const float *__restrict__, unsigned *, const int, const int);
