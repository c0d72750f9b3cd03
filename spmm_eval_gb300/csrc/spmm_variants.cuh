// Forward merge-path SpMM kernel and its variant table, shared by the
// translation units that instantiate it: csr_spmm.cu (stored or unit values)
// and csr_spmm_scaled.cu (degree-normalised binary A, SC = true).
#pragma once

#include "common.cuh"
#include "csr_spmm.cuh"
#include "feat.cuh"
#include "merge.cuh"
#include "merge_kernel.cuh"

namespace gbs {

constexpr int kSpmmThreads = 256;

// MINB: CTAs per SM the register budget must allow.  The gathers are
// latency-bound, and on GB300 more resident warps beat deeper per-warp
// unrolling: for the 232,965-node / 114.8M-edge graph at F = 256, 32 warps
// per SM with 2 (FP32) / 4 (BF16) nonzeros in flight per warp measured
// 7.12 / 5.47 ms against 7.98 / 5.67 ms for 24 warps with 4 / 8 in flight.
template <int DT, int VEC, int LPR, int CH, int U, int MINB, bool SC>
__global__ void __launch_bounds__(256, MINB) k_csr_spmm_merge(MergeArgs a) {
  MergeKernel<DT, VEC, LPR, CH, U, false, SC>::run(a);
}

template <int DT, int VEC, int LPR, int CH, bool SC>
SpmmVariant mk() {
  constexpr int UCAP = CH == 1 ? 4 : (CH == 2 ? 2 : 1);
  constexpr int U = UCAP < LPR ? UCAP : LPR;
  // register estimate: accumulators (+ blocked partials, FP32 only) + loads
  // in flight.  Without the partials the half-warp BF16 variant fits 4 CTAs
  // per SM: 4.21 against 4.78 ms (114.8M-edge graph, F = 256, 2 parts).
  constexpr int EST = 24 + (DT == DT_F32 ? 2 : 1) * CH * VEC + U * CH * 4 + U;
  constexpr int MINB = EST <= 64 ? 4 : (EST <= 80 ? 3 : (EST <= 128 ? 2 : 1));
  return SpmmVariant{(const void *)&k_csr_spmm_merge<DT, VEC, LPR, CH, U, MINB, SC>, VEC, LPR, CH};
}

// Lanes per row (LPR) and 16-byte chunks per lane (CH) for rows of nvec
// chunks.  With `halfwarp` (the gathered rows of B fit in half of L2), rows
// of 17-32 chunks of 16-bit features and 33-64 chunks of FP32 (F = 136..256)
// run on half-warps, two nonzeros per warp at a time: one shuffle pair then
// feeds two gathers, which measured 4.8 against 5.3 ms (BF16, 2 parts) and
// 6.4 against 6.7 ms (FP32, 4 parts) on the 114.8M-edge graph at F = 256.
// The half-warp variants need more registers (3 instead of 4 CTAs per SM),
// which costs more than it saves when many gathers go to DRAM.
template <int DT, int VEC, bool SC>
bool pick_lpr_ch(int nvec, bool halfwarp, SpmmVariant *v) {
  if (nvec <= 1) { *v = mk<DT, VEC, 1, 1, SC>(); return true; }
  if (nvec <= 2) { *v = mk<DT, VEC, 2, 1, SC>(); return true; }
  if (nvec <= 4) { *v = mk<DT, VEC, 4, 1, SC>(); return true; }
  if (nvec <= 8) { *v = mk<DT, VEC, 8, 1, SC>(); return true; }
  if (nvec <= 16) { *v = mk<DT, VEC, 16, 1, SC>(); return true; }
  if constexpr (VEC == 8) {
    if (halfwarp && nvec <= 32) { *v = mk<DT, VEC, 16, 2, SC>(); return true; }
  }
  if (nvec <= 32) { *v = mk<DT, VEC, 32, 1, SC>(); return true; }
  if constexpr (VEC == 4) {
    if (halfwarp && nvec <= 64) { *v = mk<DT, VEC, 16, 4, SC>(); return true; }
  }
  if (nvec <= 64) { *v = mk<DT, VEC, 32, 2, SC>(); return true; }
  if (nvec <= 128) { *v = mk<DT, VEC, 32, 4, SC>(); return true; }
  if (nvec <= 256) { *v = mk<DT, VEC, 32, 8, SC>(); return true; }
  if constexpr (VEC == 1) {
    if (nvec <= 512) { *v = mk<DT, VEC, 32, 16, SC>(); return true; }
    if (nvec <= 1024) { *v = mk<DT, VEC, 32, 32, SC>(); return true; }
  }
  return false;
}

// Variant for a column block of width Fw.  vec16 = 16-byte vector loads are
// allowed (aligned pointers, F a multiple of the vector width).
template <bool SC>
gbs_status select_variant(int dt, int Fw, bool vec16, bool halfwarp, SpmmVariant *out) {
  bool ok = false;
  if (dt == DT_F32) {
    if (vec16 && Fw % 4 == 0) ok = pick_lpr_ch<DT_F32, 4, SC>(Fw / 4, halfwarp, out);
    else ok = pick_lpr_ch<DT_F32, 1, SC>(Fw, halfwarp, out);
    if (!ok) return fail(GBS_ERR_UNSUPPORTED, "csr spmm: FP32 features need F <= 1024");
  } else {
    if (!vec16 || Fw % 8 != 0)
      return fail(GBS_ERR_UNSUPPORTED,
                  "csr spmm: 16-bit features need F % 8 == 0 and 16-byte aligned B/C");
    ok = dt == DT_BF16 ? pick_lpr_ch<DT_BF16, 8, SC>(Fw / 8, halfwarp, out)
                       : pick_lpr_ch<DT_F16, 8, SC>(Fw / 8, halfwarp, out);
    if (!ok) return fail(GBS_ERR_UNSUPPORTED, "csr spmm: 16-bit features need F <= 2048");
  }
  return GBS_OK;
}


}  // namespace gbs
