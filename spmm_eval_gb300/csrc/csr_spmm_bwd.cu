// Fused backward of C = A H in one pass over A^T's pattern:
//   dH[c]     = sum_r A[r][c] dC[r]          (merge-path SpMM on A^T)
//   dvals[e]  = <dC[r], H[c]>  for e = (r, c) (SDDMM on A's pattern)
// A warp walking row c of A^T gathers dC[r] for every entry (r, c) for the
// SpMM anyway; with H[c] held in registers the SDDMM dot product costs only
// FMAs and a butterfly reduction, and the separate SDDMM pass -- a second
// gather of every row -- disappears.  The one-pass form writes dvals in A's
// entry order through the transpose's permutation.
//
// The planned form splits A^T by column ranges (= row ranges of A, = slices
// of dC) so that each pass's dC gathers stay in L2, like the forward plan:
// the dH part of each pass accumulates, and every entry's dvals is computed
// by the one pass that holds it.  The passes write dvals in their own entry
// order (coalesced) to a temporary, and one gather pass puts them in A's
// order: dvals[e] = tmp[q[e]].  Scattering 4-byte values through the
// permutation inside the gather-bound kernel costs a 32-byte DRAM
// read-modify-write per value (about 0.9 GB of extra writes, and more reads,
// per FP32 pass on the 114.8M-edge graph); in the gather pass the reads of
// one part's block of the temporary mostly hit L2 and the writes are
// sequential.
#include <vector>

#include "common.cuh"
#include "csr_spmm.cuh"
#include "merge_kernel.cuh"
#include "transpose.cuh"
#include "util.cuh"

namespace gbs {

template <int DT, int VEC, int LPR, int CH, int U, int MINB>
__global__ void __launch_bounds__(256, MINB) k_csr_spmm_bwd(MergeArgs a) {
  MergeKernel<DT, VEC, LPR, CH, U, true>::run(a);
}

namespace {

template <int DT, int VEC, int LPR, int CH>
SpmmVariant mkb() {
  constexpr int UCAP = CH == 1 ? 4 : (CH == 2 ? 2 : 1);
  constexpr int U = UCAP < LPR ? UCAP : LPR;
  // accumulators (+ blocked partials, FP32 only) + H row + loads in flight
  constexpr int EST = 24 + (DT == DT_F32 ? 3 : 2) * CH * VEC + U * CH * 4 + 2 * U;
  constexpr int MINB = EST <= 60 ? 4 : (EST <= 80 ? 3 : (EST <= 128 ? 2 : 1));
  return SpmmVariant{(const void *)&k_csr_spmm_bwd<DT, VEC, LPR, CH, U, MINB>, VEC, LPR, CH};
}

template <int DT, int VEC>
bool pickb(int nvec, SpmmVariant *v) {
  if (nvec <= 1) { *v = mkb<DT, VEC, 1, 1>(); return true; }
  if (nvec <= 2) { *v = mkb<DT, VEC, 2, 1>(); return true; }
  if (nvec <= 4) { *v = mkb<DT, VEC, 4, 1>(); return true; }
  if (nvec <= 8) { *v = mkb<DT, VEC, 8, 1>(); return true; }
  if (nvec <= 16) { *v = mkb<DT, VEC, 16, 1>(); return true; }
  // 16-bit rows of 17-32 chunks (F = 136..256) on half-warps: one shuffle
  // pair and one dot-product butterfly serve two gathers per lane (BF16
  // backward step of the 114.8M-edge graph at F = 256: 6.69 against 7.66 ms
  // on full-warp rows)
  if constexpr (VEC == 8) {
    if (nvec <= 32) { *v = mkb<DT, VEC, 16, 2>(); return true; }
  }
  if (nvec <= 32) { *v = mkb<DT, VEC, 32, 1>(); return true; }
  if (nvec <= 64) { *v = mkb<DT, VEC, 32, 2>(); return true; }
  if (nvec <= 128) { *v = mkb<DT, VEC, 32, 4>(); return true; }
  if (nvec <= 256) { *v = mkb<DT, VEC, 32, 8>(); return true; }
  return false;
}

}  // namespace

gbs_status bwd_variant(gbs_dtype dtype, int F, SpmmVariant *v, int *dt) {
  GBS_REQUIRE(dtype == GBS_F32 || dtype == GBS_BF16 || dtype == GBS_F16, "spmm backward: bad dtype");
  GBS_REQUIRE(F >= 1, "spmm backward: F must be >= 1");
  *dt = dtype == GBS_F32 ? DT_F32 : (dtype == GBS_BF16 ? DT_BF16 : DT_F16);
  const int vec = *dt == DT_F32 ? 4 : 8;
  GBS_REQUIRE(F % vec == 0, "spmm backward: F must be a multiple of 4 (FP32) / 8 (16-bit)");
  bool ok = *dt == DT_F32 ? pickb<DT_F32, 4>(F / 4, v)
                          : (*dt == DT_BF16 ? pickb<DT_BF16, 8>(F / 8, v) : pickb<DT_F16, 8>(F / 8, v));
  if (!ok) return fail(GBS_ERR_UNSUPPORTED, "spmm backward: F too large (FP32 <= 1024, 16-bit <= 2048)");
  return GBS_OK;
}

gbs_status bwd_launch(const SpmmVariant &v, int n, int nnz, const int *rowptr, const int *colind, const float *vals,
                      const int *perm, const void *dC, const void *H, int F, float *dB, float *dvals, void *ws,
                      size_t ws_bytes, int accumulate, cudaStream_t s) {
  int P = 0;
  GBS_TRY(spmm_warps(v, n, nnz, &P));
  GBS_REQUIRE(ws != nullptr && ws_bytes >= spmm_workspace_bytes(P, F),
              "spmm backward: workspace missing or too small (size it as gbs_csr_spmm_workspace_size(ncols, nnz, F))");
  MergeArgs a;
  a.nrows = n;
  a.nnz = nnz;
  a.F = F;
  a.nvec = F / v.vec;
  a.ldb = F;
  a.ldc = F;
  a.rowptr = rowptr;
  a.rp_base = 0;
  a.colind = colind;
  a.vals = vals;
  a.rowscale = nullptr;
  a.colscale = nullptr;
  a.B = dC;
  a.C = dB;
  a.ldp = (int)align_up((size_t)F, 4);
  a.P = P;
  const long long total = (long long)n + nnz;
  a.D = (total + P - 1) / P;
  if (a.D < 1) a.D = 1;
  a.counters = reinterpret_cast<int *>(ws);
  a.partials = reinterpret_cast<float *>(reinterpret_cast<char *>(ws) + spmm_counter_bytes());
  a.accumulate = accumulate;
  a.H = H;
  a.dvals = dvals;
  a.perm = perm;
  void *args[] = {&a};
  GBS_CUDA_TRY(cudaLaunchKernel(v.fn, dim3((unsigned)((P * 32 + 255) / 256)), dim3(256), args, 0, s));
  return GBS_OK;
}

gbs_status bwd_workspace_bytes(int dt, int nrows, int nnz, int F, size_t *bytes) {
  *bytes = 0;
  const gbs_dtype d = dt == DT_F32 ? GBS_F32 : (dt == DT_BF16 ? GBS_BF16 : GBS_F16);
  SpmmVariant v{};
  int dd = 0;
  if (bwd_variant(d, F, &v, &dd) != GBS_OK) {  // no backward kernel for this shape
    clear_error();
    return GBS_OK;
  }
  int P = 0;
  GBS_TRY(spmm_warps(v, nrows, nnz, &P));
  *bytes = spmm_workspace_bytes(P, F);
  return GBS_OK;
}

}  // namespace gbs

struct gbs_spmm_backward_plan {
  int n, nnz, F;  // rows of A^T (= columns of A), entries
  gbs_dtype dtype;
  gbs::ColumnParts parts;  // A^T by column ranges; extra = transpose permutation
  int *q = nullptr;        // A entry e -> position in the part-major temporary
  std::vector<long long> off;  // first temporary position of each part
};

namespace gbs {

// q[perm_p[i]] = off_p + i for every part p.
__global__ void k_part_inverse(const int *__restrict__ perm, int n, long long off, int *__restrict__ q) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) q[perm[i]] = (int)(off + i);
}

// dvals[e] = tmp[q[e]]
__global__ void k_gather_dvals(const int *__restrict__ q, const float *__restrict__ tmp, long long n,
                               float *__restrict__ dvals) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dvals[i] = __ldg(tmp + __ldg(q + i));
}

}  // namespace gbs

using namespace gbs;

extern "C" gbs_status gbs_spmm_backward(const gbs_csr_transpose *T, const float *t_vals, const void *dC,
                                        const void *H, gbs_dtype dtype, int F, float *dB, float *dvals, void *ws,
                                        size_t ws_bytes, gbs_stream_t stream) {
  clear_error();
  GBS_REQUIRE(T != nullptr, "spmm backward: null transpose handle");
  SpmmVariant v{};
  int dt = 0;
  GBS_TRY(bwd_variant(dtype, F, &v, &dt));
  const int n = T->ncols;  // rows of A^T
  if (n == 0) return GBS_OK;
  GBS_REQUIRE(dC && H && dB && dvals, "spmm backward: null pointer");
  const uintptr_t al = reinterpret_cast<uintptr_t>(dC) | reinterpret_cast<uintptr_t>(H) |
                       reinterpret_cast<uintptr_t>(dB);
  GBS_REQUIRE((al & 15u) == 0, "spmm backward: needs 16-byte aligned dC, H and dB");
  return bwd_launch(v, n, T->nnz, T->t_rowptr, T->t_colind, t_vals, T->perm, dC, H, F, dB, dvals, ws, ws_bytes, 0,
                    (cudaStream_t)stream);
}

extern "C" gbs_status gbs_spmm_backward_plan_create(const gbs_csr_transpose *T, const float *t_vals,
                                                    gbs_dtype dtype, int F, int parts, gbs_stream_t stream,
                                                    gbs_spmm_backward_plan **out) {
  clear_error();
  GBS_REQUIRE(out != nullptr, "spmm backward plan: null output");
  *out = nullptr;
  GBS_REQUIRE(T != nullptr, "spmm backward plan: null transpose handle");
  GBS_REQUIRE(parts >= 0 && parts <= 64, "spmm backward plan: parts must be 0 (auto) .. 64");
  SpmmVariant v{};
  int dt = 0;
  GBS_TRY(bwd_variant(dtype, F, &v, &dt));
  int K = parts;
  // the gathered operand is dC: rows of A x F
  if (K == 0) GBS_TRY(auto_parts((double)T->nrows * F * (dtype == GBS_F32 ? 4.0 : 2.0), T->nnz, T->nrows, &K));
  auto *P = new gbs_spmm_backward_plan();
  P->n = T->ncols;
  P->nnz = T->nnz;
  P->F = F;
  P->dtype = dtype;
  cudaStream_t s = (cudaStream_t)stream;
  gbs_status st = partition_columns(T->ncols, T->nrows, T->nnz, T->t_rowptr, T->t_colind, t_vals, T->perm, K, s,
                                    &P->parts);
  if (st == GBS_OK && T->nnz > 0) {
    cudaError_t e = cudaMalloc(&P->q, sizeof(int) * (size_t)T->nnz);
    if (e != cudaSuccess) {
      P->q = nullptr;
      st = cuda_fail(e, "cudaMalloc");
    }
    long long off = 0;
    for (int p = 0; st == GBS_OK && p < P->parts.K; ++p) {
      P->off.push_back(off);
      const int m = P->parts.nnz[p];
      if (m > 0) {
        k_part_inverse<<<(m + 255) / 256, 256, 0, s>>>(P->parts.extra[p], m, off, P->q);
        st = check_launch("k_part_inverse");
      }
      off += m;
    }
    if (st == GBS_OK) {
      e = cudaStreamSynchronize(s);
      if (e != cudaSuccess) st = cuda_fail(e, "cudaStreamSynchronize");
    }
    // the permutation pieces are folded into q: drop the plan's copies
    if (st == GBS_OK && P->parts.owned)
      for (auto &x : P->parts.extra)
        if (x) {
          cudaFree(x);
          x = nullptr;
        }
  } else if (st == GBS_OK) {
    P->off.assign(P->parts.K, 0);
  }
  if (st != GBS_OK) {
    if (P->q) cudaFree(P->q);
    P->parts.release();
    delete P;
    return st;
  }
  *out = P;
  return GBS_OK;
}

extern "C" gbs_status gbs_spmm_backward_plan_parts(const gbs_spmm_backward_plan *P, int *parts) {
  clear_error();
  GBS_REQUIRE(P && parts, "spmm backward plan: null argument");
  *parts = P->parts.K;
  return GBS_OK;
}

extern "C" gbs_status gbs_spmm_backward_plan_destroy(gbs_spmm_backward_plan *P) {
  clear_error();
  if (P) {
    if (P->q) {
      int cur = 0;
      cudaGetDevice(&cur);
      cudaSetDevice(P->parts.device);
      cudaFree(P->q);
      cudaSetDevice(cur);
    }
    P->parts.release();
    delete P;
  }
  return GBS_OK;
}

extern "C" gbs_status gbs_spmm_backward_planned(const gbs_spmm_backward_plan *P, const void *dC, const void *H,
                                                float *dB, float *dvals, void *ws, size_t ws_bytes,
                                                gbs_stream_t stream) {
  clear_error();
  GBS_REQUIRE(P != nullptr, "spmm backward planned: null plan");
  if (P->n == 0) return GBS_OK;
  GBS_REQUIRE(dC && H && dB && dvals, "spmm backward planned: null pointer");
  const uintptr_t al = reinterpret_cast<uintptr_t>(dC) | reinterpret_cast<uintptr_t>(H) |
                       reinterpret_cast<uintptr_t>(dB);
  GBS_REQUIRE((al & 15u) == 0, "spmm backward planned: needs 16-byte aligned dC, H and dB");
  SpmmVariant v{};
  int dt = 0;
  GBS_TRY(bwd_variant(P->dtype, P->F, &v, &dt));
  const ColumnParts &cp = P->parts;
  cudaStream_t s = (cudaStream_t)stream;
  DevBuf tmp;
  GBS_TRY(tmp.alloc(sizeof(float) * (size_t)P->nnz, s));
  // Part p holds the entries of a range of A's rows, so A's entries
  // [off_p, off_p + nnz_p) take their dvals from part p's block of the
  // temporary only: part p's gather runs on the side stream while the next
  // pass runs, and only the last part's gather follows the passes.
  cudaStream_t side = nullptr;
  if (cp.K > 1) GBS_TRY(side_stream(&side));
  std::vector<cudaEvent_t> evs;
  struct EvGuard {
    std::vector<cudaEvent_t> &e;
    ~EvGuard() {
      for (auto x : e) cudaEventDestroy(x);
    }
  } guard{evs};
  auto gather = [&](int p, cudaStream_t st) -> gbs_status {
    const int m = cp.nnz[p];
    if (m == 0) return GBS_OK;
    const long long o = P->off[p];
    k_gather_dvals<<<(int)(((long long)m + 255) / 256), 256, 0, st>>>(P->q + o, tmp.as<float>(), m, dvals + o);
    return check_launch("k_gather_dvals");
  };
  for (int p = 0; p < cp.K; ++p) {
    GBS_TRY(bwd_launch(v, P->n, cp.nnz[p], cp.rowptr[p], cp.colind[p], cp.vals[p], nullptr, dC, H, P->F, dB,
                       tmp.as<float>() + P->off[p], ws, ws_bytes, p > 0 ? 1 : 0, s));
    if (p + 1 < cp.K) {
      cudaEvent_t e = nullptr;
      GBS_CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
      evs.push_back(e);
      GBS_CUDA_TRY(cudaEventRecord(e, s));
      GBS_CUDA_TRY(cudaStreamWaitEvent(side, e, 0));
      GBS_TRY(gather(p, side));
    } else {
      GBS_TRY(gather(p, s));
    }
  }
  if (cp.K > 1) {  // join: the side gathers finish before anything later on s (and the temporary's free)
    cudaEvent_t e = nullptr;
    GBS_CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    evs.push_back(e);
    GBS_CUDA_TRY(cudaEventRecord(e, side));
    GBS_CUDA_TRY(cudaStreamWaitEvent(s, e, 0));
  }
  return GBS_OK;
}
