// CSR SpMM C = A * B on sm_103a: merge-path schedule over rows + nonzeros,
// warp-wide 16-byte gathers of feature rows, FP32 accumulation.
//
// Replaces cusparseSpMM in evalCSRSpmmFloatCuSPARSE (test_spmm_full.cu:279-307:
// CSR A, alpha = 1, beta = 0, FP32) for row-major B and C.
//
// The kernel template and its schedule are described in merge_kernel.cuh.
#include <mutex>

#include "common.cuh"
#include "csr_spmm.cuh"
#include "feat.cuh"
#include "merge.cuh"
#include "merge_kernel.cuh"
#include "spmm_variants.cuh"
#include "util.cuh"

namespace gbs {

gbs_status spmm_select(int dt, int Fw, bool vec16, bool halfwarp, SpmmVariant *out, bool scaled) {
  if (scaled) return spmm_select_scaled(dt, Fw, vec16, halfwarp, out);
  return select_variant<false>(dt, Fw, vec16, halfwarp, out);
}

namespace {
constexpr int kThreads = kSpmmThreads;
constexpr long long kMinEventsPerWarp = 256;
bool aligned16(const void *p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }
}  // namespace

// Number of warps (P): one resident wave of the variant, but no warp with
// fewer than kMinEventsPerWarp merge events.
gbs_status spmm_warps(const SpmmVariant &v, int nrows, int nnz, int *P_out) {
  static std::mutex mu;
  DeviceInfo di;
  GBS_TRY(device_info(&di));
  int blocks_per_sm = 0;
  {
    std::lock_guard<std::mutex> lock(mu);
    GBS_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks_per_sm, v.fn, kThreads, 0));
  }
  if (blocks_per_sm < 1) blocks_per_sm = 1;
  const long long pmax = (long long)di.sm_count * blocks_per_sm * (kThreads / 32);
  const long long total = (long long)nrows + nnz;
  long long p = (total + kMinEventsPerWarp - 1) / kMinEventsPerWarp;
  if (p > pmax) p = pmax;
  if (p < 1) p = 1;
  *P_out = (int)p;
  return GBS_OK;
}

// Workspace layout: [arrival counters][partial-sum slots].  The counter
// region has a fixed size on a device (one int per warp the device can hold
// resident), so every call finds its counters at the same place whatever
// its shape, and that region is only ever written as counters: each call
// leaves it zero, and a workspace reused across shapes stays valid.  The
// slot region (2 P rows of the column-block width) needs no initialisation.
size_t spmm_counter_bytes() {
  DeviceInfo di;
  int warps = 152 * 64;
  if (device_info(&di) == GBS_OK) warps = di.sm_count * (di.max_threads_per_sm / 32);
  else clear_error();
  return align_up((size_t)warps * sizeof(int), 256);
}

size_t spmm_workspace_bytes(int P, int Fw) {
  const size_t ldp = align_up((size_t)Fw, 4);
  return spmm_counter_bytes() + align_up((size_t)2 * P * ldp * sizeof(float), 256);
}

// Column-block width.  col_block > 0 forces F / col_block launches of
// col_block columns (it must divide F and keep the vector alignment); each
// launch re-streams A but touches only its slice of B.  Measured on GB300 for
// the 232,965-node / 114.8M-edge graph at F = 256 (B = 238 MB > L2), every
// split was slower than one full-width launch (FP32: 8.3 ms full, 9.5 ms at
// 128, 9.9 ms at 64; BF16 likewise), because the per-nonzero work of the
// index stream is paid once per block; the default is therefore F.
gbs_status spmm_col_block(int dt, int ncols, int nnz, int F, bool vec16, int col_block, int *Fw) {
  (void)ncols;
  (void)nnz;
  const int vec = !vec16 ? 1 : (dt == DT_F32 ? 4 : 8);
  if (col_block > 0) {
    GBS_REQUIRE(col_block <= F && F % col_block == 0, "csr spmm: col_block must divide F");
    GBS_REQUIRE(col_block % vec == 0 || !vec16,
                "csr spmm: col_block must be a multiple of the 16-byte vector width");
    *Fw = col_block;
    return GBS_OK;
  }
  *Fw = F;
  return GBS_OK;
}

gbs_status spmm_launch(const SpmmVariant &v, int P, int nrows, int nnz, const int *rowptr,
                       const int *colind, const float *vals, const void *B, long long ldb, int Fw,
                       float *C, long long ldc, void *ws, cudaStream_t stream, int rp_base,
                       int accumulate, const float *rowscale, const float *colscale) {
  // the kernels address a row of B by a 32-bit byte pitch
  GBS_REQUIRE(ldb >= 0 && ldb * 4 < (1LL << 32), "csr spmm: row stride of B too large");
  MergeArgs a;
  a.rp_base = rp_base;
  a.accumulate = accumulate;
  a.H = nullptr;
  a.dvals = nullptr;
  a.perm = nullptr;
  a.nrows = nrows;
  a.nnz = nnz;
  a.F = Fw;
  a.nvec = Fw / v.vec;
  a.ldb = ldb;
  a.ldc = ldc;
  a.rowptr = rowptr;
  a.colind = colind;
  a.vals = vals;
  a.rowscale = rowscale;
  a.colscale = vals ? nullptr : colscale;
  a.B = B;
  a.C = C;
  a.ldp = (int)align_up((size_t)Fw, 4);
  a.P = P;
  const long long total = (long long)nrows + nnz;
  a.D = (total + P - 1) / P;
  if (a.D < 1) a.D = 1;
  a.counters = reinterpret_cast<int *>(ws);
  a.partials = reinterpret_cast<float *>(reinterpret_cast<char *>(ws) + spmm_counter_bytes());
  const int blocks = (P * 32 + kThreads - 1) / kThreads;
  void *args[] = {&a};
  GBS_CUDA_TRY(cudaLaunchKernel(v.fn, dim3(blocks), dim3(kThreads), args, 0, stream));
  return GBS_OK;
}

gbs_status spmm_check_args(int nrows, int ncols, int nnz, const int *rowptr, const int *colind,
                           const void *B, int F, const float *C) {
  GBS_REQUIRE(nrows >= 0 && ncols >= 0 && nnz >= 0, "csr spmm: negative size");
  GBS_REQUIRE(F >= 1, "csr spmm: F must be >= 1");
  GBS_REQUIRE(nnz == 0 || ncols > 0, "csr spmm: nnz > 0 with ncols == 0");
  if (nrows > 0) {
    GBS_REQUIRE(rowptr != nullptr && C != nullptr, "csr spmm: null rowptr or C");
  }
  if (nnz > 0) {
    GBS_REQUIRE(colind != nullptr && B != nullptr, "csr spmm: null colind or B");
  }
  return GBS_OK;
}

gbs_status spmm_plan(int dt, int nrows, int ncols, int nnz, int F, const void *B, const float *C,
                     int col_block, SpmmPlan *p, int gathered_rows, bool scaled) {
  const int vec = dt == DT_F32 ? 4 : 8;
  p->vec16 = aligned16(B) && aligned16(C) && F % vec == 0;
  GBS_TRY(spmm_col_block(dt, ncols, nnz, F, p->vec16, col_block, &p->Fw));
  DeviceInfo di;
  GBS_TRY(device_info(&di));
  const double slice = (double)(gathered_rows >= 0 ? gathered_rows : ncols) * p->Fw * (dt == DT_F32 ? 4 : 2);
  GBS_TRY(spmm_select(dt, p->Fw, p->vec16, slice <= 0.5 * (double)di.l2_bytes, &p->v, scaled));
  GBS_TRY(spmm_warps(p->v, nrows, nnz, &p->P));
  p->nblk = F / p->Fw;
  p->esize = dt == DT_F32 ? 4 : 2;
  p->ws_bytes = spmm_workspace_bytes(p->P, p->Fw);
  return GBS_OK;
}

// Workspace that covers every plan gbs_csr_spmm can choose for this shape
// (any alignment, any forced column block).
gbs_status spmm_workspace_upper(int dt, int nrows, int nnz, int F, size_t *bytes) {
  size_t best = 256;
  for (int vec16 = 0; vec16 < 2; ++vec16) {
    if (dt != DT_F32 && !vec16) continue;
    for (int Fw = 1; Fw <= F; ++Fw) {
      if (F % Fw != 0) continue;
      for (int hw = 0; hw < 4; ++hw) {  // bit 0: half-warp rows, bit 1: scaled kernels
        SpmmVariant v;
        if (spmm_select(dt, Fw, vec16 != 0, (hw & 1) != 0, &v, (hw & 2) != 0) != GBS_OK) {
          clear_error();
          continue;
        }
        int P = 1;
        GBS_TRY(spmm_warps(v, nrows, nnz, &P));
        size_t b = spmm_workspace_bytes(P, Fw);
        if (b > best) best = b;
      }
    }
  }
  size_t bb = 0;
  GBS_TRY(bwd_workspace_bytes(dt, nrows, nnz, F, &bb));
  if (bb > best) best = bb;
  *bytes = best;
  return GBS_OK;
}

gbs_status spmm_run(const SpmmPlan &p, int nrows, int nnz, const int *rowptr, const int *colind,
                    const float *vals, const void *B, int F, float *C, void *ws,
                    cudaStream_t stream, int rp_base, int accumulate, const float *rowscale,
                    const float *colscale) {
  for (int b = 0; b < p.nblk; ++b) {
    const char *Bb = reinterpret_cast<const char *>(B) + (size_t)b * p.Fw * p.esize;
    GBS_TRY(spmm_launch(p.v, p.P, nrows, nnz, rowptr, colind, vals, Bb, F, p.Fw,
                        C + (size_t)b * p.Fw, F, ws, stream, rp_base, accumulate, rowscale, colscale));
  }
  return GBS_OK;
}

}  // namespace gbs

using namespace gbs;

static int to_dt(gbs_dtype t) { return t == GBS_F32 ? DT_F32 : (t == GBS_BF16 ? DT_BF16 : DT_F16); }

extern "C" gbs_status gbs_csr_spmm_workspace_size(int nrows, int nnz, int F, gbs_dtype btype,
                                                  size_t *bytes) {
  clear_error();
  GBS_REQUIRE(bytes != nullptr, "workspace_size: null output");
  GBS_REQUIRE(nrows >= 0 && nnz >= 0 && F >= 1, "workspace_size: bad sizes");
  GBS_REQUIRE(btype == GBS_F32 || btype == GBS_BF16 || btype == GBS_F16, "workspace_size: bad dtype");
  return spmm_workspace_upper(to_dt(btype), nrows, nnz, F, bytes);
}

extern "C" gbs_status gbs_csr_spmm_workspace_init(void *ws, size_t bytes, gbs_stream_t stream) {
  clear_error();
  if (bytes == 0) return GBS_OK;
  GBS_REQUIRE(ws != nullptr, "workspace_init: null workspace");
  GBS_CUDA_TRY(cudaMemsetAsync(ws, 0, bytes, (cudaStream_t)stream));
  return GBS_OK;
}

static gbs_status csr_spmm_impl(int nrows, int ncols, int nnz, const int *rowptr, const int *colind,
                                const float *vals, const void *B, gbs_dtype btype, int F, float *C,
                                int col_block, void *ws, size_t ws_bytes, gbs_stream_t stream) {
  clear_error();
  GBS_REQUIRE(btype == GBS_F32 || btype == GBS_BF16 || btype == GBS_F16, "csr spmm: bad dtype");
  GBS_TRY(spmm_check_args(nrows, ncols, nnz, rowptr, colind, B, F, C));
  GBS_REQUIRE(col_block >= 0, "csr spmm: negative col_block");
  if (nrows == 0) return GBS_OK;
  SpmmPlan p;
  GBS_TRY(spmm_plan(to_dt(btype), nrows, ncols, nnz, F, B, C, col_block, &p));
  GBS_REQUIRE(ws != nullptr && ws_bytes >= p.ws_bytes, "csr spmm: workspace missing or too small");
  return spmm_run(p, nrows, nnz, rowptr, colind, vals, B, F, C, ws, (cudaStream_t)stream);
}

extern "C" gbs_status gbs_csr_spmm(int nrows, int ncols, int nnz, const int *rowptr,
                                   const int *colind, const float *vals, const void *B,
                                   gbs_dtype btype, int F, float *C, void *ws, size_t ws_bytes,
                                   gbs_stream_t stream) {
  return csr_spmm_impl(nrows, ncols, nnz, rowptr, colind, vals, B, btype, F, C, 0, ws, ws_bytes,
                       stream);
}

extern "C" gbs_status gbs_csr_spmm_cb(int nrows, int ncols, int nnz, const int *rowptr,
                                      const int *colind, const float *vals, const void *B,
                                      gbs_dtype btype, int F, int col_block, float *C, void *ws,
                                      size_t ws_bytes, gbs_stream_t stream) {
  return csr_spmm_impl(nrows, ncols, nnz, rowptr, colind, vals, B, btype, F, C, col_block, ws,
                       ws_bytes, stream);
}

extern "C" gbs_status gbs_csr_spmm_f32(int nrows, int ncols, int nnz, const int *rowptr,
                                       const int *colind, const float *vals, const float *B, int F,
                                       float *C, gbs_stream_t stream) {
  clear_error();
  GBS_TRY(spmm_check_args(nrows, ncols, nnz, rowptr, colind, B, F, C));
  if (nrows == 0) return GBS_OK;
  SpmmPlan p;
  GBS_TRY(spmm_plan(DT_F32, nrows, ncols, nnz, F, B, C, 0, &p));
  cudaStream_t s = (cudaStream_t)stream;
  DevBuf ws;  // library pool, stream-ordered
  GBS_TRY(ws.alloc(p.ws_bytes, s));
  GBS_CUDA_TRY(cudaMemsetAsync(ws.p, 0, p.ws_bytes, s));
  return spmm_run(p, nrows, nnz, rowptr, colind, vals, B, F, C, ws.p, s);
}
