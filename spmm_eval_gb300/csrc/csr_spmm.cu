// CSR SpMM C = A * B on sm_103a: merge-path schedule over rows + nonzeros,
// warp-wide 16-byte gathers of feature rows, FP32 accumulation.
//
// Replaces cusparseSpMM in evalCSRSpmmFloatCuSPARSE (test_spmm_full.cu:279-307:
// CSR A, alpha = 1, beta = 0, FP32) for row-major B and C.
//
// Schedule.  The merge of the row-end list rowptr[1..n] with the nonzero
// indices 0..nnz-1 has n + nnz events; warp w owns events [w*D, (w+1)*D).
// A row whose events all fall in one warp is summed by that warp in CSR
// order and written to C directly.  A row cut by a share boundary is summed
// piecewise: every warp holding a piece writes it to a workspace slot, bumps
// a per-row arrival counter, and the warp that arrives last adds the pieces
// in warp order and writes C (then resets the counter).  Nothing waits on
// another warp, and the addition order depends only on (n, nnz, P), so the
// result is bitwise reproducible for a given device and F.
//
// Lane mapping.  A feature row of F elements is nvec = F / VEC 16-byte
// chunks.  LPR = min(32, pow2 >= nvec) lanes cover one row (CH chunks each);
// the NSUB = 32 / LPR sub-groups of a warp take interleaved nonzeros of the
// same row and are folded together with xor-shuffles at the row end.
#include <mutex>

#include "common.cuh"
#include "csr_spmm.cuh"
#include "feat.cuh"
#include "merge.cuh"

namespace gbs {

struct MergeArgs {
  int nrows, nnz;
  int F;     // width of the column block handled by this launch
  int nvec;  // F / VEC
  long long ldb, ldc;  // row strides of B and C (elements)
  const int *rowptr;  // rowptr[0] == rp_base; colind/vals point at entry rp_base
  int rp_base;
  const int *colind;
  const float *vals;  // may be null: binary A
  const void *B;
  float *C;
  float *partials;  // [2P][ldp]
  int *counters;    // [P]
  int ldp;
  int P;
  long long D;
  int accumulate;  // 1: C += A B (C read, added, written); 0: C = A B
};

template <int DT, int VEC, int LPR, int CH, int U>
struct MergeKernel {
  static constexpr int NSUB = 32 / LPR;
  static constexpr int KPS = LPR;  // nonzeros per sub-group in a batch of 32
  using F_ = Feat<DT, VEC>;
  using raw = typename F_::raw;

  // Sum nonzeros [jb, je) of one row into acc (this lane's columns, this
  // lane's sub-group share).
  static __device__ __forceinline__ void accumulate(const MergeArgs &a, int jb, int je,
                                                    int lane, float (&acc)[CH][VEC]) {
    const int sub = lane / LPR;
    const int sl = lane % LPR;
#pragma unroll
    for (int c = 0; c < CH; ++c)
#pragma unroll
      for (int q = 0; q < VEC; ++q) acc[c][q] = 0.f;

    for (int base = jb; base < je; base += 32) {
      const int n_valid = min(32, je - base);
      int my_col = 0;
      float my_val = 0.f;
      if (lane < n_valid) {
        my_col = ld_stream_i32(a.colind + base + lane);
        my_val = a.vals ? ld_stream_f32(a.vals + base + lane) : 1.f;
      }
      // blocked summation: each batch of 32 nonzeros is summed into a fresh
      // partial that is then added to the row total (error ~ sqrt(32) +
      // sqrt(deg/32) roundings instead of sqrt(deg))
      float bs[CH][VEC];
#pragma unroll
      for (int c = 0; c < CH; ++c)
#pragma unroll
        for (int q = 0; q < VEC; ++q) bs[c][q] = 0.f;
      // rounds of U nonzeros per sub-group; a runtime trip count (not an
      // unrolled loop with early exits) keeps the loads of one round together
      const int rounds = (n_valid + U * NSUB - 1) / (U * NSUB);
#pragma unroll 1
      for (int rd = 0; rd < rounds; ++rd) {
        const int u0 = rd * U;
        raw bv[U][CH];
        float vv[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
          const int k = ((u0 + u) * NSUB + sub) & 31;
          const int col = __shfl_sync(0xffffffffu, my_col, k);
          const float v = __shfl_sync(0xffffffffu, my_val, k);
          const bool ok = (u0 + u) * NSUB + sub < n_valid;
          vv[u] = ok ? v : 0.f;
          const size_t rowbase = (size_t)col * (size_t)a.ldb;
#pragma unroll
          for (int c = 0; c < CH; ++c) {
            const int chunk = c * LPR + sl;
            if (ok && chunk < a.nvec) bv[u][c] = F_::load(a.B, rowbase + (size_t)chunk * VEC);
            else bv[u][c] = F_::zero();
          }
        }
#pragma unroll
        for (int u = 0; u < U; ++u)
#pragma unroll
          for (int c = 0; c < CH; ++c) F_::fma(bs[c], vv[u], bv[u][c]);
      }
#pragma unroll
      for (int c = 0; c < CH; ++c)
#pragma unroll
        for (int q = 0; q < VEC; ++q) acc[c][q] += bs[c][q];
    }
    // fold the sub-groups (fixed tree order)
#pragma unroll
    for (int off = LPR; off < 32; off <<= 1)
#pragma unroll
      for (int c = 0; c < CH; ++c)
#pragma unroll
        for (int q = 0; q < VEC; ++q) acc[c][q] += __shfl_xor_sync(0xffffffffu, acc[c][q], off);
  }

  template <bool STREAM>
  static __device__ __forceinline__ void write_row(const MergeArgs &a, float *dst, int lane,
                                                   const float (&acc)[CH][VEC]) {
    if (lane >= LPR) return;
#pragma unroll
    for (int c = 0; c < CH; ++c) {
      const int chunk = c * LPR + lane;
      if (chunk < a.nvec) store_vec<VEC, STREAM>(dst + (size_t)chunk * VEC, acc[c]);
    }
  }

  // C row += acc (accumulating launches of a column-partitioned product).
  static __device__ __forceinline__ void add_row(const MergeArgs &a, float *dst, int lane,
                                                 float (&acc)[CH][VEC]) {
    if (lane >= LPR) return;
#pragma unroll
    for (int c = 0; c < CH; ++c) {
      const int chunk = c * LPR + lane;
      if (chunk >= a.nvec) continue;
      float old[VEC];
      load_vec_cg<VEC>(dst + (size_t)chunk * VEC, old);
#pragma unroll
      for (int q = 0; q < VEC; ++q) acc[c][q] = old[q] + acc[c][q];
      store_vec<VEC, true>(dst + (size_t)chunk * VEC, acc[c]);
    }
  }

  // Called by every warp holding a piece of a split row r after it has
  // written that piece to its head or tail slot.  The last of the (w2 - w1 + 1) contributors sums the
  // pieces in warp order and writes C.
  static __device__ __forceinline__ void finish_split(const MergeArgs &a, int r, int lane) {
    const int rb = __ldg(a.rowptr + r) - a.rp_base, re = __ldg(a.rowptr + r + 1) - a.rp_base;
    const int w1 = (int)(((long long)rb + r) / a.D);
    const int w2 = (int)(((long long)re + r) / a.D);
    __threadfence();
    __syncwarp();
    int old = 0;
    if (lane == 0) old = atomicAdd(a.counters + w1, 1);
    old = __shfl_sync(0xffffffffu, old, 0);
    if (old != w2 - w1) return;
    __threadfence();
    if (lane < LPR) {
#pragma unroll
      for (int c = 0; c < CH; ++c) {
        const int chunk = c * LPR + lane;
        if (chunk >= a.nvec) continue;
        float sum[VEC], x[VEC];
        // tail piece of w1, middle pieces (tail slots), head piece of w2
        load_vec_cg<VEC>(a.partials + (size_t)(2 * w1 + 1) * a.ldp + (size_t)chunk * VEC, sum);
        for (int w = w1 + 1; w < w2; ++w) {
          load_vec_cg<VEC>(a.partials + (size_t)(2 * w + 1) * a.ldp + (size_t)chunk * VEC, x);
#pragma unroll
          for (int q = 0; q < VEC; ++q) sum[q] += x[q];
        }
        load_vec_cg<VEC>(a.partials + (size_t)(2 * w2) * a.ldp + (size_t)chunk * VEC, x);
#pragma unroll
        for (int q = 0; q < VEC; ++q) sum[q] += x[q];
        float *dst = a.C + (size_t)r * a.ldc + (size_t)chunk * VEC;
        if (a.accumulate) {
          load_vec_cg<VEC>(dst, x);
#pragma unroll
          for (int q = 0; q < VEC; ++q) sum[q] = x[q] + sum[q];
        }
        store_vec<VEC, true>(dst, sum);
      }
    }
    if (lane == 0) a.counters[w1] = 0;
  }

  static __device__ void run(const MergeArgs &a) {
    const int lane = threadIdx.x & 31;
    const int warp = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5);
    if (warp >= a.P) return;
    const long long total = (long long)a.nrows + a.nnz;
    const long long d0 = min((long long)warp * a.D, total);
    const long long d1 = min((long long)(warp + 1) * a.D, total);
    if (d0 >= d1) return;
    const int i0 = merge_search(a.rowptr, a.nrows, a.nnz, d0, a.rp_base);
    const int i1 = merge_search(a.rowptr, a.nrows, a.nnz, d1, a.rp_base);
    int j = (int)(d0 - i0);
    const int j1 = (int)(d1 - i1);

    float acc[CH][VEC];
    for (int r = i0; r < i1; ++r) {
      const int rb = __ldg(a.rowptr + r) - a.rp_base, re = __ldg(a.rowptr + r + 1) - a.rp_base;
      accumulate(a, j, re, lane, acc);
      if (j == rb) {
        if (a.accumulate) add_row(a, a.C + (size_t)r * a.ldc, lane, acc);
        else write_row<true>(a, a.C + (size_t)r * a.ldc, lane, acc);
      } else {  // head piece: the row started in an earlier warp
        write_row<false>(a, a.partials + (size_t)(2 * warp) * a.ldp, lane, acc);
        finish_split(a, r, lane);
      }
      j = re;
    }
    if (j < j1) {  // tail (or middle) piece of row i1: continues past d1
      accumulate(a, j, j1, lane, acc);
      write_row<false>(a, a.partials + (size_t)(2 * warp + 1) * a.ldp, lane, acc);
      finish_split(a, i1, lane);
    }
  }
};

// MINB: CTAs per SM the register budget must allow.  The gathers are
// latency-bound, and on GB300 more resident warps beat deeper per-warp
// unrolling: for the 232,965-node / 114.8M-edge graph at F = 256, 32 warps
// per SM with 2 (FP32) / 4 (BF16) nonzeros in flight per warp measured
// 7.12 / 5.47 ms against 7.98 / 5.67 ms for 24 warps with 4 / 8 in flight.
template <int DT, int VEC, int LPR, int CH, int U, int MINB>
__global__ void __launch_bounds__(256, MINB) k_csr_spmm_merge(MergeArgs a) {
  MergeKernel<DT, VEC, LPR, CH, U>::run(a);
}

// ---------------------------------------------------------------------------
// host side: variant selection, column blocking, grid sizing, workspace
// ---------------------------------------------------------------------------
namespace {

constexpr int kThreads = 256;
constexpr long long kMinEventsPerWarp = 256;

template <int DT, int VEC, int LPR, int CH>
SpmmVariant mk() {
  constexpr int UCAP = CH == 1 ? 4 : (CH == 2 ? 2 : 1);
  constexpr int U = UCAP < LPR ? UCAP : LPR;
  // register estimate: accumulators (+ blocked partials) + loads in flight
  constexpr int EST = 24 + 2 * CH * VEC + U * CH * 4 + U;
  constexpr int MINB = EST <= 64 ? 4 : (EST <= 80 ? 3 : (EST <= 128 ? 2 : 1));
  return SpmmVariant{(const void *)&k_csr_spmm_merge<DT, VEC, LPR, CH, U, MINB>, VEC, LPR, CH};
}

template <int DT, int VEC>
bool pick_lpr_ch(int nvec, SpmmVariant *v) {
  if (nvec <= 1) { *v = mk<DT, VEC, 1, 1>(); return true; }
  if (nvec <= 2) { *v = mk<DT, VEC, 2, 1>(); return true; }
  if (nvec <= 4) { *v = mk<DT, VEC, 4, 1>(); return true; }
  if (nvec <= 8) { *v = mk<DT, VEC, 8, 1>(); return true; }
  if (nvec <= 16) { *v = mk<DT, VEC, 16, 1>(); return true; }
  if (nvec <= 32) { *v = mk<DT, VEC, 32, 1>(); return true; }
  if (nvec <= 64) { *v = mk<DT, VEC, 32, 2>(); return true; }
  if (nvec <= 128) { *v = mk<DT, VEC, 32, 4>(); return true; }
  if (nvec <= 256) { *v = mk<DT, VEC, 32, 8>(); return true; }
  if constexpr (VEC == 1) {
    if (nvec <= 512) { *v = mk<DT, VEC, 32, 16>(); return true; }
    if (nvec <= 1024) { *v = mk<DT, VEC, 32, 32>(); return true; }
  }
  return false;
}

bool aligned16(const void *p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

}  // namespace

// Variant for a column block of width Fw.  vec16 = 16-byte vector loads are
// allowed (aligned pointers, F a multiple of the vector width).
gbs_status spmm_select(int dt, int Fw, bool vec16, SpmmVariant *out) {
  bool ok = false;
  if (dt == DT_F32) {
    if (vec16 && Fw % 4 == 0) ok = pick_lpr_ch<DT_F32, 4>(Fw / 4, out);
    else ok = pick_lpr_ch<DT_F32, 1>(Fw, out);
    if (!ok) return fail(GBS_ERR_UNSUPPORTED, "csr spmm: FP32 features need F <= 1024");
  } else {
    if (!vec16 || Fw % 8 != 0)
      return fail(GBS_ERR_UNSUPPORTED,
                  "csr spmm: 16-bit features need F % 8 == 0 and 16-byte aligned B/C");
    ok = dt == DT_BF16 ? pick_lpr_ch<DT_BF16, 8>(Fw / 8, out) : pick_lpr_ch<DT_F16, 8>(Fw / 8, out);
    if (!ok) return fail(GBS_ERR_UNSUPPORTED, "csr spmm: 16-bit features need F <= 2048");
  }
  return GBS_OK;
}

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
                       int accumulate) {
  MergeArgs a;
  a.rp_base = rp_base;
  a.accumulate = accumulate;
  a.nrows = nrows;
  a.nnz = nnz;
  a.F = Fw;
  a.nvec = Fw / v.vec;
  a.ldb = ldb;
  a.ldc = ldc;
  a.rowptr = rowptr;
  a.colind = colind;
  a.vals = vals;
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
                     int col_block, SpmmPlan *p) {
  const int vec = dt == DT_F32 ? 4 : 8;
  p->vec16 = aligned16(B) && aligned16(C) && F % vec == 0;
  GBS_TRY(spmm_col_block(dt, ncols, nnz, F, p->vec16, col_block, &p->Fw));
  GBS_TRY(spmm_select(dt, p->Fw, p->vec16, &p->v));
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
      SpmmVariant v;
      if (spmm_select(dt, Fw, vec16 != 0, &v) != GBS_OK) { clear_error(); continue; }
      int P = 1;
      GBS_TRY(spmm_warps(v, nrows, nnz, &P));
      size_t b = spmm_workspace_bytes(P, Fw);
      if (b > best) best = b;
    }
  }
  *bytes = best;
  return GBS_OK;
}

gbs_status spmm_run(const SpmmPlan &p, int nrows, int nnz, const int *rowptr, const int *colind,
                    const float *vals, const void *B, int F, float *C, void *ws,
                    cudaStream_t stream, int rp_base, int accumulate) {
  for (int b = 0; b < p.nblk; ++b) {
    const char *Bb = reinterpret_cast<const char *>(B) + (size_t)b * p.Fw * p.esize;
    GBS_TRY(spmm_launch(p.v, p.P, nrows, nnz, rowptr, colind, vals, Bb, F, p.Fw,
                        C + (size_t)b * p.Fw, F, ws, stream, rp_base, accumulate));
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
  void *ws = nullptr;
  GBS_CUDA_TRY(cudaMallocAsync(&ws, p.ws_bytes, s));
  cudaError_t e = cudaMemsetAsync(ws, 0, p.ws_bytes, s);
  gbs_status st = GBS_OK;
  if (e != cudaSuccess) st = cuda_fail(e, "cudaMemsetAsync");
  if (st == GBS_OK) st = spmm_run(p, nrows, nnz, rowptr, colind, vals, B, F, C, ws, s);
  cudaError_t e2 = cudaFreeAsync(ws, s);
  if (st == GBS_OK && e2 != cudaSuccess) st = cuda_fail(e2, "cudaFreeAsync");
  return st;
}
