// B2SR x dense SpMM on sm_103a (binary A, FP32 / BF16 / FP16 features, FP32
// out): the row-group main pass, the ordered hub pass, the order-free cut of
// long hubs, and the tile-wide pass for tiles 16 and 32 (layout in
// b2sr_common.cuh).
#include "b2sr_common.cuh"

namespace gbs {

// ---------------------------------------------------------------------------
// B2SR x dense B (binary A): one warp per (block-row, group of R tile rows).
// The 32 lanes describe 32 (tile, column j) entries of the block-row at a
// time; a ballot keeps the entries that touch any of the warp's rows, and the
// warp walks them in lane order, gathering the feature row 4*col(t)+j once
// and adding it to each of its rows whose bit is set (plain FP32 adds, no
// multiply: A is 0/1).  Entry order: ts = 4 follows spmm4_full_full_new2
// (spmm.cu:900-943): groups of 8 tiles, column j outer, tile inner, so every
// output element is the same sequence of additions as the reference and the
// result is bitwise identical for any FP32 B; other tile sizes use tile then
// column order (= CSR column order).
// ---------------------------------------------------------------------------
struct B2srSpmmArgs {
  int nrows;  // rows of C written (rows >= nrows are skipped)
  int mb;
  const int *rowptr;
  const int *colind;
  const void *val;
  const void *B;
  int nvec;
  long long ldb, ldc;
  float *C;
  // Hub split.  The main pass leaves block-rows of more than hub_min tiles
  // (0: none) to the hub pass, which reads hubs = [count, block-row ids ...]
  // and covers each hub's feature chunks in `slices` slices.
  int hub_min;
  const int *hubs;
  int slices;
  // Order-free hub split: hub_info = [segments, tiles of all hubs], segs =
  // (block-row, first tile) per segment; seg_warps = the warps the segment
  // pass keeps resident.
  const int *hub_info;
  const int2 *segs;
  long long seg_warps;
};

// One warp: block-row br (tiles [tb0, te0) of it when tb0 >= 0), tile rows
// [grp * R, grp * R + R), feature chunks chunk0 + [0, LPR * CH); U entries
// gathered per round.  The tiles are read
// G groups (of 32 / TS tiles = 32 entries) at a time; the entries of a step
// that touch the warp's rows are compacted, in order, into a per-warp list in
// shared memory (ballot + prefix popcount), and the gathers then run over the
// list U at a time while the next step's indices and tile rows are loaded.
// Entries are added in group order and, inside a group, in lane order, so
// every output element is the same sequence of FP32 additions as a
// one-group-at-a-time walk.  `list` holds 32 * G entries (col, row bits).
// ATOMIC: the sums are added into C (float atomics) instead of stored, and a
// warp whose tiles hold none of its rows adds nothing.
template <int TS, int DT, int VEC, int LPR, int CH, int RPS, bool STORE_NZ, int U, int G, bool ATOMIC = false>
__device__ __forceinline__ void b2sr_block_row(const B2srSpmmArgs &a, long long br, int grp, int chunk0,
                                               int lane, int2 *list, int tb0 = -1, int te0 = -1) {
  constexpr int NSUB = 32 / LPR;
  constexpr int R = NSUB * RPS < TS ? NSUB * RPS : TS;  // tile rows per warp
  constexpr int TPG = 32 / TS;                          // tiles per 32 entries
  constexpr int TPS = TPG * G;                          // tiles per step
  constexpr bool REF_ORDER = (TS == 4);
  using F_ = Feat<DT, VEC>;
  using raw = typename F_::raw;

  const int sub = lane / LPR, sl = lane % LPR;
  const int row0 = grp * R;
  const int my0 = sub * RPS;  // my first row inside the warp's group
  const unsigned my_mask = ((1u << RPS) - 1u) << my0;
  const unsigned lt_mask = (1u << lane) - 1u;

  float acc[RPS][CH][VEC];
#pragma unroll
  for (int k = 0; k < RPS; ++k)
#pragma unroll
    for (int c = 0; c < CH; ++c)
#pragma unroll
      for (int q = 0; q < VEC; ++q) acc[k][c][q] = 0.f;

  const int tb = tb0 >= 0 ? tb0 : __ldg(a.rowptr + br), te = te0 >= 0 ? te0 : __ldg(a.rowptr + br + 1);
  const int j = REF_ORDER ? lane / TPG : lane % TS;
  const int l = REF_ORDER ? lane % TPG : lane / TS;
  // this lane's entry (feature row, row bits) in each of G groups
  int nb[G];
  unsigned nm[G];
  auto load_step = [&](int s0) {
#pragma unroll
    for (int g = 0; g < G; ++g) {
      const int t = s0 + g * TPG + l;
      nb[g] = 0;
      nm[g] = 0;
      if (t < te) {
        nb[g] = __ldg(a.colind + t) * TS + j;
#pragma unroll
        for (int i = 0; i < R; ++i)
          if (row0 + i < TS) nm[g] |= ((tile_row<TS>(a.val, (size_t)t, row0 + i) >> (TS - 1 - j)) & 1u) << i;
      }
    }
  };
  if (tb < te) load_step(tb);
  int listed = 0;
  for (int s0 = tb; s0 < te; s0 += TPS) {
    int n = 0;
#pragma unroll
    for (int g = 0; g < G; ++g) {
      const unsigned act = __ballot_sync(0xffffffffu, nm[g] != 0);
      if (nm[g] != 0) list[n + __popc(act & lt_mask)] = make_int2(nb[g], (int)nm[g]);
      n += __popc(act);
    }
    listed += n;
    __syncwarp();
    if (s0 + TPS < te) load_step(s0 + TPS);  // next step's indices, in flight during the gathers
    for (int k0 = 0; k0 < n; k0 += U) {
      raw bv[U][CH];
      unsigned mu[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const bool live = k0 + u < n;
        const int2 en = live ? list[k0 + u] : make_int2(0, 0);
        mu[u] = (unsigned)en.y;
        const bool need = (mu[u] & my_mask) != 0;
        const size_t rb = (size_t)(unsigned)en.x * (unsigned)a.ldb;  // 32 x 32 -> 64-bit
#pragma unroll
        for (int c = 0; c < CH; ++c) {
          const int chunk = chunk0 + c * LPR + sl;
          if (need && chunk < a.nvec) bv[u][c] = F_::load(a.B, rb + (size_t)chunk * VEC);
          else bv[u][c] = F_::zero();
        }
      }
#pragma unroll
      for (int u = 0; u < U; ++u) {
#pragma unroll
        for (int c = 0; c < CH; ++c) {
          float x[VEC];
          F_::widen(x, bv[u][c]);
#pragma unroll
          for (int k = 0; k < RPS; ++k)
            if ((mu[u] >> (my0 + k)) & 1u)
#pragma unroll
              for (int q = 0; q < VEC; ++q) acc[k][c][q] = acc[k][c][q] + x[q];
        }
      }
    }
    __syncwarp();  // the list is rewritten by the next step
  }
  if (ATOMIC && listed == 0) return;
#pragma unroll
  for (int k = 0; k < RPS; ++k) {
    const int tr = row0 + my0 + k;
    if (my0 + k >= R || tr >= TS) continue;
    const long long orow = br * TS + tr;
    if (orow >= a.nrows) continue;
    float *dst = a.C + (size_t)orow * a.ldc;
#pragma unroll
    for (int c = 0; c < CH; ++c) {
      const int chunk = chunk0 + c * LPR + sl;
      if (chunk >= a.nvec) continue;
      if constexpr (ATOMIC) {
        if constexpr (VEC % 4 == 0) {
#pragma unroll
          for (int q = 0; q < VEC; q += 4)
            atomicAdd(reinterpret_cast<float4 *>(dst + (size_t)chunk * VEC + q),
                      make_float4(acc[k][c][q], acc[k][c][q + 1], acc[k][c][q + 2], acc[k][c][q + 3]));
        } else {
#pragma unroll
          for (int q = 0; q < VEC; ++q) atomicAdd(dst + (size_t)chunk * VEC + q, acc[k][c][q]);
        }
      } else if (STORE_NZ) {
#pragma unroll
        for (int q = 0; q < VEC; ++q)
          if (acc[k][c][q] != 0.f) dst[(size_t)chunk * VEC + q] = acc[k][c][q];
      } else {
        store_vec<VEC, true>(dst + (size_t)chunk * VEC, acc[k][c]);
      }
    }
  }
}

// Main pass: one warp per (block-row, group of R tile rows), all features,
// 4 entries per round.
constexpr int MAIN_G = 2;
template <int TS, int DT, int VEC, int LPR, int CH, int RPS, bool STORE_NZ>
__global__ void __launch_bounds__(256) k_b2sr_spmm(B2srSpmmArgs a) {
  constexpr int NSUB = 32 / LPR;
  constexpr int R = NSUB * RPS < TS ? NSUB * RPS : TS;
  constexpr int NG = (TS + R - 1) / R;
  const int lane = threadIdx.x & 31;
  const long long gw = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long long br = gw / NG;
  if (br >= a.mb) return;
  if (a.hub_min > 0 && __ldg(a.rowptr + br + 1) - __ldg(a.rowptr + br) > a.hub_min) return;
  __shared__ int2 lists[8][32 * MAIN_G];
  b2sr_block_row<TS, DT, VEC, LPR, CH, RPS, STORE_NZ, 4, MAIN_G>(a, br, (int)(gw % NG), 0, lane,
                                                                 lists[threadIdx.x >> 5]);
}

// Hub pass: the block-rows a single warp would walk for far longer than any
// other (power-law hubs: thousands of tiles against a mean of tens).  The
// order of additions into an output element has to stay the tile walk's,
// so a hub is not split along its tiles.  Instead a hub is split by tile row
// and by feature slices of 32 16-byte chunks: one warp walks the tiles for
// one row and one slice, so every entry it keeps is a gather all 32 lanes
// use, and with one row per warp the registers allow HUB_U = 16 gathers per
// round instead of 4 -- the warp's chain of dependent memory round trips is
// what bounds a hub, not bandwidth.  Work items (hub, row, slice) are taken
// grid-stride.
constexpr int HUB_CHUNKS = 32;
constexpr int HUB_U = 16;
template <int TS, int DT, int VEC, bool STORE_NZ>
__global__ void __launch_bounds__(256, 1) k_b2sr_spmm_hubs(B2srSpmmArgs a) {
  const int lane = threadIdx.x & 31;
  const long long gw = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
  const long long items = (long long)__ldg(a.hubs) * TS * a.slices;
  __shared__ int2 lists[8][32 * 4];
  for (long long it = gw; it < items; it += nw) {
    const int sl = (int)(it % a.slices);
    const long long rest = it / a.slices;
    const int row = (int)(rest % TS);
    const long long br = __ldg(a.hubs + 1 + rest / TS);
    b2sr_block_row<TS, DT, VEC, 32, 1, 1, STORE_NZ, HUB_U, 4>(a, br, row, sl * HUB_CHUNKS, lane,
                                                              lists[threadIdx.x >> 5]);
  }
}

// Segments of cut hubs with the main pass's layout: one warp per (segment,
// group of R tile rows), all features, items grid-stride over a grid of
// resident CTAs; partial sums added into C.
template <int TS, int DT, int VEC, int LPR, int CH, int RPS>
__global__ void __launch_bounds__(256) k_b2sr_spmm_segs(B2srSpmmArgs a) {
  constexpr int NSUB = 32 / LPR;
  constexpr int R = NSUB * RPS < TS ? NSUB * RPS : TS;
  constexpr int NG = (TS + R - 1) / R;
  const int lane = threadIdx.x & 31;
  const long long gw = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
  const long long items = (long long)__ldcg(a.hub_info) * NG;
  const long long mean_work = (long long)__ldcg(a.hub_info + 1) * NG / a.seg_warps;
  __shared__ int2 lists[8][32 * MAIN_G];
  for (long long it = gw; it < items; it += nw) {
    const int2 sg = a.segs[it / NG];
    const int te = __ldg(a.rowptr + sg.x + 1);
    const int len = hub_segments(te - __ldg(a.rowptr + sg.x), mean_work).y;
    b2sr_block_row<TS, DT, VEC, LPR, CH, RPS, false, 4, MAIN_G, true>(a, sg.x, (int)(it % NG), 0, lane,
                                                                      lists[threadIdx.x >> 5], sg.y,
                                                                      min(te, sg.y + len));
  }
}

// SpMM body: this lane's 4 features [f0, f0 + 4) of the slice, the TS row
// sums acc[row * 32 + lane] in shared memory.
template <int TS, int DT>
struct WideSpmm {
  const B2srSpmmArgs &a;
  int f0, lane;
  bool mine;
  float4 *acc;
  // the n listed entries, WIDE_U gathers at a time, each 4-feature chunk
  // added to its row's sums
  __device__ __forceinline__ void flush(const uint16_t *list, int n, int tc_lane) {
    __syncwarp();
    for (int k0 = 0; k0 < n; k0 += WIDE_U) {
      float4 x[WIDE_U];
      int rr[WIDE_U];
#pragma unroll
      for (int u = 0; u < WIDE_U; ++u) {
        const bool live = k0 + u < n;
        const int e = live ? (int)list[k0 + u] : 0;
        rr[u] = (e >> 5) & 31;
        const int tc = __shfl_sync(0xffffffffu, tc_lane, e >> 10);
        const size_t col = (size_t)(unsigned)tc * TS + (e & 31);
        x[u] = (live && mine) ? wide_load<DT>(a.B, col * (size_t)a.ldb + f0) : make_float4(0.f, 0.f, 0.f, 0.f);
      }
#pragma unroll
      for (int u = 0; u < WIDE_U; ++u) {
        if (k0 + u < n) {
          float4 t = acc[rr[u] * 32 + lane];
          t.x = t.x + x[u].x;
          t.y = t.y + x[u].y;
          t.z = t.z + x[u].z;
          t.w = t.w + x[u].w;
          acc[rr[u] * 32 + lane] = t;
        }
      }
    }
    __syncwarp();
  }
};

// One warp: tiles [tb, te) of block-row br, features [sl * 128, +128).
template <int TS, int DT>
__device__ __forceinline__ void wide_block_row(const B2srSpmmArgs &a, long long br, int tb, int te, int sl,
                                               bool atomic, int lane, float4 *acc, uint16_t *list) {
  const int f0 = sl * WIDE_FEATS + lane * 4;
  WideSpmm<TS, DT> body{a, f0, lane, f0 < (int)a.ldc, acc};  // F % 4 == 0: all 4 features in range
#pragma unroll
  for (int q = 0; q < TS; ++q) acc[q * 32 + lane] = make_float4(0.f, 0.f, 0.f, 0.f);
  wide_walk<TS>(a.colind, a.val, tb, te, lane, list, body);
  if (!body.mine) return;
  for (int q = 0; q < TS; ++q) {
    const long long orow = br * TS + q;
    if (orow >= a.nrows) break;
    const float4 v = acc[q * 32 + lane];
    float *dst = a.C + (size_t)orow * a.ldc + f0;
    if (atomic) atomicAdd(reinterpret_cast<float4 *>(dst), v);
    else *reinterpret_cast<float4 *>(dst) = v;
  }
}

// Items: (block-row, slice) for every block-row not cut, then (segment,
// slice) for the segments of the cut ones; grid-stride over resident CTAs.
template <int TS, int DT>
__global__ void __launch_bounds__(WIDE_WARPS * 32, 1) k_b2sr_spmm_wide(B2srSpmmArgs a) {
  extern __shared__ __align__(16) unsigned char wide_sm[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  float4 *acc = reinterpret_cast<float4 *>(wide_sm) + (size_t)warp * TS * 32;
  uint16_t *list = reinterpret_cast<uint16_t *>(wide_sm + (size_t)WIDE_WARPS * TS * 32 * sizeof(float4)) +
                   (size_t)warp * wide_cap<TS>();
  const long long gw = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
  const long long cut = wide_cut(__ldg(a.rowptr + a.mb), a.slices, a.seg_warps);
  const long long main_items = (long long)a.mb * a.slices;
  const long long items = main_items + (long long)__ldcg(a.hub_info) * a.slices;
  for (long long it = gw; it < items; it += nw) {
    const int sl = (int)(it % a.slices);
    if (it < main_items) {
      const long long br = it / a.slices;
      const int tb = __ldg(a.rowptr + br), te = __ldg(a.rowptr + br + 1);
      if (te - tb > cut) continue;  // done by its segments
      wide_block_row<TS, DT>(a, br, tb, te, sl, false, lane, acc, list);
    } else {
      const int2 sg = a.segs[(it - main_items) / a.slices];
      const int te = __ldg(a.rowptr + sg.x + 1);
      const int len = wide_segments(te - __ldg(a.rowptr + sg.x), cut).y;
      wide_block_row<TS, DT>(a, sg.x, sg.y, min(te, sg.y + len), sl, true, lane, acc, list);
    }
  }
}

namespace {

struct B2srVariant {
  const void *fn;
  int vec, lpr, ch, rows_per_warp, groups;
  const void *hub_fn;      // ordered hub pass (32-chunk slices), same tile size and type
  const void *hub_seg_fn;  // segments of split hubs (full stores only)
};

template <int TS, int DT, int VEC, int LPR, int CH, bool NZ>
B2srVariant mk_b2sr() {
  constexpr int NSUB = 32 / LPR;
  constexpr int RPS0 = (32 / (CH * VEC)) > 0 ? (32 / (CH * VEC)) : 1;
  constexpr int RPS1 = RPS0 > 4 ? 4 : RPS0;
  constexpr int RPS = (NSUB * RPS1 > TS) ? ((TS / NSUB) > 0 ? TS / NSUB : 1) : RPS1;
  constexpr int R = NSUB * RPS < TS ? NSUB * RPS : TS;
  return B2srVariant{(const void *)&k_b2sr_spmm<TS, DT, VEC, LPR, CH, RPS, NZ>, VEC, LPR, CH, R,
                     (TS + R - 1) / R, (const void *)&k_b2sr_spmm_hubs<TS, DT, VEC, NZ>,
                     NZ ? nullptr : (const void *)&k_b2sr_spmm_segs<TS, DT, VEC, LPR, CH, RPS>};
}

template <int TS, int DT, int VEC, bool NZ>
bool pick_b2sr(int nvec, B2srVariant *v) {
  if (nvec <= 1) { *v = mk_b2sr<TS, DT, VEC, 1, 1, NZ>(); return true; }
  if (nvec <= 2) { *v = mk_b2sr<TS, DT, VEC, 2, 1, NZ>(); return true; }
  if (nvec <= 4) { *v = mk_b2sr<TS, DT, VEC, 4, 1, NZ>(); return true; }
  if (nvec <= 8) { *v = mk_b2sr<TS, DT, VEC, 8, 1, NZ>(); return true; }
  if (nvec <= 16) { *v = mk_b2sr<TS, DT, VEC, 16, 1, NZ>(); return true; }
  if (nvec <= 32) { *v = mk_b2sr<TS, DT, VEC, 32, 1, NZ>(); return true; }
  if (nvec <= 64) { *v = mk_b2sr<TS, DT, VEC, 32, 2, NZ>(); return true; }
  if (nvec <= 128) { *v = mk_b2sr<TS, DT, VEC, 32, 4, NZ>(); return true; }
  if (nvec <= 256) { *v = mk_b2sr<TS, DT, VEC, 32, 8, NZ>(); return true; }
  return false;
}

template <int TS, bool NZ>
bool pick_ts(int dt, int F, bool vec16, B2srVariant *v) {
  if (dt == DT_F32) {
    if (vec16 && F % 4 == 0) return pick_b2sr<TS, DT_F32, 4, NZ>(F / 4, v);
    return pick_b2sr<TS, DT_F32, 1, NZ>(F, v);
  }
  if (!vec16 || F % 8 != 0) return false;
  if (dt == DT_BF16) return pick_b2sr<TS, DT_BF16, 8, NZ>(F / 8, v);
  return pick_b2sr<TS, DT_F16, 8, NZ>(F / 8, v);
}

bool is_aligned16(const void *p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }



template <int TS, int DT>
gbs_status launch_wide(B2srSpmmArgs &a, cudaStream_t s) {
  const void *fn = (const void *)&k_b2sr_spmm_wide<TS, DT>;
  const size_t smem = wide_smem<TS>();
  GBS_CUDA_TRY(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  DeviceInfo di;
  GBS_TRY(device_info(&di));
  int per_sm = 0;
  GBS_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, WIDE_WARPS * 32, smem));
  const dim3 grid(di.sm_count * (per_sm > 0 ? per_sm : 1));
  a.seg_warps = (long long)grid.x * WIDE_WARPS;
  DevBuf info, segs;
  GBS_TRY(info.alloc(sizeof(int), s));
  GBS_TRY(segs.alloc(sizeof(int2) * (size_t)a.mb * kSegMax, s));
  GBS_CUDA_TRY(cudaMemsetAsync(info.p, 0, sizeof(int), s));
  k_wide_segments<TS><<<(int)(((long long)a.mb * 32 + 255) / 256), 256, 0, s>>>(
      a.rowptr, a.mb, a.nrows, (int)a.ldc, a.slices, a.seg_warps, reinterpret_cast<uint32_t *>(a.C), info.as<int>(),
      segs.as<int2>());
  GBS_TRY(check_launch("k_wide_segments"));
  a.hub_info = info.as<int>();
  a.segs = segs.as<int2>();
  void *args[] = {&a};
  GBS_CUDA_TRY(cudaLaunchKernel(fn, grid, dim3(WIDE_WARPS * 32), args, smem, s));
  return GBS_OK;
}

gbs_status b2sr_spmm_wide(int ts, int nrows, int mb, const int *rowptr, const int *colind, const void *val,
                          const void *B, int dt, int F, float *C, cudaStream_t s) {
  B2srSpmmArgs a{};
  a.nrows = nrows;
  a.mb = mb;
  a.rowptr = rowptr;
  a.colind = colind;
  a.val = val;
  a.B = B;
  a.nvec = F / 4;
  a.ldb = F;
  a.ldc = F;
  a.C = C;
  a.slices = (F + WIDE_FEATS - 1) / WIDE_FEATS;
#define GBS_WIDE(TS)                                           \
  if (ts == TS) {                                               \
    if (dt == DT_F32) return launch_wide<TS, DT_F32>(a, s);    \
    if (dt == DT_BF16) return launch_wide<TS, DT_BF16>(a, s);  \
    return launch_wide<TS, DT_F16>(a, s);                      \
  }
  GBS_WIDE(16)
  GBS_WIDE(32)
#undef GBS_WIDE
  return fail(GBS_ERR_UNSUPPORTED, "b2sr spmm: the tile-wide pass takes tiles 16 and 32");
}

}  // namespace

gbs_status b2sr_spmm_run(int ts, bool store_nz, int nrows, int mb, const int *rowptr, const int *colind,
                         const void *val, const void *B, int dt, int F, float *C, cudaStream_t s) {
  const bool vec16 = is_aligned16(B) && is_aligned16(C) && F % (dt == DT_F32 ? 4 : 8) == 0;
  B2srVariant v{};
  bool ok = false;
  switch (ts) {
    case 4: ok = store_nz ? pick_ts<4, true>(dt, F, vec16, &v) : pick_ts<4, false>(dt, F, vec16, &v); break;
    case 8: ok = store_nz ? pick_ts<8, true>(dt, F, vec16, &v) : pick_ts<8, false>(dt, F, vec16, &v); break;
    case 16: ok = store_nz ? pick_ts<16, true>(dt, F, vec16, &v) : pick_ts<16, false>(dt, F, vec16, &v); break;
    case 32: ok = store_nz ? pick_ts<32, true>(dt, F, vec16, &v) : pick_ts<32, false>(dt, F, vec16, &v); break;
    default: return fail(GBS_ERR_UNSUPPORTED, "b2sr spmm: tile size must be 4, 8, 16 or 32");
  }
  if (!ok)
    return fail(GBS_ERR_UNSUPPORTED,
                "b2sr spmm: F too large (FP32 <= 1024 with 16-byte alignment, else <= 256; 16-bit "
                "features need F % 8 == 0, F <= 2048)");
  if (mb == 0) return GBS_OK;
  // tiles 16 / 32 of the full-output entry point: the tile-wide pass (4
  // features per lane: FP32 16-byte or 16-bit 8-byte aligned B, F % 4 ==
  // 0).  At tile 8 the row-group kernels above are faster (flickr-shaped
  // graph, F = 256: 0.33 against 0.46 ms).
  if (!store_nz && ts >= 16 && F % 4 == 0 && is_aligned16(C) &&
      (dt == DT_F32 ? is_aligned16(B) : (reinterpret_cast<uintptr_t>(B) & 7u) == 0))
    return b2sr_spmm_wide(ts, nrows, mb, rowptr, colind, val, B, dt, F, C, s);
  B2srSpmmArgs a;
  a.nrows = nrows;
  a.mb = mb;
  a.rowptr = rowptr;
  a.colind = colind;
  a.val = val;
  a.B = B;
  a.nvec = F / v.vec;
  a.ldb = F;
  a.ldc = F;
  a.C = C;
  a.hub_min = 0;
  a.hubs = nullptr;
  a.slices = (a.nvec + HUB_CHUNKS - 1) / HUB_CHUNKS;
  a.hub_info = nullptr;
  a.segs = nullptr;
  a.seg_warps = 1;
  const long long warps = (long long)mb * v.groups;
  const int blocks = (int)((warps * 32 + 255) / 256);
  if (mb < kHubMinBlockRows) {
    void *args[] = {&a};
    GBS_CUDA_TRY(cudaLaunchKernel(v.fn, dim3(blocks), dim3(256), args, 0, s));
    return GBS_OK;
  }
  // Hub block-rows go to concurrent passes on side streams:
  //   s: find hubs [-> cut hubs] -> fork -> main pass (hubs skipped) -> join
  //   side 0:                           -> whole hubs --------------/
  //   side 1:                           -> [segments of cut hubs] -/
  // buf = [segments, tiles of all hubs, hub count, hub ids ...]
  DevBuf buf, segs, whole;
  GBS_TRY(buf.alloc(sizeof(int) * ((size_t)mb + 3), s));
  GBS_CUDA_TRY(cudaMemsetAsync(buf.p, 0, 3 * sizeof(int), s));
  int *info = buf.as<int>(), *hubs = info + 2;
  k_find_hubs<<<(mb + 255) / 256, 256, 0, s>>>(rowptr, mb, kHubTiles, hubs, info + 1);
  GBS_TRY(check_launch("k_find_hubs"));
  a.hub_min = kHubTiles;
  a.hubs = hubs;
  DeviceInfo di;
  GBS_TRY(device_info(&di));
  B2srSpmmArgs aw = a;  // the ordered pass: all hubs, or those not cut
  dim3 seg_grid;
  if (v.hub_seg_fn) {
    int per_sm = 0;
    GBS_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, v.hub_seg_fn, 256, 0));
    seg_grid = dim3(di.sm_count * (per_sm > 0 ? per_sm : 1));
    GBS_TRY(segs.alloc(sizeof(int2) * (size_t)mb * kSegMax, s));
    GBS_TRY(whole.alloc(sizeof(int) * ((size_t)mb + 1), s));
    GBS_CUDA_TRY(cudaMemsetAsync(whole.p, 0, sizeof(int), s));
    a.hub_info = info;
    a.segs = segs.as<int2>();
    a.seg_warps = (long long)seg_grid.x * 8;
    k_hub_segments<<<(mb + 7) / 8, 256, 0, s>>>(hubs, rowptr, info, segs.as<int2>(), whole.as<int>(), v.groups,
                                                a.seg_warps, ts, nrows, F, reinterpret_cast<uint32_t *>(C));
    GBS_TRY(check_launch("k_hub_segments"));
    aw.hubs = whole.as<int>();
  }
  cudaStream_t side = nullptr, side1 = nullptr;
  GBS_TRY(side_stream(&side, 0));
  if (v.hub_seg_fn) GBS_TRY(side_stream(&side1, 1));
  Events ev;
  GBS_TRY(ev.create(3));
  GBS_CUDA_TRY(cudaEventRecord(ev.e[0], s));
  GBS_CUDA_TRY(cudaStreamWaitEvent(side, ev.e[0], 0));
  if (side1) GBS_CUDA_TRY(cudaStreamWaitEvent(side1, ev.e[0], 0));
  void *args[] = {&a};
  void *wargs[] = {&aw};
  gbs_status st = GBS_OK;
  cudaError_t e = cudaSuccess;
  if (side1) {
    e = cudaLaunchKernel(v.hub_seg_fn, seg_grid, dim3(256), args, 0, side1);
    if (e != cudaSuccess) st = cuda_fail(e, "k_b2sr_spmm_segs");
    GBS_CUDA_TRY(cudaEventRecord(ev.e[2], side1));
  }
  // enough warps that every (hub, group, slice) item of a typical graph gets
  // its own warp (surplus warps exit at once)
  e = cudaLaunchKernel(v.hub_fn, dim3(di.sm_count * 8), dim3(256), wargs, 0, side);
  if (e != cudaSuccess && st == GBS_OK) st = cuda_fail(e, "k_b2sr_spmm_hubs");
  GBS_CUDA_TRY(cudaEventRecord(ev.e[1], side));
  e = cudaLaunchKernel(v.fn, dim3(blocks), dim3(256), args, 0, s);
  if (e != cudaSuccess && st == GBS_OK) st = cuda_fail(e, "k_b2sr_spmm");
  // join even on failure, so the side streams' work is ordered before
  // anything the caller enqueues next (and before the lists are freed)
  GBS_CUDA_TRY(cudaStreamWaitEvent(s, ev.e[1], 0));
  if (side1) GBS_CUDA_TRY(cudaStreamWaitEvent(s, ev.e[2], 0));
  return st;
}

}  // namespace gbs

// ===========================================================================
// C ABI
// ===========================================================================
using namespace gbs;

extern "C" gbs_status gbs_b2sr_spmm(int tile, int nrows, int nblockrows, const int *rowptr, const int *colind,
                                    const void *val, const void *B, gbs_dtype btype, int F, float *C,
                                    gbs_stream_t stream) {
  clear_error();
  GBS_REQUIRE(valid_tile(tile), "b2sr spmm: tile must be 4, 8, 16 or 32");
  GBS_REQUIRE(btype == GBS_F32 || btype == GBS_BF16 || btype == GBS_F16, "b2sr spmm: bad dtype");
  GBS_REQUIRE(nrows >= 0 && F >= 1, "b2sr spmm: bad sizes");
  GBS_REQUIRE(nblockrows == (nrows + tile - 1) / tile, "b2sr spmm: nblockrows must be ceil(nrows / tile)");
  if (nrows == 0) return GBS_OK;
  GBS_REQUIRE(rowptr && C && B, "b2sr spmm: null pointer");
  const int dt = btype == GBS_F32 ? DT_F32 : (btype == GBS_BF16 ? DT_BF16 : DT_F16);
  return b2sr_spmm_run(tile, false, nrows, nblockrows, rowptr, colind, val, B, dt, F, C,
                       (cudaStream_t)stream);
}

extern "C" gbs_status gbs_spmm4_full_full(const uint8_t *A, const float *B, float *C, const int *rowptr,
                                          const int *colind, int nblockrows, int B_cols,
                                          gbs_stream_t stream) {
  clear_error();
  GBS_REQUIRE(nblockrows >= 0 && B_cols >= 1, "spmm4_full_full: bad sizes");
  if (nblockrows == 0) return GBS_OK;
  GBS_REQUIRE(rowptr && B && C, "spmm4_full_full: null pointer");
  return b2sr_spmm_run(4, true, nblockrows * 4, nblockrows, rowptr, colind, A, B, DT_F32, B_cols, C,
                       (cudaStream_t)stream);
}

