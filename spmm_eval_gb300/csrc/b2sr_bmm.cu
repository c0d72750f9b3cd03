// B2SR x bit-packed features on sm_103a (int32 popcounts or the +-1 form):
// the row-group main pass, the hub pass, the order-free cut of long hubs,
// the aligned B2SR-8/16 reads and the tile-wide pass for tile 32 (layout in
// b2sr_common.cuh).
#include "b2sr_common.cuh"

namespace gbs {

// ---------------------------------------------------------------------------
// B2SR x packed-bit features -> int32 counts (BMV for F = 32, BMM above).
// X row j = W = ceil(F/32) uint32 words, column 32w+b at bit 31-b of word w
// (ToBit32RowDenseSign layout, spmm.cu:75-91).  C01[i][k] = sum_j A_ij
// bit_jk; signed form 2*C01 - deg(i) is the +-1 product.  Lane l owns columns
// l, l+32, ...; one warp per (block-row, group of R tile rows), R*W <= 32
// counters per lane.
// ---------------------------------------------------------------------------
struct B2srBmmArgs {
  int nrows, mb, F, W;
  const int *rowptr;
  const int *colind;
  const void *val;
  const uint32_t *X;
  int32_t *C;
  int signed_form;
  int hub_min;      // main pass: leave block-rows of more tiles to the hub pass (0: none)
  const int *hubs;  // hub pass: [count, block-row ids ...]
  // hub split, as in B2srSpmmArgs
  const int *hub_info;
  const int2 *segs;
  long long seg_warps;
};

// One warp: block-row br, tile rows [grp * R, grp * R + R).  Entries of G
// groups at a time are compacted into the per-warp shared-memory list (as
// in b2sr_block_row), then gathered U at a time while the next step's
// indices load.  Integer counts: the order of entries does not matter here.
// AL: the tiles come in the aligned B2SR-8/16 layout (padding tiles carry
// no bits, so they drop out at the compaction).
// With tb0 >= 0 only tiles [tb0, te0) are walked; ATOMIC adds the counts of
// the rows with entries (and the +-1 form's additive 2 count - entries) into
// C.
template <int TS, int WMAX, int R, int U, int G, bool AL, bool ATOMIC = false>
__device__ __forceinline__ void bmm_block_row(const B2srBmmArgs &a, long long br, int grp, int lane, int2 *list,
                                              int tb0 = -1, int te0 = -1) {
  constexpr int TPG = 32 / TS;
  constexpr int TPS = TPG * G;
  const int row0 = grp * R;
  const unsigned lt_mask = (1u << lane) - 1u;
  int cnt[R][WMAX];
  int deg[R];
#pragma unroll
  for (int i = 0; i < R; ++i) {
    deg[i] = 0;
#pragma unroll
    for (int k = 0; k < WMAX; ++k) cnt[i][k] = 0;
  }
  const int tb = tb0 >= 0 ? tb0 : __ldg(a.rowptr + br), te = tb0 >= 0 ? te0 : __ldg(a.rowptr + br + 1);
  const int j = lane % TS, l = lane / TS;
  const int shift = 31 - lane;
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
          if (row0 + i < TS)
            nm[g] |= ((tile_row_any<TS, AL>(a.val, (size_t)t, row0 + i) >> (TS - 1 - j)) & 1u) << i;
      }
    }
  };
  if (tb < te) load_step(tb);
  for (int s0 = tb; s0 < te; s0 += TPS) {
    int n = 0;
#pragma unroll
    for (int g = 0; g < G; ++g) {
      const unsigned act = __ballot_sync(0xffffffffu, nm[g] != 0);
      if (nm[g] != 0) list[n + __popc(act & lt_mask)] = make_int2(nb[g], (int)nm[g]);
      n += __popc(act);
    }
    __syncwarp();
    if (s0 + TPS < te) load_step(s0 + TPS);
    for (int k0 = 0; k0 < n; k0 += U) {
      uint32_t w[U][WMAX];
      unsigned mu[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const bool live = k0 + u < n;
        const int2 en = live ? list[k0 + u] : make_int2(0, 0);
        mu[u] = (unsigned)en.y;
        const uint32_t *xr = a.X + (size_t)(unsigned)en.x * (unsigned)a.W;
#pragma unroll
        for (int k = 0; k < WMAX; ++k) w[u][k] = (live && k < a.W) ? __ldg(xr + k) : 0u;
      }
#pragma unroll
      for (int u = 0; u < U; ++u)
#pragma unroll
        for (int i = 0; i < R; ++i)
          if ((mu[u] >> i) & 1u) {
            ++deg[i];
#pragma unroll
            for (int k = 0; k < WMAX; ++k) cnt[i][k] += (int)((w[u][k] >> shift) & 1u);
          }
    }
    __syncwarp();
  }
#pragma unroll
  for (int i = 0; i < R; ++i) {
    const int tr = row0 + i;
    if (tr >= TS) continue;
    const long long orow = br * TS + tr;
    if (orow >= a.nrows || (ATOMIC && deg[i] == 0)) continue;
    int32_t *dst = a.C + (size_t)orow * a.F;
#pragma unroll
    for (int k = 0; k < WMAX; ++k) {
      const int c = k * 32 + lane;
      const int v = a.signed_form ? 2 * cnt[i][k] - deg[i] : cnt[i][k];
      if (c < a.F) {
        if constexpr (ATOMIC) atomicAdd(dst + c, v);
        else dst[c] = v;
      }
    }
  }
}

template <int WMAX>
struct BmmShape {
  static constexpr int R0 = 32 / WMAX > 0 ? 32 / WMAX : 1;
  static constexpr int U = 32 / WMAX > 8 ? 8 : (32 / WMAX > 0 ? 32 / WMAX : 1);  // words in flight
};

// Main pass: one warp per (block-row, group of R rows), R * WMAX <= 32
// counters per lane.
template <int TS, int WMAX, bool AL>
__global__ void __launch_bounds__(256) k_b2sr_bmm(B2srBmmArgs a) {
  constexpr int R = BmmShape<WMAX>::R0 < TS ? BmmShape<WMAX>::R0 : TS;
  constexpr int NG = (TS + R - 1) / R;
  const int lane = threadIdx.x & 31;
  const long long gw = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long long br = gw / NG;
  if (br >= a.mb) return;
  if (a.hub_min > 0 && __ldg(a.rowptr + br + 1) - __ldg(a.rowptr + br) > a.hub_min) return;
  __shared__ int2 lists[8][32 * 2];
  bmm_block_row<TS, WMAX, R, BmmShape<WMAX>::U, 2, AL>(a, br, (int)(gw % NG), lane, lists[threadIdx.x >> 5]);
}

// One warp, one tile row `row` of a hub block-row.  The entries of 4 groups
// that set the row's bit are compacted into `list`; the feature rows of 32
// listed entries are then loaded in one round with the lanes spread over
// (entry, word) -- 32 / WMAX entries per warp-wide load, so a round needs
// WMAX loads per lane and no more registers -- and each word is broadcast to
// the lanes by a shuffle when its bits are counted.  The chain of dependent
// round trips is (entries / 32) deep instead of (entries / U).
template <int TS, int WMAX, bool AL>
__device__ __forceinline__ void bmm_hub_row(const B2srBmmArgs &a, long long br, int row, int lane, int2 *list) {
  constexpr int G = 4;
  constexpr int TPG = 32 / TS;
  constexpr int TPS = TPG * G;
  constexpr int EPL = 32 / WMAX;  // entries per warp-wide load
  const unsigned lt_mask = (1u << lane) - 1u;
  int cnt[WMAX];
  int deg = 0;
#pragma unroll
  for (int k = 0; k < WMAX; ++k) cnt[k] = 0;
  const int tb = __ldg(a.rowptr + br), te = __ldg(a.rowptr + br + 1);
  const int j = lane % TS, l = lane / TS;
  const int shift = 31 - lane;
  const int my_e = lane / WMAX, my_w = lane % WMAX;  // (entry, word) this lane loads
  for (int s0 = tb; s0 < te; s0 += TPS) {
    int n = 0;
#pragma unroll
    for (int g = 0; g < G; ++g) {
      const int t = s0 + g * TPG + l;
      int col = 0;
      bool set = false;
      if (t < te) {
        col = __ldg(a.colind + t) * TS + j;
        set = (tile_row_any<TS, AL>(a.val, (size_t)t, row) >> (TS - 1 - j)) & 1u;
      }
      const unsigned act = __ballot_sync(0xffffffffu, set);
      if (set) list[n + __popc(act & lt_mask)] = make_int2(col, 0);
      n += __popc(act);
    }
    __syncwarp();
    for (int k0 = 0; k0 < n; k0 += 32) {
      uint32_t w[WMAX];
#pragma unroll
      for (int it = 0; it < WMAX; ++it) {
        const int u = k0 + it * EPL + my_e;
        w[it] = (u < n && my_w < a.W) ? __ldg(a.X + (size_t)(unsigned)list[u].x * (unsigned)a.W + my_w) : 0u;
      }
      const int m = min(32, n - k0);
      deg += m;
#pragma unroll
      for (int it = 0; it < WMAX; ++it)
#pragma unroll
        for (int e = 0; e < EPL; ++e) {
          if (it * EPL + e >= m) break;  // warp-uniform
#pragma unroll
          for (int k = 0; k < WMAX; ++k)
            cnt[k] += (int)((__shfl_sync(0xffffffffu, w[it], e * WMAX + k) >> shift) & 1u);
        }
    }
    __syncwarp();
  }
  const long long orow = br * TS + row;
  if (orow >= a.nrows) return;
  int32_t *dst = a.C + (size_t)orow * a.F;
#pragma unroll
  for (int k = 0; k < WMAX; ++k) {
    const int c = k * 32 + lane;
    if (c < a.F) dst[c] = a.signed_form ? 2 * cnt[k] - deg : cnt[k];
  }
}

// Hub pass: one warp per (hub block-row, tile row), items grid-stride.
template <int TS, int WMAX, bool AL>
__global__ void __launch_bounds__(256) k_b2sr_bmm_hubs(B2srBmmArgs a) {
  const int lane = threadIdx.x & 31;
  const long long gw = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
  const long long items = (long long)__ldg(a.hubs) * TS;
  __shared__ int2 lists[8][32 * 4];
  for (long long it = gw; it < items; it += nw) {
    const long long br = __ldg(a.hubs + 1 + it / TS);
    bmm_hub_row<TS, WMAX, AL>(a, br, (int)(it % TS), lane, lists[threadIdx.x >> 5]);
  }
}

// Segments of cut hubs (k_hub_segments) with the main pass's layout: one
// warp per (segment, group of R rows), counts added into C.
template <int TS, int WMAX, bool AL>
__global__ void __launch_bounds__(256) k_b2sr_bmm_segs(B2srBmmArgs a) {
  constexpr int R = BmmShape<WMAX>::R0 < TS ? BmmShape<WMAX>::R0 : TS;
  constexpr int NG = (TS + R - 1) / R;
  const int lane = threadIdx.x & 31;
  const long long gw = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
  const long long items = (long long)__ldcg(a.hub_info) * NG;
  const long long mean_work = (long long)__ldcg(a.hub_info + 1) * NG / a.seg_warps;
  __shared__ int2 lists[8][32 * 2];
  for (long long it = gw; it < items; it += nw) {
    const int2 sg = a.segs[it / NG];
    const int te = __ldg(a.rowptr + sg.x + 1);
    const int len = hub_segments(te - __ldg(a.rowptr + sg.x), mean_work).y;
    bmm_block_row<TS, WMAX, R, BmmShape<WMAX>::U, 2, AL, true>(a, sg.x, (int)(it % NG), lane,
                                                               lists[threadIdx.x >> 5], sg.y, min(te, sg.y + len));
  }
}

// Tile-wide BMM (gbs_b2sr_bmm at tile 32, plain layout): the walk
// of the tile-wide SpMM with integer counts.  An item is a block-row and a
// slice of 4 feature words (128 features); lane l counts features
// 32 (w0 + k) + l, k < 4, of every row in acc[row * 32 + l] (shared memory).
// Each entry adds its feature bits (or 2 bit - 1 for the +-1 form, whose
// sum is 2 count - entries), so segments of a cut block-row add exactly.
template <int TS>
struct WideBmm {
  const B2srBmmArgs &a;
  int w0, lane;
  int4 *acc;
  __device__ __forceinline__ void flush(const uint16_t *list, int n, int tc_lane) {
    __syncwarp();
    const int nwords = min(4, a.W - w0);
    const int shift = 31 - lane;
    const int sgn = a.signed_form;
    for (int k0 = 0; k0 < n; k0 += WIDE_U) {
      uint32_t x[WIDE_U][4];
      int rr[WIDE_U];
#pragma unroll
      for (int u = 0; u < WIDE_U; ++u) {
        const bool live = k0 + u < n;
        const int e = live ? (int)list[k0 + u] : 0;
        rr[u] = (e >> 5) & 31;
        const int tc = __shfl_sync(0xffffffffu, tc_lane, e >> 10);
        const uint32_t *xp = a.X + ((size_t)(unsigned)tc * TS + (e & 31)) * (size_t)a.W + w0;
#pragma unroll
        for (int k = 0; k < 4; ++k) x[u][k] = (live && k < nwords) ? __ldg(xp + k) : 0u;
      }
#pragma unroll
      for (int u = 0; u < WIDE_U; ++u) {
        if (k0 + u < n) {
          int b[4];
#pragma unroll
          for (int k = 0; k < 4; ++k) {
            b[k] = (int)((x[u][k] >> shift) & 1u);
            if (sgn) b[k] = 2 * b[k] - 1;
          }
          int4 t = acc[rr[u] * 32 + lane];
          t.x += b[0];
          t.y += b[1];
          t.z += b[2];
          t.w += b[3];
          acc[rr[u] * 32 + lane] = t;
        }
      }
    }
    __syncwarp();
  }
};

template <int TS>
__global__ void __launch_bounds__(WIDE_WARPS * 32, 1) k_b2sr_bmm_wide(B2srBmmArgs a) {
  extern __shared__ __align__(16) unsigned char wide_sm[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int4 *acc = reinterpret_cast<int4 *>(wide_sm) + (size_t)warp * TS * 32;
  uint16_t *list = reinterpret_cast<uint16_t *>(wide_sm + (size_t)WIDE_WARPS * TS * 32 * sizeof(int4)) +
                   (size_t)warp * wide_cap<TS>();
  const int slices = (a.W + 3) / 4;
  const long long gw = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
  const long long cut = wide_cut(__ldg(a.rowptr + a.mb), slices, a.seg_warps);
  const long long main_items = (long long)a.mb * slices;
  const long long items = main_items + (long long)__ldcg(a.hub_info) * slices;
  for (long long it = gw; it < items; it += nw) {
    const int sl = (int)(it % slices);
    long long br;
    int tb, te;
    bool atomic;
    if (it < main_items) {
      br = it / slices;
      tb = __ldg(a.rowptr + br);
      te = __ldg(a.rowptr + br + 1);
      if (te - tb > cut) continue;  // done by its segments
      atomic = false;
    } else {
      const int2 sg = a.segs[(it - main_items) / slices];
      br = sg.x;
      const int te_row = __ldg(a.rowptr + sg.x + 1);
      tb = sg.y;
      te = min(te_row, sg.y + wide_segments(te_row - __ldg(a.rowptr + sg.x), cut).y);
      atomic = true;
    }
    WideBmm<TS> body{a, sl * 4, lane, acc};
#pragma unroll
    for (int q = 0; q < TS; ++q) acc[q * 32 + lane] = make_int4(0, 0, 0, 0);
    wide_walk<TS>(a.colind, a.val, tb, te, lane, list, body);
    for (int q = 0; q < TS; ++q) {
      const long long orow = br * TS + q;
      if (orow >= a.nrows) break;
      const int4 v = acc[q * 32 + lane];
      const int vk[4] = {v.x, v.y, v.z, v.w};
      int32_t *dst = a.C + (size_t)orow * a.F;
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const int f = (sl * 4 + k) * 32 + lane;
        if (f < a.F) {
          if (atomic) atomicAdd(dst + f, vk[k]);
          else dst[f] = vk[k];
        }
      }
    }
  }
}

template <int TS>
gbs_status launch_bmm_wide(B2srBmmArgs &a, cudaStream_t s) {
  const void *fn = (const void *)&k_b2sr_bmm_wide<TS>;
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
      a.rowptr, a.mb, a.nrows, a.F, (a.W + 3) / 4, a.seg_warps, reinterpret_cast<uint32_t *>(a.C), info.as<int>(),
      segs.as<int2>());
  GBS_TRY(check_launch("k_wide_segments"));
  a.hub_info = info.as<int>();
  a.segs = segs.as<int2>();
  void *args[] = {&a};
  GBS_CUDA_TRY(cudaLaunchKernel(fn, grid, dim3(WIDE_WARPS * 32), args, smem, s));
  return GBS_OK;
}

template <int TS, bool AL = false>
gbs_status launch_bmm(B2srBmmArgs &a, cudaStream_t s) {
  const void *fn = nullptr, *hub_fn = nullptr, *seg_fn = nullptr;
  int wmax = 0;
#define GBS_BMM_CASE(WM)                                     \
  {                                                          \
    fn = (const void *)&k_b2sr_bmm<TS, WM, AL>;              \
    hub_fn = (const void *)&k_b2sr_bmm_hubs<TS, WM, AL>;     \
    seg_fn = (const void *)&k_b2sr_bmm_segs<TS, WM, AL>;     \
    wmax = WM;                                               \
  }
  if (a.W <= 1) GBS_BMM_CASE(1)
  else if (a.W <= 2) GBS_BMM_CASE(2)
  else if (a.W <= 4) GBS_BMM_CASE(4)
  else if (a.W <= 8) GBS_BMM_CASE(8)
  else if (a.W <= 16) GBS_BMM_CASE(16)
  else if (a.W <= 32) GBS_BMM_CASE(32)
  else return fail(GBS_ERR_UNSUPPORTED, "b2sr bmm: F must be <= 1024");
#undef GBS_BMM_CASE
  const int R0 = 32 / wmax > 0 ? 32 / wmax : 1;
  const int R = R0 < TS ? R0 : TS;
  const int NG = (TS + R - 1) / R;
  const long long warps = (long long)a.mb * NG;
  const int blocks = (int)((warps * 32 + 255) / 256);
  if (blocks == 0) return GBS_OK;
  a.hub_min = 0;
  a.hubs = nullptr;
  a.hub_info = nullptr;
  a.segs = nullptr;
  a.seg_warps = 1;
  // plain-layout tile 32: the tile-wide pass (flickr-shaped graph, F = 256
  // / 1024: 0.77 / 3.02 against 1.54 / 4.02 ms; at tile 16 it lost, 0.77 /
  // 3.01 against 0.46 / 1.89 ms: each tile is walked once per 4-word slice,
  // the row kernels above walk it once per row for all words)
  if constexpr (!AL && TS == 32) return launch_bmm_wide<TS>(a, s);
  if (a.mb < kHubMinBlockRows) {
    void *args[] = {&a};
    GBS_CUDA_TRY(cudaLaunchKernel(fn, dim3(blocks), dim3(256), args, 0, s));
    return GBS_OK;
  }
  // main pass on s, whole hubs and segments of cut hubs on the side streams
  // (as in b2sr_spmm_run; integer counts, so the split is exact)
  DevBuf buf, segs, whole;
  GBS_TRY(buf.alloc(sizeof(int) * ((size_t)a.mb + 3), s));
  GBS_CUDA_TRY(cudaMemsetAsync(buf.p, 0, 3 * sizeof(int), s));
  int *info = buf.as<int>(), *hubs = info + 2;
  k_find_hubs<<<(a.mb + 255) / 256, 256, 0, s>>>(a.rowptr, a.mb, kHubTiles, hubs, info + 1);
  GBS_TRY(check_launch("k_find_hubs"));
  a.hub_min = kHubTiles;
  a.hubs = hubs;
  DeviceInfo di;
  GBS_TRY(device_info(&di));
  int per_sm = 0;
  GBS_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, seg_fn, 256, 0));
  const dim3 seg_grid(di.sm_count * (per_sm > 0 ? per_sm : 1));
  GBS_TRY(segs.alloc(sizeof(int2) * (size_t)a.mb * kSegMax, s));
  GBS_TRY(whole.alloc(sizeof(int) * ((size_t)a.mb + 1), s));
  GBS_CUDA_TRY(cudaMemsetAsync(whole.p, 0, sizeof(int), s));
  a.hub_info = info;
  a.segs = segs.as<int2>();
  a.seg_warps = (long long)seg_grid.x * 8;
  k_hub_segments<<<(a.mb + 7) / 8, 256, 0, s>>>(hubs, a.rowptr, info, segs.as<int2>(), whole.as<int>(), NG,
                                                a.seg_warps, TS, a.nrows, a.F, reinterpret_cast<uint32_t *>(a.C));
  GBS_TRY(check_launch("k_hub_segments"));
  B2srBmmArgs aw = a;
  aw.hubs = whole.as<int>();
  cudaStream_t side = nullptr, side1 = nullptr;
  GBS_TRY(side_stream(&side, 0));
  GBS_TRY(side_stream(&side1, 1));
  Events ev;
  GBS_TRY(ev.create(3));
  GBS_CUDA_TRY(cudaEventRecord(ev.e[0], s));
  GBS_CUDA_TRY(cudaStreamWaitEvent(side, ev.e[0], 0));
  GBS_CUDA_TRY(cudaStreamWaitEvent(side1, ev.e[0], 0));
  void *args[] = {&a};
  void *wargs[] = {&aw};
  gbs_status st = GBS_OK;
  cudaError_t e = cudaLaunchKernel(seg_fn, seg_grid, dim3(256), args, 0, side1);
  if (e != cudaSuccess) st = cuda_fail(e, "k_b2sr_bmm_segs");
  GBS_CUDA_TRY(cudaEventRecord(ev.e[2], side1));
  e = cudaLaunchKernel(hub_fn, dim3(di.sm_count * 4), dim3(256), wargs, 0, side);
  if (e != cudaSuccess && st == GBS_OK) st = cuda_fail(e, "k_b2sr_bmm_hubs");
  GBS_CUDA_TRY(cudaEventRecord(ev.e[1], side));
  e = cudaLaunchKernel(fn, dim3(blocks), dim3(256), args, 0, s);
  if (e != cudaSuccess && st == GBS_OK) st = cuda_fail(e, "k_b2sr_bmm");
  GBS_CUDA_TRY(cudaStreamWaitEvent(s, ev.e[1], 0));
  GBS_CUDA_TRY(cudaStreamWaitEvent(s, ev.e[2], 0));
  return st;
}

}  // namespace gbs

// ===========================================================================
// C ABI
// ===========================================================================
using namespace gbs;

extern "C" gbs_status gbs_b2sr_bmm(int tile, int nrows, int nblockrows, const int *rowptr, const int *colind,
                                   const void *val, const uint32_t *X, int F, int signed_form, int32_t *C,
                                   gbs_stream_t stream) {
  clear_error();
  GBS_REQUIRE(valid_tile(tile), "b2sr bmm: tile must be 4, 8, 16 or 32");
  GBS_REQUIRE(nrows >= 0 && F >= 1 && F <= 1024, "b2sr bmm: need 1 <= F <= 1024");
  GBS_REQUIRE(nblockrows == (nrows + tile - 1) / tile, "b2sr bmm: nblockrows must be ceil(nrows / tile)");
  if (nrows == 0) return GBS_OK;
  GBS_REQUIRE(rowptr && C && X, "b2sr bmm: null pointer");
  B2srBmmArgs a;
  a.nrows = nrows;
  a.mb = nblockrows;
  a.F = F;
  a.W = (F + 31) / 32;
  a.rowptr = rowptr;
  a.colind = colind;
  a.val = val;
  a.X = X;
  a.C = C;
  a.signed_form = signed_form ? 1 : 0;
  cudaStream_t s = (cudaStream_t)stream;
  switch (tile) {
    case 4: return launch_bmm<4>(a, s);
    case 8: return launch_bmm<8>(a, s);
    case 16: return launch_bmm<16>(a, s);
    default: return launch_bmm<32>(a, s);
  }
}

extern "C" gbs_status gbs_b2sr_bmm_aligned(int tile, int nrows, int nblockrows, const int *new_rowptr,
                                           const int *new_colind, const uint32_t *new_val, const uint32_t *X,
                                           int F, int signed_form, int32_t *C, gbs_stream_t stream) {
  clear_error();
  GBS_REQUIRE(tile == 8 || tile == 16, "b2sr bmm aligned: tile must be 8 or 16");
  GBS_REQUIRE(nrows >= 0 && F >= 1 && F <= 1024, "b2sr bmm aligned: need 1 <= F <= 1024");
  GBS_REQUIRE(nblockrows == (nrows + tile - 1) / tile, "b2sr bmm aligned: nblockrows must be ceil(nrows / tile)");
  if (nrows == 0) return GBS_OK;
  GBS_REQUIRE(new_rowptr && C && X, "b2sr bmm aligned: null pointer");
  B2srBmmArgs a;
  a.nrows = nrows;
  a.mb = nblockrows;
  a.F = F;
  a.W = (F + 31) / 32;
  a.rowptr = new_rowptr;
  a.colind = new_colind;
  a.val = new_val;
  a.X = X;
  a.C = C;
  a.signed_form = signed_form ? 1 : 0;
  cudaStream_t s = (cudaStream_t)stream;
  return tile == 8 ? launch_bmm<8, true>(a, s) : launch_bmm<16, true>(a, s);
}

