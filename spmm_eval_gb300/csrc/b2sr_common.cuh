// Shared parts of the B2SR kernels (b2sr.cu: packing, aligned formats and
// sign packers; b2sr_spmm.cu: B2SR x dense SpMM; b2sr_bmm.cu: B2SR x bits
// BMM): the tile layout, the hub constants and the order-free hub cut, the
// tile-wide walk, and per-call fork/join events.
//
// Layout (the reference's, csr2bsr_batch_bsrbmv.cu + spmm.cu ToBit*Col):
// block-row i covers CSR rows [i*ts, (i+1)*ts); it has one tile per distinct
// floor(col / ts) of those rows, in ascending order; tile b stores its ts rows
// as ts-bit words, element ts*b + r = row r, column 0 in the most significant
// of the ts bits (uint8 for ts 4 (low nibble) and 8, uint16 for 16, uint32
// for 32).  Any stored CSR entry sets its bit (values are ignored, as the
// reference forces them to 1.0 before packing, csr2bsr_batch_bsrbmv.cu:296).
#pragma once

#include <climits>
#include <vector>

#include "common.cuh"
#include "feat.cuh"
#include "util.cuh"

namespace gbs {

// Block-rows (strips) of more tiles (entries) than kHubTiles (kHubStripNnz)
// go to the hub passes of the SpMM / BMM (packer): the mean of a power-law
// graph's tile-4 block-rows is ~40 tiles, its largest hubs have thousands.
// Matrices of fewer than kHubMinBlockRows block-rows run in one pass.
constexpr int kHubTiles = 256;
constexpr int kHubStripNnz = 256;
constexpr int kHubMinBlockRows = 1024;

template <int TS> struct TileT;
template <> struct TileT<4> { using T = uint8_t; };
template <> struct TileT<8> { using T = uint8_t; };
template <> struct TileT<16> { using T = uint16_t; };
template <> struct TileT<32> { using T = uint32_t; };

template <int TS>
__device__ __forceinline__ uint32_t tile_row(const void *val, size_t t, int r) {
  using VT = typename TileT<TS>::T;
  return (uint32_t)__ldg(reinterpret_cast<const VT *>(val) + t * TS + r);
}

// Row r of tile t in the aligned B2SR-8/16 layout (packUchar2AlignedUnsigned /
// packUshort2AlignedUnsigned): tiles in groups of g = 32 / TS per uint32 word,
// word (t / g) * TS + r holds row r of the group's tiles, the first tile in
// the most significant byte / half.  t indexes the padded tile list.
template <int TS, bool AL>
__device__ __forceinline__ uint32_t tile_row_any(const void *val, size_t t, int r) {
  if constexpr (AL) {
    static_assert(TS == 8 || TS == 16, "aligned B2SR exists for tiles 8 and 16");
    constexpr int g = 32 / TS;
    const uint32_t w = __ldg(reinterpret_cast<const uint32_t *>(val) + (t / g) * TS + r);
    return (w >> (TS * (g - 1 - (int)(t % g)))) & ((1u << TS) - 1u);
  } else {
    return tile_row<TS>(val, t, r);
  }
}

// Order-free hub split (gbs_b2sr_spmm).  The ordered hub pass above gives
// one warp all of a hub's tiles for its (row, slice), so the largest hubs are
// chains far longer than the mean work of a warp and the SMs idle behind
// them.  A hub whose walk is longer than 1/kSegShare of the mean work per
// resident warp (and than kSegMinTiles tiles) is cut into equal segments of
// consecutive tiles (at most kSegMax); a segment is then an ordinary short
// block-row: one warp per (segment, group of tile rows) walks it with the
// main pass's layout (all features, 4 gathers per round, every tile read
// once per group) and adds its partial sums into C, which the segment
// builder zeroed.  The other hubs go to the ordered pass whole.  Sums of a
// split hub are formed in an order that depends on scheduling: exact for 0/1
// and +-1 features (integer partial sums), within FP32 rounding otherwise.
constexpr int kSegMax = 64;
constexpr int kSegMinTiles = 128;
constexpr int kSegShare = 2;

// (segments, tiles per segment) of a hub of T tiles; mean_work = tiles of
// all hubs * items per hub / resident warps.
__device__ __forceinline__ int2 hub_segments(int T, long long mean_work) {
  const long long cut = max((long long)kSegMinTiles, mean_work / kSegShare);
  if (T <= cut) return make_int2(1, T);
  const int n = (int)min((long long)kSegMax, ((long long)T + cut - 1) / cut);
  return make_int2(n, (T + n - 1) / n);
}

namespace {
// One warp per hub: a hub that is cut appends its segments (block-row, first
// tile) to segs and zeroes its rows of C (32-bit elements, F per row), any
// other is appended to whole = [count, block-row ids ...].  info =
// [segments, tiles of all hubs]; per = items per hub.
__global__ void k_hub_segments(const int *__restrict__ hubs, const int *__restrict__ rowptr, int *__restrict__ info,
                               int2 *__restrict__ segs, int *__restrict__ whole, long long per, long long warps,
                               int ts, int nrows, int F, uint32_t *__restrict__ C) {
  const int h = (int)(((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
  if (h >= __ldg(hubs)) return;
  const int br = __ldg(hubs + 1 + h);
  const int tb = __ldg(rowptr + br), te = __ldg(rowptr + br + 1);
  const int2 sg = hub_segments(te - tb, (long long)__ldcg(info + 1) * per / warps);
  if (sg.x == 1) {
    if (lane == 0) whole[1 + atomicAdd(whole, 1)] = br;
    return;
  }
  int base = 0;
  if (lane == 0) base = atomicAdd(info, sg.x);
  base = __shfl_sync(0xffffffffu, base, 0);
  for (int i = lane; i < sg.x; i += 32) segs[base + i] = make_int2(br, tb + i * sg.y);
  const long long r0 = (long long)br * ts;
  const int rows = (int)min((long long)ts, (long long)nrows - r0);
  for (int q = 0; q < rows; ++q) {
    uint32_t *row = C + (r0 + q) * F;
    for (int c = lane; c < F; c += 32) row[c] = 0u;
  }
}

}  // namespace

// ---------------------------------------------------------------------------
// Tile-wide B2SR SpMM (gbs_b2sr_spmm, tiles 16 / 32).  The kernels above
// give a warp R rows of a block-row, so at large tiles every tile is walked
// TS / R times (and TS times in the hub pass): at tile 32 the walk of the
// tile indices and row words, not the gathers, is the work.  Here one warp
// owns all TS rows of a block-row and a slice of 128 features (4 per lane),
// with the row sums in shared memory, and reads each tile once: per step
// the indices of 32 tiles (one per lane) and their row words (TS per lane,
// all issued together), whose set bits are appended to a per-warp
// list of (tile, row, column) entries; the list is then gathered U at a
// time, every gathered 4-feature chunk added to its row's sums.  Entries of
// a row come in column order, as in the kernels above, so a row's sums are
// the same sequence of FP32 additions.  Block-rows longer than half the mean
// work per resident warp are cut into segments (k_wide_segments) whose sums
// are added into C with atomics, as the hub split above.
constexpr int WIDE_WARPS = 4;    // warps per CTA
constexpr int WIDE_FEATS = 128;  // features per item: 4 per lane
constexpr int WIDE_U = 8;        // gathers in flight per lane
constexpr int kWideCutMin = 256; // tiles: shorter block-rows are never cut

template <int TS>
constexpr int wide_cap() { return 32 * TS; }  // list entries (a step with more bits goes tile by tile)
template <int TS>
constexpr size_t wide_smem() {
  return (size_t)WIDE_WARPS * (TS * 32 * sizeof(float4) + wide_cap<TS>() * sizeof(uint16_t));
}

// Block-rows of more tiles than this are cut: half the mean work per
// resident warp, in tiles (nnzb tiles x slices items / warps).
__device__ __forceinline__ long long wide_cut(long long nnzb, int slices, long long warps) {
  return max((long long)kWideCutMin, nnzb * slices / (2 * warps));
}
// (segments, tiles per segment) of a cut block-row of T tiles.
__device__ __forceinline__ int2 wide_segments(int T, long long cut) {
  const int n = (int)min((long long)kSegMax, ((long long)T + cut - 1) / cut);
  return make_int2(n, (T + n - 1) / n);
}

// 4 features of a B row as FP32 (16-byte FP32 or 8-byte 16-bit load).
template <int DT>
__device__ __forceinline__ float4 wide_load(const void *B, size_t elem) {
  if constexpr (DT == DT_F32) {
    return ld_nc_f4(reinterpret_cast<const float *>(B) + elem);
  } else {
    const uint2 w = __ldg(reinterpret_cast<const uint2 *>(reinterpret_cast<const uint16_t *>(B) + elem));
    if constexpr (DT == DT_BF16) {
      return make_float4(bf16lo(w.x), bf16hi(w.x), bf16lo(w.y), bf16hi(w.y));
    } else {
      const float2 p = h2f2(w.x), q = h2f2(w.y);
      return make_float4(p.x, p.y, q.x, q.y);
    }
  }
}

// One warp per block-row: a block-row longer than the cut appends its
// segments (block-row, first tile) to segs, counted in *nsegs, and zeroes its
// rows of C (32-bit elements, F per row).
template <int TS>
__global__ void k_wide_segments(const int *__restrict__ rowptr, int mb, int nrows, int F, int slices,
                                long long warps, uint32_t *__restrict__ C, int *__restrict__ nsegs,
                                int2 *__restrict__ segs) {
  const long long br = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (br >= mb) return;
  const int tb = __ldg(rowptr + br), te = __ldg(rowptr + br + 1);
  const long long cut = wide_cut(__ldg(rowptr + mb), slices, warps);
  if (te - tb <= cut) return;
  const int2 sg = wide_segments(te - tb, cut);
  int base = 0;
  if (lane == 0) base = atomicAdd(nsegs, sg.x);
  base = __shfl_sync(0xffffffffu, base, 0);
  for (int i = lane; i < sg.x; i += 32) segs[base + i] = make_int2((int)br, tb + i * sg.y);
  const long long r0 = br * TS;
  const int rows = (int)min((long long)TS, (long long)nrows - r0);
  for (int q = 0; q < rows; ++q) {
    uint32_t *row = C + (r0 + q) * F;
    for (int c = lane; c < F; c += 32) row[c] = 0u;
  }
}

// A step whose bits overflow the list (more than 32 * TS of them), out of
// line: its tiles one at a time (lane = tile row), flushing whenever the
// next tile might not fit.  Rows still come in tile and column order.
template <int TS, class P>
__device__ __noinline__ void wide_step_dense(const void *val, int s0, int nt, int tc_lane, int lane,
                                             uint16_t *list, P &body) {
  constexpr int CAP = wide_cap<TS>();
  int n = 0;
  for (int i = 0; i < nt; ++i) {
    uint32_t w = lane < TS ? tile_row<TS>(val, (size_t)(s0 + i), lane) : 0u;
    const int cnt = __popc(w);
    const int tot = __reduce_add_sync(0xffffffffu, cnt);
    if (n + tot > CAP) {  // one tile (TS * TS bits) always fits in an empty list
      body.flush(list, n, tc_lane);
      n = 0;
    }
    int incl = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += y;
    }
    int pos = n + incl - cnt;
    while (w) {
      const int b = 31 - __clz(w);
      list[pos++] = (uint16_t)((i << 10) | (lane << 5) | (TS - 1 - b));
      w &= ~(1u << b);
    }
    n += tot;
  }
  body.flush(list, n, tc_lane);
}

// One warp walks tiles [tb, te) of a block-row and hands the set bits to
// body.flush as (tile, row, column) entries (entry = tile << 10 | row << 5 |
// column; the tile's block column is lane `tile`'s tc_lane).  Per step of
// 32 tiles, lane (k, r) = (lane / TS, lane % TS) loads row r of tiles
// k * TS + [0, TS) (all TS loads in flight together) and writes its set bits
// (tiles ascending, columns ascending) at its place in the list (one prefix
// sum per step), so every row's entries are in tile and column order.
template <int TS, class P>
__device__ __forceinline__ void wide_walk(const int *colind, const void *val, int tb, int te, int lane,
                                          uint16_t *list, P &body) {
  constexpr int CAP = wide_cap<TS>();
  const int k0 = (lane / TS) * TS, r = lane % TS;
  for (int s0 = tb; s0 < te; s0 += 32) {
    const int nt = min(32, te - s0);
    const int my_tc = lane < nt ? __ldg(colind + s0 + lane) : 0;
    uint32_t wv[TS];
    int cnt = 0;
#pragma unroll
    for (int g = 0; g < TS; ++g) {
      wv[g] = k0 + g < nt ? tile_row<TS>(val, (size_t)(s0 + k0 + g), r) : 0u;
      cnt += __popc(wv[g]);
    }
    const int tot = __reduce_add_sync(0xffffffffu, cnt);
    if (tot > CAP) {
      wide_step_dense<TS>(val, s0, nt, my_tc, lane, list, body);
      continue;
    }
    int incl = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += y;
    }
    int pos = incl - cnt;
#pragma unroll
    for (int g = 0; g < TS; ++g) {
      uint32_t w = wv[g];
      while (w) {  // column 0 is the most significant of the TS bits: ascending columns
        const int b = 31 - __clz(w);
        list[pos++] = (uint16_t)(((k0 + g) << 10) | (r << 5) | (TS - 1 - b));
        w &= ~(1u << b);
      }
    }
    body.flush(list, tot, my_tc);
  }
}

namespace {
// hubs[0] = number of block-rows with more than hub_min tiles, hubs[1..] =
// their ids (any order); *tiles (if given) += their tiles.
__global__ void k_find_hubs(const int *__restrict__ rowptr, int mb, int hub_min, int *__restrict__ hubs,
                            int *__restrict__ tiles = nullptr) {
  const int br = blockIdx.x * blockDim.x + threadIdx.x;
  if (br >= mb) return;
  const int t = rowptr[br + 1] - rowptr[br];
  if (t > hub_min) {
    hubs[1 + atomicAdd(hubs, 1)] = br;
    if (tiles) atomicAdd(tiles, t);
  }
}
}  // namespace

namespace {
// Per-call events (created and destroyed around one fork/join).
struct Events {
  static constexpr int kMax = 3;
  cudaEvent_t e[kMax] = {};
  int n = 0;
  gbs_status create(int k) {
    if (k > kMax) return fail(GBS_ERR_INVALID_ARG, "too many events");
    for (n = 0; n < k; ++n) GBS_CUDA_TRY(cudaEventCreateWithFlags(&e[n], cudaEventDisableTiming));
    return GBS_OK;
  }
  ~Events() {
    for (int i = 0; i < n; ++i) cudaEventDestroy(e[i]);
  }
};
}  // namespace

}  // namespace gbs

static inline bool valid_tile(int t) { return t == 4 || t == 8 || t == 16 || t == 32; }
