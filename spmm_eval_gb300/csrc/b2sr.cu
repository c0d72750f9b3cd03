// B2SR ("binarised BSR") on sm_103a: CSR -> B2SR packing for tiles 4/8/16/32,
// the "aligned" B2SR-8/16 variants, B2SR x dense SpMM, B2SR x packed-bit BMM
// and the dense sign packers.
//
// Layout (the reference's, csr2bsr_batch_bsrbmv.cu + spmm.cu ToBit*Col):
// block-row i covers CSR rows [i*ts, (i+1)*ts); it has one tile per distinct
// floor(col / ts) of those rows, in ascending order; tile b stores its ts rows
// as ts-bit words, element ts*b + r = row r, column 0 in the most significant
// of the ts bits (uint8 for ts 4 (low nibble) and 8, uint16 for 16, uint32
// for 32).  Any stored CSR entry sets its bit (values are ignored, as the
// reference forces them to 1.0 before packing, csr2bsr_batch_bsrbmv.cu:296).
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

// ---------------------------------------------------------------------------
// Packing.  A group of ts lanes owns one block-row (lane r walks CSR row
// i*ts + r).  Each step takes the smallest tile column m at the heads of the
// ts rows (__reduce_min_sync over the group), every lane consumes its
// entries in that tile column and ORs their bits into its tile row; the tiles
// therefore come out in ascending order with no sort and no atomics.
// ---------------------------------------------------------------------------
template <int TS, bool FILL>
__global__ void __launch_bounds__(256)
    k_b2sr_pack(int nrows, int ncols, int mb, const int *__restrict__ rowptr,
                const int *__restrict__ colind, int *__restrict__ counts, const int *__restrict__ brp,
                int *__restrict__ bcol, typename TileT<TS>::T *__restrict__ bval, int *__restrict__ err,
                int hub_min) {
  using VT = typename TileT<TS>::T;
  constexpr int G = 32 / TS;
  const int lane = threadIdx.x & 31;
  const int g = lane / TS, r = lane % TS;
  const long long gw = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long long strip = gw * G + g;
  if (strip >= mb) return;  // the whole group leaves together
  if (hub_min > 0) {  // strips of more entries belong to the hub pass
    const long long r0 = strip * TS;
    const long long r1 = r0 + TS < nrows ? r0 + TS : nrows;
    if (__ldg(rowptr + r1) - __ldg(rowptr + r0) > hub_min) return;
  }
  const unsigned gmask = (TS == 32) ? 0xffffffffu : (((1u << TS) - 1u) << (g * TS));
  const long long row = strip * TS + r;
  int p = 0, e = 0;
  if (row < nrows) {
    p = __ldg(rowptr + row);
    e = __ldg(rowptr + row + 1);
  }
  const int rs = p;
  const int out = FILL ? __ldg(brp + strip) : 0;
  int cnt = 0, prev_m = -1;
  while (true) {
    int head = INT_MAX;
    if (p < e) {
      const int c = __ldg(colind + p);
      if (!FILL && (c < 0 || c >= ncols || (p > rs && __ldg(colind + p - 1) > c))) {
        atomicOr(err, 1);
        p = e;
      } else {
        head = c / TS;
      }
    }
    const int m = __reduce_min_sync(gmask, head);
    if (m == INT_MAX) break;
    if (!FILL && m < prev_m) atomicOr(err, 1);  // unreachable for sorted, in-range input
    prev_m = m;
    uint32_t bits = 0;
    while (p < e) {
      const int c = __ldg(colind + p);
      if (c / TS != m) break;
      if (!FILL && (c >= ncols || (p > rs && __ldg(colind + p - 1) > c))) {
        atomicOr(err, 1);
        p = e;
        break;
      }
      bits |= 1u << (TS - 1 - (c % TS));
      ++p;
    }
    if (FILL) {
      if (r == 0) bcol[out + cnt] = m;
      bval[(size_t)(out + cnt) * TS + r] = (VT)bits;
    }
    ++cnt;
  }
  if (!FILL && r == 0) counts[strip] = cnt;
}

// Hub strips: strips with thousands of entries walk their tile columns one
// at a time above, a chain of dependent loads per tile column.  Here one CTA
// takes such a strip: every thread marks the tile columns of its entries in
// a shared-memory bitmap (atomicOr), the count is the bitmap's population;
// the fill pass turns the bitmap into tile positions (prefix popcounts per
// word), writes the tile columns in ascending order and ORs every entry's
// bit into its tile row with 32-bit global atomics (the strip's tile rows are
// zeroed first).  Same output as the lane-group walk.  hubs = [count, strip
// ids ...]; strips taken grid-stride.
__global__ void k_find_hub_strips(const int *__restrict__ rowptr, int nrows, int mb, int ts, int min_nnz,
                                  int *__restrict__ hubs) {
  const long long strip = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (strip >= mb) return;
  const long long r0 = strip * ts;
  const long long r1 = r0 + ts < nrows ? r0 + ts : nrows;
  if (rowptr[r1] - rowptr[r0] > min_nnz) hubs[1 + atomicAdd(hubs, 1)] = (int)strip;
}

// Block-wide exclusive sum of one int per thread (256 threads); returns the
// total through *total.
__device__ __forceinline__ int block_exclusive_sum(int x, int *scratch, int *total) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int inc = x;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += y;
  }
  if (lane == 31) scratch[w] = inc;
  __syncthreads();
  if (w == 0) {
    int v = lane < 8 ? scratch[lane] : 0;
#pragma unroll
    for (int o = 1; o < 8; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, v, o);
      if (lane >= o) v += y;
    }
    if (lane < 8) scratch[8 + lane] = v;  // inclusive warp totals
  }
  __syncthreads();
  const int before = (w > 0 ? scratch[8 + w - 1] : 0) + inc - x;
  *total = scratch[15];
  __syncthreads();
  return before;
}

template <int TS, bool FILL>
__global__ void __launch_bounds__(256)
    k_b2sr_pack_hubs(int nrows, int ncols, const int *__restrict__ rowptr, const int *__restrict__ colind,
                     int *__restrict__ counts, const int *__restrict__ brp, int *__restrict__ bcol,
                     uint32_t *__restrict__ bval32, int *__restrict__ err, const int *__restrict__ hubs, int words) {
  using VT = typename TileT<TS>::T;
  extern __shared__ uint32_t sm[];
  uint32_t *bm = sm;                                          // tile-column bitmap
  int *pre = reinterpret_cast<int *>(sm + words);             // fill: tiles before each word
  int *srp = pre + (FILL ? words : 0);                        // the strip's row pointers
  int *scratch = srp + TS + 1;                                // 16 ints
  const int tid = threadIdx.x;
  const int nh = hubs[0];
  for (int h = blockIdx.x; h < nh; h += gridDim.x) {
    const int strip = hubs[1 + h];
    const int r0 = strip * TS;
    const int nr = nrows - r0 < TS ? nrows - r0 : TS;
    if (tid <= nr) srp[tid] = rowptr[r0 + tid];
    for (int w = tid; w < words; w += 256) bm[w] = 0u;
    __syncthreads();
    const int eb = srp[0], ee = srp[nr];
    for (int e = eb + tid; e < ee; e += 256) {
      const int c = colind[e];
      if (FILL && (c < 0 || c >= ncols)) continue;  // a CSR the count pass would have rejected
      if (!FILL) {
        int lo = 0, hi = nr - 1;  // row of e: last r with srp[r] <= e
        while (lo < hi) {
          const int mid = (lo + hi + 1) >> 1;
          if (srp[mid] <= e) lo = mid;
          else hi = mid - 1;
        }
        if (c < 0 || c >= ncols || (e > srp[lo] && colind[e - 1] > c)) {
          atomicOr(err, 1);
          continue;
        }
      }
      const int key = c / TS;
      atomicOr(bm + (key >> 5), 1u << (key & 31));
    }
    __syncthreads();
    if (!FILL) {
      int cnt = 0;
      for (int w = tid; w < words; w += 256) cnt += __popc(bm[w]);
      int total = 0;
      block_exclusive_sum(cnt, scratch, &total);
      if (tid == 0) counts[strip] = total;
    } else {
      const int per = (words + 255) / 256;
      const int w0 = tid * per < words ? tid * per : words;
      const int w1 = w0 + per < words ? w0 + per : words;
      int local = 0;
      for (int w = w0; w < w1; ++w) local += __popc(bm[w]);
      int total = 0;
      int run = block_exclusive_sum(local, scratch, &total);
      for (int w = w0; w < w1; ++w) {
        pre[w] = run;
        run += __popc(bm[w]);
      }
      const int out = brp[strip], end = brp[strip + 1];
      // zero the strip's tile rows, then OR the entries' bits in
      const long long wb = (long long)out * TS * (long long)sizeof(VT) / 4;
      const long long nwords = (long long)(brp[strip + 1] - out) * TS * (long long)sizeof(VT) / 4;
      for (long long i = tid; i < nwords; i += 256) bval32[wb + i] = 0u;
      __syncthreads();
      for (int w = tid; w < words; w += 256) {
        uint32_t m = bm[w];
        int t = out + pre[w];
        while (m && t < end) {
          const int b = __ffs(m) - 1;
          m &= m - 1u;
          bcol[t++] = w * 32 + b;
        }
      }
      for (int e = eb + tid; e < ee; e += 256) {
        int lo = 0, hi = nr - 1;
        while (lo < hi) {
          const int mid = (lo + hi + 1) >> 1;
          if (srp[mid] <= e) lo = mid;
          else hi = mid - 1;
        }
        const int c = colind[e];
        if (c < 0 || c >= ncols) continue;
        const int key = c / TS, w = key >> 5, b = key & 31;
        const int t = out + pre[w] + __popc(bm[w] & ((1u << b) - 1u));
        if (t >= end) continue;  // tile counts from another matrix
        const uint32_t bit = 1u << (TS - 1 - (c % TS));
        const long long byte = ((long long)t * TS + lo) * (long long)sizeof(VT);
        atomicOr(bval32 + byte / 4, bit << (8 * (int)(byte % 4)));
      }
    }
    __syncthreads();  // the next strip reuses the shared arrays
  }
}

// The packer's hub pass is used while its bitmap and prefix arrays fit in
// kHubPackSmem bytes of shared memory.
constexpr int kHubPackSmem = 96 * 1024;

template <int TS>
gbs_status launch_pack(bool fill, int nrows, int ncols, int mb, const int *rowptr, const int *colind,
                       int *counts, const int *brp, int *bcol, void *bval, int *err, cudaStream_t s) {
  constexpr int G = 32 / TS;
  const long long warps = ((long long)mb + G - 1) / G;
  const int blocks = (int)((warps * 32 + 255) / 256);
  using VT = typename TileT<TS>::T;
  if (blocks == 0) return GBS_OK;
  // hub pass: needs the bitmap in shared memory and 4-byte aligned tile rows
  const long long words = (((long long)ncols + TS - 1) / TS + 31) / 32;
  const size_t smem = sizeof(uint32_t) * (size_t)words * (fill ? 2 : 1) + sizeof(int) * (TS + 1 + 16);
  const bool hub = mb >= kHubMinBlockRows && smem <= (size_t)kHubPackSmem &&
                   (!fill || (reinterpret_cast<uintptr_t>(bval) & 3u) == 0);
  DevBuf hubs;
  if (hub) {
    GBS_TRY(hubs.alloc(sizeof(int) * ((size_t)mb + 1), s));
    GBS_CUDA_TRY(cudaMemsetAsync(hubs.p, 0, sizeof(int), s));
    k_find_hub_strips<<<(mb + 255) / 256, 256, 0, s>>>(rowptr, nrows, mb, TS, kHubStripNnz, hubs.as<int>());
    GBS_TRY(check_launch("k_find_hub_strips"));
  }
  const int hub_min = hub ? kHubStripNnz : 0;
  if (fill)
    k_b2sr_pack<TS, true><<<blocks, 256, 0, s>>>(nrows, ncols, mb, rowptr, colind, counts, brp, bcol,
                                                 reinterpret_cast<VT *>(bval), err, hub_min);
  else
    k_b2sr_pack<TS, false><<<blocks, 256, 0, s>>>(nrows, ncols, mb, rowptr, colind, counts, brp, bcol,
                                                  reinterpret_cast<VT *>(bval), err, hub_min);
  GBS_TRY(check_launch("k_b2sr_pack"));
  if (!hub) return GBS_OK;
  DeviceInfo di;
  GBS_TRY(device_info(&di));
  const void *fn = fill ? (const void *)&k_b2sr_pack_hubs<TS, true> : (const void *)&k_b2sr_pack_hubs<TS, false>;
  if (smem > 48 * 1024) GBS_CUDA_TRY(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int iwords = (int)words;
  uint32_t *bval32 = reinterpret_cast<uint32_t *>(bval);
  const int *hp = hubs.as<int>();
  void *args[] = {&nrows, &ncols, &rowptr, &colind, &counts, &brp, &bcol, &bval32, &err, &hp, &iwords};
  GBS_CUDA_TRY(cudaLaunchKernel(fn, dim3(di.sm_count * 2), dim3(256), args, smem, s));
  return GBS_OK;
}

gbs_status pack_dispatch(int ts, bool fill, int nrows, int ncols, int mb, const int *rowptr,
                         const int *colind, int *counts, const int *brp, int *bcol, void *bval,
                         int *err, cudaStream_t s) {
  switch (ts) {
    case 4: return launch_pack<4>(fill, nrows, ncols, mb, rowptr, colind, counts, brp, bcol, bval, err, s);
    case 8: return launch_pack<8>(fill, nrows, ncols, mb, rowptr, colind, counts, brp, bcol, bval, err, s);
    case 16: return launch_pack<16>(fill, nrows, ncols, mb, rowptr, colind, counts, brp, bcol, bval, err, s);
    case 32: return launch_pack<32>(fill, nrows, ncols, mb, rowptr, colind, counts, brp, bcol, bval, err, s);
    default: return fail(GBS_ERR_UNSUPPORTED, "b2sr: tile size must be 4, 8, 16 or 32");
  }
}


// counts -> bsrRowPtr (exclusive scan, total in [mb]) and nnzb / validity to
// the host.
gbs_status b2sr_nnzb(int nrows, int ncols, int nnz, const int *rowptr, const int *colind, int ts,
                     int *bsr_rowptr, int *h_nnzb, cudaStream_t s) {
  const int mb = (nrows + ts - 1) / ts;
  DevBuf counts, err;
  GBS_TRY(counts.alloc(sizeof(int) * ((size_t)mb + 1), s));
  GBS_TRY(err.alloc(sizeof(int), s));
  GBS_CUDA_TRY(cudaMemsetAsync(counts.p, 0, sizeof(int) * ((size_t)mb + 1), s));
  GBS_CUDA_TRY(cudaMemsetAsync(err.p, 0, sizeof(int), s));
  GBS_TRY(pack_dispatch(ts, false, nrows, ncols, mb, rowptr, colind, counts.as<int>(), nullptr, nullptr,
                        nullptr, err.as<int>(), s));
  GBS_TRY(exclusive_scan_i32(counts.as<int>(), bsr_rowptr, mb + 1, s));
  int h[2] = {0, 0};
  GBS_CUDA_TRY(cudaMemcpyAsync(&h[0], bsr_rowptr + mb, sizeof(int), cudaMemcpyDeviceToHost, s));
  GBS_CUDA_TRY(cudaMemcpyAsync(&h[1], err.p, sizeof(int), cudaMemcpyDeviceToHost, s));
  GBS_CUDA_TRY(cudaStreamSynchronize(s));
  if (h[1]) return fail(GBS_ERR_INVALID_ARG, "csr2b2sr: column index out of range or columns of a row not ascending");
  (void)nnz;
  *h_nnzb = h[0];
  return GBS_OK;
}

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

// ---------------------------------------------------------------------------
// Aligned B2SR-8 / B2SR-16 (packUchar2AlignedUnsigned, :608-648;
// packUshort2AlignedUnsigned, :859-888): tiles of a block-row padded to a
// multiple of g = 4 (ts 8) / 2 (ts 16) with colind 0; word j of a group of g
// tiles holds row j of each, the first tile in the most significant byte
// (ts 8) / half (ts 16).
// ---------------------------------------------------------------------------
__global__ void k_aligned_counts(int mb, int g, const int *__restrict__ brp, int *__restrict__ counts) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < mb) {
    const int nt = brp[i + 1] - brp[i];
    counts[i] = (nt + g - 1) / g * g;
  } else if (i == mb) {
    counts[i] = 0;
  }
}

template <int TS>
__global__ void __launch_bounds__(256)
    k_aligned_fill(int mb, const int *__restrict__ brp, const int *__restrict__ bcol, const void *__restrict__ bval,
                   const int *__restrict__ nrp, int *__restrict__ ncol, uint32_t *__restrict__ nval) {
  constexpr int g = TS == 8 ? 4 : 2;
  constexpr int sh = 32 / g;
  const int lane = threadIdx.x & 31;
  const long long br = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (br >= mb) return;
  const int start = brp[br], nt = brp[br + 1] - start;
  const int pstart = nrp[br], padded = nrp[br + 1] - pstart;
  for (int i = lane; i < padded; i += 32) ncol[pstart + i] = i < nt ? bcol[start + i] : 0;
  const long long wbase = (long long)pstart / g * TS;
  const int nwords = padded / g * TS;
  for (int w = lane; w < nwords; w += 32) {
    const int gi = w / TS, j = w % TS;
    uint32_t word = 0;
#pragma unroll
    for (int q = 0; q < g; ++q) {
      const int ti = gi * g + q;
      const uint32_t a = ti < nt ? tile_row<TS>(bval, (size_t)start + ti, j) : 0u;
      word |= a << ((g - 1 - q) * sh);
    }
    nval[wbase + w] = word;
  }
}

// ---------------------------------------------------------------------------
// Dense sign packers: bit = (x >= 0), first column in bit 31.
//   rows : ToBit32RowDenseSign (spmm.cu:75-91), out[r*W + w]
//   colud: ToBit32ColUd (spmm.cu:93-111), out[w*Hp + r], Hp = 32*ceil(H/32)
// Elements outside the matrix read as -1 (bit 0).
// ---------------------------------------------------------------------------
template <bool COLUD>
__global__ void __launch_bounds__(256)
    k_pack_sign(const float *__restrict__ X, int H, int Wd, int Hp, uint32_t *__restrict__ out) {
  const int lane = threadIdx.x & 31;
  const long long row = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int rows = COLUD ? Hp : H;
  if (row >= rows) return;
  const int W = (Wd + 31) / 32;
  for (int w = 0; w < W; ++w) {
    const int c = w * 32 + lane;
    const float x = (row < H && c < Wd) ? __ldg(X + (size_t)row * Wd + c) : -1.0f;
    const uint32_t word = __brev(__ballot_sync(0xffffffffu, x >= 0.0f));
    if (lane == 0) {
      if (COLUD) out[(size_t)w * Hp + row] = word;
      else out[(size_t)row * W + w] = word;
    }
  }
}

}  // namespace gbs

// ===========================================================================
// C ABI
// ===========================================================================
using namespace gbs;

static bool valid_tile(int t) { return t == 4 || t == 8 || t == 16 || t == 32; }

extern "C" gbs_status gbs_csr2b2sr_nnzb(int nrows, int ncols, int nnz, const int *rowptr,
                                        const int *colind, int tile, int *bsr_rowptr, int *h_nnzb,
                                        gbs_stream_t stream) {
  clear_error();
  GBS_REQUIRE(valid_tile(tile), "csr2b2sr: tile must be 4, 8, 16 or 32");
  GBS_REQUIRE(nrows >= 0 && ncols >= 0 && nnz >= 0, "csr2b2sr: negative size");
  GBS_REQUIRE(h_nnzb != nullptr, "csr2b2sr: null nnzb output");
  GBS_REQUIRE(nrows == 0 || (rowptr != nullptr && bsr_rowptr != nullptr), "csr2b2sr: null pointer");
  GBS_REQUIRE(nnz == 0 || colind != nullptr, "csr2b2sr: null colind");
  if (nrows == 0) {
    *h_nnzb = 0;
    if (bsr_rowptr) GBS_CUDA_TRY(cudaMemsetAsync(bsr_rowptr, 0, sizeof(int), (cudaStream_t)stream));
    return GBS_OK;
  }
  return b2sr_nnzb(nrows, ncols, nnz, rowptr, colind, tile, bsr_rowptr, h_nnzb, (cudaStream_t)stream);
}

extern "C" gbs_status gbs_csr2b2sr(int nrows, int ncols, int nnz, const int *rowptr, const int *colind,
                                   int tile, const int *bsr_rowptr, int *bsr_colind, void *bsr_val,
                                   gbs_stream_t stream) {
  clear_error();
  GBS_REQUIRE(valid_tile(tile), "csr2b2sr: tile must be 4, 8, 16 or 32");
  GBS_REQUIRE(nrows >= 0 && ncols >= 0 && nnz >= 0, "csr2b2sr: negative size");
  if (nrows == 0) return GBS_OK;
  GBS_REQUIRE(rowptr && bsr_rowptr, "csr2b2sr: null pointer");
  GBS_REQUIRE(nnz == 0 || (colind && bsr_colind && bsr_val), "csr2b2sr: null pointer");
  const int mb = (nrows + tile - 1) / tile;
  return pack_dispatch(tile, true, nrows, ncols, mb, rowptr, colind, nullptr, bsr_rowptr, bsr_colind,
                       bsr_val, nullptr, (cudaStream_t)stream);
}

extern "C" gbs_status gbs_csr2bsr_batch(const int *h_rowptr, const int *h_colind, int nrows, int ncols,
                                        int nnz, int *bsr_rowptr, int *bsr_colind, void *bsr_val,
                                        int blocksize, int nblockrows, int nblocks) {
  clear_error();
  GBS_REQUIRE(valid_tile(blocksize), "csr2bsr_batch: blocksize must be 4, 8, 16 or 32");
  GBS_REQUIRE(nrows >= 0 && ncols >= 0 && nnz >= 0 && nblocks >= 0, "csr2bsr_batch: negative size");
  GBS_REQUIRE(nblockrows == (nrows + blocksize - 1) / blocksize,
              "csr2bsr_batch: nblockrows must be ceil(nrows / blocksize)");
  GBS_REQUIRE(nrows == 0 || (h_rowptr && bsr_rowptr), "csr2bsr_batch: null pointer");
  if (nrows == 0) return GBS_OK;
  GBS_REQUIRE(h_rowptr[0] == 0 && h_rowptr[nrows] == nnz, "csr2bsr_batch: rowptr[0] != 0 or rowptr[nrows] != nnz");
  cudaStream_t s = 0;
  DevBuf drp, dci;
  GBS_TRY(drp.alloc(sizeof(int) * ((size_t)nrows + 1), s));
  GBS_TRY(dci.alloc(sizeof(int) * (size_t)nnz, s));
  GBS_CUDA_TRY(cudaMemcpyAsync(drp.p, h_rowptr, sizeof(int) * ((size_t)nrows + 1), cudaMemcpyHostToDevice, s));
  if (nnz > 0)
    GBS_CUDA_TRY(cudaMemcpyAsync(dci.p, h_colind, sizeof(int) * (size_t)nnz, cudaMemcpyHostToDevice, s));
  int got = 0;
  GBS_TRY(b2sr_nnzb(nrows, ncols, nnz, drp.as<int>(), dci.as<int>(), blocksize, bsr_rowptr, &got, s));
  if (got != nblocks)
    return fail(GBS_ERR_INVALID_ARG, "csr2bsr_batch: nblocks = " + std::to_string(nblocks) +
                                         " but the matrix has " + std::to_string(got) + " tiles");
  if (nblocks > 0) {
    GBS_REQUIRE(bsr_colind && bsr_val, "csr2bsr_batch: null output");
    GBS_TRY(pack_dispatch(blocksize, true, nrows, ncols, nblockrows, drp.as<int>(), dci.as<int>(), nullptr,
                          bsr_rowptr, bsr_colind, bsr_val, nullptr, s));
  }
  GBS_CUDA_TRY(cudaStreamSynchronize(s));
  return GBS_OK;
}

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

extern "C" gbs_status gbs_b2sr_aligned_nnzb(int tile, int nblockrows, const int *bsr_rowptr, int *new_rowptr,
                                            int *h_ntiles, gbs_stream_t stream) {
  clear_error();
  GBS_REQUIRE(tile == 8 || tile == 16, "b2sr aligned: tile must be 8 or 16");
  GBS_REQUIRE(nblockrows >= 0 && h_ntiles, "b2sr aligned: bad arguments");
  GBS_REQUIRE(bsr_rowptr && new_rowptr, "b2sr aligned: null pointer");
  cudaStream_t s = (cudaStream_t)stream;
  DevBuf counts;
  GBS_TRY(counts.alloc(sizeof(int) * ((size_t)nblockrows + 1), s));
  const int g = tile == 8 ? 4 : 2;
  k_aligned_counts<<<(nblockrows + 1 + 255) / 256, 256, 0, s>>>(nblockrows, g, bsr_rowptr, counts.as<int>());
  GBS_TRY(check_launch("k_aligned_counts"));
  GBS_TRY(exclusive_scan_i32(counts.as<int>(), new_rowptr, nblockrows + 1, s));
  int h = 0;
  GBS_CUDA_TRY(cudaMemcpyAsync(&h, new_rowptr + nblockrows, sizeof(int), cudaMemcpyDeviceToHost, s));
  GBS_CUDA_TRY(cudaStreamSynchronize(s));
  *h_ntiles = h;
  return GBS_OK;
}

extern "C" gbs_status gbs_b2sr_pack_aligned(int tile, int nblockrows, const int *bsr_rowptr,
                                            const int *bsr_colind, const void *bsr_val, const int *new_rowptr,
                                            int *new_colind, uint32_t *new_val, gbs_stream_t stream) {
  clear_error();
  GBS_REQUIRE(tile == 8 || tile == 16, "b2sr aligned: tile must be 8 or 16");
  GBS_REQUIRE(nblockrows >= 0, "b2sr aligned: bad sizes");
  if (nblockrows == 0) return GBS_OK;
  GBS_REQUIRE(bsr_rowptr && new_rowptr && new_colind && new_val, "b2sr aligned: null pointer");
  cudaStream_t s = (cudaStream_t)stream;
  const int blocks = (int)(((long long)nblockrows * 32 + 255) / 256);
  if (tile == 8)
    k_aligned_fill<8><<<blocks, 256, 0, s>>>(nblockrows, bsr_rowptr, bsr_colind, bsr_val, new_rowptr, new_colind, new_val);
  else
    k_aligned_fill<16><<<blocks, 256, 0, s>>>(nblockrows, bsr_rowptr, bsr_colind, bsr_val, new_rowptr, new_colind, new_val);
  return check_launch("k_aligned_fill");
}

extern "C" gbs_status gbs_pack_sign_rows(const float *X, int n, int F, uint32_t *out, gbs_stream_t stream) {
  clear_error();
  GBS_REQUIRE(n >= 0 && F >= 1, "pack_sign_rows: bad sizes");
  if (n == 0) return GBS_OK;
  GBS_REQUIRE(X && out, "pack_sign_rows: null pointer");
  const int blocks = (int)(((long long)n * 32 + 255) / 256);
  k_pack_sign<false><<<blocks, 256, 0, (cudaStream_t)stream>>>(X, n, F, 0, out);
  return check_launch("k_pack_sign");
}

extern "C" gbs_status gbs_pack_sign_colud(const float *A, int H, int Wd, uint32_t *out, gbs_stream_t stream) {
  clear_error();
  GBS_REQUIRE(H >= 0 && Wd >= 1, "pack_sign_colud: bad sizes");
  if (H == 0) return GBS_OK;
  GBS_REQUIRE(A && out, "pack_sign_colud: null pointer");
  const int Hp = (H + 31) / 32 * 32;
  const int blocks = (int)(((long long)Hp * 32 + 255) / 256);
  k_pack_sign<true><<<blocks, 256, 0, (cudaStream_t)stream>>>(A, H, Wd, Hp, out);
  return check_launch("k_pack_sign");
}
