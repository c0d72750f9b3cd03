// B2SR ("binarised BSR") on sm_103a: CSR -> B2SR packing for tiles 4/8/16/32,
// the "aligned" B2SR-8/16 variants and the dense sign packers (layout in
// b2sr_common.cuh).
#include "b2sr_common.cuh"

namespace gbs {

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
