// Merge-path CSR SpMM kernel template shared by the forward entry points
// (csr_spmm.cu) and the fused backward (csr_spmm_bwd.cu).
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
//
// SD (fused SDDMM, backward only): the warp also keeps row r of H in
// registers and, for every entry (r, c) it gathers, reduces <B[c], H[r]>
// across the row's lanes and stores it at dvals[perm[e]] -- the value
// gradient of A in C = A^T-pass order mapped back to A's order.
#pragma once

#include "common.cuh"
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
  // degree-normalised binary A (vals null): entry (r, c) counts as
  // colscale[c] and row r of the result is multiplied by rowscale[r]; either
  // may be null (= 1).  Forward kernels only.
  const float *rowscale;
  const float *colscale;
  const void *B;
  float *C;
  float *partials;  // [2P][ldp]
  int *counters;    // [P]
  int ldp;
  int P;
  long long D;
  int accumulate;  // 1: C += A B (C read, added, written); 0: C = A B
  // fused SDDMM (SD kernels only)
  const void *H;     // rows indexed like C, F elements, B's type
  float *dvals;      // output, indexed through perm (or by entry when perm is null)
  const int *perm;   // entry e of this matrix -> index in dvals
};

// SC: degree-normalised binary A (rowscale / colscale, forward only);
// a separate instantiation, so the other kernels carry no extra registers.
template <int DT, int VEC, int LPR, int CH, int U, bool SD = false, bool SC = false>
struct MergeKernel {
  static constexpr int NSUB = 32 / LPR;
  static constexpr int KPS = LPR;  // nonzeros per sub-group in a batch of 32
  // Blocked summation (a fresh partial per batch of 32 nonzeros) for FP32
  // features only: it holds the FP32 error bound on rows of 20,000 entries,
  // while for 16-bit features the input rounding dominates and the second
  // set of accumulators would cost a CTA per SM (32 -> 24 warps).
  static constexpr bool BLK = DT == DT_F32;
  using F_ = Feat<DT, VEC>;
  using raw = typename F_::raw;

  // One forward round: U nonzeros per sub-group, entries u0 .. u0 + U - 1
  // of the sub-group's share of the batch.  TAIL: some entries may lie past
  // n_valid (their loads are skipped and their values zeroed); otherwise
  // every entry exists and the loads go out unpredicated.  Lanes whose chunk
  // lies past the row gather the row's last chunk; their sums are never
  // stored.  The (column, value) pairs come from the warp's batch staged in
  // shared memory sub-group-major, so one 16-byte load gives a sub-group two
  // entries where two shuffles per entry broadcast them before (114.8M-edge
  // graph, F = 256: FP32 5.81 against 5.92 ms, BF16 3.35 against 3.46 ms;
  // in the fused backward the same staging measured slower, 6.10 against
  // 6.00 ms, so it keeps the shuffles).
  template <bool TAIL>
  static __device__ __forceinline__ void round(const MergeArgs &a, int u0, int n_valid, int sub, int sl,
                                               const int2 *stage, float (&bs)[CH][VEC]) {
    raw bv[U][CH];
    float vv[U];
    int2 ent[U];
    if constexpr (U % 2 == 0) {
#pragma unroll
      for (int u = 0; u < U; u += 2) {
        const int4 q = *reinterpret_cast<const int4 *>(stage + sub * (32 / NSUB) + ((u0 + u) & (32 / NSUB - 1)));
        ent[u] = make_int2(q.x, q.y);
        ent[u + 1] = make_int2(q.z, q.w);
      }
    } else {
#pragma unroll
      for (int u = 0; u < U; ++u) ent[u] = stage[sub * (32 / NSUB) + ((u0 + u) & (32 / NSUB - 1))];
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int col = ent[u].x;
      const float v = __int_as_float(ent[u].y);
      const bool ok = !TAIL || (u0 + u) * NSUB + sub < n_valid;
      vv[u] = ok ? v : 0.f;
      // 32 x 32 -> 64-bit row offset (row strides are checked below 2^32 bytes)
      const size_t rowbase = (size_t)(unsigned)col * (unsigned)a.ldb;
#pragma unroll
      for (int c = 0; c < CH; ++c) {
        if (ok) bv[u][c] = F_::load(a.B, rowbase + (size_t)(min(c * LPR + sl, a.nvec - 1) * VEC));
        else bv[u][c] = F_::zero();
      }
    }
#pragma unroll
    for (int u = 0; u < U; ++u)
#pragma unroll
      for (int c = 0; c < CH; ++c) F_::fma(bs[c], vv[u], bv[u][c]);
  }

  // Value of entry e (column col): the stored value (or 1: binary A), or
  // the column's scale of a degree-normalised binary A.
  static __device__ __forceinline__ float entry_value(const MergeArgs &a, int e, int col) {
    if constexpr (SC) {
      return a.colscale ? __ldg(a.colscale + col) : 1.f;
    } else {
      return a.vals ? ld_stream_f32(a.vals + e) : 1.f;
    }
  }

  static __device__ __forceinline__ void scale_row(const MergeArgs &a, int r, float (&acc)[CH][VEC]) {
    if constexpr (!SC) return;
    if (!a.rowscale) return;
    const float s = __ldg(a.rowscale + r);
#pragma unroll
    for (int c = 0; c < CH; ++c)
#pragma unroll
      for (int q = 0; q < VEC; ++q) acc[c][q] *= s;
  }

  // Sum nonzeros [jb, je) of one row into acc (this lane's columns, this
  // lane's sub-group share).
  static __device__ __forceinline__ void accumulate(const MergeArgs &a, int jb, int je,
                                                    int lane, float (&acc)[CH][VEC],
                                                    const float (&h)[CH][VEC]) {
    const int sub = lane / LPR;
    const int sl = lane % LPR;
#pragma unroll
    for (int c = 0; c < CH; ++c)
#pragma unroll
      for (int q = 0; q < VEC; ++q) acc[c][q] = 0.f;

    // fused backward addressing: chunk c of row col of B starts at
    // lane_b[c] + col * pitch bytes (one 32 x 32 -> 64-bit multiply-add per
    // gathered chunk).  A lane whose chunk lies past the row reads the row's
    // last chunk instead, so every gather is an unconditional in-bounds load:
    // its FMAs land in accumulator slots that are never stored and its
    // dot-product terms meet a zero H element.  Entries past the end of a
    // batch gather the row of a column the lane held before (a valid row)
    // with weight 0, and their dot products are not stored.  (Predicated
    // loads with zero fill measured 9.61 / 7.66 ms against 8.82 / 6.83 ms
    // per FP32 / BF16 backward step of the 114.8M-edge graph.)
    const char *lane_b[CH];
#pragma unroll
    for (int c = 0; c < CH; ++c)
      lane_b[c] = static_cast<const char *>(a.B) +
                  (size_t)min(c * LPR + sl, a.nvec - 1) * VEC * sizeof(typename F_::storage_t);
    const unsigned pitch = (unsigned)(a.ldb * (long long)sizeof(typename F_::storage_t));
    raw bv[U][CH];
#pragma unroll
    for (int u = 0; u < U; ++u)
#pragma unroll
      for (int c = 0; c < CH; ++c) bv[u][c] = F_::zero();
    int nx_col = 0;
    float nx_val = 0.f;
    if (jb + lane < je) {
      nx_col = ld_stream_i32(a.colind + jb + lane);
      nx_val = entry_value(a, jb + lane, nx_col);
    }
    for (int base = jb; base < je; base += 32) {
      const int n_valid = min(32, je - base);
      const int my_col = nx_col;
      const float my_val = nx_val;
      // the next batch of this row is loaded while this one is gathered
      if (base + 32 + lane < je) {
        nx_col = ld_stream_i32(a.colind + base + 32 + lane);
        nx_val = entry_value(a, base + 32 + lane, nx_col);
      }
      // blocked summation: each batch of 32 nonzeros is summed into a fresh
      // partial that is then added to the row total (error ~ sqrt(32) +
      // sqrt(deg/32) roundings instead of sqrt(deg))
      float blk[CH][VEC];
      float (&bs)[CH][VEC] = BLK ? blk : acc;
      if constexpr (BLK) {
#pragma unroll
        for (int c = 0; c < CH; ++c)
#pragma unroll
          for (int q = 0; q < VEC; ++q) bs[c][q] = 0.f;
      }
      // rounds of U nonzeros per sub-group; a runtime trip count (not an
      // unrolled loop with early exits) keeps the loads of one round
      // together.  Only the last round of a batch can hold missing entries:
      // the forward runs the others unpredicated (BF16 3.66 against 4.21 ms,
      // 114.8M-edge graph, F = 256); the fused backward runs one loop of
      // unconditional loads with zero weights past the batch (a split into
      // full rounds and a tail measured 10.9 against 10.0 ms in FP32).
      if constexpr (SD) {
        const int rounds = (n_valid + U * NSUB - 1) / (U * NSUB);
#pragma unroll 1
        for (int rd = 0; rd < rounds; ++rd) {
          const int u0 = rd * U;
          float vv[U];
#pragma unroll
          for (int u = 0; u < U; ++u) {
            const int k = ((u0 + u) * NSUB + sub) & 31;
            const int col = __shfl_sync(0xffffffffu, my_col, k);
            const float v = __shfl_sync(0xffffffffu, my_val, k);
            const bool ok = (u0 + u) * NSUB + sub < n_valid;
            vv[u] = ok ? v : 0.f;
            const size_t rowoff = (size_t)(unsigned)col * pitch;
#pragma unroll
            for (int c = 0; c < CH; ++c) bv[u][c] = F_::load(lane_b[c] + rowoff, 0);
          }
          // each gathered chunk is widened once and feeds both the row sum
          // and the dot product with the H row (even / odd columns as the
          // two halves of FFMA2s, added at the end)
          float sd[U];
#pragma unroll
          for (int u = 0; u < U; ++u) {
            float s0 = 0.f, s1 = 0.f;
#pragma unroll
            for (int c = 0; c < CH; ++c) {
              float x[VEC];
              F_::widen(x, bv[u][c]);
              if constexpr (VEC % 2 == 0) {
#pragma unroll
                for (int q = 0; q < VEC; q += 2) {
                  fma2(bs[c][q], bs[c][q + 1], vv[u], x[q], x[q + 1]);
                  fma2v(s0, s1, h[c][q], h[c][q + 1], x[q], x[q + 1]);
                }
              } else {
#pragma unroll
                for (int q = 0; q < VEC; ++q) {
                  bs[c][q] = fmaf(vv[u], x[q], bs[c][q]);
                  s0 = fmaf(h[c][q], x[q], s0);
                }
              }
            }
            sd[u] = s0 + s1;
          }
          sddmm_reduce(a, base, u0, n_valid, sub, sl, sd);
        }
      } else {
        // stage the batch: entry k at position (k % NSUB) * (32 / NSUB) + k / NSUB
        __shared__ __align__(16) int2 fstage_all[8][32];
        int2 *stage = fstage_all[threadIdx.x >> 5];
        __syncwarp();
        stage[(lane % NSUB) * (32 / NSUB) + lane / NSUB] = make_int2(my_col, __float_as_int(my_val));
        __syncwarp();
        const int full = n_valid / (U * NSUB);
#pragma unroll 1
        for (int rd = 0; rd < full; ++rd) round<false>(a, rd * U, n_valid, sub, sl, stage, bs);
        if (full * U * NSUB < n_valid) round<true>(a, full * U, n_valid, sub, sl, stage, bs);
      }
      if constexpr (BLK) {
#pragma unroll
        for (int c = 0; c < CH; ++c)
#pragma unroll
          for (int q = 0; q < VEC; ++q) acc[c][q] += bs[c][q];
      }
    }
    // fold the sub-groups (fixed tree order)
#pragma unroll
    for (int off = LPR; off < 32; off <<= 1)
#pragma unroll
      for (int c = 0; c < CH; ++c)
#pragma unroll
        for (int q = 0; q < VEC; ++q) acc[c][q] += __shfl_xor_sync(0xffffffffu, acc[c][q], off);
  }

  // Fused SDDMM for one round of U entries per sub-group: the per-lane
  // partial dot products s[u] (gathered row . H row) are reduced over the LPR
  // lanes by a multi-value butterfly ((U - 1) + log2(LPR / U) shuffles per U
  // entries) and stored.
  static __device__ __forceinline__ void sddmm_reduce(const MergeArgs &a, int base, int u0, int n_valid, int sub,
                                                      int sl, float (&s)[U]) {
    int nv = U;
#pragma unroll
    for (int off = LPR / 2; off >= 1; off >>= 1) {
      if (nv > 1) {
        const int half = nv / 2;
        const bool upper = (sl & off) != 0;
#pragma unroll
        for (int i = 0; i < U / 2; ++i) {
          if (i < half) {
            const float send = upper ? s[i] : s[i + half];
            const float keep = upper ? s[i + half] : s[i];
            s[i] = keep + __shfl_xor_sync(0xffffffffu, send, off);
          }
        }
        nv = half;
      } else {
        s[0] += __shfl_xor_sync(0xffffffffu, s[0], off);
      }
    }
    const int span = LPR / U;
    const int k = (u0 + sl / span) * NSUB + sub;
    if (sl % span == 0 && k < n_valid) {
      const long long e = (long long)a.rp_base + base + k;
      a.dvals[a.perm ? (long long)__ldg(a.perm + e) : e] = s[0];
    }
  }

  // H row r (this lane's chunks), widened to FP32.
  static __device__ __forceinline__ void load_h(const MergeArgs &a, int r, int lane, float (&h)[CH][VEC]) {
    const int sl = lane % LPR;
#pragma unroll
    for (int c = 0; c < CH; ++c) {
      const int chunk = c * LPR + sl;
      if (SD && chunk < a.nvec) F_::widen(h[c], F_::load(a.H, (size_t)r * a.F + (size_t)chunk * VEC));
      else
#pragma unroll
        for (int q = 0; q < VEC; ++q) h[c][q] = 0.f;
    }
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
        if (SC && a.rowscale) {
          const float s = __ldg(a.rowscale + r);
#pragma unroll
          for (int q = 0; q < VEC; ++q) sum[q] *= s;
        }
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
    float h[CH][VEC];
    for (int r = i0; r < i1; ++r) {
      const int rb = __ldg(a.rowptr + r) - a.rp_base, re = __ldg(a.rowptr + r + 1) - a.rp_base;
      if constexpr (SD) load_h(a, r, lane, h);
      accumulate(a, j, re, lane, acc, h);
      if (j == rb) {
        scale_row(a, r, acc);
        if (a.accumulate) add_row(a, a.C + (size_t)r * a.ldc, lane, acc);
        else write_row<true>(a, a.C + (size_t)r * a.ldc, lane, acc);
      } else {  // head piece: the row started in an earlier warp
        write_row<false>(a, a.partials + (size_t)(2 * warp) * a.ldp, lane, acc);
        finish_split(a, r, lane);
      }
      j = re;
    }
    if (j < j1) {  // tail (or middle) piece of row i1: continues past d1
      if constexpr (SD) load_h(a, i1, lane, h);
      accumulate(a, j, j1, lane, acc, h);
      write_row<false>(a, a.partials + (size_t)(2 * warp + 1) * a.ldp, lane, acc);
      finish_split(a, i1, lane);
    }
  }
};

}  // namespace gbs
