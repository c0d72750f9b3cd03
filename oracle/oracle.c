/*
 * oracle.c -- CPU restatement of the spmm_eval reference path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker the tests, the smoke
 * run and the CPU-baseline leg of bench.py compare against; the product
 * (libgbspmm.so) never links, loads or calls it.
 *
 * Every function cites the reference file:line whose behaviour it restates
 * (paths inside the spmm_eval project).  Pinning: see tests/golden/ (the
 * .mtx ingest goldens made by the reference's own readMtx.hpp compiled by
 * oracle/Makefile) and the GPU tests that compare these layouts with
 * cuSPARSE csr2bsr / cusparseSpMM, the library the reference itself calls.
 *
 * Plain C11 + OpenMP; no SIMD intrinsics; identical results on x86-64 and
 * aarch64 (integer and FP64 paths; the FP32 baseline uses fmaf explicitly).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------------ */
/* CSR SpMM                                                                  */
/* ------------------------------------------------------------------------ */

/* FP64 oracle of C = A*B for the rows in `rows` (or all rows if rows==NULL)
 * plus the magnitude sum M = |A|*|B| used as the relative-error scale.
 * Standard definition; the reference checks against cusparseSpMM
 * (test_spmm_full.cu:303-307).  vals == NULL means every entry is 1.0. */
void orc_csr_spmm_f64(int nrows, const int *rowptr, const int *colind, const float *vals,
                      const float *B, int F, const int *rows, int nsel, double *C,
                      double *M) {
  int count = rows ? nsel : nrows;
#pragma omp parallel for schedule(dynamic, 16)
  for (int t = 0; t < count; ++t) {
    int r = rows ? rows[t] : t;
    double *c = C + (size_t)t * F;
    double *m = M ? M + (size_t)t * F : NULL;
    for (int k = 0; k < F; ++k) {
      c[k] = 0.0;
      if (m) m[k] = 0.0;
    }
    for (int e = rowptr[r]; e < rowptr[r + 1]; ++e) {
      double v = vals ? (double)vals[e] : 1.0;
      const float *b = B + (size_t)colind[e] * F;
      for (int k = 0; k < F; ++k) {
        c[k] += v * (double)b[k];
        if (m) m[k] += fabs(v) * fabs((double)b[k]);
      }
    }
  }
}

/* FP32 CPU baseline with the reference's semantics: row-major B and C, each
 * row accumulated in CSR order (the order coo2csr gives, readMtx.hpp:284-292),
 * one fmaf per product, rows [r0, r1) only, dynamic schedule of 64 rows. */
void orc_csr_spmm_f32(int r0, int r1, const int *rowptr, const int *colind, const float *vals,
                      const float *B, int F, float *C, int nthreads) {
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
#pragma omp parallel for schedule(dynamic, 64)
  for (int r = r0; r < r1; ++r) {
    float *c = C + (size_t)(r - r0) * F;
    for (int k = 0; k < F; ++k) c[k] = 0.0f;
    for (int e = rowptr[r]; e < rowptr[r + 1]; ++e) {
      float v = vals ? vals[e] : 1.0f;
      const float *b = B + (size_t)colind[e] * F;
      for (int k = 0; k < F; ++k) c[k] = fmaf(v, b[k], c[k]);
    }
  }
}

int orc_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

/* ------------------------------------------------------------------------ */
/* CSR -> B2SR packing                                                       */
/* ------------------------------------------------------------------------ */
/*
 * csr2bsr_batch_{4,8,16,32} (csr2bsr_batch_bsrbmv.cu:207-397, :403-579,
 * :654-830, :894-1070) walk the block-rows serially.  Block-row i covers CSR
 * rows [i*ts, min((i+1)*ts, nrows)) (:240; the last strip's row pointer is
 * padded with temp_nnz, :271-276, i.e. the missing rows are empty).  Each
 * strip goes through cusparseScsr2bsr with every value forced to 1.0
 * (:296-297), so a tile exists for every distinct floor(col/ts) of the strip,
 * in ascending order, and every stored entry (even a stored 0.0) sets its
 * bit.  ToBit{4,8,16,32}Col (spmm.cu:165-194, :226-246, :272-291, :318-335)
 * then packs tile row r into element ts*b + r, column 0 at the most
 * significant of the ts bits: uchar for ts 4 (low nibble) and 8, ushort for
 * 16, uint32 for 32.  bsrRowPtr is the running sum of tile counts (:332-334).
 */

/* Tiles in each block-row; returns nnzb, fills bsr_rowptr[mb+1].
 * Returns -1 if a row's columns are not ascending or out of range. */
long long orc_b2sr_count(int nrows, int ncols, const int *rowptr, const int *colind, int ts,
                         int *bsr_rowptr) {
  int mb = (nrows + ts - 1) / ts;
  int nbc = (ncols + ts - 1) / ts;
  int *mark = (int *)malloc(sizeof(int) * (size_t)(nbc > 0 ? nbc : 1));
  for (int i = 0; i < nbc; ++i) mark[i] = -1;
  long long total = 0;
  bsr_rowptr[0] = 0;
  for (int i = 0; i < mb; ++i) {
    int cnt = 0;
    int rend = (i + 1) * ts < nrows ? (i + 1) * ts : nrows;
    for (int r = i * ts; r < rend; ++r) {
      for (int e = rowptr[r]; e < rowptr[r + 1]; ++e) {
        int c = colind[e];
        if (c < 0 || c >= ncols || (e > rowptr[r] && colind[e - 1] > c)) {
          free(mark);
          return -1;
        }
        int bc = c / ts;
        if (mark[bc] != i) {
          mark[bc] = i;
          ++cnt;
        }
      }
    }
    total += cnt;
    bsr_rowptr[i + 1] = (int)total;
  }
  free(mark);
  return total;
}

static int cmp_int(const void *a, const void *b) {
  int x = *(const int *)a, y = *(const int *)b;
  return (x > y) - (x < y);
}

/* Fill colind / packed values; bsr_val element size = 1 (ts 4, 8), 2 (16),
 * 4 (32).  Uses bsr_rowptr from orc_b2sr_count. */
void orc_b2sr_fill(int nrows, int ncols, const int *rowptr, const int *colind, int ts,
                   const int *bsr_rowptr, int *bsr_colind, void *bsr_val) {
  int mb = (nrows + ts - 1) / ts;
  int nbc = (ncols + ts - 1) / ts;
  int *slot = (int *)malloc(sizeof(int) * (size_t)(nbc > 0 ? nbc : 1));
  for (int i = 0; i < mb; ++i) {
    int base = bsr_rowptr[i], n = 0;
    int rend = (i + 1) * ts < nrows ? (i + 1) * ts : nrows;
    for (int r = i * ts; r < rend; ++r)
      for (int e = rowptr[r]; e < rowptr[r + 1]; ++e) {
        int bc = colind[e] / ts;
        int seen = 0;
        for (int q = 0; q < n; ++q)
          if (bsr_colind[base + q] == bc) { seen = 1; break; }
        if (!seen) bsr_colind[base + n++] = bc;
      }
    qsort(bsr_colind + base, (size_t)n, sizeof(int), cmp_int);
    for (int q = 0; q < n; ++q) slot[bsr_colind[base + q]] = base + q;
    for (int q = 0; q < n * ts; ++q) {
      size_t at = (size_t)base * ts + q;
      if (ts <= 8) ((uint8_t *)bsr_val)[at] = 0;
      else if (ts == 16) ((uint16_t *)bsr_val)[at] = 0;
      else ((uint32_t *)bsr_val)[at] = 0;
    }
    for (int r = i * ts; r < rend; ++r)
      for (int e = rowptr[r]; e < rowptr[r + 1]; ++e) {
        int c = colind[e], b = slot[c / ts], rr = r - i * ts, j = c % ts;
        size_t at = (size_t)b * ts + rr;
        if (ts <= 8) ((uint8_t *)bsr_val)[at] |= (uint8_t)(1u << (ts - 1 - j));
        else if (ts == 16) ((uint16_t *)bsr_val)[at] |= (uint16_t)(1u << (15 - j));
        else ((uint32_t *)bsr_val)[at] |= 1u << (31 - j);
      }
  }
  free(slot);
}

static inline uint32_t tile_row(const void *val, int ts, size_t tile, int r) {
  size_t at = tile * ts + r;
  if (ts <= 8) return ((const uint8_t *)val)[at];
  if (ts == 16) return ((const uint16_t *)val)[at];
  return ((const uint32_t *)val)[at];
}

/* "Aligned" B2SR-8 / B2SR-16 for the BMV kernels: countUcharUnsignedSize /
 * packUchar2AlignedUnsigned (csr2bsr_batch_bsrbmv.cu:586-648) and
 * countUshortUnsignedSize / packUshort2AlignedUnsigned (:837-888).  Tiles of
 * a block-row are padded to a multiple of g = 4 (ts 8) or 2 (ts 16); padded
 * colind entries are 0; word j of a group packs row j of its g tiles, the
 * first tile in the most significant byte / half.  Returns the number of
 * uint32 words (the count function's result). */
long long orc_b2sr_aligned(int ts, int nblockrows, const int *bsr_rowptr, const int *bsr_colind,
                           const void *bsr_val, int *new_rowptr, int *new_colind,
                           uint32_t *new_val) {
  int g = ts == 8 ? 4 : 2;
  long long cnt = 0, colcnt = 0;
  if (new_rowptr) new_rowptr[0] = 0;
  for (int row = 0; row < nblockrows; ++row) {
    int nt = bsr_rowptr[row + 1] - bsr_rowptr[row], start = bsr_rowptr[row];
    int padded = (nt + g - 1) / g * g;
    for (int i = 0; i < padded; i += g)
      for (int j = 0; j < ts; ++j) {
        uint32_t w = 0;
        for (int q = 0; q < g; ++q) {
          uint32_t a = (i + q < nt) ? tile_row(bsr_val, ts, (size_t)start + i + q, j) : 0u;
          w |= a << ((g - 1 - q) * (32 / g));
        }
        if (new_val) new_val[cnt] = w;
        ++cnt;
      }
    for (int i = 0; i < padded; ++i) {
      if (new_colind) new_colind[colcnt] = i < nt ? bsr_colind[start + i] : 0;
      ++colcnt;
    }
    if (new_rowptr) new_rowptr[row + 1] = new_rowptr[row] + padded;
  }
  return cnt;
}

/* ------------------------------------------------------------------------ */
/* B2SR x dense SpMM                                                         */
/* ------------------------------------------------------------------------ */

/* spmm4_full_full_new2 (spmm.cu:877-956), summation order restated exactly:
 * block-row r, output row 4r+i, column c: result starts at +0.0f and, for
 * each group of 8 tiles (:900), for j = 0..3 (:930) and tile l = 0..7 of the
 * group (:931), adds B[(4*colind[t]+j)*F + c] if bit (3-j) of byte 4t+i is
 * set (:907-909, :936-940).  A result equal to 0 is not stored (:947-954),
 * so C must come in zero-filled and padding rows >= nrows are never written
 * (they have no bits). */
void orc_b2sr4_spmm_ref(int nblockrows, const int *rowptr, const int *colind, const uint8_t *A,
                        const float *B, int F, float *C, long long crows) {
#pragma omp parallel for schedule(dynamic, 16)
  for (int r = 0; r < nblockrows; ++r) {
    for (int i = 0; i < 4; ++i) {
      long long orow = 4LL * r + i;
      for (int c = 0; c < F; ++c) {
        float res = 0.0f;
        for (int g = rowptr[r]; g < rowptr[r + 1]; g += 8)
          for (int j = 0; j < 4; ++j)
            for (int l = 0; l < 8; ++l) {
              int t = g + l;
              if (t >= rowptr[r + 1]) continue;
              if ((A[(size_t)t * 4 + i] >> (3 - j)) & 1u)
                res = res + B[((size_t)colind[t] * 4 + j) * F + c];
            }
        if (res != 0.0f && orow < crows) C[orow * F + c] = res;
      }
    }
  }
}

/* B2SR (ts 4/8/16/32) x FP32 B, natural order (tile, then column j), every
 * row < nrows written.  Equals the CSR product of the 0/1 matrix; exact for
 * integer-valued B.  No reference kernel exists for ts != 4. */
void orc_b2sr_spmm(int ts, int nrows, int nblockrows, const int *rowptr, const int *colind,
                   const void *val, const float *B, int F, float *C) {
#pragma omp parallel for schedule(dynamic, 16)
  for (int r = 0; r < nblockrows; ++r)
    for (int i = 0; i < ts; ++i) {
      long long orow = (long long)r * ts + i;
      if (orow >= nrows) continue;
      float *c = C + orow * F;
      for (int k = 0; k < F; ++k) c[k] = 0.0f;
      for (int t = rowptr[r]; t < rowptr[r + 1]; ++t) {
        uint32_t bits = tile_row(val, ts, (size_t)t, i);
        for (int j = 0; j < ts; ++j)
          if ((bits >> (ts - 1 - j)) & 1u) {
            const float *b = B + ((size_t)colind[t] * ts + j) * F;
            for (int k = 0; k < F; ++k) c[k] += b[k];
          }
      }
    }
}

/* ------------------------------------------------------------------------ */
/* Bit packing of dense matrices                                             */
/* ------------------------------------------------------------------------ */

/* ToBit32RowDenseSign (spmm.cu:75-91): bit = (x >= 0), row-major words
 * [n][W], W = ceil(F/32), column 32w at bit 31; columns >= F read as -1 (0). */
void orc_pack_sign_rows(const float *X, int n, int F, uint32_t *out) {
  int W = (F + 31) / 32;
  for (int r = 0; r < n; ++r)
    for (int w = 0; w < W; ++w) {
      uint32_t v = 0;
      for (int b = 0; b < 32; ++b) {
        int c = w * 32 + b;
        float x = c < F ? X[(size_t)r * F + c] : -1.0f;
        v = (v << 1) | (x >= 0.0f ? 1u : 0u);
      }
      out[(size_t)r * W + w] = v;
    }
}

/* ToBit32ColUd (spmm.cu:93-111): bit = (x >= 0) for an H x Wd matrix; word
 * (by, row) at out[by * Hp + row] with Hp = 32*ceil(H/32), column 32*by at
 * bit 31; rows >= H and columns >= Wd read as -1 (0). */
void orc_pack_sign_colud(const float *A, int H, int Wd, uint32_t *out) {
  int Hp = (H + 31) / 32 * 32, Wb = (Wd + 31) / 32;
  for (int by = 0; by < Wb; ++by)
    for (int row = 0; row < Hp; ++row) {
      uint32_t v = 0;
      for (int b = 0; b < 32; ++b) {
        int c = by * 32 + b;
        float x = (row < H && c < Wd) ? A[(size_t)row * Wd + c] : -1.0f;
        v = (v << 1) | (x >= 0.0f ? 1u : 0u);
      }
      out[(size_t)by * Hp + row] = v;
    }
}

/* ------------------------------------------------------------------------ */
/* B2SR x packed-bit features (BMV / BMM)                                    */
/* ------------------------------------------------------------------------ */

/* C01[i][k] = sum_j A_ij * bit_jk over the 0/1 B2SR matrix and features
 * packed by orc_pack_sign_rows; signed_form = 1 gives 2*C01 - deg(i), the
 * float result of the reference driver for +-1 features
 * (test_spmm_full.cu:488-491 with spmm.cu:877-956). */
void orc_b2sr_bmm(int ts, int nrows, int nblockrows, const int *rowptr, const int *colind,
                  const void *val, const uint32_t *X, int F, int signed_form, int32_t *C) {
  int W = (F + 31) / 32;
#pragma omp parallel for schedule(dynamic, 16)
  for (int r = 0; r < nblockrows; ++r)
    for (int i = 0; i < ts; ++i) {
      long long orow = (long long)r * ts + i;
      if (orow >= nrows) continue;
      int32_t *c = C + orow * F;
      for (int k = 0; k < F; ++k) c[k] = 0;
      int deg = 0;
      for (int t = rowptr[r]; t < rowptr[r + 1]; ++t) {
        uint32_t bits = tile_row(val, ts, (size_t)t, i);
        for (int j = 0; j < ts; ++j)
          if ((bits >> (ts - 1 - j)) & 1u) {
            ++deg;
            const uint32_t *x = X + ((size_t)colind[t] * ts + j) * W;
            for (int k = 0; k < F; ++k) c[k] += (int32_t)((x[k / 32] >> (31 - k % 32)) & 1u);
          }
      }
      if (signed_form)
        for (int k = 0; k < F; ++k) c[k] = 2 * c[k] - deg;
    }
}

/* ------------------------------------------------------------------------ */
/* Dense binary GEMM (backend/mm.cu)                                         */
/* ------------------------------------------------------------------------ */
/* A: [Kw][M] words, B: [Kw][N] words (the ToBit32ColUd layout; mm.cu:30-31
 * reads A[i*A_height + row], B[i*B_width + col]).  xorcount = sum_i
 * popc(A[i][r] ^ B[i][c]). */
static inline int popc32(uint32_t x) {
  x = x - ((x >> 1) & 0x55555555u);
  x = (x & 0x33333333u) + ((x >> 2) & 0x33333333u);
  x = (x + (x >> 4)) & 0x0F0F0F0Fu;
  return (int)((x * 0x01010101u) >> 24);
}

/* mode 0: XOR count, 1: AND count, 2: 32*Kw - 2*xor (the value BMM32_Arow_Brow
 * stores, mm.cu:44-51, as int32).  C row-major M x N. */
void orc_bmm_counts(const uint32_t *A, const uint32_t *B, int M, int N, int Kw, int mode,
                    int32_t *C) {
#pragma omp parallel for schedule(static)
  for (int r = 0; r < M; ++r)
    for (int c = 0; c < N; ++c) {
      int acc = 0;
      for (int i = 0; i < Kw; ++i) {
        uint32_t a = A[(size_t)i * M + r], b = B[(size_t)i * N + c];
        acc += popc32(mode == 1 ? (a & b) : (a ^ b));
      }
      C[(size_t)r * N + c] = mode == 2 ? 32 * Kw - 2 * acc : acc;
    }
}

/* BMM32_Arow_Brow<float> (mm.cu:17-53): C[r*N + c] = 32*Kw - 2*xor as float. */
void orc_bmm32_arow_brow(const uint32_t *A, const uint32_t *B, int M, int Kw, int N, float *C) {
#pragma omp parallel for schedule(static)
  for (int r = 0; r < M; ++r)
    for (int c = 0; c < N; ++c) {
      int acc = 0;
      for (int i = 0; i < Kw; ++i) acc += popc32(A[(size_t)i * M + r] ^ B[(size_t)i * N + c]);
      C[(size_t)r * N + c] = (float)(32 * Kw) - (float)acc * 2.0f;
    }
}

/* BMM32_BIN (mm.cu:79-105), launched <<<(m/32, k/32), 32>>>: word of row
 * bx*32+lane over columns by*32..by*32+31 (first column in bit 31), bit =
 * (n - 2*xor >= 0) with n the number of bits, stored at C[by*m + bx*32 +
 * lane].  The loop (i*32) < n reads ceil(n/32) words. */
void orc_bmm32_bin(const uint32_t *A, const uint32_t *B, int m, int n, int k, uint32_t *C) {
  int Kw = (n + 31) / 32;
  for (int by = 0; by < k / 32; ++by)
    for (int row = 0; row < m; ++row) {
      uint32_t w = 0;
      for (int j = 0; j < 32; ++j) {
        int col = by * 32 + j, acc = 0;
        for (int i = 0; i < Kw; ++i) acc += popc32(A[(size_t)i * m + row] ^ B[(size_t)i * k + col]);
        float t = (float)n - 2.0f * (float)acc;
        w = w + w + (t >= 0.0f ? 1u : 0u);
      }
      C[(size_t)by * m + row] = w;
    }
}

/* BMM32S_BIN (mm.cu:108-125), launched <<<(m/32, k/32), 1024>>>: warp w of
 * block (bx, by) handles row bx*32+w; lane l column by*32+l; bit = (n - 2*xor
 * >= 0); ballot + brev puts lane 0 in bit 31; stored at C[bx*k*32 + by*32 +
 * w] (k = number of columns). */
void orc_bmm32s_bin(const uint32_t *A, const uint32_t *B, int m, int n, int k, uint32_t *C) {
  int Kw = (n + 31) / 32;
  for (int bx = 0; bx < m / 32; ++bx)
    for (int by = 0; by < k / 32; ++by)
      for (int w = 0; w < 32; ++w) {
        int row = bx * 32 + w;
        uint32_t word = 0;
        for (int l = 0; l < 32; ++l) {
          int col = by * 32 + l, acc = 0;
          for (int i = 0; i < Kw; ++i) acc += popc32(A[(size_t)i * m + row] ^ B[(size_t)i * k + col]);
          float t = (float)n - 2.0f * (float)acc;
          if (t >= 0.0f) word |= 1u << (31 - l);
        }
        C[(size_t)bx * k * 32 + (size_t)by * 32 + w] = word;
      }
}

/* ------------------------------------------------------------------------ */
/* Backward support                                                          */
/* ------------------------------------------------------------------------ */

/* CSR transpose with rows ascending inside each column, as csr2csc does
 * (readMtx.hpp:319-345 via coo2csr's stable per-row fill); perm[i] is the
 * index in A of transposed entry i. */
void orc_csr_transpose(int nrows, int ncols, const int *rowptr, const int *colind,
                       int *t_rowptr, int *t_colind, int *perm) {
  for (int c = 0; c <= ncols; ++c) t_rowptr[c] = 0;
  int nnz = rowptr[nrows];
  for (int e = 0; e < nnz; ++e) t_rowptr[colind[e] + 1]++;
  for (int c = 0; c < ncols; ++c) t_rowptr[c + 1] += t_rowptr[c];
  int *fill = (int *)malloc(sizeof(int) * (size_t)(ncols > 0 ? ncols : 1));
  for (int c = 0; c < ncols; ++c) fill[c] = t_rowptr[c];
  for (int r = 0; r < nrows; ++r)
    for (int e = rowptr[r]; e < rowptr[r + 1]; ++e) {
      int at = fill[colind[e]]++;
      t_colind[at] = r;
      perm[at] = e;
    }
  free(fill);
}

/* SDDMM over A's pattern in FP64: out[e] = <G[row(e), :], H[col(e), :]>. */
void orc_sddmm_f64(int nrows, const int *rowptr, const int *colind, const float *G,
                   const float *H, int F, double *out) {
#pragma omp parallel for schedule(dynamic, 16)
  for (int r = 0; r < nrows; ++r)
    for (int e = rowptr[r]; e < rowptr[r + 1]; ++e) {
      const float *g = G + (size_t)r * F, *h = H + (size_t)colind[e] * F;
      double s = 0.0;
      for (int k = 0; k < F; ++k) s += (double)g[k] * (double)h[k];
      out[e] = s;
    }
}
