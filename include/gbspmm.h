/*
 * gbspmm.h -- C ABI of the GB300 (sm_103a) SpMM library.
 *
 * Drop-in boundary for the SpMM evaluation path of spmm_eval.  Every entry
 * point takes plain device pointers, sizes and a CUDA stream, returns a
 * gbs_status, never traps on the device and never synchronises the device
 * unless its comment says so (a size that must reach the host).
 *
 * Conventions
 *   - CSR matrices use int32 row pointers / column indices, zero based, with
 *     the column indices of a row ascending (what coo2csr in the reference's
 *     backend/readMtx.hpp:246-304 produces).
 *   - Dense feature matrices (B, C, dC, X) are row-major, leading dimension F.
 *   - The caller owns every input, output and workspace buffer.  Opaque
 *     objects (gbs_csr_transpose) are created and destroyed explicitly.
 *   - gbs_stream_t is a cudaStream_t; NULL is the legacy default stream.
 *   - Errors: a non-zero gbs_status; gbs_last_error() gives a message for the
 *     calling thread.
 */
#ifndef GBSPMM_H_
#define GBSPMM_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define GBS_API __attribute__((visibility("default")))
#else
#define GBS_API
#endif

typedef struct CUstream_st *gbs_stream_t;

typedef enum gbs_status {
  GBS_OK = 0,
  GBS_ERR_INVALID_ARG = 1, /* bad size, null pointer, malformed CSR      */
  GBS_ERR_UNSUPPORTED = 2, /* valid request this build does not support  */
  GBS_ERR_CUDA = 3,        /* a CUDA runtime call failed                 */
  GBS_ERR_OOM = 4,         /* device allocation failed                   */
  GBS_ERR_INTERNAL = 5
} gbs_status;

/* Element type of a dense feature / gradient matrix.  Accumulation is
 * always FP32 and outputs are FP32. */
typedef enum gbs_dtype { GBS_F32 = 0, GBS_BF16 = 1, GBS_F16 = 2 } gbs_dtype;

/* Message describing the last failure on the calling thread ("" if none). */
GBS_API const char *gbs_last_error(void);
/* ABI version of this header (bumped on incompatible change). */
GBS_API int gbs_abi_version(void);
/* Entry points that document temporary allocations take them from a
 * library-owned stream-ordered pool on the current device, which keeps up to
 * 8 GiB of freed temporaries mapped between calls.  This returns all of the
 * pool's unused memory to the device.  No counterpart in the reference. */
GBS_API gbs_status gbs_pool_trim(void);

/* ------------------------------------------------------------------------
 * Matrix Market ingest (host).  Same result as readMtx<float>(...,
 * directed = 0, ...) + coo2csr in the reference (test_spmm_full.cu:99-113,
 * backend/readMtx.hpp:351-422, :246-304): 0-based, sorted by (row, col),
 * duplicates kept, symmetric files not expanded, pattern values 1.0.
 * Errors (not undefined state) for truncated files, out-of-range indices,
 * complex or dense files.
 * ------------------------------------------------------------------------ */
typedef struct gbs_host_csr {
  int nrows, ncols, nnz;
  int *rowptr;  /* nrows + 1 */
  int *colind;  /* nnz */
  float *vals;  /* nnz */
} gbs_host_csr;

GBS_API gbs_status gbs_mtx_read(const char *path, gbs_host_csr *out);
GBS_API void gbs_host_csr_free(gbs_host_csr *csr);
/* Binary CSR cache, so a large .mtx is parsed once (the reference derives
 * .bin cache names for the same purpose, readMtx.hpp:227-244, but never
 * writes one).  Host byte order: "GBSCSR1\0", int32 nrows, ncols, nnz,
 * has_vals, rowptr, colind, [vals].  write: vals NULL stores a pattern
 * (read back as 1.0).  read: fills *out (free with gbs_host_csr_free); a
 * truncated file, a row pointer that is not monotone or a column outside
 * [0, ncols) is an error.  No counterpart in the reference's code path. */
GBS_API gbs_status gbs_csr_write_bin(const char *path, const gbs_host_csr *csr);
GBS_API gbs_status gbs_csr_read_bin(const char *path, gbs_host_csr *out);

/* Host copy of a B2SR matrix (the layout of gbs_csr2b2sr's outputs):
 * rowptr[nblockrows + 1], colind[nnzb] (tile columns ascending per block
 * row), val[nnzb * tile] tile rows of 1 (tile 4, 8), 2 (16) or 4 (32)
 * bytes, bit (tile - 1 - j) = column j of the tile. */
typedef struct gbs_host_b2sr {
  int nrows, ncols, tile, nblockrows, nnzb;
  int *rowptr;
  int *colind;
  void *val;
} gbs_host_b2sr;

/* Binary B2SR cache: "GBSB2SR1", int32 nrows, ncols, tile, nblockrows, nnzb,
 * rowptr, colind, val (host byte order), so packed tiles are kept between
 * runs.  Both directions check the arrays (pointers from 0 to nnzb, tile
 * columns ascending and inside the matrix, no bit past the last row or
 * column); read fills *out (free with gbs_host_b2sr_free).  No counterpart
 * in the reference's code path. */
GBS_API gbs_status gbs_b2sr_write_bin(const char *path, const gbs_host_b2sr *b);
GBS_API gbs_status gbs_b2sr_read_bin(const char *path, gbs_host_b2sr *out);
GBS_API void gbs_host_b2sr_free(gbs_host_b2sr *b);

/* ------------------------------------------------------------------------
 * CSR SpMM  C = A * B   (A: nrows x ncols CSR, B: ncols x F, C: nrows x F)
 *
 * Replaces the cuSPARSE call of evalCSRSpmmFloatCuSPARSE
 * (test_spmm_full.cu:212-342: cusparseSpMM, CSR, alpha = 1, beta = 0) with
 * row-major B and C instead of the column-major copies made at :215-223 and
 * :321-329.  C is overwritten (every row, including empty ones).
 *
 * Schedule: merge-path over (rows + nonzeros); each warp owns an equal share
 * and a row cut by a share boundary is finished by whichever warp arrives
 * last at it (no spin-waits), summing the pieces in a fixed order, so the
 * result is deterministic for a given device and F.
 *
 * vals may be NULL: every stored entry then counts as 1.0 (binary A).
 * B may be FP32, BF16 or FP16 (btype); accumulation and C are FP32.
 * ------------------------------------------------------------------------ */

/* Bytes of workspace gbs_csr_spmm / gbs_csr_spmm_cb need for this shape on
 * the current device (any alignment, any column block).  The workspace must
 * be zero-filled before its first use (gbs_csr_spmm_workspace_init); its
 * arrival counters are back to zero after every call, so one workspace can
 * serve calls of any shape in sequence.  It must not be used by two calls
 * that can overlap on the GPU. */
GBS_API gbs_status gbs_csr_spmm_workspace_size(int nrows, int nnz, int F,
                                       gbs_dtype btype, size_t *bytes);
GBS_API gbs_status gbs_csr_spmm_workspace_init(void *d_workspace, size_t bytes,
                                       gbs_stream_t stream);

GBS_API gbs_status gbs_csr_spmm(int nrows, int ncols, int nnz, const int *d_rowptr,
                        const int *d_colind, const float *d_vals,
                        const void *d_B, gbs_dtype btype, int F, float *d_C,
                        void *d_workspace, size_t workspace_bytes,
                        gbs_stream_t stream);

/* Same as gbs_csr_spmm with an explicit column-block width: F is processed
 * in F / col_block launches of col_block columns each (col_block must
 * divide F; 0 selects the width gbs_csr_spmm would use).  Smaller blocks
 * keep the touched slice of B resident in L2 at the cost of re-reading A. */
GBS_API gbs_status gbs_csr_spmm_cb(int nrows, int ncols, int nnz, const int *d_rowptr,
                           const int *d_colind, const float *d_vals,
                           const void *d_B, gbs_dtype btype, int F, int col_block,
                           float *d_C, void *d_workspace, size_t workspace_bytes,
                           gbs_stream_t stream);

/* Column-partitioned plan.  When B is larger than L2, splitting A by column
 * ranges into `parts` pieces (0 = choose: the smallest power of two <= 8
 * whose B slice fits in L2; 1 when B fits in L2 or rows of B are reused
 * fewer than 64 times on average) and accumulating one merge-path pass per
 * piece keeps each pass's row gathers in L2 (232,965 x 256 FP32 on GB300:
 * 6.10 ms in one pass, 5.79 ms as 2 parts, 6.33 ms as 4).  The plan copies
 * A's pattern and values into the parts (values captured at creation;
 * rebuild after changing them); with one part it only records the caller's
 * arrays, which must outlive it.  Synchronises the stream.  Workspace as
 * gbs_csr_spmm_workspace_size(nrows, nnz, F, btype). */
typedef struct gbs_csr_spmm_plan gbs_csr_spmm_plan;
GBS_API gbs_status gbs_csr_spmm_plan_create(int nrows, int ncols, int nnz,
                                    const int *d_rowptr, const int *d_colind,
                                    const float *d_vals, gbs_dtype btype, int F,
                                    int parts, gbs_stream_t stream,
                                    gbs_csr_spmm_plan **out);
GBS_API gbs_status gbs_csr_spmm_plan_parts(const gbs_csr_spmm_plan *plan, int *parts);
GBS_API gbs_status gbs_csr_spmm_planned(const gbs_csr_spmm_plan *plan, const void *d_B,
                                float *d_C, void *d_workspace,
                                size_t workspace_bytes, gbs_stream_t stream);
GBS_API gbs_status gbs_csr_spmm_plan_destroy(gbs_csr_spmm_plan *plan);

/* Degree-normalised binary A: C[r] = rowscale[r] * sum over the stored
 * entries (r, c) of colscale[c] * B[c] -- the GCN propagation
 * D^-1/2 A D^-1/2 B with the normalisation folded into the kernel instead of
 * a value array (no 4-byte value per nonzero is streamed; each nonzero reads
 * its column's scale, an array of ncols floats that stays in cache, and each
 * row is scaled once in the epilogue).  A's values are not used: every
 * stored entry counts as 1, as in the reference's binary B2SR path
 * (spmm.cu:877-956), and the scaling is that of the normalised graphs the
 * evaluation runs on.  rowscale / colscale may be NULL (= 1).  Workspace,
 * schedule and feature types as gbs_csr_spmm. */
GBS_API gbs_status gbs_csr_spmm_scaled(int nrows, int ncols, int nnz, const int *d_rowptr,
                               const int *d_colind, const float *d_rowscale,
                               const float *d_colscale, const void *d_B, gbs_dtype btype,
                               int F, float *d_C, void *d_workspace, size_t workspace_bytes,
                               gbs_stream_t stream);
/* The column-partitioned plan of gbs_csr_spmm_scaled (run with
 * gbs_csr_spmm_planned); the plan keeps copies of the scales. */
GBS_API gbs_status gbs_csr_spmm_plan_create_scaled(int nrows, int ncols, int nnz,
                                           const int *d_rowptr, const int *d_colind,
                                           const float *d_rowscale, const float *d_colscale,
                                           gbs_dtype btype, int F, int parts,
                                           gbs_stream_t stream, gbs_csr_spmm_plan **out);
/* out[r] = 1 / sqrt(deg(r)), deg = rowptr[r+1] - rowptr[r], computed in
 * FP64 on the device and rounded once to FP32 (0 for an empty row): the
 * D^-1/2 factors of a symmetric adjacency. */
GBS_API gbs_status gbs_degree_rsqrt(int nrows, const int *d_rowptr, float *d_out,
                            gbs_stream_t stream);

/* Host-buffer form for callers that hold A, B and C in host memory, as the
 * reference's evalCSRSpmmFloatCuSPARSE does (test_spmm_full.cu:212-342):
 * copies in, C = A * B, copies out, and returns when h_C is filled.  A is
 * sent in row ranges of ~nnz/16 nonzeros so the copies overlap the kernels
 * (pinned host buffers are needed for the overlap; pageable ones work,
 * serialised); the ranges' kernels alternate between `stream` and a
 * library-owned compute stream so one range's tail overlaps the next.  ctx (optional) keeps device buffers, streams and events
 * between calls; with ctx == NULL each call allocates its buffers
 * stream-ordered on `stream`.  A context serves one call at a time. */
typedef struct gbs_spmm_host_ctx gbs_spmm_host_ctx;
GBS_API gbs_status gbs_spmm_host_ctx_create(gbs_spmm_host_ctx **out);
GBS_API gbs_status gbs_spmm_host_ctx_destroy(gbs_spmm_host_ctx *ctx);
GBS_API gbs_status gbs_csr_spmm_host(gbs_spmm_host_ctx *ctx, int nrows, int ncols, int nnz,
                             const int *h_rowptr, const int *h_colind,
                             const float *h_vals, const void *h_B, gbs_dtype btype,
                             int F, float *h_C, gbs_stream_t stream);

/* One-call FP32 form with the argument meaning of the cuSPARSE generic
 * SpMM used by the reference (alpha = 1, beta = 0, FP32 everywhere).
 * Allocates and frees its workspace with stream-ordered allocation. */
GBS_API gbs_status gbs_csr_spmm_f32(int nrows, int ncols, int nnz,
                            const int *d_rowptr, const int *d_colind,
                            const float *d_vals, const float *d_B, int F,
                            float *d_C, gbs_stream_t stream);

/* ------------------------------------------------------------------------
 * Backward of C = A * B (no counterpart in the reference, which has no
 * differentiation): dB = A^T dC through a cached transpose, and
 * d(values)[e] = <dC[row(e)], B[col(e)]> (SDDMM on A's pattern).
 * ------------------------------------------------------------------------ */
typedef struct gbs_csr_transpose gbs_csr_transpose;

/* Builds A^T (ncols x nrows CSR, rows ascending inside each column, as
 * csr2csc in backend/readMtx.hpp:319-345) and perm (A^T entry i is A entry
 * perm[i]).  Allocates the handle's device arrays; synchronises the stream. */
GBS_API gbs_status gbs_csr_transpose_create(int nrows, int ncols, int nnz,
                                    const int *d_rowptr, const int *d_colind,
                                    gbs_stream_t stream, gbs_csr_transpose **out);
/* Device arrays owned by the handle (any output pointer may be NULL). */
GBS_API gbs_status gbs_csr_transpose_arrays(const gbs_csr_transpose *T,
                                    const int **d_t_rowptr, const int **d_t_colind,
                                    const int **d_perm);
/* Copies the handle's arrays into caller buffers (any may be NULL). */
GBS_API gbs_status gbs_csr_transpose_copy(const gbs_csr_transpose *T, int *d_t_rowptr,
                                  int *d_t_colind, int *d_perm, gbs_stream_t stream);
/* t_vals[i] = vals[perm[i]]: A's values in A^T order. */
GBS_API gbs_status gbs_csr_transpose_values(const gbs_csr_transpose *T,
                                    const float *d_vals, float *d_t_vals,
                                    gbs_stream_t stream);
GBS_API gbs_status gbs_csr_transpose_destroy(gbs_csr_transpose *T);
/* dB (ncols x F, FP32) = A^T dC (dC nrows x F in dtype) with the merge-path
 * SpMM; t_vals from gbs_csr_transpose_values (NULL: binary A).  Workspace
 * as gbs_csr_spmm for (ncols, nnz, F, dtype). */
GBS_API gbs_status gbs_csr_spmm_transposed(const gbs_csr_transpose *T,
                                   const float *d_t_vals, const void *d_dC,
                                   gbs_dtype dtype, int F, float *d_dB,
                                   void *d_workspace, size_t workspace_bytes,
                                   gbs_stream_t stream);
/* Fused backward of C = A H: dB = A^T dC (as gbs_csr_spmm_transposed) and
 * dvals[e] = <dC[row(e)], H[col(e)]> (as gbs_sddmm, in A's entry order) in
 * one pass over A^T's pattern, gathering each row of dC once for both.  dC,
 * H: same dtype, 16-byte aligned, F a multiple of 4 (FP32) or 8 (16-bit).
 * Workspace as gbs_csr_spmm_workspace_size(ncols, nnz, F, dtype). */
GBS_API gbs_status gbs_spmm_backward(const gbs_csr_transpose *T, const float *d_t_vals,
                             const void *d_dC, const void *d_H, gbs_dtype dtype,
                             int F, float *d_dB, float *d_dvals, void *d_workspace,
                             size_t workspace_bytes, gbs_stream_t stream);
/* Planned fused backward: A^T split by column ranges (= row ranges of A,
 * slices of dC) into `parts` pieces (0 = automatic: the fewest whose dC
 * slice fits in half of L2, 1 while dC already does) so that every pass's
 * dC gathers stay in L2; the dB part of each pass accumulates and every
 * entry's dvals comes from the one pass holding it.  The plan copies the
 * pieces of T's arrays and of t_vals (NULL: binary A) at creation and
 * synchronises the stream; with 1 part it keeps pointers to T's arrays and
 * t_vals, which must then outlive it.  Recreate it when the values change.
 * No counterpart in the reference (its repo has no backward). */
typedef struct gbs_spmm_backward_plan gbs_spmm_backward_plan;
GBS_API gbs_status gbs_spmm_backward_plan_create(const gbs_csr_transpose *T,
                                         const float *d_t_vals, gbs_dtype dtype,
                                         int F, int parts, gbs_stream_t stream,
                                         gbs_spmm_backward_plan **out);
GBS_API gbs_status gbs_spmm_backward_plan_parts(const gbs_spmm_backward_plan *plan,
                                        int *parts);
GBS_API gbs_status gbs_spmm_backward_plan_destroy(gbs_spmm_backward_plan *plan);
/* Same results as gbs_spmm_backward (dB to FP32 rounding of a different
 * summation split, dvals bitwise when the dot products' lane order is
 * unchanged); workspace as gbs_spmm_backward.  The passes write dvals in
 * their own entry order to nnz * 4 bytes of temporaries (library pool,
 * stream-ordered) and a final gather puts them in A's order. */
GBS_API gbs_status gbs_spmm_backward_planned(const gbs_spmm_backward_plan *plan,
                                     const void *d_dC, const void *d_H,
                                     float *d_dB, float *d_dvals,
                                     void *d_workspace, size_t workspace_bytes,
                                     gbs_stream_t stream);
/* out[e] = sum_k G[row(e)][k] * H[col(e)][k], FP32 accumulation; G nrows x F
 * and H ncols x F in dtype. */
GBS_API gbs_status gbs_sddmm(int nrows, int ncols, int nnz, const int *d_rowptr,
                     const int *d_colind, const void *d_G, const void *d_H,
                     gbs_dtype dtype, int F, float *d_out, gbs_stream_t stream);

/* ------------------------------------------------------------------------
 * CSR -> B2SR packing (tile = 4, 8, 16 or 32)
 *
 * B2SR layout (the reference's): block-row i covers CSR rows [i*tile,
 * (i+1)*tile); it holds one tile per distinct floor(col/tile) of those rows,
 * ascending; tile b stores row r as a tile-bit word at element tile*b + r,
 * column 0 in the most significant of the tile bits.  Element type: uint8
 * (tile 4: low nibble; tile 8), uint16 (16), uint32 (32).  Every stored CSR
 * entry sets its bit; values are ignored.
 * ------------------------------------------------------------------------ */

/* Tile counts: writes bsr_rowptr[0..mb] (mb = ceil(nrows/tile)) and returns
 * the number of tiles in *h_nnzb.  Validates the CSR (column range, columns
 * ascending within a row).  Synchronises the stream.  Replaces
 * cusparseXcsr2bsrNnz in CSR2B2SR (test_spmm_full.cu:147-151). */
GBS_API gbs_status gbs_csr2b2sr_nnzb(int nrows, int ncols, int nnz,
                             const int *d_rowptr, const int *d_colind,
                             int tile, int *d_bsr_rowptr, int *h_nnzb,
                             gbs_stream_t stream);
/* Fills bsr_colind[nnzb] and bsr_val[nnzb*tile] (bsr_rowptr from
 * gbs_csr2b2sr_nnzb on the same CSR).  Replaces the per-block-row loop of
 * csr2bsr_batch_{4,8,16,32} (csr2bsr_batch_bsrbmv.cu:207-397, :403-579,
 * :654-830, :894-1070) with one kernel. */
GBS_API gbs_status gbs_csr2b2sr(int nrows, int ncols, int nnz, const int *d_rowptr,
                        const int *d_colind, int tile, const int *d_bsr_rowptr,
                        int *d_bsr_colind, void *d_bsr_val, gbs_stream_t stream);
/* Drop-in with the argument list of csr2bsr_batch_{4,8,16,32}
 * (csr2bsr_batch_bsrbmv.cu:207): host CSR in, caller-allocated device B2SR
 * out, nblocks as computed by cusparseXcsr2bsrNnz (checked).  Synchronous,
 * legacy default stream; allocates device copies of the CSR internally. */
GBS_API gbs_status gbs_csr2bsr_batch(const int *h_csrRowPtr, const int *h_csrColInd,
                             int nrows, int ncols, int nnz, int *d_bsrRowPtr,
                             int *d_bsrColInd, void *d_bsrVal, int blocksize,
                             int nblockrows, int nblocks);

/* "Aligned" B2SR-8/16 (packUchar2AlignedUnsigned / packUshort2Aligned-
 * Unsigned, csr2bsr_batch_bsrbmv.cu:586-648, :837-888): tiles of a
 * block-row padded to a multiple of 4 (tile 8) / 2 (tile 16), padded colind
 * 0; uint32 word j of a group packs row j of its tiles, first tile in the
 * most significant byte/half.  nnzb writes new_rowptr (padded tile counts)
 * and returns the padded tile total (words = total*tile/g) synchronously. */
GBS_API gbs_status gbs_b2sr_aligned_nnzb(int tile, int nblockrows,
                                 const int *d_bsr_rowptr, int *d_new_rowptr,
                                 int *h_ntiles, gbs_stream_t stream);
GBS_API gbs_status gbs_b2sr_pack_aligned(int tile, int nblockrows,
                                 const int *d_bsr_rowptr, const int *d_bsr_colind,
                                 const void *d_bsr_val, const int *d_new_rowptr,
                                 int *d_new_colind, uint32_t *d_new_val,
                                 gbs_stream_t stream);

/* ------------------------------------------------------------------------
 * B2SR x dense (binary A):  C = A01 * B, C FP32 nrows x F (every row
 * written).  Order-free: a block-row whose tile walk is far longer than the
 * mean work per warp (a power-law hub) is cut into segments whose partial
 * sums are added into C with atomics, so such rows are exact for 0/1 and
 * +-1 (integer-valued) B and within FP32 rounding otherwise, and may differ
 * in the last bits from run to run.  Rows of other block-rows, and every
 * row of a matrix of fewer than 1024 block-rows, add tile by tile; at tile 4
 * in the order of spmm4_full_full_new2 (spmm.cu:877-956).  The reference's
 * order for every row is gbs_spmm4_full_full below.
 * ------------------------------------------------------------------------ */
GBS_API gbs_status gbs_b2sr_spmm(int tile, int nrows, int nblockrows,
                         const int *d_bsr_rowptr, const int *d_bsr_colind,
                         const void *d_bsr_val, const void *d_B, gbs_dtype btype,
                         int F, float *d_C, gbs_stream_t stream);
/* Drop-in for the launch of spmm4_full_full_new2 (test_spmm_full.cu:351-361,
 * same arguments plus a stream): C must be zero-filled by the caller, only
 * nonzero results are stored (as the reference does, spmm.cu:947-954). */
GBS_API gbs_status gbs_spmm4_full_full(const uint8_t *A, const float *B, float *C,
                               const int *rowptr, const int *colind,
                               int nblockrows, int B_cols, gbs_stream_t stream);

/* B2SR x packed-bit features -> int32 (BMV for F <= 32, BMM above; the
 * reference names these kernels but does not ship them,
 * csr2bsr_batch_bsrbmv.cu:1).  X: ceil(F/32) uint32 words per row as
 * gbs_pack_sign_rows writes them.  C[i][k] = sum_j A_ij * bit_jk, or with
 * signed_form != 0: 2*C01 - deg(i), the +-1 product. F <= 1024. */
GBS_API gbs_status gbs_b2sr_bmm(int tile, int nrows, int nblockrows,
                        const int *d_bsr_rowptr, const int *d_bsr_colind,
                        const void *d_bsr_val, const uint32_t *d_X, int F,
                        int signed_form, int32_t *d_C, gbs_stream_t stream);

/* The same product on the aligned B2SR-8/16 arrays of gbs_b2sr_pack_aligned
 * (new_rowptr, new_colind, new_val): the consumer the reference builds those
 * formats for ("bsrbmv", named at csr2bsr_batch_bsrbmv.cu:1, not shipped).
 * Each uint32 word holds one row of 4 (tile 8) / 2 (tile 16) consecutive
 * tiles; padding tiles carry no bits.  Same int32 result as gbs_b2sr_bmm on
 * the plain arrays. */
GBS_API gbs_status gbs_b2sr_bmm_aligned(int tile, int nrows, int nblockrows,
                                const int *d_new_rowptr, const int *d_new_colind,
                                const uint32_t *d_new_val, const uint32_t *d_X, int F,
                                int signed_form, int32_t *d_C, gbs_stream_t stream);

/* Dense sign packing, bit = (x >= 0), first column in bit 31, elements
 * outside the matrix read as -1 (bit 0).
 * rows : ToBit32RowDenseSign (spmm.cu:75-91), out[r*ceil(F/32) + w].
 * colud: ToBit32ColUd (spmm.cu:93-111), out[w*Hp + r], Hp = 32*ceil(H/32),
 *        the word-major layout the binary GEMM reads. */
GBS_API gbs_status gbs_pack_sign_rows(const float *d_X, int n, int F, uint32_t *d_out,
                              gbs_stream_t stream);
GBS_API gbs_status gbs_pack_sign_colud(const float *d_A, int H, int W, uint32_t *d_out,
                               gbs_stream_t stream);

/* ------------------------------------------------------------------------
 * Dense binary matmul (backend/mm.cu).  A: Kw x M and B: Kw x N uint32
 * words in the word-major layout of ToBit32ColUd (spmm.cu:93-111), word kw
 * of row r = K-bits 32kw..32kw+31.  M and N multiples of 4, A and B 16-byte
 * aligned.
 * ------------------------------------------------------------------------ */
/* C (M x N int32, row-major): mode 0 = sum popc(a ^ b), 1 = sum popc(a & b),
 * 2 = 32*Kw - 2*xor (the +-1 dot product).  algo 0 = default (= 4, the
 * fastest on GB300), 1 = CUDA-core __popc, 2 = tensor-core mma.sync .b1
 * AND-popc (XOR from row popcounts), 3 = tcgen05 tensor cores on the bits
 * expanded to FP8 {0, 1}, one CTA per 128 x 256 tile, 4 = the same MMAs in
 * a persistent warp-specialised kernel (one CTA per SM, two TMEM
 * accumulators so a tile's epilogue overlaps the next tile's MMAs).  3 and
 * 4 are exact and allocate (M+N)*K bytes of temporaries, stream-ordered.
 * 8192^3 XOR on GB300: 0.39 / 0.60 / 3.59 / 7.51 ms for 4 / 3 / 1 / 2. */
GBS_API gbs_status gbs_bmm_b1(const uint32_t *d_A, const uint32_t *d_B, int M, int N,
                      int Kw, int mode, int algo, int32_t *d_C, gbs_stream_t stream);
/* Number of bounded mbarrier waits that ran out in algo-3/4 launches of this
 * process (0 in normal operation; each timeout also skips that tile's
 * stores).  Synchronises with the device. */
GBS_API gbs_status gbs_bmm_tc_timeouts(int *count);
/* Drop-in for BMM32_Arow_Brow<float> (mm.cu:17-53) and BMM32_MT_M_S
 * (:59-75): C[r*B_width + c] = 32*A_width - 2*xor as float. */
GBS_API gbs_status gbs_bmm32_arow_brow(const uint32_t *d_A, const uint32_t *d_B, float *d_C,
                               int A_height, int A_width, int B_width,
                               gbs_stream_t stream);
/* Drop-ins for BMM32_BIN (mm.cu:79-105) and BMM32S_BIN (:108-125): bit =
 * (n - 2*xor >= 0) with n the number of K bits, 32 output columns per word,
 * first column in bit 31, stored at C[by*m + r] (BIN) or
 * C[(r/32)*k*32 + by*32 + r%32] (S_BIN).  m, k multiples of 32.  The
 * persistent tcgen05 GEMM thresholds its counts in the epilogue and writes
 * only the words (no count matrix); temporaries as gbs_bmm_b1 algo 4. */
GBS_API gbs_status gbs_bmm32_bin(const uint32_t *d_A, const uint32_t *d_B, uint32_t *d_C,
                         int m, int n, int k, gbs_stream_t stream);
GBS_API gbs_status gbs_bmm32s_bin(const uint32_t *d_A, const uint32_t *d_B, uint32_t *d_C,
                          int m, int n, int k, gbs_stream_t stream);
/* The sign-word product of gbs_bmm32_bin (layout 0) / gbs_bmm32s_bin
 * (layout 1) with the algorithm chosen: algo 0 = thresholded in the tcgen05
 * epilogue (what the drop-ins run), 1 = int32 XOR counts into an m x k
 * temporary, then a separate sign-word pass.  Same words either way.  No
 * counterpart in the reference beyond the two kernels named above. */
GBS_API gbs_status gbs_bmm_bin(const uint32_t *d_A, const uint32_t *d_B, uint32_t *d_C, int m,
                       int n, int k, int layout, int algo, gbs_stream_t stream);

/* CSR SpMM that allocates no device memory.  No counterpart in the
 * reference: it exists for callers that may not allocate while they run (a
 * framework that reserves its device memory up front in its own pool, a
 * serving loop that bans cudaMalloc/cudaFree because they can synchronise
 * the device).  Same arguments and result as gbs_csr_spmm minus the
 * workspace: the kernel's scratch is a fixed 8 MiB array compiled into the
 * library, held on every GPU that loads the library until the process exits.
 * The warp count is reduced until the scratch fits, so rows wider than about
 * 128 FP32 columns run with fewer warps than a full wave (slower, same
 * result); widths gbs_csr_spmm does not support fail with
 * GBS_ERR_UNSUPPORTED as there.  The device address of the array is looked
 * up on every call; the first call in a CUDA context loads the library's
 * device code, so make that first call before any stream capture starts.
 * All calls share the array: calls that can overlap on the GPU race and
 * must be serialised by the caller. */
GBS_API gbs_status gbs_csr_spmm_noalloc(int nrows, int ncols, int nnz,
                                const int *d_rowptr, const int *d_colind,
                                const float *d_vals, const void *d_B,
                                gbs_dtype btype, int F, float *d_C,
                                gbs_stream_t stream);

#ifdef __cplusplus
}
#endif

#endif /* GBSPMM_H_ */
