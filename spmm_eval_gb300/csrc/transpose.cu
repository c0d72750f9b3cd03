// Cached CSR transpose for the backward pass (dB = A^T dC) and the
// value-gradient bookkeeping.
//
// Built once per sparsity pattern: column histogram -> t_rowptr, row ids of
// the nonzeros, and a stable radix sort of the nonzero indices by column
// (CUB), so inside every column of A^T the rows come out ascending, as
// csr2csc does in the reference (backend/readMtx.hpp:319-345 through
// coo2csr's stable fill).  perm[i] is the index in A of entry i of A^T, so
// A^T's values are vals[perm[i]] for any value array on A's pattern.
#include "common.cuh"
#include "csr_spmm.cuh"
#include "util.cuh"

#include "transpose.cuh"

namespace gbs {

__global__ void k_col_hist(const int *__restrict__ colind, int nnz, int ncols, int *__restrict__ counts,
                           int *__restrict__ err) {
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < nnz;
       e += (long long)gridDim.x * blockDim.x) {
    const int c = colind[e];
    if (c < 0 || c >= ncols) {
      atomicOr(err, 1);
      continue;
    }
    atomicAdd(counts + c, 1);
  }
}

__global__ void k_row_ids(const int *__restrict__ rowptr, int nrows, int *__restrict__ rowid) {
  const long long r = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (r >= nrows) return;
  const int b = rowptr[r], e = rowptr[r + 1];
  for (int i = b + lane; i < e; i += 32) rowid[i] = (int)r;
}

__global__ void k_iota(int *__restrict__ x, int n) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    x[i] = (int)i;
}

template <typename T>
__global__ void k_gather(const T *__restrict__ src, const int *__restrict__ idx, int n, T *__restrict__ dst) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    dst[i] = src[idx[i]];
}

static int grid_for(long long n) {
  long long b = (n + 255) / 256;
  if (b > 152 * 64) b = 152 * 64;
  return (int)(b < 1 ? 1 : b);
}

}  // namespace gbs

using namespace gbs;

extern "C" gbs_status gbs_csr_transpose_create(int nrows, int ncols, int nnz, const int *rowptr,
                                               const int *colind, gbs_stream_t stream,
                                               gbs_csr_transpose **out) {
  clear_error();
  GBS_REQUIRE(out != nullptr, "csr transpose: null output handle");
  *out = nullptr;
  GBS_REQUIRE(nrows >= 0 && ncols >= 0 && nnz >= 0, "csr transpose: negative size");
  GBS_REQUIRE(nrows == 0 || rowptr, "csr transpose: null rowptr");
  GBS_REQUIRE(nnz == 0 || colind, "csr transpose: null colind");
  cudaStream_t s = (cudaStream_t)stream;
  gbs_csr_transpose *T = new gbs_csr_transpose{nrows, ncols, nnz, 0, nullptr, nullptr, nullptr};
  auto cleanup = [&](gbs_status st) {
    if (T->t_rowptr) cudaFree(T->t_rowptr);
    if (T->t_colind) cudaFree(T->t_colind);
    if (T->perm) cudaFree(T->perm);
    delete T;
    return st;
  };
  cudaGetDevice(&T->device);
  cudaError_t e;
  if ((e = cudaMalloc(&T->t_rowptr, sizeof(int) * ((size_t)ncols + 1))) != cudaSuccess)
    return cleanup(cuda_fail(e, "cudaMalloc"));
  if ((e = cudaMalloc(&T->t_colind, sizeof(int) * (size_t)(nnz > 0 ? nnz : 1))) != cudaSuccess)
    return cleanup(cuda_fail(e, "cudaMalloc"));
  if ((e = cudaMalloc(&T->perm, sizeof(int) * (size_t)(nnz > 0 ? nnz : 1))) != cudaSuccess)
    return cleanup(cuda_fail(e, "cudaMalloc"));

  gbs_status st = GBS_OK;
  {
    DevBuf counts, err, rowid, iota, keys;
    if ((st = counts.alloc(sizeof(int) * ((size_t)ncols + 1), s)) != GBS_OK) return cleanup(st);
    if ((st = err.alloc(sizeof(int), s)) != GBS_OK) return cleanup(st);
    if ((st = rowid.alloc(sizeof(int) * (size_t)nnz, s)) != GBS_OK) return cleanup(st);
    if ((st = iota.alloc(sizeof(int) * (size_t)nnz, s)) != GBS_OK) return cleanup(st);
    if ((st = keys.alloc(sizeof(int) * (size_t)nnz, s)) != GBS_OK) return cleanup(st);
    cudaMemsetAsync(counts.p, 0, sizeof(int) * ((size_t)ncols + 1), s);
    cudaMemsetAsync(err.p, 0, sizeof(int), s);
    if (nnz > 0) {
      k_col_hist<<<grid_for(nnz), 256, 0, s>>>(colind, nnz, ncols, counts.as<int>(), err.as<int>());
      k_row_ids<<<(int)(((long long)nrows * 32 + 255) / 256), 256, 0, s>>>(rowptr, nrows, rowid.as<int>());
      k_iota<<<grid_for(nnz), 256, 0, s>>>(iota.as<int>(), nnz);
      if ((st = check_launch("transpose kernels")) != GBS_OK) return cleanup(st);
    }
    if ((st = exclusive_scan_i32(counts.as<int>(), T->t_rowptr, ncols + 1, s)) != GBS_OK) return cleanup(st);
    if (nnz > 0) {
      if ((st = stable_sort_pairs_i32(colind, keys.as<int>(), iota.as<int>(), T->perm, nnz,
                                      bits_for(ncols > 0 ? ncols - 1 : 0), s)) != GBS_OK)
        return cleanup(st);
      k_gather<int><<<grid_for(nnz), 256, 0, s>>>(rowid.as<int>(), T->perm, nnz, T->t_colind);
      if ((st = check_launch("k_gather")) != GBS_OK) return cleanup(st);
    }
    int h_err = 0;
    if ((e = cudaMemcpyAsync(&h_err, err.p, sizeof(int), cudaMemcpyDeviceToHost, s)) != cudaSuccess)
      return cleanup(cuda_fail(e, "cudaMemcpyAsync"));
    if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return cleanup(cuda_fail(e, "cudaStreamSynchronize"));
    if (h_err) return cleanup(fail(GBS_ERR_INVALID_ARG, "csr transpose: column index out of range"));
  }
  *out = T;
  return GBS_OK;
}

extern "C" gbs_status gbs_csr_transpose_arrays(const gbs_csr_transpose *T, const int **t_rowptr,
                                               const int **t_colind, const int **perm) {
  clear_error();
  GBS_REQUIRE(T != nullptr, "csr transpose: null handle");
  if (t_rowptr) *t_rowptr = T->t_rowptr;
  if (t_colind) *t_colind = T->t_colind;
  if (perm) *perm = T->perm;
  return GBS_OK;
}

extern "C" gbs_status gbs_csr_transpose_copy(const gbs_csr_transpose *T, int *t_rowptr, int *t_colind,
                                             int *perm, gbs_stream_t stream) {
  clear_error();
  GBS_REQUIRE(T != nullptr, "csr transpose: null handle");
  cudaStream_t s = (cudaStream_t)stream;
  if (t_rowptr)
    GBS_CUDA_TRY(cudaMemcpyAsync(t_rowptr, T->t_rowptr, sizeof(int) * ((size_t)T->ncols + 1),
                                 cudaMemcpyDeviceToDevice, s));
  if (T->nnz > 0 && t_colind)
    GBS_CUDA_TRY(cudaMemcpyAsync(t_colind, T->t_colind, sizeof(int) * (size_t)T->nnz, cudaMemcpyDeviceToDevice, s));
  if (T->nnz > 0 && perm)
    GBS_CUDA_TRY(cudaMemcpyAsync(perm, T->perm, sizeof(int) * (size_t)T->nnz, cudaMemcpyDeviceToDevice, s));
  return GBS_OK;
}

extern "C" gbs_status gbs_csr_transpose_values(const gbs_csr_transpose *T, const float *vals, float *t_vals,
                                               gbs_stream_t stream) {
  clear_error();
  GBS_REQUIRE(T != nullptr, "csr transpose: null handle");
  if (T->nnz == 0) return GBS_OK;
  GBS_REQUIRE(vals && t_vals, "csr transpose: null values");
  k_gather<float><<<grid_for(T->nnz), 256, 0, (cudaStream_t)stream>>>(vals, T->perm, T->nnz, t_vals);
  return check_launch("k_gather");
}

extern "C" gbs_status gbs_csr_transpose_destroy(gbs_csr_transpose *T) {
  clear_error();
  if (!T) return GBS_OK;
  int cur = 0;
  cudaGetDevice(&cur);
  cudaSetDevice(T->device);
  cudaFree(T->t_rowptr);
  cudaFree(T->t_colind);
  cudaFree(T->perm);
  cudaSetDevice(cur);
  delete T;
  return GBS_OK;
}

extern "C" gbs_status gbs_csr_spmm_transposed(const gbs_csr_transpose *T, const float *t_vals, const void *dC,
                                              gbs_dtype dtype, int F, float *dB, void *ws, size_t ws_bytes,
                                              gbs_stream_t stream) {
  clear_error();
  GBS_REQUIRE(T != nullptr, "spmm transposed: null handle");
  return gbs_csr_spmm(T->ncols, T->nrows, T->nnz, T->t_rowptr, T->t_colind, t_vals, dC, dtype, F, dB, ws,
                      ws_bytes, stream);
}
