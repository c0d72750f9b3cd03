// Column-partitioned CSR SpMM plan.
//
// When the feature matrix B is larger than L2 (FP32 B of the 232,965-node
// graph at F = 256 is 238 MB against 129 MB of L2), a quarter of the row
// gathers miss L2.  Splitting A by column ranges into K parts whose slices of
// B fit in half of L2, and running the merge-path SpMM once per part with the
// later parts accumulating into C (C += A_p B_p), keeps every pass's gathers
// in L2 at the price of reading and writing C K-1 more times.  Measured on
// GB300 for that graph: 8.0 ms in one pass, 6.6 ms as 4 parts.
//
// The plan copies A into the K parts once (rows in the same order, each
// part's columns still ascending); it is reused for any B of the planned
// width and type.  With K = 1 the plan only records the caller's arrays,
// which must then outlive it.
#include <vector>

#include "common.cuh"
#include "csr_spmm.cuh"
#include "util.cuh"

struct gbs_csr_spmm_plan {
  int nrows, ncols, nnz, F, K;
  gbs_dtype btype;
  int device;
  bool owned;
  std::vector<int *> rowptr, colind;
  std::vector<float *> vals;
  std::vector<int> part_nnz;
};

namespace gbs {

// Per row: the first entry of each column range (columns ascending).
__global__ void k_part_bounds(const int *__restrict__ rowptr, const int *__restrict__ colind, int nrows, int K,
                              int S, int *__restrict__ len) {
  const long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (r > nrows) return;
  if (r == nrows) {
    for (int p = 0; p < K; ++p) len[(size_t)p * (nrows + 1) + nrows] = 0;
    return;
  }
  const int rb = rowptr[r], re = rowptr[r + 1];
  int prev = rb;
  for (int p = 0; p < K; ++p) {
    int b;
    if (p == K - 1) {
      b = re;
    } else {
      const long long lim = (long long)(p + 1) * S;
      int lo = prev, hi = re;  // first index with colind >= lim
      while (lo < hi) {
        const int mid = lo + (hi - lo) / 2;
        if (colind[mid] < lim) lo = mid + 1;
        else hi = mid;
      }
      b = lo;
    }
    len[(size_t)p * (nrows + 1) + r] = b - prev;
    prev = b;
  }
}

// Warp per row: copy each column range to its part.
__global__ void k_part_copy(const int *__restrict__ rowptr, const int *__restrict__ colind,
                            const float *__restrict__ vals, int nrows, int K, int *const *__restrict__ prp,
                            int *const *__restrict__ pci, float *const *__restrict__ pv) {
  const long long r = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (r >= nrows) return;
  int src = rowptr[r];
  for (int p = 0; p < K; ++p) {
    const int d0 = prp[p][r], n = prp[p][r + 1] - d0;
    for (int i = lane; i < n; i += 32) {
      pci[p][d0 + i] = colind[src + i];
      if (vals) pv[p][d0 + i] = vals[src + i];
    }
    src += n;
  }
}

}  // namespace gbs

using namespace gbs;

static void free_plan(gbs_csr_spmm_plan *P) {
  if (!P) return;
  if (P->owned) {
    int cur = 0;
    cudaGetDevice(&cur);
    cudaSetDevice(P->device);
    for (auto p : P->rowptr) cudaFree(p);
    for (auto p : P->colind) cudaFree(p);
    for (auto p : P->vals)
      if (p) cudaFree(p);
    cudaSetDevice(cur);
  }
  delete P;
}

extern "C" gbs_status gbs_csr_spmm_plan_create(int nrows, int ncols, int nnz, const int *rowptr, const int *colind,
                                               const float *vals, gbs_dtype btype, int F, int parts,
                                               gbs_stream_t stream, gbs_csr_spmm_plan **out) {
  clear_error();
  GBS_REQUIRE(out != nullptr, "spmm plan: null output");
  *out = nullptr;
  GBS_REQUIRE(btype == GBS_F32 || btype == GBS_BF16 || btype == GBS_F16, "spmm plan: bad dtype");
  GBS_TRY(spmm_check_args(nrows, ncols, nnz, rowptr, colind, (const void *)1, F, (const float *)1));
  GBS_REQUIRE(parts >= 0 && parts <= 64, "spmm plan: parts must be 0 (auto) .. 64");
  cudaStream_t s = (cudaStream_t)stream;
  int K = parts;
  if (K == 0) {
    DeviceInfo di;
    GBS_TRY(device_info(&di));
    const double bbytes = (double)ncols * F * (btype == GBS_F32 ? 4.0 : 2.0);
    K = 1;
    if (bbytes > (double)di.l2_bytes && (double)nnz >= 8.0 * ncols) {
      while (K < 8 && bbytes / K > 0.5 * (double)di.l2_bytes) K *= 2;
    }
  }
  if (K > ncols && ncols > 0) K = ncols;
  if (K < 1) K = 1;
  auto *P = new gbs_csr_spmm_plan();
  P->nrows = nrows;
  P->ncols = ncols;
  P->nnz = nnz;
  P->F = F;
  P->K = K;
  P->btype = btype;
  cudaGetDevice(&P->device);
  if (K == 1) {
    P->owned = false;
    P->rowptr.push_back(const_cast<int *>(rowptr));
    P->colind.push_back(const_cast<int *>(colind));
    P->vals.push_back(const_cast<float *>(vals));
    P->part_nnz.push_back(nnz);
    *out = P;
    return GBS_OK;
  }
  P->owned = true;
  const int S = (ncols + K - 1) / K;
  gbs_status st = GBS_OK;
  {
    DevBuf len, tables;
    if ((st = len.alloc(sizeof(int) * (size_t)K * (nrows + 1), s)) != GBS_OK) {
      free_plan(P);
      return st;
    }
    k_part_bounds<<<(nrows + 1 + 255) / 256, 256, 0, s>>>(rowptr, colind, nrows, K, S, len.as<int>());
    if ((st = check_launch("k_part_bounds")) != GBS_OK) {
      free_plan(P);
      return st;
    }
    std::vector<int> totals(K);
    for (int p = 0; p < K; ++p) {
      int *rp = nullptr;
      cudaError_t e = cudaMalloc(&rp, sizeof(int) * ((size_t)nrows + 1));
      if (e != cudaSuccess) {
        free_plan(P);
        return cuda_fail(e, "cudaMalloc");
      }
      P->rowptr.push_back(rp);
      if ((st = exclusive_scan_i32(len.as<int>() + (size_t)p * (nrows + 1), rp, nrows + 1, s)) != GBS_OK) {
        free_plan(P);
        return st;
      }
      cudaMemcpyAsync(&totals[p], rp + nrows, sizeof(int), cudaMemcpyDeviceToHost, s);
    }
    cudaError_t e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
      free_plan(P);
      return cuda_fail(e, "cudaStreamSynchronize");
    }
    for (int p = 0; p < K; ++p) {
      int *ci = nullptr;
      float *v = nullptr;
      if ((e = cudaMalloc(&ci, sizeof(int) * (size_t)(totals[p] > 0 ? totals[p] : 1))) != cudaSuccess) {
        free_plan(P);
        return cuda_fail(e, "cudaMalloc");
      }
      P->colind.push_back(ci);
      if (vals) {
        if ((e = cudaMalloc(&v, sizeof(float) * (size_t)(totals[p] > 0 ? totals[p] : 1))) != cudaSuccess) {
          free_plan(P);
          return cuda_fail(e, "cudaMalloc");
        }
      }
      P->vals.push_back(v);
      P->part_nnz.push_back(totals[p]);
    }
    if ((st = tables.alloc(sizeof(void *) * 3 * (size_t)K, s)) != GBS_OK) {
      free_plan(P);
      return st;
    }
    std::vector<void *> host(3 * (size_t)K);
    for (int p = 0; p < K; ++p) {
      host[p] = P->rowptr[p];
      host[K + p] = P->colind[p];
      host[2 * K + p] = P->vals[p];
    }
    cudaMemcpyAsync(tables.p, host.data(), sizeof(void *) * host.size(), cudaMemcpyHostToDevice, s);
    void **tab = tables.as<void *>();
    k_part_copy<<<(int)(((long long)nrows * 32 + 255) / 256), 256, 0, s>>>(
        rowptr, colind, vals, nrows, K, reinterpret_cast<int *const *>(tab), reinterpret_cast<int *const *>(tab + K),
        reinterpret_cast<float *const *>(tab + 2 * K));
    if ((st = check_launch("k_part_copy")) != GBS_OK) {
      free_plan(P);
      return st;
    }
    if ((e = cudaStreamSynchronize(s)) != cudaSuccess) {
      free_plan(P);
      return cuda_fail(e, "cudaStreamSynchronize");
    }
  }
  *out = P;
  return GBS_OK;
}

extern "C" gbs_status gbs_csr_spmm_plan_parts(const gbs_csr_spmm_plan *P, int *parts) {
  clear_error();
  GBS_REQUIRE(P && parts, "spmm plan: null argument");
  *parts = P->K;
  return GBS_OK;
}

extern "C" gbs_status gbs_csr_spmm_plan_destroy(gbs_csr_spmm_plan *P) {
  clear_error();
  free_plan(P);
  return GBS_OK;
}

extern "C" gbs_status gbs_csr_spmm_planned(const gbs_csr_spmm_plan *P, const void *B, float *C, void *ws,
                                           size_t ws_bytes, gbs_stream_t stream) {
  clear_error();
  GBS_REQUIRE(P != nullptr, "spmm planned: null plan");
  if (P->nrows == 0) return GBS_OK;
  GBS_REQUIRE(B && C, "spmm planned: null B or C");
  const int dt = P->btype == GBS_F32 ? 0 : (P->btype == GBS_BF16 ? 1 : 2);
  for (int p = 0; p < P->K; ++p) {
    SpmmPlan sp;
    GBS_TRY(spmm_plan(dt, P->nrows, P->ncols, P->part_nnz[p], P->F, B, C, 0, &sp));
    GBS_REQUIRE(ws != nullptr && ws_bytes >= sp.ws_bytes, "spmm planned: workspace missing or too small");
    GBS_TRY(spmm_run(sp, P->nrows, P->part_nnz[p], P->rowptr[p], P->colind[p], P->vals[p], B, P->F, C, ws,
                     (cudaStream_t)stream, 0, p > 0 ? 1 : 0));
  }
  return GBS_OK;
}
