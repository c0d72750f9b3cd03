// Column-partitioned CSR SpMM plan.
//
// When the feature matrix B is larger than L2 (FP32 B of the 232,965-node
// graph at F = 256 is 238 MB against 129 MB of L2 split over two dies), many
// row gathers miss L2.  Splitting A by column ranges into K parts and running
// the merge-path SpMM once per part with the later parts accumulating into C
// (C += A_p B_p) keeps more of every pass's gathers in L2 at the price of
// reading and writing C K-1 more times.  Measured on GB300 for that graph
// with the current kernels: FP32 6.10 ms in one pass, 5.79 ms as 2 parts,
// 6.33 ms as 4; BF16 (B = 119 MB, inside L2) 3.31 ms in one pass, 3.34 ms as
// 2 parts, 3.65 ms as 4.
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
  int nrows, ncols, nnz, F;
  gbs_dtype btype;
  gbs::ColumnParts parts;
  // degree-normalised binary A: copies of the row and column scales (null
  // for a plan with stored values)
  float *rowscale = nullptr, *colscale = nullptr;
  bool scaled = false;
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
                            const float *__restrict__ vals, const int *__restrict__ extra, int nrows, int K,
                            int *const *__restrict__ prp, int *const *__restrict__ pci, float *const *__restrict__ pv,
                            int *const *__restrict__ pex) {
  const long long r = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (r >= nrows) return;
  int src = rowptr[r];
  for (int p = 0; p < K; ++p) {
    const int d0 = prp[p][r], n = prp[p][r + 1] - d0;
    for (int i = lane; i < n; i += 32) {
      pci[p][d0 + i] = colind[src + i];
      if (vals) pv[p][d0 + i] = vals[src + i];
      if (extra) pex[p][d0 + i] = extra[src + i];
    }
    src += n;
  }
}

void ColumnParts::release() {
  if (owned) {
    int cur = 0;
    cudaGetDevice(&cur);
    cudaSetDevice(device);
    for (auto p : rowptr) cudaFree(p);
    for (auto p : colind) cudaFree(p);
    for (auto p : vals)
      if (p) cudaFree(p);
    for (auto p : extra)
      if (p) cudaFree(p);
    cudaSetDevice(cur);
  }
  rowptr.clear();
  colind.clear();
  vals.clear();
  extra.clear();
  nnz.clear();
  owned = false;
  K = 0;
}

// Column parts pay one pass over A's rows (and one read-modify-write of C)
// each, so they need rows of B gathered many times over: a mean of 64 or
// more nonzeros per column.  (The 89,250-node flickr-shaped graph, ~10 per
// column, ran its F = 256 FP32 product in 0.358 ms as 2 parts against
// 0.109 ms in one pass; the 114.8M-edge graph, ~492 per column, gains.)
constexpr double kMinReuseForParts = 64.0;

// Forward plans: once B is larger than L2, at least 2 parts, then the
// smallest power of two whose slice fits in L2.
gbs_status auto_parts_forward(double bbytes, long long nnz, int ncols, int *K) {
  DeviceInfo di;
  GBS_TRY(device_info(&di));
  const double l2 = (double)di.l2_bytes;
  int k = 1;
  if (bbytes > l2 && (double)nnz >= kMinReuseForParts * ncols) {
    k = 2;
    while (k < 8 && bbytes / k > l2) k *= 2;
  }
  *K = k;
  return GBS_OK;
}

// Backward plans (row ranges of A): the smallest power of two whose dC slice
// fits in half of L2.
gbs_status auto_parts(double bbytes, long long nnz, int ncols, int *K) {
  DeviceInfo di;
  GBS_TRY(device_info(&di));
  const double half_l2 = 0.5 * (double)di.l2_bytes;
  int k = 1;
  if (bbytes > half_l2 && (double)nnz >= kMinReuseForParts * ncols)
    while (k < 8 && bbytes / k > half_l2) k *= 2;
  *K = k;
  return GBS_OK;
}

namespace {
template <typename T>
gbs_status dev_alloc(T **p, size_t count) {
  cudaError_t e = cudaMalloc(p, sizeof(T) * (count > 0 ? count : 1));
  if (e != cudaSuccess) {
    *p = nullptr;
    return cuda_fail(e, "cudaMalloc");
  }
  return GBS_OK;
}

gbs_status partition_impl(int nrows, int ncols, int nnz, const int *rowptr, const int *colind, const float *vals,
                          const int *extra, int K, cudaStream_t s, ColumnParts *P) {
  const int S = (ncols + K - 1) / K;
  DevBuf len, tables;
  GBS_TRY(len.alloc(sizeof(int) * (size_t)K * (nrows + 1), s));
  k_part_bounds<<<(nrows + 1 + 255) / 256, 256, 0, s>>>(rowptr, colind, nrows, K, S, len.as<int>());
  GBS_TRY(check_launch("k_part_bounds"));
  std::vector<int> totals(K);
  for (int p = 0; p < K; ++p) {
    int *rp = nullptr;
    GBS_TRY(dev_alloc(&rp, (size_t)nrows + 1));
    P->rowptr.push_back(rp);
    GBS_TRY(exclusive_scan_i32(len.as<int>() + (size_t)p * (nrows + 1), rp, nrows + 1, s));
    GBS_CUDA_TRY(cudaMemcpyAsync(&totals[p], rp + nrows, sizeof(int), cudaMemcpyDeviceToHost, s));
  }
  GBS_CUDA_TRY(cudaStreamSynchronize(s));
  for (int p = 0; p < K; ++p) {
    int *ci = nullptr, *ex = nullptr;
    float *v = nullptr;
    GBS_TRY(dev_alloc(&ci, (size_t)totals[p]));
    P->colind.push_back(ci);
    if (vals) GBS_TRY(dev_alloc(&v, (size_t)totals[p]));
    P->vals.push_back(v);
    if (extra) GBS_TRY(dev_alloc(&ex, (size_t)totals[p]));
    P->extra.push_back(ex);
    P->nnz.push_back(totals[p]);
  }
  GBS_TRY(tables.alloc(sizeof(void *) * 4 * (size_t)K, s));
  std::vector<void *> host(4 * (size_t)K);
  for (int p = 0; p < K; ++p) {
    host[p] = P->rowptr[p];
    host[K + p] = P->colind[p];
    host[2 * K + p] = P->vals[p];
    host[3 * K + p] = P->extra[p];
  }
  GBS_CUDA_TRY(cudaMemcpyAsync(tables.p, host.data(), sizeof(void *) * host.size(), cudaMemcpyHostToDevice, s));
  void **tab = tables.as<void *>();
  k_part_copy<<<(int)(((long long)nrows * 32 + 255) / 256), 256, 0, s>>>(
      rowptr, colind, vals, extra, nrows, K, reinterpret_cast<int *const *>(tab),
      reinterpret_cast<int *const *>(tab + K), reinterpret_cast<float *const *>(tab + 2 * K),
      reinterpret_cast<int *const *>(tab + 3 * K));
  GBS_TRY(check_launch("k_part_copy"));
  // the host table is read by the copy above: wait before it goes out of scope
  GBS_CUDA_TRY(cudaStreamSynchronize(s));
  return GBS_OK;
}
}  // namespace

gbs_status partition_columns(int nrows, int ncols, int nnz, const int *rowptr, const int *colind,
                             const float *vals, const int *extra, int K, cudaStream_t s, ColumnParts *P) {
  P->release();
  if (K > ncols && ncols > 0) K = ncols;
  if (K < 1) K = 1;
  GBS_CUDA_TRY(cudaGetDevice(&P->device));
  P->K = K;
  if (K == 1) {
    P->owned = false;
    P->rowptr.push_back(const_cast<int *>(rowptr));
    P->colind.push_back(const_cast<int *>(colind));
    P->vals.push_back(const_cast<float *>(vals));
    P->extra.push_back(const_cast<int *>(extra));
    P->nnz.push_back(nnz);
    return GBS_OK;
  }
  P->owned = true;
  gbs_status st = partition_impl(nrows, ncols, nnz, rowptr, colind, vals, extra, K, s, P);
  if (st != GBS_OK) P->release();
  return st;
}

}  // namespace gbs

using namespace gbs;

static gbs_status plan_create(int nrows, int ncols, int nnz, const int *rowptr, const int *colind,
                              const float *vals, const float *rowscale, const float *colscale,
                              gbs_dtype btype, int F, int parts, gbs_stream_t stream,
                              gbs_csr_spmm_plan **out);

static void plan_free(gbs_csr_spmm_plan *P) {
  if (!P) return;
  P->parts.release();
  if (P->rowscale) cudaFree(P->rowscale);
  if (P->colscale) cudaFree(P->colscale);
  delete P;
}

extern "C" gbs_status gbs_csr_spmm_plan_create(int nrows, int ncols, int nnz, const int *rowptr, const int *colind,
                                               const float *vals, gbs_dtype btype, int F, int parts,
                                               gbs_stream_t stream, gbs_csr_spmm_plan **out) {
  clear_error();
  return plan_create(nrows, ncols, nnz, rowptr, colind, vals, nullptr, nullptr, btype, F, parts, stream, out);
}

extern "C" gbs_status gbs_csr_spmm_plan_create_scaled(int nrows, int ncols, int nnz, const int *rowptr,
                                                      const int *colind, const float *rowscale,
                                                      const float *colscale, gbs_dtype btype, int F,
                                                      int parts, gbs_stream_t stream, gbs_csr_spmm_plan **out) {
  clear_error();
  return plan_create(nrows, ncols, nnz, rowptr, colind, nullptr, rowscale, colscale, btype, F, parts, stream, out);
}

static gbs_status plan_create(int nrows, int ncols, int nnz, const int *rowptr, const int *colind,
                              const float *vals, const float *rowscale, const float *colscale,
                              gbs_dtype btype, int F, int parts, gbs_stream_t stream,
                              gbs_csr_spmm_plan **out) {
  GBS_REQUIRE(out != nullptr, "spmm plan: null output");
  *out = nullptr;
  GBS_REQUIRE(btype == GBS_F32 || btype == GBS_BF16 || btype == GBS_F16, "spmm plan: bad dtype");
  GBS_TRY(spmm_check_args(nrows, ncols, nnz, rowptr, colind, (const void *)1, F, (const float *)1));
  GBS_REQUIRE(parts >= 0 && parts <= 64, "spmm plan: parts must be 0 (auto) .. 64");
  int K = parts;
  if (K == 0) GBS_TRY(auto_parts_forward((double)ncols * F * (btype == GBS_F32 ? 4.0 : 2.0), nnz, ncols, &K));
  auto *P = new gbs_csr_spmm_plan();
  P->nrows = nrows;
  P->ncols = ncols;
  P->nnz = nnz;
  P->F = F;
  P->btype = btype;
  P->scaled = rowscale != nullptr || colscale != nullptr;
  gbs_status st = partition_columns(nrows, ncols, nnz, rowptr, colind, vals, nullptr, K, (cudaStream_t)stream,
                                    &P->parts);
  // the scales are copied, so the caller's arrays need not outlive the plan
  auto copy_scale = [&](const float *src, int count, float **dst) -> gbs_status {
    if (!src || count == 0) return GBS_OK;
    GBS_CUDA_TRY(cudaMalloc(dst, sizeof(float) * (size_t)count));
    GBS_CUDA_TRY(cudaMemcpyAsync(*dst, src, sizeof(float) * (size_t)count, cudaMemcpyDeviceToDevice,
                                 (cudaStream_t)stream));
    return GBS_OK;
  };
  if (st == GBS_OK) st = copy_scale(rowscale, nrows, &P->rowscale);
  if (st == GBS_OK) st = copy_scale(colscale, ncols, &P->colscale);
  if (st == GBS_OK && (P->rowscale || P->colscale)) {
    cudaError_t e = cudaStreamSynchronize((cudaStream_t)stream);
    if (e != cudaSuccess) st = cuda_fail(e, "spmm plan: scale copies");
  }
  if (st != GBS_OK) {
    plan_free(P);
    return st;
  }
  *out = P;
  return GBS_OK;
}

extern "C" gbs_status gbs_csr_spmm_plan_parts(const gbs_csr_spmm_plan *P, int *parts) {
  clear_error();
  GBS_REQUIRE(P && parts, "spmm plan: null argument");
  *parts = P->parts.K;
  return GBS_OK;
}

extern "C" gbs_status gbs_csr_spmm_plan_destroy(gbs_csr_spmm_plan *P) {
  clear_error();
  plan_free(P);
  return GBS_OK;
}

extern "C" gbs_status gbs_csr_spmm_planned(const gbs_csr_spmm_plan *P, const void *B, float *C, void *ws,
                                           size_t ws_bytes, gbs_stream_t stream) {
  clear_error();
  GBS_REQUIRE(P != nullptr, "spmm planned: null plan");
  if (P->nrows == 0) return GBS_OK;
  GBS_REQUIRE(B && C, "spmm planned: null B or C");
  const int dt = P->btype == GBS_F32 ? 0 : (P->btype == GBS_BF16 ? 1 : 2);
  const ColumnParts &cp = P->parts;
  for (int p = 0; p < cp.K; ++p) {
    SpmmPlan sp;
    GBS_TRY(spmm_plan(dt, P->nrows, P->ncols, cp.nnz[p], P->F, B, C, 0, &sp, (P->ncols + cp.K - 1) / cp.K,
                      P->scaled));
    GBS_REQUIRE(ws != nullptr && ws_bytes >= sp.ws_bytes, "spmm planned: workspace missing or too small");
    GBS_TRY(spmm_run(sp, P->nrows, cp.nnz[p], cp.rowptr[p], cp.colind[p], cp.vals[p], B, P->F, C, ws,
                     (cudaStream_t)stream, 0, p > 0 ? 1 : 0, P->rowscale, P->colscale));
  }
  return GBS_OK;
}
