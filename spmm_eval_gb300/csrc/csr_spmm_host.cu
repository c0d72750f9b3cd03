// CSR SpMM from host buffers, pipelined: the call a host-side caller of
// evalCSRSpmmFloatCuSPARSE (test_spmm_full.cu:212-342) makes -- host CSR and
// host B in, host C out -- with the copies overlapped with the kernels.
//
// B goes to the device first (every row needs it).  A is copied in K row
// ranges of about nnz/K nonzeros each on a copy stream; the merge-path SpMM
// of range k starts as soon as range k and B have arrived, on the caller's
// stream for even k and on a second compute stream (with its own workspace)
// for odd k, so one range's tail overlaps the next range's start (e2e 7.86
// against 8.19 ms on one stream, 232,965-node graph, F = 256); range k of C
// is copied back on a third stream as soon as it is computed.  With pinned
// host buffers the copies and the kernels overlap; with pageable buffers the
// copies are still correct, only serialised.
//
// A gbs_spmm_host_ctx keeps the device buffers (grow-only), the two side
// streams and the events between calls, so repeated calls allocate nothing;
// without one, each call allocates and frees its buffers stream-ordered.
#include <mutex>
#include <vector>

#include "common.cuh"
#include "csr_spmm.cuh"
#include "util.cuh"

namespace gbs {
namespace {

constexpr int kChunks = 16;

struct StreamPair {
  cudaStream_t h2d = nullptr, d2h = nullptr, c1 = nullptr;
};

gbs_status side_streams(StreamPair *out) {
  static std::mutex mu;
  static StreamPair per_dev[64];
  int dev = 0;
  GBS_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return fail(GBS_ERR_UNSUPPORTED, "csr spmm host: device ordinal >= 64");
  std::lock_guard<std::mutex> lock(mu);
  StreamPair &p = per_dev[dev];
  if (!p.h2d) {
    GBS_CUDA_TRY(cudaStreamCreateWithFlags(&p.h2d, cudaStreamNonBlocking));
    GBS_CUDA_TRY(cudaStreamCreateWithFlags(&p.d2h, cudaStreamNonBlocking));
    GBS_CUDA_TRY(cudaStreamCreateWithFlags(&p.c1, cudaStreamNonBlocking));
  }
  *out = p;
  return GBS_OK;
}

// Waits for the side streams when the call leaves early on an error, so the
// device buffers (freed on the caller's stream) are no longer in use.
struct SideSync {
  StreamPair sp;
  ~SideSync() {
    if (sp.h2d) cudaStreamSynchronize(sp.h2d);
    if (sp.d2h) cudaStreamSynchronize(sp.d2h);
    if (sp.c1) cudaStreamSynchronize(sp.c1);
  }
};

struct Events {
  std::vector<cudaEvent_t> ev;
  gbs_status make(int n) {
    ev.resize(n, nullptr);
    for (auto &e : ev) GBS_CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    return GBS_OK;
  }
  ~Events() {
    for (auto e : ev)
      if (e) cudaEventDestroy(e);
  }
};

}  // namespace
}  // namespace gbs

using namespace gbs;

struct gbs_spmm_host_ctx {
  int device = 0;
  StreamPair sp;
  void *buf[7] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
  size_t cap[7] = {0, 0, 0, 0, 0, 0, 0};
  std::vector<cudaEvent_t> ev;
};

namespace {

// Device buffer `i` of at least `bytes`, from the context (grow-only) or a
// temporary.
gbs_status ctx_buffer(gbs_spmm_host_ctx *ctx, int i, size_t bytes, DevBuf &tmp, cudaStream_t s, void **out) {
  if (bytes == 0) bytes = 16;
  if (!ctx) {
    GBS_TRY(tmp.alloc(bytes, s));
    *out = tmp.p;
    return GBS_OK;
  }
  if (ctx->cap[i] < bytes) {
    if (ctx->buf[i]) {
      GBS_CUDA_TRY(cudaStreamSynchronize(s));
      cudaFree(ctx->buf[i]);
      ctx->buf[i] = nullptr;
      ctx->cap[i] = 0;
    }
    GBS_CUDA_TRY(cudaMalloc(&ctx->buf[i], bytes));
    ctx->cap[i] = bytes;
  }
  *out = ctx->buf[i];
  return GBS_OK;
}

}  // namespace

extern "C" gbs_status gbs_spmm_host_ctx_create(gbs_spmm_host_ctx **out) {
  clear_error();
  GBS_REQUIRE(out != nullptr, "spmm host ctx: null output");
  auto *c = new gbs_spmm_host_ctx();
  cudaGetDevice(&c->device);
  cudaError_t e = cudaStreamCreateWithFlags(&c->sp.h2d, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->sp.d2h, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->sp.c1, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    if (c->sp.h2d) cudaStreamDestroy(c->sp.h2d);
    if (c->sp.d2h) cudaStreamDestroy(c->sp.d2h);
    delete c;
    return cuda_fail(e, "cudaStreamCreateWithFlags");
  }
  *out = c;
  return GBS_OK;
}

extern "C" gbs_status gbs_spmm_host_ctx_destroy(gbs_spmm_host_ctx *c) {
  clear_error();
  if (!c) return GBS_OK;
  int cur = 0;
  cudaGetDevice(&cur);
  cudaSetDevice(c->device);
  cudaStreamSynchronize(c->sp.h2d);
  cudaStreamSynchronize(c->sp.d2h);
  cudaStreamSynchronize(c->sp.c1);
  for (auto &b : c->buf)
    if (b) cudaFree(b);
  for (auto e : c->ev) cudaEventDestroy(e);
  cudaStreamDestroy(c->sp.h2d);
  cudaStreamDestroy(c->sp.d2h);
  cudaStreamDestroy(c->sp.c1);
  cudaSetDevice(cur);
  delete c;
  return GBS_OK;
}

extern "C" gbs_status gbs_csr_spmm_host(gbs_spmm_host_ctx *ctx, int nrows, int ncols, int nnz,
                                        const int *h_rowptr, const int *h_colind, const float *h_vals,
                                        const void *h_B, gbs_dtype btype, int F, float *h_C,
                                        gbs_stream_t stream) {
  clear_error();
  GBS_REQUIRE(btype == GBS_F32 || btype == GBS_BF16 || btype == GBS_F16, "csr spmm host: bad dtype");
  GBS_TRY(spmm_check_args(nrows, ncols, nnz, h_rowptr, h_colind, h_B, F, h_C));
  if (nrows == 0) return GBS_OK;
  GBS_REQUIRE(h_rowptr[0] == 0 && h_rowptr[nrows] == nnz, "csr spmm host: rowptr[0] != 0 or rowptr[n] != nnz");
  const int dt = btype == GBS_F32 ? 0 : (btype == GBS_BF16 ? 1 : 2);
  const size_t esz = btype == GBS_F32 ? 4 : 2;
  cudaStream_t s0 = (cudaStream_t)stream;
  StreamPair sp;
  if (ctx) sp = ctx->sp;
  else GBS_TRY(side_streams(&sp));

  // row ranges with ~nnz/K nonzeros each
  std::vector<int> cut{0};
  for (int k = 1; k < kChunks; ++k) {
    const long long target = (long long)nnz * k / kChunks;
    int lo = cut.back(), hi = nrows;
    while (lo < hi) {  // first row whose start is >= target
      const int mid = lo + (hi - lo) / 2;
      if (h_rowptr[mid] < target) lo = mid + 1;
      else hi = mid;
    }
    if (lo > cut.back() && lo < nrows) cut.push_back(lo);
  }
  cut.push_back(nrows);
  const int K = (int)cut.size() - 1;

  DevBuf tB, trp, tci, tv, tC, tws, tws2;
  void *pB, *prp, *pci, *pv = nullptr, *pC;
  GBS_TRY(ctx_buffer(ctx, 0, (size_t)ncols * F * esz, tB, s0, &pB));
  GBS_TRY(ctx_buffer(ctx, 1, sizeof(int) * ((size_t)nrows + 1), trp, s0, &prp));
  GBS_TRY(ctx_buffer(ctx, 2, sizeof(int) * (size_t)nnz, tci, s0, &pci));
  if (h_vals) GBS_TRY(ctx_buffer(ctx, 3, sizeof(float) * (size_t)nnz, tv, s0, &pv));
  GBS_TRY(ctx_buffer(ctx, 4, sizeof(float) * (size_t)nrows * F, tC, s0, &pC));
  int *drp = (int *)prp, *dci = (int *)pci;
  float *dv = (float *)pv, *dC = (float *)pC;
  // plan for the largest range (workspace sized for it, reused by every range)
  SpmmPlan plan;
  size_t ws_bytes = 256;
  for (int k = 0; k < K; ++k) {
    const int rows = cut[k + 1] - cut[k], nz = h_rowptr[cut[k + 1]] - h_rowptr[cut[k]];
    GBS_TRY(spmm_plan(dt, rows, ncols, nz, F, pB, dC, 0, &plan));
    if (plan.ws_bytes > ws_bytes) ws_bytes = plan.ws_bytes;
  }
  void *ws = nullptr, *ws2 = nullptr;
  GBS_TRY(ctx_buffer(ctx, 5, ws_bytes, tws, s0, &ws));
  GBS_TRY(ctx_buffer(ctx, 6, ws_bytes, tws2, s0, &ws2));
  SideSync guard{sp};  // destroyed before the buffers above
  // The counter region must be zero; the kernels leave it zero, a freshly
  // allocated buffer is cleared here (cheap: one memset of the workspace).
  GBS_CUDA_TRY(cudaMemsetAsync(ws, 0, ws_bytes, s0));
  GBS_CUDA_TRY(cudaMemsetAsync(ws2, 0, ws_bytes, s0));

  Events own;
  std::vector<cudaEvent_t> *evp = &own.ev;
  if (ctx) {
    while ((int)ctx->ev.size() < 2 + 2 * K + 1) {
      cudaEvent_t e;
      GBS_CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
      ctx->ev.push_back(e);
    }
    evp = &ctx->ev;
  } else {
    GBS_TRY(own.make(2 + 2 * K + 1));
  }
  std::vector<cudaEvent_t> &ev = *evp;
  cudaEvent_t ready = ev[0], haveB = ev[1], done = ev[2 + 2 * K];
  GBS_CUDA_TRY(cudaEventRecord(ready, s0));  // allocations are ordered before the copies
  GBS_CUDA_TRY(cudaStreamWaitEvent(sp.h2d, ready, 0));
  GBS_CUDA_TRY(cudaStreamWaitEvent(sp.d2h, ready, 0));
  GBS_CUDA_TRY(cudaStreamWaitEvent(sp.c1, ready, 0));
  GBS_CUDA_TRY(cudaMemcpyAsync(pB, h_B, (size_t)ncols * F * esz, cudaMemcpyHostToDevice, sp.h2d));
  GBS_CUDA_TRY(cudaEventRecord(haveB, sp.h2d));
  for (int k = 0; k < K; ++k) {
    const int r0 = cut[k], r1 = cut[k + 1];
    const int e0 = h_rowptr[r0], e1 = h_rowptr[r1];
    cudaEvent_t haveA = ev[2 + 2 * k], haveC = ev[3 + 2 * k];
    GBS_CUDA_TRY(cudaMemcpyAsync(drp + r0, h_rowptr + r0, sizeof(int) * (size_t)(r1 - r0 + 1),
                                 cudaMemcpyHostToDevice, sp.h2d));
    if (e1 > e0) {
      GBS_CUDA_TRY(cudaMemcpyAsync(dci + e0, h_colind + e0, sizeof(int) * (size_t)(e1 - e0),
                                   cudaMemcpyHostToDevice, sp.h2d));
      if (h_vals)
        GBS_CUDA_TRY(cudaMemcpyAsync(dv + e0, h_vals + e0, sizeof(float) * (size_t)(e1 - e0),
                                     cudaMemcpyHostToDevice, sp.h2d));
    }
    GBS_CUDA_TRY(cudaEventRecord(haveA, sp.h2d));
    cudaStream_t cs = (k & 1) ? sp.c1 : s0;
    GBS_CUDA_TRY(cudaStreamWaitEvent(cs, haveA, 0));
    if (k < 2) GBS_CUDA_TRY(cudaStreamWaitEvent(cs, haveB, 0));
    GBS_TRY(spmm_plan(dt, r1 - r0, ncols, e1 - e0, F, pB, dC, 0, &plan));
    GBS_TRY(spmm_run(plan, r1 - r0, e1 - e0, drp + r0, dci + e0, h_vals ? dv + e0 : nullptr, pB, F,
                     dC + (size_t)r0 * F, (k & 1) ? ws2 : ws, cs, e0));
    GBS_CUDA_TRY(cudaEventRecord(haveC, cs));
    GBS_CUDA_TRY(cudaStreamWaitEvent(sp.d2h, haveC, 0));
    GBS_CUDA_TRY(cudaMemcpyAsync(h_C + (size_t)r0 * F, dC + (size_t)r0 * F,
                                 sizeof(float) * (size_t)(r1 - r0) * F, cudaMemcpyDeviceToHost, sp.d2h));
  }
  GBS_CUDA_TRY(cudaEventRecord(done, sp.d2h));
  GBS_CUDA_TRY(cudaStreamWaitEvent(s0, done, 0));  // frees below are ordered after all copies
  GBS_CUDA_TRY(cudaStreamSynchronize(s0));
  return GBS_OK;
}
