// CSR SpMM that allocates nothing: the merge-path kernel of csr_spmm.cu run
// with its scratch (split-row partial sums and arrival counters) in a
// fixed-size array compiled into this library instead of a caller-provided
// workspace.
//
// Who needs it: a caller that may not allocate device memory while it runs.
// Typical cases are a host application or framework that reserves all of its
// device memory up front in its own pool (an extra cudaMalloc from a library
// would fail or fragment that pool), and latency-critical serving loops that
// ban cudaMalloc/cudaFree on the request path because those calls can
// synchronise the whole device.  Such a caller still owns A, B and C; only
// the kernel's scratch comes from here.
//
// Costs of the fixed array: every GPU that loads the library holds
// kNoAllocScratchBytes of device memory until the process exits, and all
// calls share it, so two calls that can overlap on the GPU (different
// streams, or different host threads on one device) race on it and must be
// serialised by the caller.
#include "common.cuh"
#include "csr_spmm.cuh"

namespace gbs {

// 8 MiB.  The scratch of a launch is a fixed counter region (one int per
// warp the device can hold) plus two partial-sum rows of F floats per warp,
// so 8 MiB holds a full resident wave of warps up to about F = 128 FP32
// columns; wider rows run with fewer warps (fit_warps), which is correct but
// slower, down to 8 KiB per warp at F = 1024.  Widths the library does not
// support at all fail as they do in gbs_csr_spmm (GBS_ERR_UNSUPPORTED).
constexpr size_t kNoAllocScratchBytes = 8u << 20;

static __device__ __align__(256) unsigned char g_spmm_scratch[kNoAllocScratchBytes];

namespace {

// Device address of g_spmm_scratch on the current device.  In host code the
// name g_spmm_scratch is only a host-side stand-in for the symbol; the
// address a kernel may use comes from cudaGetSymbolAddress with that device
// current.  It is looked up on every call (no allocation, cheap) rather than
// cached, so a call after cudaDeviceReset or with a new primary context never
// uses an address from the old context.  The first lookup in a context loads
// the library's device code (which reserves the array), so that first call
// must come before any stream capture.
gbs_status scratch_address(void **out) {
  void *p = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&p, g_spmm_scratch);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_spmm_scratch)");
  *out = p;
  return GBS_OK;
}

// Largest warp count whose partial slots and counters fit in the array.
int fit_warps(int P, int Fw) {
  while (P > 1 && spmm_workspace_bytes(P, Fw) > kNoAllocScratchBytes) P = P * 3 / 4;
  return P;
}

}  // namespace
}  // namespace gbs

using namespace gbs;

extern "C" gbs_status gbs_csr_spmm_noalloc(int nrows, int ncols, int nnz, const int *rowptr,
                                           const int *colind, const float *vals, const void *B,
                                           gbs_dtype btype, int F, float *C,
                                           gbs_stream_t stream) {
  clear_error();
  GBS_REQUIRE(btype == GBS_F32 || btype == GBS_BF16 || btype == GBS_F16,
              "csr spmm noalloc: bad dtype");
  GBS_TRY(spmm_check_args(nrows, ncols, nnz, rowptr, colind, B, F, C));
  if (nrows == 0) return GBS_OK;
  const int dt = btype == GBS_F32 ? 0 : (btype == GBS_BF16 ? 1 : 2);
  SpmmPlan p;
  GBS_TRY(spmm_plan(dt, nrows, ncols, nnz, F, B, C, 0, &p));
  p.P = fit_warps(p.P, p.Fw);
  p.ws_bytes = spmm_workspace_bytes(p.P, p.Fw);
  // a guard: with one warp every supported width fits (at most 16 KiB of
  // partial rows beside the counters)
  if (p.ws_bytes > kNoAllocScratchBytes)
    return fail(GBS_ERR_INVALID_ARG,
                "csr spmm noalloc: F = " + std::to_string(F) + " needs " +
                    std::to_string(p.ws_bytes) + " bytes of scratch, more than the " +
                    std::to_string(kNoAllocScratchBytes) + "-byte static array");
  void *ws = nullptr;
  GBS_TRY(scratch_address(&ws));
  cudaStream_t s = (cudaStream_t)stream;
  // The array keeps whatever the previous call left in it.  Only the arrival
  // counters (the first P ints) must start at zero -- partial slots are
  // written before they are read -- so clear exactly those.
  GBS_CUDA_TRY(cudaMemsetAsync(ws, 0, (size_t)p.P * sizeof(int), s));
  return spmm_run(p, nrows, nnz, rowptr, colind, vals, B, F, C, ws, s);
}
