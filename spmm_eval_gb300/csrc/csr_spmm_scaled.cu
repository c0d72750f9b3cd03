// Degree-normalised CSR SpMM: C[r] = rowscale[r] * sum over the stored
// entries (r, c) of colscale[c] * B[c], the GCN propagation D^-1/2 A D^-1/2 B
// with the normalisation folded into the merge-path kernel (SC = true
// instantiations of merge_kernel.cuh) instead of a value array: no value
// stream, one cached 4-byte scale per gathered row, one multiply per output
// row.  Also the FP64 D^-1/2 factors of a CSR pattern.
#include "common.cuh"
#include "csr_spmm.cuh"
#include "spmm_variants.cuh"
#include "util.cuh"

namespace gbs {

gbs_status spmm_select_scaled(int dt, int Fw, bool vec16, bool halfwarp, SpmmVariant *out) {
  return select_variant<true>(dt, Fw, vec16, halfwarp, out);
}

}  // namespace gbs

using namespace gbs;

static int to_dt(gbs_dtype t) { return t == GBS_F32 ? DT_F32 : (t == GBS_BF16 ? DT_BF16 : DT_F16); }

extern "C" gbs_status gbs_csr_spmm_scaled(int nrows, int ncols, int nnz, const int *rowptr,
                                          const int *colind, const float *rowscale,
                                          const float *colscale, const void *B, gbs_dtype btype,
                                          int F, float *C, void *ws, size_t ws_bytes,
                                          gbs_stream_t stream) {
  clear_error();
  GBS_REQUIRE(btype == GBS_F32 || btype == GBS_BF16 || btype == GBS_F16, "csr spmm scaled: bad dtype");
  GBS_TRY(spmm_check_args(nrows, ncols, nnz, rowptr, colind, B, F, C));
  if (nrows == 0) return GBS_OK;
  SpmmPlan p;
  GBS_TRY(spmm_plan(to_dt(btype), nrows, ncols, nnz, F, B, C, 0, &p, -1, true));
  GBS_REQUIRE(ws != nullptr && ws_bytes >= p.ws_bytes, "csr spmm scaled: workspace missing or too small");
  return spmm_run(p, nrows, nnz, rowptr, colind, nullptr, B, F, C, ws, (cudaStream_t)stream, 0, 0,
                  rowscale, colscale);
}

// out[r] = 1 / sqrt(rowptr[r+1] - rowptr[r]) computed in FP64 and rounded
// once to FP32 (0 for an empty row).
__global__ void k_degree_rsqrt(const int *__restrict__ rowptr, int n, float *__restrict__ out) {
  const long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  const int d = __ldg(rowptr + r + 1) - __ldg(rowptr + r);
  out[r] = d > 0 ? (float)(1.0 / sqrt((double)d)) : 0.f;
}

extern "C" gbs_status gbs_degree_rsqrt(int nrows, const int *rowptr, float *out, gbs_stream_t stream) {
  clear_error();
  GBS_REQUIRE(nrows >= 0, "degree rsqrt: negative size");
  if (nrows == 0) return GBS_OK;
  GBS_REQUIRE(rowptr && out, "degree rsqrt: null pointer");
  k_degree_rsqrt<<<(nrows + 255) / 256, 256, 0, (cudaStream_t)stream>>>(rowptr, nrows, out);
  return check_launch("k_degree_rsqrt");
}

