// SDDMM on A's pattern: out[e] = <G[row(e), :], H[col(e), :]> with FP32
// accumulation -- the gradient of the values of A in C = A H given dC = G.
//
// Same merge-path partition as the SpMM (each warp an equal share of rows +
// nonzeros).  A warp keeps its current row of G in registers and, per
// nonzero, gathers the row of H, multiplies, and reduces across the LPR
// lanes that cover the row with a fixed xor-shuffle tree; nothing is shared
// between warps, so there is no fix-up pass and the result is deterministic.
#include "common.cuh"
#include "feat.cuh"
#include "merge.cuh"

namespace gbs {

struct SddmmArgs {
  int nrows, nnz, F, nvec;
  const int *rowptr;
  const int *colind;
  const void *G;
  const void *H;
  float *out;
  int P;
  long long D;
};

template <int DT, int VEC, int LPR, int CH, int U, int MINB>
__global__ void __launch_bounds__(256, MINB) k_sddmm(SddmmArgs a) {
  constexpr int NSUB = 32 / LPR;
  constexpr int KPS = LPR;
  using F_ = Feat<DT, VEC>;
  using raw = typename F_::raw;
  const int lane = threadIdx.x & 31, sub = lane / LPR, sl = lane % LPR;
  const int warp = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5);
  if (warp >= a.P) return;
  const long long total = (long long)a.nrows + a.nnz;
  const long long d0 = min((long long)warp * a.D, total), d1 = min((long long)(warp + 1) * a.D, total);
  if (d0 >= d1) return;
  const int i0 = merge_search(a.rowptr, a.nrows, a.nnz, d0);
  const int i1 = merge_search(a.rowptr, a.nrows, a.nnz, d1);
  int j = (int)(d0 - i0);
  const int j1 = (int)(d1 - i1);
  for (int r = i0; r <= i1 && r < a.nrows; ++r) {
    const int re = r < i1 ? __ldg(a.rowptr + r + 1) : j1;
    if (j < re) {
      float g[CH][VEC];
#pragma unroll
      for (int c = 0; c < CH; ++c) {
        const int chunk = c * LPR + sl;
        if (chunk < a.nvec) F_::widen(g[c], F_::load(a.G, (size_t)r * a.F + (size_t)chunk * VEC));
        else
#pragma unroll
          for (int q = 0; q < VEC; ++q) g[c][q] = 0.f;
      }
      for (int base = j; base < re; base += 32) {
        const int n_valid = min(32, re - base);
        const int my_col = lane < n_valid ? ld_stream_i32(a.colind + base + lane) : 0;
        for (int u0 = 0; u0 < KPS; u0 += U) {
          if (u0 * NSUB >= n_valid) break;
          raw hv[U][CH];
#pragma unroll
          for (int u = 0; u < U; ++u) {
            const int k = (u0 + u) * NSUB + sub;
            const int col = __shfl_sync(0xffffffffu, my_col, k);
            const bool ok = k < n_valid;
#pragma unroll
            for (int c = 0; c < CH; ++c) {
              const int chunk = c * LPR + sl;
              if (ok && chunk < a.nvec) hv[u][c] = F_::load(a.H, (size_t)(unsigned)col * (unsigned)a.F + (size_t)chunk * VEC);
              else hv[u][c] = F_::zero();
            }
          }
          float s[U];
#pragma unroll
          for (int u = 0; u < U; ++u) {
            s[u] = 0.f;
#pragma unroll
            for (int c = 0; c < CH; ++c) {
              float h[VEC];
              F_::widen(h, hv[u][c]);
#pragma unroll
              for (int q = 0; q < VEC; ++q) s[u] = fmaf(g[c][q], h[q], s[u]);
            }
          }
          // Multi-value butterfly over the LPR lanes of the sub-group: each
          // of the first log2(U) levels halves the values a lane holds (the
          // lane keeps the half selected by its own offset bit and adds the
          // partner's copy), the remaining levels finish one value.  Lane sl
          // ends with the full dot product of nonzero sl / (LPR / U):
          // (U - 1) + log2(LPR / U) shuffles per U nonzeros instead of
          // U * log2(LPR).  Fixed order, so deterministic.
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
          {
            const int span = LPR / U;  // lanes sharing one finished value
            const int idx = sl / span;
            const int k = (u0 + idx) * NSUB + sub;
            if (sl % span == 0 && k < n_valid) a.out[base + k] = s[0];
          }
        }
      }
    }
    j = re;
  }
}

namespace {

struct SVar {
  const void *fn;
  int vec;
};

template <int DT, int VEC, int LPR, int CH>
SVar mks() {
  constexpr int UCAP = CH == 1 ? 4 : (CH == 2 ? 2 : 1);
  constexpr int U = UCAP < LPR ? UCAP : LPR;
  // register estimate: accumulators (+ blocked partials) + loads in flight
  constexpr int EST = 24 + 2 * CH * VEC + U * CH * 4 + U;
  constexpr int MINB = EST <= 64 ? 4 : (EST <= 80 ? 3 : (EST <= 128 ? 2 : 1));
  return SVar{(const void *)&k_sddmm<DT, VEC, LPR, CH, U, MINB>, VEC};
}

template <int DT, int VEC>
bool pick(int nvec, SVar *v) {
  if (nvec <= 1) { *v = mks<DT, VEC, 1, 1>(); return true; }
  if (nvec <= 2) { *v = mks<DT, VEC, 2, 1>(); return true; }
  if (nvec <= 4) { *v = mks<DT, VEC, 4, 1>(); return true; }
  if (nvec <= 8) { *v = mks<DT, VEC, 8, 1>(); return true; }
  if (nvec <= 16) { *v = mks<DT, VEC, 16, 1>(); return true; }
  if (nvec <= 32) { *v = mks<DT, VEC, 32, 1>(); return true; }
  if (nvec <= 64) { *v = mks<DT, VEC, 32, 2>(); return true; }
  if (nvec <= 128) { *v = mks<DT, VEC, 32, 4>(); return true; }
  if (nvec <= 256) { *v = mks<DT, VEC, 32, 8>(); return true; }
  return false;
}

}  // namespace
}  // namespace gbs

using namespace gbs;

extern "C" gbs_status gbs_sddmm(int nrows, int ncols, int nnz, const int *rowptr, const int *colind,
                                const void *G, const void *H, gbs_dtype dtype, int F, float *out,
                                gbs_stream_t stream) {
  clear_error();
  GBS_REQUIRE(dtype == GBS_F32 || dtype == GBS_BF16 || dtype == GBS_F16, "sddmm: bad dtype");
  GBS_REQUIRE(nrows >= 0 && ncols >= 0 && nnz >= 0 && F >= 1, "sddmm: bad sizes");
  GBS_REQUIRE(nnz == 0 || ncols > 0, "sddmm: nnz > 0 with ncols == 0");
  if (nrows == 0 || nnz == 0) return GBS_OK;
  GBS_REQUIRE(rowptr && colind && G && H && out, "sddmm: null pointer");
  const int dt = dtype == GBS_F32 ? DT_F32 : (dtype == GBS_BF16 ? DT_BF16 : DT_F16);
  const bool al = ((reinterpret_cast<uintptr_t>(G) | reinterpret_cast<uintptr_t>(H)) & 15u) == 0;
  SVar v{};
  bool ok;
  if (dt == DT_F32) ok = (al && F % 4 == 0) ? pick<DT_F32, 4>(F / 4, &v) : pick<DT_F32, 1>(F, &v);
  else if (!al || F % 8 != 0) ok = false;
  else ok = dt == DT_BF16 ? pick<DT_BF16, 8>(F / 8, &v) : pick<DT_F16, 8>(F / 8, &v);
  if (!ok)
    return fail(GBS_ERR_UNSUPPORTED, "sddmm: FP32 needs F <= 1024 (16-byte aligned) or <= 256; 16-bit needs "
                                     "F % 8 == 0, F <= 2048, 16-byte aligned");
  DeviceInfo di;
  GBS_TRY(device_info(&di));
  int bps = 0;
  GBS_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, v.fn, 256, 0));
  if (bps < 1) bps = 1;
  const long long total = (long long)nrows + nnz;
  long long P = (long long)di.sm_count * bps * 8;
  const long long pmin = (total + 255) / 256;
  if (P > pmin) P = pmin;
  if (P < 1) P = 1;
  SddmmArgs a;
  a.nrows = nrows;
  a.nnz = nnz;
  a.F = F;
  a.nvec = F / v.vec;
  a.rowptr = rowptr;
  a.colind = colind;
  a.G = G;
  a.H = H;
  a.out = out;
  a.P = (int)P;
  a.D = (total + P - 1) / P;
  void *args[] = {&a};
  GBS_CUDA_TRY(cudaLaunchKernel(v.fn, dim3((unsigned)((P * 32 + 255) / 256)), dim3(256), args, 0,
                                (cudaStream_t)stream));
  return GBS_OK;
}
