// L2 -> SM gather ceiling of this GPU: the rate at which warps can pull
// random feature rows of an L2-resident table into registers, the same
// access the CSR SpMM makes (half-warp per row, 16-byte loads, one index
// batch of 32 rows per warp, FP32 multiply-add of every element).  The
// SpMM's achieved gather rate is quoted against this number, since for a
// power-law graph most row gathers hit L2 and DRAM is not the limit.
//
//   gather_ceiling [--json]
//
// Rows: 1 KB (F = 256 FP32) and 512 B (F = 256 BF16, widened to FP32), of a
// table of 8,192 or 32,768 rows; 16M row indices uniform over the table
// (64 MB, streamed).  Each variant: 3 warm-up launches, 10 timed launches
// (CUDA events), grid = SMs x resident CTAs.  Indices are generated on the
// host, so every access stays inside the table.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#define CK(x)                                                                  \
  do {                                                                         \
    cudaError_t e_ = (x);                                                      \
    if (e_ != cudaSuccess) {                                                   \
      std::fprintf(stderr, "CUDA error %s at line %d\n", cudaGetErrorString(e_), __LINE__); \
      std::exit(1);                                                            \
    }                                                                          \
  } while (0)

__device__ __forceinline__ uint4 ld_nc(const uint4 *p) {
  uint4 v;
  asm volatile("ld.global.nc.v4.u32 {%0,%1,%2,%3}, [%4];"
               : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
               : "l"(p));
  return v;
}
__device__ __forceinline__ float bf_lo(unsigned x) { return __uint_as_float(x << 16); }
__device__ __forceinline__ float bf_hi(unsigned x) { return __uint_as_float(x & 0xffff0000u); }

// CH 16-byte chunks per lane per row (4: 1 KB rows, 2: 512 B rows); BF: the
// chunks hold bf16 pairs; U rows per half-warp in flight.
template <int CH, bool BF, int U>
__global__ void __launch_bounds__(256) k_gather(const uint4 *__restrict__ tab, const int *__restrict__ idx,
                                                long long n_idx, float *out) {
  const int lane = threadIdx.x & 31, sub = lane >> 4, sl = lane & 15;
  const long long warp = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
  const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
  constexpr int NA = BF ? CH * 8 : CH * 4;
  float acc[NA];
#pragma unroll
  for (int i = 0; i < NA; ++i) acc[i] = 0.f;
  const float v = 0.5f;
  for (long long b = warp * 32; b < n_idx; b += nwarps * 32) {
    const int my = idx[b + lane];  // n_idx is a multiple of 32
#pragma unroll 1
    for (int r = 0; r < 16; r += U) {
      uint4 x[U][CH];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int row = __shfl_sync(0xffffffffu, my, (r + u) * 2 + sub);
        const uint4 *p = tab + (size_t)row * (CH * 16) + sl;
#pragma unroll
        for (int c = 0; c < CH; ++c) x[u][c] = ld_nc(p + c * 16);
      }
#pragma unroll
      for (int u = 0; u < U; ++u)
#pragma unroll
        for (int c = 0; c < CH; ++c) {
          const unsigned w[4] = {x[u][c].x, x[u][c].y, x[u][c].z, x[u][c].w};
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            if (BF) {
              acc[c * 8 + 2 * q] = fmaf(v, bf_lo(w[q]), acc[c * 8 + 2 * q]);
              acc[c * 8 + 2 * q + 1] = fmaf(v, bf_hi(w[q]), acc[c * 8 + 2 * q + 1]);
            } else {
              acc[c * 4 + q] = fmaf(v, __uint_as_float(w[q]), acc[c * 4 + q]);
            }
          }
        }
    }
  }
  float s = 0.f;
#pragma unroll
  for (int i = 0; i < NA; ++i) s += acc[i];
  out[blockIdx.x * (long long)blockDim.x + threadIdx.x] = s;
}

struct Result {
  const char *name;
  int table_rows, ctas_per_sm;
  double ms, tbs;
};

template <int CH, bool BF, int U>
Result run(const char *name, int table_rows, const uint4 *tab, const int *idx, long long n, float *out,
           int sms) {
  auto k = k_gather<CH, BF, U>;
  int per = 0;
  CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k, 256, 0));
  if (per > 8) per = 8;  // the output buffer holds 8 CTAs per SM
  const int grid = sms * per;
  for (int i = 0; i < 3; ++i) k<<<grid, 256>>>(tab, idx, n, out);
  CK(cudaGetLastError());
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  const int reps = 10;
  CK(cudaEventRecord(e0));
  for (int i = 0; i < reps; ++i) k<<<grid, 256>>>(tab, idx, n, out);
  CK(cudaEventRecord(e1));
  CK(cudaEventSynchronize(e1));
  float ms = 0.f;
  CK(cudaEventElapsedTime(&ms, e0, e1));
  CK(cudaEventDestroy(e0));
  CK(cudaEventDestroy(e1));
  ms /= reps;
  const double bytes = (double)n * CH * 16 * 16;  // rows x row bytes
  return Result{name, table_rows, per, ms, bytes / (ms * 1e-3) / 1e12};
}

int main(int argc, char **argv) {
  const bool json = argc > 1 && std::strcmp(argv[1], "--json") == 0;
  cudaDeviceProp pr;
  CK(cudaGetDeviceProperties(&pr, 0));
  const int sms = pr.multiProcessorCount;
  const long long n = 16LL << 20;
  std::vector<Result> res;
  for (int T : {8192, 32768}) {
    std::vector<int> h(n);
    unsigned s = 12345u;
    for (long long i = 0; i < n; ++i) {
      s = s * 1664525u + 1013904223u;
      h[i] = (int)((s >> 8) % (unsigned)T);
    }
    uint4 *tab;
    int *idx;
    float *out;
    CK(cudaMalloc(&tab, (size_t)T * 1024));
    CK(cudaMemset(tab, 0, (size_t)T * 1024));
    CK(cudaMalloc(&idx, n * sizeof(int)));
    CK(cudaMemcpy(idx, h.data(), n * sizeof(int), cudaMemcpyHostToDevice));
    CK(cudaMalloc(&out, (size_t)sms * 8 * 256 * sizeof(float)));
    res.push_back(run<4, false, 1>("fp32_1KB_rows_U1", T, tab, idx, n, out, sms));
    res.push_back(run<4, false, 2>("fp32_1KB_rows_U2", T, tab, idx, n, out, sms));
    res.push_back(run<2, true, 2>("bf16_512B_rows_U2", T, tab, idx, n, out, sms));
    res.push_back(run<2, true, 4>("bf16_512B_rows_U4", T, tab, idx, n, out, sms));
    CK(cudaFree(tab));
    CK(cudaFree(idx));
    CK(cudaFree(out));
  }
  if (json) {
    std::printf("{\"device\": \"%s\", \"sms\": %d, \"l2_mb\": %d, \"results\": [", pr.name, sms,
                pr.l2CacheSize >> 20);
    for (size_t i = 0; i < res.size(); ++i)
      std::printf("%s{\"kernel\": \"%s\", \"table_rows\": %d, \"ctas_per_sm\": %d, \"ms\": %.4f, \"tbs\": %.3f}",
                  i ? ", " : "", res[i].name, res[i].table_rows, res[i].ctas_per_sm, res[i].ms, res[i].tbs);
    std::printf("]}\n");
  } else {
    std::printf("%s: %d SMs, L2 %d MB; 16M random rows per launch\n", pr.name, sms, pr.l2CacheSize >> 20);
    for (const Result &r : res)
      std::printf("%-20s table %6d rows  %d CTAs/SM  %.3f ms  %.2f TB/s gathered\n", r.name, r.table_rows,
                  r.ctas_per_sm, r.ms, r.tbs);
  }
  return 0;
}
