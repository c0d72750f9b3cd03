// Shared helpers for the sm_103a kernels and the C ABI: status plumbing,
// cached device properties, vector load/store wrappers with cache hints and
// the BF16/FP16 -> FP32 widening used by the feature gathers.
#pragma once

#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <string>

#include "gbspmm.h"

namespace gbs {

// ---- error plumbing --------------------------------------------------------
void set_error(const std::string &msg);
void clear_error();

inline gbs_status fail(gbs_status st, const std::string &msg) {
  set_error(msg);
  return st;
}

inline gbs_status cuda_fail(cudaError_t e, const char *what) {
  set_error(std::string(what) + ": " + cudaGetErrorString(e));
  return e == cudaErrorMemoryAllocation ? GBS_ERR_OOM : GBS_ERR_CUDA;
}

#define GBS_CUDA_TRY(expr)                                   \
  do {                                                       \
    cudaError_t e_ = (expr);                                 \
    if (e_ != cudaSuccess) return gbs::cuda_fail(e_, #expr); \
  } while (0)

#define GBS_TRY(expr)                    \
  do {                                   \
    gbs_status s_ = (expr);              \
    if (s_ != GBS_OK) return s_;         \
  } while (0)

#define GBS_REQUIRE(cond, msg)                                     \
  do {                                                             \
    if (!(cond)) return gbs::fail(GBS_ERR_INVALID_ARG, (msg));     \
  } while (0)

// Checks the launch that was just enqueued.
inline gbs_status check_launch(const char *what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, what);
  return GBS_OK;
}

// ---- device properties (cached per device) --------------------------------
struct DeviceInfo {
  int device;
  int sm_count;
  int max_threads_per_sm;
  int regs_per_sm;
  size_t smem_per_block_optin;
  int l2_bytes;
};
gbs_status device_info(DeviceInfo *out);

inline size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

// ---- device-side helpers ----------------------------------------------------
__device__ __forceinline__ unsigned lane_id() {
  unsigned l;
  asm volatile("mov.u32 %0, %%laneid;" : "=r"(l));
  return l;
}

// Read-only gather through the non-coherent path (L1 allocate).
__device__ __forceinline__ float4 ld_nc_f4(const void *p) {
  float4 v;
  asm("ld.global.nc.v4.f32 {%0,%1,%2,%3}, [%4];"
               : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
               : "l"(p));
  return v;
}
__device__ __forceinline__ uint4 ld_nc_u4(const void *p) {
  uint4 v;
  asm("ld.global.nc.v4.u32 {%0,%1,%2,%3}, [%4];"
               : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
               : "l"(p));
  return v;
}
// Streamed once: do not allocate in L1.
__device__ __forceinline__ int ld_stream_i32(const int *p) {
  int v;
  asm("ld.global.nc.L1::no_allocate.b32 %0, [%1];"
               : "=r"(v)
               : "l"(p));
  return v;
}
__device__ __forceinline__ float ld_stream_f32(const float *p) {
  float v;
  asm("ld.global.nc.L1::no_allocate.f32 %0, [%1];"
               : "=f"(v)
               : "l"(p));
  return v;
}
// Output rows are written once and not re-read by the kernel.
__device__ __forceinline__ void st_stream_f4(void *p, float4 v) {
  asm volatile("st.global.cs.v4.f32 [%0], {%1,%2,%3,%4};" ::"l"(p), "f"(v.x),
               "f"(v.y), "f"(v.z), "f"(v.w)
               : "memory");
}
__device__ __forceinline__ void st_stream_f32(float *p, float v) {
  asm volatile("st.global.cs.f32 [%0], %1;" ::"l"(p), "f"(v) : "memory");
}

// Widening of packed 16-bit features to FP32.
__device__ __forceinline__ float bf16lo(uint32_t w) {
  return __uint_as_float(w << 16);
}
__device__ __forceinline__ float bf16hi(uint32_t w) {
  return __uint_as_float(w & 0xffff0000u);
}
// FP16 pairs are widened on the FMA pipe as x * 1 + (-0), exact (the
// mixed-precision fma.rn.f32.f16 of sm_100+): the conversion instruction it
// replaces measured FP16 SpMM 4.02 against 3.38 ms (114.8M-edge graph, F =
// 256).  BF16 keeps its shift / mask on the ALU: the same FMA form measured
// 3.38 against 3.30 ms there.
__device__ __forceinline__ float2 h2f2(uint32_t w) {
  float lo, hi;
  asm("{\n .reg .b16 l, h, one;\n mov.b32 {l, h}, %2;\n mov.b16 one, 0x3C00;\n"
      " fma.rn.f32.f16 %0, l, one, 0f80000000;\n fma.rn.f32.f16 %1, h, one, 0f80000000;\n}"
      : "=f"(lo), "=f"(hi)
      : "r"(w));
  return make_float2(lo, hi);
}

}  // namespace gbs
