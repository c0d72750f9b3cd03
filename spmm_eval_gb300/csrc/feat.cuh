// Feature-row access for the gather kernels: one 16-byte (or 4-byte) load
// of a dense row chunk, kept in its storage type in registers, widened to
// FP32 only at the multiply-add.
#pragma once

#include "common.cuh"

namespace gbs {

enum { DT_F32 = 0, DT_BF16 = 1, DT_F16 = 2 };

inline int dt_bytes(int dt) { return dt == DT_F32 ? 4 : 2; }

template <int DT, int VEC>
struct Feat;

template <>
struct Feat<DT_F32, 4> {
  using raw = float4;
  using storage_t = float;
  static __device__ __forceinline__ raw load(const void *base, size_t elem) {
    return ld_nc_f4(reinterpret_cast<const float *>(base) + elem);
  }
  static __device__ __forceinline__ raw zero() { return make_float4(0.f, 0.f, 0.f, 0.f); }
  static __device__ __forceinline__ void fma(float *acc, float v, const raw &r) {
    acc[0] = fmaf(v, r.x, acc[0]);
    acc[1] = fmaf(v, r.y, acc[1]);
    acc[2] = fmaf(v, r.z, acc[2]);
    acc[3] = fmaf(v, r.w, acc[3]);
  }
  static __device__ __forceinline__ void widen(float *out, const raw &r) {
    out[0] = r.x; out[1] = r.y; out[2] = r.z; out[3] = r.w;
  }
};

template <>
struct Feat<DT_F32, 1> {
  using raw = float;
  using storage_t = float;
  static __device__ __forceinline__ raw load(const void *base, size_t elem) {
    return __ldg(reinterpret_cast<const float *>(base) + elem);
  }
  static __device__ __forceinline__ raw zero() { return 0.f; }
  static __device__ __forceinline__ void fma(float *acc, float v, const raw &r) {
    acc[0] = fmaf(v, r, acc[0]);
  }
  static __device__ __forceinline__ void widen(float *out, const raw &r) { out[0] = r; }
};

template <>
struct Feat<DT_BF16, 8> {
  using raw = uint4;
  using storage_t = uint16_t;
  static __device__ __forceinline__ raw load(const void *base, size_t elem) {
    return ld_nc_u4(reinterpret_cast<const uint16_t *>(base) + elem);
  }
  static __device__ __forceinline__ raw zero() { return make_uint4(0, 0, 0, 0); }
  static __device__ __forceinline__ void fma(float *acc, float v, const raw &r) {
    acc[0] = fmaf(v, bf16lo(r.x), acc[0]);
    acc[1] = fmaf(v, bf16hi(r.x), acc[1]);
    acc[2] = fmaf(v, bf16lo(r.y), acc[2]);
    acc[3] = fmaf(v, bf16hi(r.y), acc[3]);
    acc[4] = fmaf(v, bf16lo(r.z), acc[4]);
    acc[5] = fmaf(v, bf16hi(r.z), acc[5]);
    acc[6] = fmaf(v, bf16lo(r.w), acc[6]);
    acc[7] = fmaf(v, bf16hi(r.w), acc[7]);
  }
  static __device__ __forceinline__ void widen(float *out, const raw &r) {
    out[0] = bf16lo(r.x); out[1] = bf16hi(r.x); out[2] = bf16lo(r.y); out[3] = bf16hi(r.y);
    out[4] = bf16lo(r.z); out[5] = bf16hi(r.z); out[6] = bf16lo(r.w); out[7] = bf16hi(r.w);
  }
};

template <>
struct Feat<DT_F16, 8> {
  using raw = uint4;
  using storage_t = uint16_t;
  static __device__ __forceinline__ raw load(const void *base, size_t elem) {
    return ld_nc_u4(reinterpret_cast<const uint16_t *>(base) + elem);
  }
  static __device__ __forceinline__ raw zero() { return make_uint4(0, 0, 0, 0); }
  static __device__ __forceinline__ void fma(float *acc, float v, const raw &r) {
    float2 a = h2f2(r.x), b = h2f2(r.y), c = h2f2(r.z), d = h2f2(r.w);
    acc[0] = fmaf(v, a.x, acc[0]);
    acc[1] = fmaf(v, a.y, acc[1]);
    acc[2] = fmaf(v, b.x, acc[2]);
    acc[3] = fmaf(v, b.y, acc[3]);
    acc[4] = fmaf(v, c.x, acc[4]);
    acc[5] = fmaf(v, c.y, acc[5]);
    acc[6] = fmaf(v, d.x, acc[6]);
    acc[7] = fmaf(v, d.y, acc[7]);
  }
  static __device__ __forceinline__ void widen(float *out, const raw &r) {
    float2 a = h2f2(r.x), b = h2f2(r.y), c = h2f2(r.z), d = h2f2(r.w);
    out[0] = a.x; out[1] = a.y; out[2] = b.x; out[3] = b.y;
    out[4] = c.x; out[5] = c.y; out[6] = d.x; out[7] = d.y;
  }
};

// Store VEC FP32 values.  stream=true marks data the kernel never re-reads.
template <int VEC, bool STREAM>
__device__ __forceinline__ void store_vec(float *p, const float *v) {
  if constexpr (VEC == 1) {
    if (STREAM) st_stream_f32(p, v[0]); else p[0] = v[0];
  } else {
#pragma unroll
    for (int q = 0; q < VEC; q += 4) {
      float4 x = make_float4(v[q], v[q + 1], v[q + 2], v[q + 3]);
      if (STREAM) st_stream_f4(p + q, x);
      else *reinterpret_cast<float4 *>(p + q) = x;
    }
  }
}

// Load VEC FP32 values through L2 only (data written by other warps of the
// same launch).
template <int VEC>
__device__ __forceinline__ void load_vec_cg(const float *p, float *v) {
  if constexpr (VEC == 1) {
    v[0] = __ldcg(p);
  } else {
#pragma unroll
    for (int q = 0; q < VEC; q += 4) {
      float4 x = __ldcg(reinterpret_cast<const float4 *>(p + q));
      v[q] = x.x; v[q + 1] = x.y; v[q + 2] = x.z; v[q + 3] = x.w;
    }
  }
}

}  // namespace gbs
