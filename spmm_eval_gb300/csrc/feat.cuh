// Feature-row access for the gather kernels: one 16-byte (or 4-byte) load
// of a dense row chunk, kept in its storage type in registers, widened to
// FP32 only at the multiply-add.
#pragma once

#include "common.cuh"

namespace gbs {

enum { DT_F32 = 0, DT_BF16 = 1, DT_F16 = 2 };

inline int dt_bytes(int dt) { return dt == DT_F32 ? 4 : 2; }

// acc0 += v * x0, acc1 += v * x1 as one packed sm_100+ FFMA2 (each half
// rounds exactly like fmaf).
__device__ __forceinline__ void fma2(float &acc0, float &acc1, float v, float x0, float x1) {
  asm("{\n .reg .b64 va, xa, ca;\n mov.b64 va, {%2, %2};\n mov.b64 xa, {%3, %4};\n"
      " mov.b64 ca, {%0, %1};\n fma.rn.f32x2 ca, va, xa, ca;\n mov.b64 {%0, %1}, ca;\n}"
      : "+f"(acc0), "+f"(acc1)
      : "f"(v), "f"(x0), "f"(x1));
}

// (acc0, acc1) += (a0 * b0, a1 * b1) as one FFMA2: two interleaved partial
// sums of a dot product.
__device__ __forceinline__ void fma2v(float &acc0, float &acc1, float a0, float a1, float b0, float b1) {
  asm("{\n .reg .b64 aa, bb, cc;\n mov.b64 aa, {%2, %3};\n mov.b64 bb, {%4, %5};\n"
      " mov.b64 cc, {%0, %1};\n fma.rn.f32x2 cc, aa, bb, cc;\n mov.b64 {%0, %1}, cc;\n}"
      : "+f"(acc0), "+f"(acc1)
      : "f"(a0), "f"(a1), "f"(b0), "f"(b1));
}

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
    fma2(acc[0], acc[1], v, r.x, r.y);
    fma2(acc[2], acc[3], v, r.z, r.w);
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
    fma2(acc[0], acc[1], v, bf16lo(r.x), bf16hi(r.x));
    fma2(acc[2], acc[3], v, bf16lo(r.y), bf16hi(r.y));
    fma2(acc[4], acc[5], v, bf16lo(r.z), bf16hi(r.z));
    fma2(acc[6], acc[7], v, bf16lo(r.w), bf16hi(r.w));
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
    fma2(acc[0], acc[1], v, a.x, a.y);
    fma2(acc[2], acc[3], v, b.x, b.y);
    fma2(acc[4], acc[5], v, c.x, c.y);
    fma2(acc[6], acc[7], v, d.x, d.y);
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
