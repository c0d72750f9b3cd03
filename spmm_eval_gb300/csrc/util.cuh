// Internal device-wide primitives (scan.cu) and small shared helpers.
#pragma once

#include "common.cuh"

namespace gbs {

// out[i] = sum in[0..i-1]; n elements.
gbs_status exclusive_scan_i32(const int *in, int *out, int n, cudaStream_t s);
gbs_status exclusive_scan_i64(const long long *in, long long *out, int n, cudaStream_t s);
// Stable radix sort of (key, value) pairs on the low key_bits bits of key.
gbs_status stable_sort_pairs_i32(const int *keys_in, int *keys_out, const int *vals_in,
                                 int *vals_out, int n, int key_bits, cudaStream_t s);

inline int bits_for(long long v) {
  int b = 1;
  while (b < 62 && (1ll << b) <= v) ++b;
  return b;
}

// RAII device buffer from stream-ordered allocation (freed on the same
// stream).  Used only where an entry point documents that it allocates.
struct DevBuf {
  void *p = nullptr;
  cudaStream_t s = nullptr;
  DevBuf() = default;
  DevBuf(const DevBuf &) = delete;
  DevBuf &operator=(const DevBuf &) = delete;
  gbs_status alloc(size_t bytes, cudaStream_t stream) {
    s = stream;
    if (bytes == 0) bytes = 16;
    cudaError_t e = cudaMallocAsync(&p, bytes, stream);
    if (e != cudaSuccess) {
      p = nullptr;
      return cuda_fail(e, "cudaMallocAsync");
    }
    return GBS_OK;
  }
  template <typename T>
  T *as() const { return reinterpret_cast<T *>(p); }
  ~DevBuf() {
    if (p) cudaFreeAsync(p, s);
  }
};

}  // namespace gbs
