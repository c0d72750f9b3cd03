// Internal device-wide primitives (scan.cu) and small shared helpers.
#pragma once

#include "common.cuh"

namespace gbs {

// out[i] = sum in[0..i-1]; n elements.
gbs_status exclusive_scan_i32(const int *in, int *out, int n, cudaStream_t s);
// Stable radix sort of (key, value) pairs on the low key_bits bits of key.
gbs_status stable_sort_pairs_i32(const int *keys_in, int *keys_out, const int *vals_in,
                                 int *vals_out, int n, int key_bits, cudaStream_t s);

inline int bits_for(long long v) {
  int b = 1;
  while (b < 62 && (1ll << b) <= v) ++b;
  return b;
}

// The library's own stream-ordered memory pool on the current device.  It
// keeps up to kPoolKeepBytes of freed temporaries mapped across
// synchronisations, so back-to-back calls do not pay for mapping fresh
// memory each time (the device's default pool returns everything at every
// synchronisation).  gbs_pool_trim releases what it keeps.
constexpr unsigned long long kPoolKeepBytes = 8ull << 30;
gbs_status lib_pool(cudaMemPool_t *out);
// Non-blocking streams per device (kSideStreams of them, by index) for
// sub-passes that run beside the caller's stream (forked and joined with
// events inside one call).
constexpr int kSideStreams = 2;
gbs_status side_stream(cudaStream_t *out, int which = 0);

// RAII device buffer from stream-ordered allocation in the library pool
// (freed on the same stream).  Used only where an entry point documents that
// it allocates.
struct DevBuf {
  void *p = nullptr;
  cudaStream_t s = nullptr;
  DevBuf() = default;
  DevBuf(const DevBuf &) = delete;
  DevBuf &operator=(const DevBuf &) = delete;
  gbs_status alloc(size_t bytes, cudaStream_t stream) {
    s = stream;
    if (bytes == 0) bytes = 16;
    cudaMemPool_t pool;
    GBS_TRY(lib_pool(&pool));
    cudaError_t e = cudaMallocFromPoolAsync(&p, bytes, pool, stream);
    if (e != cudaSuccess) {
      p = nullptr;
      return cuda_fail(e, "cudaMallocFromPoolAsync");
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
