// Device-wide scans and the stable key sort used by the packers and the
// transpose, on CUB (header library shipped with the CUDA toolkit).  Kept in
// one translation unit so CUB is compiled once.  Temporary storage comes from
// the library's stream-ordered pool (DevBuf).
#include <cub/cub.cuh>

#include "common.cuh"
#include "util.cuh"

namespace gbs {

gbs_status exclusive_scan_i32(const int *in, int *out, int n, cudaStream_t s) {
  if (n <= 0) return GBS_OK;
  size_t tmp = 0;
  GBS_CUDA_TRY(cub::DeviceScan::ExclusiveSum(nullptr, tmp, in, out, n, s));
  DevBuf buf;
  GBS_TRY(buf.alloc(tmp, s));
  GBS_CUDA_TRY(cub::DeviceScan::ExclusiveSum(buf.p, tmp, in, out, n, s));
  return GBS_OK;
}

gbs_status stable_sort_pairs_i32(const int *keys_in, int *keys_out, const int *vals_in,
                                 int *vals_out, int n, int key_bits, cudaStream_t s) {
  if (n <= 0) return GBS_OK;
  size_t tmp = 0;
  GBS_CUDA_TRY(cub::DeviceRadixSort::SortPairs(nullptr, tmp, keys_in, keys_out, vals_in, vals_out,
                                               n, 0, key_bits, s));
  DevBuf buf;
  GBS_TRY(buf.alloc(tmp, s));
  GBS_CUDA_TRY(cub::DeviceRadixSort::SortPairs(buf.p, tmp, keys_in, keys_out, vals_in, vals_out,
                                               n, 0, key_bits, s));
  return GBS_OK;
}

}  // namespace gbs
