// Error strings, ABI version and the cached device-property table shared by
// every entry point of the C ABI.
#include <mutex>

#include "common.cuh"
#include "util.cuh"

namespace gbs {

static thread_local std::string g_last_error;

void set_error(const std::string &msg) { g_last_error = msg; }
void clear_error() { g_last_error.clear(); }

gbs_status device_info(DeviceInfo *out) {
  static std::mutex mu;
  static DeviceInfo cache[64];
  static bool have[64] = {false};
  int dev = 0;
  GBS_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return fail(GBS_ERR_UNSUPPORTED, "device ordinal >= 64");
  std::lock_guard<std::mutex> lock(mu);
  if (!have[dev]) {
    DeviceInfo d{};
    d.device = dev;
    GBS_CUDA_TRY(cudaDeviceGetAttribute(&d.sm_count, cudaDevAttrMultiProcessorCount, dev));
    GBS_CUDA_TRY(cudaDeviceGetAttribute(&d.max_threads_per_sm,
                                        cudaDevAttrMaxThreadsPerMultiProcessor, dev));
    GBS_CUDA_TRY(cudaDeviceGetAttribute(&d.regs_per_sm, cudaDevAttrMaxRegistersPerMultiprocessor, dev));
    int smem = 0;
    GBS_CUDA_TRY(cudaDeviceGetAttribute(&smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    d.smem_per_block_optin = (size_t)smem;
    GBS_CUDA_TRY(cudaDeviceGetAttribute(&d.l2_bytes, cudaDevAttrL2CacheSize, dev));
    cache[dev] = d;
    have[dev] = true;
  }
  *out = cache[dev];
  return GBS_OK;
}

gbs_status lib_pool(cudaMemPool_t *out) {
  static std::mutex mu;
  static cudaMemPool_t pools[64] = {};
  int dev = 0;
  GBS_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return fail(GBS_ERR_UNSUPPORTED, "device ordinal >= 64");
  std::lock_guard<std::mutex> lock(mu);
  if (!pools[dev]) {
    cudaMemPoolProps props{};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = dev;
    cudaMemPool_t p;
    GBS_CUDA_TRY(cudaMemPoolCreate(&p, &props));
    unsigned long long keep = kPoolKeepBytes;
    cudaError_t e = cudaMemPoolSetAttribute(p, cudaMemPoolAttrReleaseThreshold, &keep);
    if (e != cudaSuccess) {
      cudaMemPoolDestroy(p);
      return cuda_fail(e, "cudaMemPoolSetAttribute");
    }
    pools[dev] = p;
  }
  *out = pools[dev];
  return GBS_OK;
}

gbs_status side_stream(cudaStream_t *out, int which) {
  static std::mutex mu;
  static cudaStream_t streams[64][kSideStreams] = {};
  int dev = 0;
  GBS_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return fail(GBS_ERR_UNSUPPORTED, "device ordinal >= 64");
  if (which < 0 || which >= kSideStreams) return fail(GBS_ERR_INVALID_ARG, "side stream index");
  std::lock_guard<std::mutex> lock(mu);
  cudaStream_t &st = streams[dev][which];
  if (!st) GBS_CUDA_TRY(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
  *out = st;
  return GBS_OK;
}

}  // namespace gbs

extern "C" gbs_status gbs_pool_trim(void) {
  gbs::clear_error();
  cudaMemPool_t p;
  GBS_TRY(gbs::lib_pool(&p));
  GBS_CUDA_TRY(cudaMemPoolTrimTo(p, 0));
  return GBS_OK;
}

extern "C" const char *gbs_last_error(void) { return gbs::g_last_error.c_str(); }

extern "C" int gbs_abi_version(void) { return 1; }
