// Host-side launch bookkeeping shared by every kernel file: the dynamic shared memory cap of each kernel.
#include <mutex>
#include <utility>
#include <map>

#include "common.cuh"

namespace ffno {

// One cap per (kernel, device), found and set once under a lock. cudaFuncSetAttribute changes a process-wide attribute,
// so it runs only here, with the same value every time; later launches from any thread read the cached cap.
bool smem_cap_lookup(const void* kernel, size_t* cap) {
  static std::mutex mu;
  static std::map<std::pair<const void*, int>, size_t> caps;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return false;
  std::lock_guard<std::mutex> lock(mu);
  auto it = caps.find({kernel, dev});
  if (it != caps.end()) {
    *cap = it->second;
    return true;
  }
  int optin = 0;
  if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) return false;
  cudaFuncAttributes fa;
  if (cudaFuncGetAttributes(&fa, kernel) != cudaSuccess) return false;
  if ((size_t)optin <= fa.sharedSizeBytes) return false;
  const size_t c = (size_t)optin - fa.sharedSizeBytes;
  if (cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)c) != cudaSuccess) return false;
  caps[{kernel, dev}] = c;
  *cap = c;
  return true;
}

}  // namespace ffno
