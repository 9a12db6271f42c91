// device.cu -- per-device SM counts and dynamic shared-memory limits.
#include <map>
#include <mutex>
#include <utility>

#include "device.cuh"

namespace g3m3 {

cudaError_t prepare_fcsmooth();
cudaError_t prepare_push_ion();
namespace contracted {
cudaError_t prepare_push_ion();
}

namespace {

constexpr int kMaxDevices = 64;
std::mutex mu;
int sms[kMaxDevices];                                   // 0: not queried yet
std::map<std::pair<int, const void*>, cudaError_t> smem_done;

int current_device() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return dev;
}

}  // namespace

int sm_count() {
  const int dev = current_device();
  if (dev < 0 || dev >= kMaxDevices) return 148;
  std::lock_guard<std::mutex> lock(mu);
  if (!sms[dev]) {
    int n = 0;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) {
      cudaGetLastError();
      n = 148;
    }
    sms[dev] = n;
  }
  return sms[dev];
}

cudaError_t prepare_smem(const void* func, int bytes) {
  const int dev = current_device();
  std::lock_guard<std::mutex> lock(mu);
  auto key = std::make_pair(dev, func);
  auto it = smem_done.find(key);
  if (it != smem_done.end()) return it->second;
  cudaError_t e = cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  if (e != cudaSuccess) cudaGetLastError();
  smem_done[key] = e;
  return e;
}

cudaError_t prepare_device_kernels() {
  cudaError_t e = prepare_fcsmooth();
  if (e == cudaSuccess) e = prepare_push_ion();
  if (e == cudaSuccess) e = contracted::prepare_push_ion();
  return e;
}

}  // namespace g3m3
