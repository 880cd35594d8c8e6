// Fixed device scratch for rkdg_limit_static (include/rkdg_gpu.h).
//
// The cell means that the limiter reads live in one file-scope device array
// of RKDG_LIMIT_STATIC_MAX_VALUES doubles (16 MiB), created with the module on
// every device that loads the library.  Its device address is looked up once
// per device, with that device current, and cached.  Every context on a device
// shares the array, so two rkdg_limit_static calls in flight at the same time
// on one device (two host threads, or two contexts on different streams)
// overwrite each other's means.
#include <cuda_runtime.h>

#include <mutex>

#include "rkdg_gpu.h"
#include "rkdg_launch.h"

namespace {

constexpr int kMaxDevices = 64;

__device__ __align__(256) double g_static_means[RKDG_LIMIT_STATIC_MAX_VALUES];

std::mutex g_mutex;
double* g_addr[kMaxDevices] = {};

}  // namespace

namespace rkdg {

// Device address of the fixed means scratch on `device`, which the caller has
// made current.  Returns the error of cudaGetSymbolAddress, if any.
cudaError_t static_means_scratch(int device, double** out) {
  *out = nullptr;
  if (device < 0 || device >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_mutex);
  if (!g_addr[device]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_static_means);
    if (e != cudaSuccess) return e;
    g_addr[device] = static_cast<double*>(p);
  }
  *out = g_addr[device];
  return cudaSuccess;
}

}  // namespace rkdg
