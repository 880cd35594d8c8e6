// Fixed device scratch for rkdg_limit_static (include/rkdg_gpu.h).
//
// Some callers may not allocate device memory while they step: a host code
// whose device memory belongs to its own memory manager or to a framework's
// caching pool, or a time loop that must not stall the device (cudaMalloc and
// cudaFree can synchronise it).  For them the cell means that the limiter
// reads live in one file-scope device array of RKDG_LIMIT_STATIC_MAX_VALUES
// doubles (16 MiB), which every GPU that loads the library holds until the
// process exits.  In host code the array's name is only a stand-in, not a
// device address: the first rkdg_limit_static call on a device looks the
// address up with cudaGetSymbolAddress (that device current) and caches it for
// the life of the process, so that first call should come before any stream
// capture, and a device reset (which would invalidate the cached address) ends
// the use of rkdg_limit_static in the process.  Every context on a
// device shares the array, so two rkdg_limit_static calls in flight at the
// same time on one device (two host threads, or two contexts on different
// streams) overwrite each other's means; nothing in it needs to start at zero,
// because the means kernel writes every entry the limiter then reads.
#include <cuda_runtime.h>

#include <mutex>

#include "rkdg_gpu.h"
#include "rkdg_launch.h"

namespace {

constexpr int kMaxDevices = 64;

static __device__ __align__(256) double g_static_means[RKDG_LIMIT_STATIC_MAX_VALUES];

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
