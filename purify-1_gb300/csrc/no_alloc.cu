// Fixed scratch for purify_gb300_grid_no_alloc.
//
// Some callers may not allocate device memory once they are running: codes
// that hand all GPU memory to one pool at start-up and forbid cudaMalloc /
// cudaFree afterwards (fragmentation, latency spikes on a real-time path), or
// processes that share a GPU under a hard memory cap.  The gridding entry
// point for them takes its scratch — the per-task accumulation windows and
// the slot-ordered visibility buffer — from the array below instead of from
// buffers of its own.  The array is a fixed part of the library image: every
// GPU that loads the library holds PURIFY_GB300_STATIC_SCRATCH_BYTES of it
// until the process exits.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/purify_gb300.h"
#include "no_alloc.h"

namespace pg {
namespace {

constexpr size_t kBytes = PURIFY_GB300_STATIC_SCRATCH_BYTES;
static __device__ __align__(256) unsigned char g_static_scratch[kBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
void *g_address[kMaxDevices] = {};

}  // namespace

size_t static_scratch_bytes() { return kBytes; }

// In host code `g_static_scratch` only names the symbol; the device address
// comes from cudaGetSymbolAddress, asked once per device with that device
// current.  The first call on a device does this set-up and the address is
// kept for the life of the process.  It belongs to the device's primary
// context: after cudaDeviceReset the module may load at another address, so
// a reset after the first call is not supported (the reset also frees every
// operator's device state, which makes the operators unusable anyway).
cudaError_t static_scratch_address(void **out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_address[dev]) {
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_static_scratch);
    if (e != cudaSuccess) return e;
    g_address[dev] = p;
  }
  *out = g_address[dev];
  return cudaSuccess;
}

}  // namespace pg
