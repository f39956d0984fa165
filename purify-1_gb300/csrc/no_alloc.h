// Fixed device scratch of the allocation-free gridding entry point.
#pragma once
#include <cuda_runtime_api.h>

#include <cstddef>

namespace pg {
// Size of the scratch array (PURIFY_GB300_STATIC_SCRATCH_BYTES).
size_t static_scratch_bytes();
// Device address of the scratch array on the current device.  The first
// call on a device looks it up (cudaGetSymbolAddress) and caches it.
cudaError_t static_scratch_address(void **out);
}  // namespace pg
