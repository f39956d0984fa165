// Programmatic dependent launch between the kernels of an apply chain.
//
// A chain kernel is launched with the programmatic-stream-serialization
// attribute.  Its CTAs may then be scheduled as soon as every CTA of the
// previous kernel in the stream has started (each chain kernel signals that
// at its start, pdl_launch_next), instead of after the previous kernel has
// finished.  Before it reads anything the previous kernels wrote, and before
// it writes any global memory, every CTA of a chain kernel waits for the
// previous kernel to complete (pdl_wait, griddepcontrol.wait; its memory is
// then visible).  What may run before the wait: reads of the immutable
// coverage state and twiddle tables, index arithmetic, and shared-memory
// writes.  Every CTA executes the wait, including CTAs with no work, so a
// chain kernel never completes before its predecessor: the order of the
// whole chain stays the stream order.  A kernel whose predecessor did not
// signal (a library kernel, a copy, an event) starts after it completes, as
// without the attribute.  In a CUDA graph captured from the stream the
// attribute becomes a programmatic edge.
#pragma once
#include <cuda_runtime.h>

#include <utility>

namespace pg {

// Launch chain kernels with the attribute (false: plain stream order).
constexpr bool kChainPdl = true;

namespace dev {
__device__ __forceinline__ void pdl_launch_next() {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
}  // namespace dev

template <typename... KArgs, typename... Args>
cudaError_t launch_chain(void (*fn)(KArgs...), dim3 grid, dim3 block, size_t smem,
                         cudaStream_t s, Args &&...args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = kChainPdl ? 1 : 0;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, fn, std::forward<Args>(args)...);
}

}  // namespace pg
