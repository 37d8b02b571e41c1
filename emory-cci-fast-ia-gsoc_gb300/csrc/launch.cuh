// Programmatic dependent launch helpers for the labelling and output kernels.
#pragma once

#include <cuda_runtime.h>

#include <utility>

namespace nsgb {

// Programmatic dependent launch.  A kernel launched by launch_dependent() may be scheduled
// while the kernel before it on the stream drains; pdl_wait() holds it until that kernel has
// completed and its writes are visible, and pdl_release() lets the next such kernel be
// scheduled once every CTA of this one has started.  Both are no-ops in a kernel launched the
// ordinary way, so kernels shared with other paths call them unconditionally, first thing.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_release() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

template <typename... KArgs, typename... Args>
inline cudaError_t launch_dependent(void (*kernel)(KArgs...), dim3 grid, dim3 block, cudaStream_t s,
                                    Args&&... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = 0;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}

}  // namespace nsgb
