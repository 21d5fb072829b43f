// Programmatic dependent launch: a kernel launched with launch_pdl may start
// while the previous kernel of its stream finishes.  Every such kernel calls
// pdl_trigger() (its dependents may launch once all its blocks have started)
// and pdl_wait() before it reads anything the previous kernels wrote; wait
// returns once those grids have completed and their writes are visible.
// Launched without the attribute, both instructions are no-ops.
#pragma once
#include <cuda_runtime.h>

namespace lcp {

__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

template <class K, class... Args>
inline cudaError_t launch_pdl(K* kernel, dim3 grid, dim3 block, size_t smem, cudaStream_t st, Args... args) {
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kernel, args...);
}

}  // namespace lcp
