// Programmatic dependent launch: a kernel launched with programmatic stream
// serialisation may start while its predecessor in the stream drains.  Such a
// kernel reads nothing its predecessor writes before grid_dep_wait(), and
// releases its own successor only after that wait, so no kernel's early part
// runs before the kernel two launches back has completed.  One exception: the
// motion-compensated row-local iteration (rowlocal.cuh) releases at its start
// and waits only before its update; its successor (the fused tTV kernel of
// the next iteration) waits before reading anything, and its own early part
// reads only what the launch three back wrote.
#pragma once

#include <cuda_runtime.h>

namespace gbn {

__device__ __forceinline__ void grid_dep_wait() { asm volatile("griddepcontrol.wait;\n" ::: "memory"); }
__device__ __forceinline__ void grid_dep_release() { asm volatile("griddepcontrol.launch_dependents;\n" ::: "memory"); }

// launch with programmatic stream serialisation
template <typename... KArgs, typename... Args>
inline void launch_pdl(void (*kernel)(KArgs...), dim3 grid, int threads, int smem, cudaStream_t s, Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = dim3(threads);
  cfg.dynamicSmemBytes = size_t(smem);
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  cudaLaunchKernelEx(&cfg, kernel, args...);
}

}  // namespace gbn
