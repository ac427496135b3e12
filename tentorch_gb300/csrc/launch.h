// Programmatic dependent launch for the engine's kernels.  The ops of a plan run back to back on
// one stream, each reading what the one before wrote; launched with programmatic stream
// serialisation, the next kernel is scheduled while the previous one drains (its launch and CTA
// set-up overlap the previous kernel's tail) and holds at griddepcontrol.wait until the previous
// grid has completed and its writes are visible.  Every kernel launched this way calls
// dependent_entry() before it touches global memory.
#pragma once

#include <cuda_runtime.h>

#include <utility>

namespace ttg
{
  __device__ __forceinline__ void dependent_entry()
  {
    asm volatile("griddepcontrol.wait;\n" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;\n" ::: "memory");
  }

  template <typename... Params, typename... Args>
  cudaError_t launch_dependent(void (*kernel)(Params...), dim3 grid, dim3 block, size_t smem, cudaStream_t stream,
                               Args &&...args)
  {
    cudaLaunchConfig_t config = {};
    config.gridDim = grid;
    config.blockDim = block;
    config.dynamicSmemBytes = smem;
    config.stream = stream;
    cudaLaunchAttribute attribute[1];
    attribute[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attribute[0].val.programmaticStreamSerializationAllowed = 1;
    config.attrs = attribute;
    config.numAttrs = 1;
    return cudaLaunchKernelEx(&config, kernel, std::forward<Args>(args)...);
  }
} // namespace ttg
