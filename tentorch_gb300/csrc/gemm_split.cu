// Split-precision grouped GEMM (placeholder until the tensor-core kernel lands): reports that the
// mode is not available so a caller never gets FP64 results under a split-precision name.
#include "executor.h"

namespace ttg
{
  cudaError_t launch_gemm_split(const Program &, const Op &, DeviceTables &, size_t, const double *, const double *,
                                double *, int32_t, cudaStream_t)
  {
    return cudaErrorNotSupported;
  }
} // namespace ttg
