// The plain per-block FP64 form of a GEMM op: one cuBLAS DGEMM (ZGEMM for complex128) per block
// pair, issued from the host in the order the pairs are listed, the way the reference runs its
// block products on a CUDA device (one at::matmul per matching block pair,
// tentorch/linalg/graded/contract.cpp:148-163).  It is the comparison arm of the grouped kernels:
// same program, same recouplings, only the block products differ.
#include <cublas_v2.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <map>
#include <mutex>

#include "executor.h"

namespace ttg
{
  namespace
  {
    std::mutex handle_mutex;
    std::map<int, cublasHandle_t> handles;

    cublasHandle_t handle_of_current_device(cudaError_t &error)
    {
      int device = 0;
      error = cudaGetDevice(&device);
      if (error != cudaSuccess) return nullptr;
      std::lock_guard<std::mutex> lock(handle_mutex);
      auto found = handles.find(device);
      if (found != handles.end()) return found->second;
      cublasHandle_t handle = nullptr;
      if (cublasCreate(&handle) != CUBLAS_STATUS_SUCCESS)
      {
        error = cudaErrorUnknown;
        return nullptr;
      }
      handles.emplace(device, handle);
      return handle;
    }
  } // namespace

  cudaError_t launch_gemm_per_block(const Program &p, const Op &op, const void *A, const void *B, void *C, bool complex,
                                    cudaStream_t stream)
  {
    cudaError_t error = cudaSuccess;
    cublasHandle_t handle = handle_of_current_device(error);
    if (!handle) return error == cudaSuccess ? cudaErrorUnknown : error;
    if (cublasSetStream(handle, stream) != CUBLAS_STATUS_SUCCESS) return cudaErrorUnknown;
    const size_t esize = complex ? 16 : 8;
    for (int64_t b = op.begin; b < op.begin + op.count; ++b)
    {
      const GemmBlock &blk = p.gemm_blocks[static_cast<size_t>(b)];
      char *c = static_cast<char *>(C) + static_cast<size_t>(blk.c) * esize;
      const int64_t entries = static_cast<int64_t>(blk.m) * blk.n;
      // an arena pads every block to an even number of entries; the pad stays zero
      const int64_t padded = entries + (entries & 1);
      if (entries == 0) continue;
      if (blk.pair_count == 0)
      {
        if ((error = cudaMemsetAsync(c, 0, static_cast<size_t>(padded) * esize, stream)) != cudaSuccess) return error;
        continue;
      }
      if (padded != entries &&
          (error = cudaMemsetAsync(c + entries * esize, 0, esize, stream)) != cudaSuccess)
        return error;
      for (int32_t k = 0; k < blk.pair_count; ++k)
      {
        const GemmPair &pr = p.gemm_pairs[static_cast<size_t>(blk.pair_begin + k)];
        const char *a = static_cast<const char *>(A) + static_cast<size_t>(pr.a) * esize;
        const char *bb = static_cast<const char *>(B) + static_cast<size_t>(pr.b) * esize;
        // row-major C (m x n) = A (m x k) B (k x n) is column-major C^T = B^T A^T
        cublasStatus_t status;
        if (complex)
        {
          const cuDoubleComplex one = make_cuDoubleComplex(1.0, 0.0), zero = make_cuDoubleComplex(0.0, 0.0);
          status = cublasZgemm(handle, CUBLAS_OP_N, CUBLAS_OP_N, blk.n, blk.m, pr.k, &one,
                               reinterpret_cast<const cuDoubleComplex *>(bb), blk.n,
                               reinterpret_cast<const cuDoubleComplex *>(a), std::max(1, pr.k), k == 0 ? &zero : &one,
                               reinterpret_cast<cuDoubleComplex *>(c), blk.n);
        }
        else
        {
          const double one = 1.0, zero = 0.0;
          status = cublasDgemm(handle, CUBLAS_OP_N, CUBLAS_OP_N, blk.n, blk.m, pr.k, &one,
                               reinterpret_cast<const double *>(bb), blk.n, reinterpret_cast<const double *>(a),
                               std::max(1, pr.k),
                               k == 0 ? &zero : &one, reinterpret_cast<double *>(c), blk.n);
        }
        if (status != CUBLAS_STATUS_SUCCESS) return cudaErrorUnknown;
      }
    }
    return cudaGetLastError();
  }

} // namespace ttg
