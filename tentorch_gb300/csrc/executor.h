// The device side of a compiled program: its descriptor tables on the GPU and the executor that
// launches its operations on one stream.
#pragma once

#include <cuda_runtime.h>

#include <mutex>
#include <vector>

#include "program.h"

namespace ttg
{
  // The descriptor tables of one program, uploaded on first execution (plan-compile time, never
  // inside a timed or captured region once warmed up).
  struct DeviceTables
  {
    std::mutex mutex;
    bool ready = false;
    int32_t *gather = nullptr;
    Chunk *chunks = nullptr;
    Term *terms = nullptr;
    GemmBlock *blocks = nullptr;
    GemmPair *pairs = nullptr;
    int32_t *tiles = nullptr;  // (block, m0, n0, 0) per 32x32 output tile
    std::vector<int64_t> tile_begin, tile_count;
    // split-precision scratch layout (see gemm_split.cu), per GEMM op
    std::vector<int64_t> split_tile_begin, split_tile_count;
    int32_t *split_tiles = nullptr;

    cudaError_t ensure(const Program &p);
    ~DeviceTables();
  };

  struct ExecArgs
  {
    bool complex = false;                  // complex128 arenas (else float64)
    int32_t precision = 0;                 // 0: FP64 products; k > 0: split products with k slices
    const void *const *inputs = nullptr;   // one arena per operand
    const void *const *prepared = nullptr; // per operand: its prepared arena, or null
    void *output = nullptr;
    void *workspace = nullptr;
    cudaStream_t stream = nullptr;
    int32_t only_phase = -1;               // >= 0: run only this operand's prepare phase
    void *prepared_out = nullptr;          // where that phase writes its prepared arena
    cudaEvent_t *events = nullptr;         // when set: 2 per op, recorded around every op that runs
  };

  cudaError_t execute(const Program &p, DeviceTables &t, const ExecArgs &args);

  // The split-precision grouped GEMM of one op (gemm_split.cu).
  cudaError_t launch_gemm_split(const Program &p, const Op &op, DeviceTables &t, size_t op_index, const double *A,
                                const double *B, double *C, int32_t slices, cudaStream_t stream);

  constexpr int kDotParts = 120;
  // out[2j], out[2j+1] = re, im of <a_j, b> for j < count; partial holds 2*kDotParts*count doubles.
  cudaError_t arena_dots(const double *const *dev_as, int32_t count, const double *b, int64_t n_doubles, bool complex,
                         double *partial, double *out, cudaStream_t stream);

} // namespace ttg
