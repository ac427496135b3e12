// The device side of a compiled program: its descriptor tables on the GPU and the executor that
// launches its operations on one stream.
#pragma once

#include <cuda_runtime.h>

#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "gemm.h"
#include "program.h"

namespace ttg
{
  // Host tables gathered into one device allocation: each add() reserves a 256-byte aligned slot
  // and records where its device address goes; commit() makes one cudaMalloc and one copy.
  struct TableStaging
  {
    std::vector<char> host;
    std::vector<std::pair<size_t, void **>> slots;

    template <typename T>
    void add(const std::vector<T> &table, void **device)
    {
      *device = nullptr;
      if (table.empty()) return;
      const size_t at = (host.size() + 255) / 256 * 256;
      host.resize(at + table.size() * sizeof(T));
      std::memcpy(host.data() + at, table.data(), table.size() * sizeof(T));
      slots.emplace_back(at, device);
    }
    cudaError_t commit(void **base);
  };

  // A non-blocking stream of this library per device, for building tables before any launch reads
  // them (each build is waited for on the host).
  cudaError_t upload_stream(cudaStream_t *stream);

  // The descriptor tables of one program, uploaded on first execution (plan-compile time, never
  // inside a timed or captured region once warmed up), all in one device allocation.
  struct DeviceTables
  {
    std::mutex mutex;
    bool ready = false;
    void *base = nullptr;
    int32_t *gather = nullptr;
    Tile *tiles = nullptr;
    TileChunk *tile_chunks = nullptr;
    Chunk *chunks = nullptr;
    Term *terms = nullptr;
    GemmBlock *blocks = nullptr;
    GemmPair *pairs = nullptr;
    // per op: the balanced work items of a GEMM (FP64 tiles and split-precision tiles) and, for
    // the split path, the rows and columns to slice
    struct GemmTables
    {
      bool ready = false;            // built on the op's first FP64 launch, in an allocation of its own
      void *base = nullptr;
      GemmItem *items = nullptr;
      GemmReduce *reduces = nullptr;
      int32_t *cta_begin = nullptr;  // per CTA, the start of its list of items (n_ctas + 1 entries)
      int32_t n_ctas = 0;
      int64_t longest = 0;           // the longest list
      int64_t n_items = 0, n_reduces = 0, slots = 0;
    };
    struct SplitTables
    {
      bool ready = false;      // built on the op's first split launch, in an allocation of its own
      void *base = nullptr;
      int32_t *cta_begin = nullptr;  // per CTA, the start of its list of items (n_ctas + 1 entries)
      int32_t n_ctas = 0;
      int64_t longest = 0;
      void *items = nullptr, *pairs = nullptr, *lines = nullptr;
      GemmReduce *reduces = nullptr;
      int64_t n_items = 0, n_reduces = 0, n_lines_a = 0, n_lines_b = 0, slice_a = 0, slice_b = 0, exps_a = 0, exps = 0,
              slots = 0;
    };
    // the tile lists of split products on the tensor cores (split_tc.cu), built on first use
    struct TcTables
    {
      bool ready = false;
      void *base = nullptr;
      void *items = nullptr;
      int32_t *cta_begin = nullptr;
      int32_t n_ctas = 0;
    };
    std::vector<GemmTables> gemm;
    std::vector<SplitTables> split;
    std::vector<TcTables> tc;
    // the program's product chain (chain.cu): the relabelling table of its move (built on its first
    // launch in any form) and the one-launch FP64 tables (built on its first FP64 launch)
    struct ChainTables
    {
      bool tried = false, ok = false;                  // the one-launch FP64 tables
      bool relabel_tried = false, relabel_ok = false;  // the relabelling table
      void *base = nullptr;
      const ChainItem *items = nullptr;
      const int32_t *cta_begin = nullptr;
      const ChainReduce *reduces = nullptr;
      void *relabel_base = nullptr;
      const int32_t *relabel = nullptr;    // per entry of the first product's result: its place after the move, or -1
      int32_t n_ctas = 0;
      int64_t longest = 0, n_items = 0, n_reduces = 0, first_tiles = 0, slots = 0, moved_from = 0;
      std::vector<ChainItem> host_items;  // every item, first product first, before the deal (for batches)
      std::vector<double> host_work;      // their work estimates
    } chain;

    cudaError_t ensure(const Program &p);
    ~DeviceTables();
  };

  struct ExecArgs
  {
    bool complex = false;                  // complex128 arenas (else float64)
    int32_t precision = 0;                 // 0: FP64 products; k > 0: split products with k slices;
                                           // -1: the plain per-block FP64 form (one cuBLAS call per pair)
    const void *const *inputs = nullptr;   // one arena per operand
    const void *const *prepared = nullptr; // per operand: its prepared arena, or null
    void *output = nullptr;
    void *workspace = nullptr;
    cudaStream_t stream = nullptr;
    int32_t only_phase = -1;               // >= 0: run only this operand's prepare phase
    void *prepared_out = nullptr;          // where that phase writes its prepared arena
    cudaEvent_t *events = nullptr;         // when set: 2 per op, recorded around every op that runs
    bool *chain_ran = nullptr;             // when set: whether the product chain ran as one launch
                                           // (its events are those of the chain's first op)
    bool phases_only = false;              // run only the prepare phases that have to run
    int32_t forms = -1;                    // kForm* bits; -1: the autotuner's choice for the plan's
                                           // histogram (autotune.cpp), 0 when it has none
  };

  // The forms a plan's products can run in (autotune.cpp).
  constexpr int32_t kFormSeparate = 1;       // a product chain as separate launches
  constexpr int32_t kFormNoTensorCores = 2;  // split products of large blocks on mma.sync, not tcgen05
  // The cached forms for a key, or -1.
  int32_t tuned_forms(uint64_t key, bool complex, int32_t precision);
  void store_forms(uint64_t key, bool complex, int32_t precision, int32_t forms);
  void clear_forms();
  // The forms worth timing for a plan, the plain one first.
  std::vector<int32_t> candidate_forms(const Program &p, bool complex, int32_t precision);
  // Times every candidate form on `base`'s operands (two untimed and five timed executions each, on
  // base.stream, waited for), keeps the fastest in the cache under the plan's key, and returns it
  // with its median time.
  cudaError_t autotune(const Program &p, DeviceTables &t, const ExecArgs &base, int32_t *best, float *best_ms);

  cudaError_t execute(const Program &p, DeviceTables &t, const ExecArgs &args);
  // Where every buffer of the program lives for these arguments (inputs, output, prepared arenas,
  // workspace offsets).
  std::vector<char *> buffer_pointers(const Program &p, const ExecArgs &args);

  // The grouped GEMM of one op (gemm.cu): FP64 / complex128, or split precision with `slices`.
  // `tickets` is the workspace's ticket region (kTicketInts ints, zero, left zero).
  cudaError_t launch_gemm_f64(const Program &p, DeviceTables &t, size_t op_index, const void *A, const void *B, void *C,
                              bool complex, void *scratch, int *tickets, cudaStream_t stream);
  // `prepared`: the caller's prepared arenas (or null); a side read from one uses the slices cut
  // into it by fill_slice_caches.  With `relabel` (chain_relabel) every entry of C is stored at its
  // place after the program's chain move instead (C then being the move's destination).
  cudaError_t launch_gemm_split(const Program &p, const Op &op, DeviceTables &t, size_t op_index, const double *A,
                                const double *B, double *C, int32_t slices, void *scratch, int *tickets,
                                const void *const *prepared, cudaStream_t stream, const int32_t *relabel = nullptr,
                                bool tensor_cores = true);
  // The device table of the program's chain move (chain.cu): per entry of the first product's
  // result its place after the move, or -1; built on first use, null when the move does not write
  // every entry the second product reads.
  cudaError_t chain_relabel(const Program &p, DeviceTables &t, const int32_t **relabel);
  // Cut the slices of the GEMM operands that are operand `operand`'s prepared value into its arena.
  cudaError_t fill_slice_caches(const Program &p, DeviceTables &t, int32_t operand, const void *arena,
                                cudaStream_t stream);
  void stage_gemm(const Program &p, DeviceTables &t, TableStaging &staging);
  // The product chain of a program (Program::chain_*) in one FP64 launch (chain.cu): the first
  // product A1 B1 lands in the moved layout `moved`, the second reads it as its A.  *used is false
  // when the chain cannot run as one launch (then nothing is launched and the ops run one by one).
  cudaError_t launch_chain_f64(const Program &p, DeviceTables &t, const double *A1, const double *B1, double *moved,
                               const double *B2, double *C, void *workspace, cudaStream_t stream, bool *used);
  // `count` programs' chains (one per window of a batch) as ONE FP64 launch: per program its operands,
  // outputs and its own workspace (tickets at its head, scratch at p.scratch_offset).  *used is false
  // when some program's chain cannot join (then nothing is launched).  The deal of all the programs'
  // items is cached per list of programs (clear_chain_batches forgets them with the plans).
  struct ChainBatchEntry
  {
    const Program *program;
    DeviceTables *tables;
    const double *a1, *b1, *b2;
    double *moved, *c;
    void *workspace;
  };
  cudaError_t launch_chain_batch(const std::vector<ChainBatchEntry> &entries, cudaStream_t stream, bool *used);
  void clear_chain_batches();
  // Split products on the tensor cores (split_tc.cu): whether an op's blocks fill its 128 x 64 tiles
  // well enough, and the launch (slices and exponents as launch_gemm_split lays them out; `error`
  // an int of the workspace's ticket region, raised when a wait gives up).
  bool split_tc_suits(const Program &p, const Op &op, int32_t slices);
  cudaError_t launch_split_tc(const Program &p, const Op &op, DeviceTables &t, size_t op_index, int32_t slices,
                              const uint16_t *sa, const uint16_t *sb, const int16_t *exps_a, const int16_t *exps_b,
                              int64_t stride_a, int64_t stride_b, const void *spairs, double *C, int *error,
                              cudaStream_t stream);
  // The plain per-block form (per_block.cu): one cuBLAS call per block pair.
  cudaError_t launch_gemm_per_block(const Program &p, const Op &op, const void *A, const void *B, void *C, bool complex,
                                    cudaStream_t stream);

  // Record a failure for tt_last_error() and return its status code (capi.cpp).
  int32_t report(int32_t code, const std::string &message);

  // Thin SVDs of float64 blocks in one launch (svd.cu): `table` is a device array of 7 int64 per
  // block (a_off, rows, cols, u_off, s_off, vh_off, ws_off); info[i] = Jacobi sweeps, -1 when block
  // i did not converge.  svd_keep writes the kept factors into the split's arenas (12 int64-sized
  // fields per block, see svd.cu).
  cudaError_t svd_blocks(int32_t count, int64_t largest, const void *table, const double *a, double *u, double *s, double *vh,
                         void *workspace, int32_t *info, cudaStream_t stream);
  // doubles of global workspace one block needs (0 when its working set fits in shared memory)
  int64_t svd_workspace_doubles(int64_t rows, int64_t cols);
  // The ranking of a split's singular values (svd.cu rank_kernel): per block the values it keeps;
  // shared memory rank_bytes(...) at most kRankMaxBytes.
  constexpr int64_t kRankMaxBytes = 200 * 1024;
  int64_t rank_bytes(int32_t n_values, int32_t n_blocks, int32_t n_sectors);
  cudaError_t svd_rank(const double *values, int32_t n_values, const int32_t *block_k, const int32_t *block_sector,
                       int32_t n_blocks, const int32_t *dual, int32_t n_sectors, double tol, int64_t max_bond, int32_t *kept,
                       cudaStream_t stream);
  cudaError_t svd_keep(int32_t count, const void *table, const double *u, const double *s, const double *vh,
                       double *first, double *second, double *values, cudaStream_t stream);

  // The Lanczos loop of a window (lanczos.cu): `base` carries the plan's operands (the vector
  // operand's pointer is replaced by each basis vector), prepared arenas and workspace; scratch holds
  // lanczos_scratch_doubles() doubles; the normalised Ritz vector goes to `result`, the lowest Ritz
  // value to *energy_dev and the Krylov size to *size_dev (device memory), all on base.stream with no
  // host wait.  lanczos_energy_slot() is a place for both in the scratch (the energy, then the size).
  int64_t lanczos_scratch_doubles(int64_t n_doubles, int32_t n_iter);
  cudaError_t lanczos(const Program &p, DeviceTables &t, const ExecArgs &base, int32_t vector_operand,
                      const double *start, int64_t n_doubles, int32_t n_iter, double tol, double *scratch,
                      double *result, double *energy_dev, int32_t *size_dev);
  double *lanczos_energy_slot(double *scratch, int64_t n_doubles, int32_t n_iter);

  constexpr int kDotParts = 120;
  // out[2j], out[2j+1] = re, im of <a_j, b> for j < count; partial holds 2*kDotParts*count doubles.
  cudaError_t arena_dots(const double *const *dev_as, int32_t count, const double *b, int64_t n_doubles, bool complex,
                         double *partial, double *out, cudaStream_t stream);

} // namespace ttg
