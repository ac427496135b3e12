// Grouped block-pair GEMM schedules and launchers.
//
// A GEMM op of a program computes every output block C_b = sum over its pairs A_p B_p.  Its output
// tiles are cut into work items of roughly equal multiply-add count, each covering a contiguous
// range of the tile's K (concatenated over the tile's pairs), so one long block product is spread
// over many SMs.  An item that covers its whole tile writes C; otherwise it writes a partial tile
// to scratch and a reduction sums the partials of the tile in a fixed order (deterministic, no
// atomics).
//
// Split precision (gemm.cu): every row of A and column of B is scaled by a power of two so that
// its entries lie in [-1, 1], then cut into `s` slices of 7 bits held exactly as bf16 integers
// (|q_1| <= 128, |q_t| <= 64).  The products of slices are sums of integers that fp32 accumulates
// exactly over a K-chunk of up to 256, so the only rounding is the final FP64 combination and the
// truncation after s slices (about 2^-7s of the row and column maxima): Ozaki's error-free
// splitting (K. Ozaki, T. Ogita, S. Oishi, S. M. Rump, Numer. Algorithms 59 (2012)) on bf16
// tensor cores with fp32 accumulation.
#pragma once

#include <cstdint>
#include <vector>

#include "program.h"

namespace ttg
{
  struct GemmItem
  {
    int32_t block, m0, n0, k0, k1, slot;  // slot -1: the item covers its tile and writes C
    int32_t reduce, pad;                   // the tile's GemmReduce when slot >= 0
  };
  struct GemmReduce
  {
    int32_t block, m0, n0, slot0, nslots, pad;
  };
  struct GemmSchedule
  {
    std::vector<GemmItem> items;     // grouped by the CTA that runs them
    std::vector<GemmReduce> reduces;
    std::vector<int32_t> cta_begin;  // CTA b runs items [cta_begin[b], cta_begin[b + 1])
    int64_t slots = 0;               // partial tiles of bm x bn doubles
    int64_t n_items = 0;             // items (also when only the sizes were computed)
  };
  // The SMs of the current device (cached per device), or 152, a GB300's count, when no device is
  // visible (plans compiled on a host without a GPU).  A plan's persistent GEMM launches spread
  // their items over this many CTAs, one per SM (Program::ctas, fixed when the plan is compiled).
  int device_sms();

  // Split precision works pair by pair: an item is one pair's K range (a multiple of 32 long, but
  // for the pair's last one), so a tile with several pairs or chunks always goes through partials.
  struct SplitItem
  {
    int32_t block, m0, n0, pair, k0, k1, slot, reduce;
  };
  // Where a pair's slices and exponents sit in scratch: A slices rows of `kp` (K padded to 32),
  // B slices transposed, one row of `kp` per column.
  struct SplitPair
  {
    int64_t sa, sb;
    int32_t kp, ea, eb, pad;
  };
  struct SplitLine
  {
    int64_t src, dst;
    int32_t len, src_stride, padded, exp;
  };
  struct SplitSchedule
  {
    std::vector<SplitItem> items;
    std::vector<GemmReduce> reduces;
    std::vector<SplitPair> pairs;  // one per GemmPair of the program (only this op's are filled)
    std::vector<SplitLine> lines;  // rows of A then columns of B
    int64_t lines_a = 0;
    int64_t slice_a = 0, slice_b = 0;  // elements of one slice of all A (B) rows
    int64_t exps_a = 0, exps_b = 0;    // int16 exponents of the rows of A, of the columns of B
    int64_t exps = 0;                  // both
    int64_t slots = 0;
    std::vector<int32_t> cta_begin;    // CTA b runs items [cta_begin[b], cta_begin[b + 1])
  };
  // The split-precision schedule of a GEMM op; with full = false only its sizes (slices, exponents,
  // partial slots, reductions), for sizing the scratch without building its tables.
  SplitSchedule schedule_split(const Program &p, const Op &op, bool full = true);

  // Tile sizes of the two kernels.
  constexpr int kF64TileM = 32, kF64TileN = 32;
  constexpr int kDmmaStepK = 32;  // K staged per step (two stages in flight) in the DMMA kernel
  constexpr int kSplitTileM = 32, kSplitTileN = 32, kSplitStepK = 32;
  // Persistent launches: one CTA per SM (held there by its shared memory), several workers of 128
  // threads per CTA taking items round robin.
  constexpr int kF64Workers = 4, kSplitWorkers = 2, kWorkerThreads = 128;
  constexpr int kMaxSlices = 8;
  constexpr int kExactChunk = 256;  // K over which fp32 sums of slice products stay exact

  // The FP64 schedule of a GEMM op; with full = false only its sizes (items, partial slots,
  // reductions), for sizing the scratch: the items are dealt on the op's first FP64 launch.
  GemmSchedule schedule_gemm(const Program &p, const Op &op, int bm, int bn, bool full = true);
  // The partial tiles (32 x 32 doubles each) the one launch of a program's product chain may hold
  // (chain.cu; 0 without a chain).
  int64_t chain_partial_slots(const Program &p);
  // The key of a plan's block-size histogram (autotune.cpp).
  uint64_t tune_key(const Program &p);

  // Scratch doubles a program's GEMM ops need at most (FP64 partials, or slices + exponents +
  // partials for split precision), laid out per op from offset 0.
  // Per op of a program (empty for the ops that are not GEMMs): the FP64 and the split schedules.
  // The slices of a GEMM operand that is an operand's prepared value (fixed while the arena is
  // unchanged: the head and tail of a Lanczos window) are cut once, when the arena is prepared,
  // into the arena after the prepared value: kMaxSlices slices (any fewer are a prefix of them)
  // and the exponents, laid out as the launch's scratch lays them out.
  struct SliceCache
  {
    int32_t op;       // the GEMM op
    int32_t side;     // 0: its A (rows), 1: its B (columns)
    int32_t operand;  // whose prepared arena holds it
    int64_t offset;   // bytes into that arena: the slices, then the exponents at exps_offset
    int64_t exps_offset;
    int64_t bytes;
  };
  struct GemmPlans
  {
    std::vector<GemmSchedule> f64;
    std::vector<SplitSchedule> split;
    std::vector<SliceCache> caches;
    std::vector<int32_t> cache_a, cache_b;  // per op: its A's (B's) cache, -1 for none
    std::vector<int64_t> prepared_bytes;    // per operand: bytes of its prepared arena with caches
  };
  // Schedule every GEMM op of the program into p.gemm_plans and return the scratch elements the
  // launches need (partial tiles, tickets, slices).
  int64_t plan_gemms(Program &p);

  // Find a product -> leg move -> product chain among the program's ops (Program::chain_*), from
  // the ops alone; whether the move is a one-to-one relabelling is checked on its first launch.
  void detect_chain(Program &p);
  // One FP64 work item of a chain: stage 0 items belong to the first product (their results go to
  // the moved layout), stage 1 items to the second (they start once every stage 0 tile is done).
  struct ChainItem
  {
    int32_t stage, block, m0, n0, k0, k1, slot, reduce, window, pad;  // window: the program of a batched launch
  };
  struct ChainReduce
  {
    int32_t stage, block, m0, n0, slot0, nslots, pad0, pad1;
  };
  // Programs a batched chain launch takes at most (tt_plan_execute_batch).
  constexpr int kChainBatch = 64;

  // The distinct left blocks (offset, rows, cols) and right blocks of one GEMM op.
  struct OperandBlock
  {
    int64_t offset;
    int32_t rows, cols;
  };
  void gemm_operands(const Program &p, const Op &op, std::vector<OperandBlock> &left, std::vector<OperandBlock> &right);

} // namespace ttg
