// The plan compiler: a place, a contraction or a whole einsum compiled once per shape into a
// device program, a short list of operations over arenas with their descriptor tables.
//
//   TILES    a chain of leg moves whose every coefficient is 1 (abelian groups) as strided
//            rectangles: each tile is one (row tree, column tree) piece of an input block landing
//            as a rows x cols rectangle of an output block, its entries found from the copies of
//            every leg by mixed-radix strides; one pass however many steps the chain has, and a
//            descriptor per tile instead of an index per entry.
//   GATHER   dst[i] = src[index[i]] (index -1 writes 0): the same, composed with an earlier move
//            or for more legs than a tile describes.
//   RUNS     dst[d + t*ds] (+)= sum_k c_k src[s_k + t*ss_k] over chunks of runs: one leg-move step
//            (or a trace) with F/R coefficients, grouped by destination so the pass is atomic free.
//   GEMM     C_blk = sum_pairs A_blk(m x k) B_blk(k x n) over all output blocks of a contraction in
//            one grouped launch (every output block written, zero when it has no pair).
//   ADD      dst += src over a whole arena (the sum over charge alternatives of an einsum).
//   COPY     dst = src.
//   ZERO     dst = 0.
//
// Buffers are the operands, the output, and temporaries placed in one caller-provided workspace.
// Operations that depend on one operand alone form that operand's "prepare" phase; a caller can
// run it once and pass the prepared arena on later calls (the loop-invariant head and tail of a
// Lanczos matvec).
#pragma once

#include <cstdint>
#include <memory>
#include <string>
#include <vector>

#include "engine.h"

namespace ttg
{
  enum class OpKind : int32_t
  {
    zero = 0,
    gather = 1,
    runs = 2,
    gemm = 3,
    add = 4,
    copy = 5,
    tiles = 6,
  };

  struct Op
  {
    OpKind kind;
    int32_t src = -1, src2 = -1, dst = -1;
    int64_t begin = 0, count = 0;  // range in the op's descriptor table
    int64_t elements = 0;          // destination elements (zero/add/copy/gather)
    int32_t phase = -1;            // operand whose prepare phase this belongs to, -1 for the core
    int32_t flags = 0;             // tiles: 1 = conjugate the values (complex arenas)
  };

  // One destination run of a RUNS pass, already cut to at most kChunk elements.
  struct Chunk
  {
    int64_t dst;
    int32_t len;
    int32_t dst_step;
    int32_t term_begin;
    int32_t term_count;
  };
  struct Term
  {
    int64_t src;
    int64_t src_step;
    double re, im;
  };
  constexpr int32_t kChunk = 128;

  // One piece of a relabelling move: dst[out_base + r * out_ld + c] = src[in_base + sum over the
  // legs of copy_l * stride_l] for r < rows, c < cols, where r runs over the copies of the n_row
  // output codomain legs and c over those of the n_col output domain legs, the last leg of each
  // side fastest (extent[0..n_row) then extent[n_row..n_row+n_col)).
  constexpr int kTileLegs = 12;
  struct Tile
  {
    int64_t in_base, out_base;
    int32_t out_ld, rows, cols, n_row, n_col, pad;
    int32_t extent[kTileLegs];
    int64_t stride[kTileLegs];
  };
  // A launch unit: rows [row0, row0 + nrows) of one tile (about 2K entries).
  struct TileChunk
  {
    int32_t tile, row0, nrows, pad;
  };

  // One output block of a grouped GEMM and the block pairs summed into it.
  struct GemmBlock
  {
    int64_t c;
    int32_t m, n;
    int32_t pair_begin, pair_count;
  };
  struct GemmPair
  {
    int64_t a, b;
    int32_t k, pad;
  };

  enum class BufferKind : int32_t
  {
    input = 0,
    output = 1,
    temp = 2,
  };

  struct Buffer
  {
    BufferKind kind;
    int32_t index;   // operand number for inputs
    int64_t offset;  // elements into the workspace for temporaries
    int64_t size;    // elements
    int32_t prepared_of = -1;  // the operand whose prepared value this temporary holds
  };

  // Programs with GEMM ops keep their tickets (the counters by which the last partial tile of a
  // split output tile is found) in the first kTicketInts ints of the workspace, ahead of their
  // temporaries.  That region is zero when a workspace is first used, and every execution leaves
  // it zero (the last finisher of a tile resets its ticket), so no launch has to clear it.
  constexpr int64_t kTicketInts = 16384;
  constexpr int64_t kTicketElements = kTicketInts * 4 / 8;  // elements of 8 bytes or more

  struct Program
  {
    int32_t n_inputs = 0;
    std::vector<Space> input_spaces;
    Space output_space = nullptr;
    std::vector<Buffer> buffers;
    std::vector<Op> ops;
    int64_t workspace = 0;  // elements
    int64_t scratch_offset = 0;  // elements: GEMM scratch (partial tiles, slices) at the end of the workspace
    int32_t ctas = 152;          // CTAs of its persistent GEMM launches: the SMs of the device it was compiled for
    std::vector<int32_t> fold;   // an einsum's operands in the order it folds them (empty for other plans)
    // A product whose result only a leg move with unit coefficients reads, whose result in turn only
    // the A side of a second product reads (the two-site matvec): in FP64 the three ops run as one
    // launch, in split precision the first product stores through the move (chain.cu).  Ops between
    // the move and the second product belong to prepare phases.
    int32_t chain_first = -1, chain_move = -1, chain_second = -1;
    int64_t chain_slots = 0;  // partial tiles the chain's one launch may hold (its scratch is sized for them)
    uint64_t tune_key = 0;    // its block-size histogram's key (autotune.cpp)
    // per operand: the buffer holding its prepared value (the input itself when no op prepares it)
    std::vector<int32_t> prepared;
    // descriptor tables
    std::vector<int32_t> gather_index;
    std::vector<Chunk> chunks;
    std::vector<Term> terms;
    std::vector<GemmBlock> gemm_blocks;
    std::vector<GemmPair> gemm_pairs;
    std::vector<Tile> tiles;
    std::vector<TileChunk> tile_chunks;
    // the work schedules of the GEMM ops (gemm.h), computed once with the program
    std::shared_ptr<const struct GemmPlans> gemm_plans;
    // bookkeeping for the roofline: useful flops of the GEMMs, elements moved by recouplings
    double gemm_flops = 0;
    int64_t moved_elements = 0;
    bool complex_coefficients = false;  // some RUNS term has an imaginary part
  };

  // The entry-by-entry index a TILES or GATHER op amounts to: output entry i reads input entry
  // index[i], -1 where it writes zero (op.elements entries).
  std::vector<int32_t> expand_move(const Program &p, const Op &op);

  // Compile the conjugate-transpose of a tensor (its bra): every block (r, s, c) becomes block
  // (s, r, c) of the space with codomain and domain swapped and the dual charge, transposed and,
  // for complex arenas, conjugated (tentorch/tensors/tensor.cpp:99-107).
  std::shared_ptr<Program> compile_conj(Space space);

  // Compile one leg move of an arena of `space` into `above` / `below`.
  std::shared_ptr<Program> compile_place(Space space, const std::vector<int32_t> &above,
                                         const std::vector<int32_t> &below);
  // Compile a contraction (tentorch/linalg/graded/contract.cpp:117-175).  `has_charge` false takes
  // the charge of `left` and requires a neutral `right`.
  std::shared_ptr<Program> compile_contract(Space left, Space right, const std::vector<int32_t> &left_legs,
                                            const std::vector<int32_t> &right_legs, bool has_charge,
                                            const Sector &charge);
  // Compile an einsum (tentorch/linalg/graded/einsum.cpp:444-605).
  std::shared_ptr<Program> compile_einsum(const std::string &spec, const std::vector<Space> &operands,
                                          bool has_charge, const Sector &charge);

} // namespace ttg
