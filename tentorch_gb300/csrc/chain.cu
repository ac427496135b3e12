// One launch for a block product whose result is moved and multiplied again: the two-site
// effective-Hamiltonian matvec of DMRG, head' theta -> X, X -> X' (a leg move with unit
// coefficients, a relabelling of entries for abelian symmetries), X' tail'' -> image
// (tentorch/linalg/graded/einsum.cpp:351-376 folds it as two contractions with a recoupling between
// them, tentorch/linalg/graded/contract.cpp:148-163 one product per block pair).
//
// The persistent FP64 kernel runs the work items of both products from one list per SM (4 workers
// of 128 threads claiming from it, FP64 FMA lanes, see the kernel):
//   - a first-product tile writes its entries straight to their places after the move (a table of
//     one int32 per entry of X, built on the device once per plan from the move's tile
//     descriptors, replaces the move's own pass), then counts itself done (per worker, published
//     once before the worker's first wait);
//   - a second-product item waits until every first-product tile of its program is done, then runs
//     like any other tile;
//   - a tile cut along K adds its chunks into a per-tile accumulator with FP64 atomics; the
//     accumulators, in the workspace's scratch, are zeroed by all CTAs at the start of the launch,
//     and no chunk adds before every CTA has zeroed its share.
// Each SM's list holds its first-product items before its second-product items and every SM runs
// its own list, so every wait ends once the first-product items of the running SMs are done; a wait
// still gives up after two seconds and raises an error flag (no hang on a fault elsewhere).  The
// counters sit in the workspace's ticket region; the last CTA to leave resets them, so every launch
// leaves the region zero, as the other grouped kernels do.  Many programs (the windows of a batch)
// can share one launch: their items are dealt together and each names its program.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <map>
#include <mutex>
#include <numeric>
#include <set>
#include <vector>

#include "executor.h"
#include "gemm.h"
#include "gemm_device.cuh"
#include "launch.h"

namespace ttg
{
  // ------------------------------------------------------------------------------------------
  // host: finding the chain
  // ------------------------------------------------------------------------------------------

  void detect_chain(Program &p)
  {
    p.chain_first = p.chain_move = p.chain_second = -1;
    const auto reads = [](const Op &op, int32_t buffer) { return op.src == buffer || op.src2 == buffer; };
    for (size_t i = 0; i + 2 < p.ops.size(); ++i)
    {
      const Op &first = p.ops[i], &move = p.ops[i + 1];
      if (first.kind != OpKind::gemm || first.phase >= 0 || move.kind != OpKind::tiles || move.phase >= 0 ||
          move.src != first.dst || move.flags != 0)
        continue;
      if (p.buffers[static_cast<size_t>(first.dst)].kind != BufferKind::temp ||
          p.buffers[static_cast<size_t>(move.dst)].kind != BufferKind::temp)
        continue;
      size_t k = i + 2;
      while (k < p.ops.size() && p.ops[k].phase >= 0) ++k;
      if (k >= p.ops.size()) continue;
      const Op &second = p.ops[k];
      if (second.kind != OpKind::gemm || second.src != move.dst || second.src2 == first.dst || second.src2 == move.dst)
        continue;
      // X is read by the move alone and X' by the second product alone; nothing else writes them
      bool alone = true;
      for (size_t j = 0; j < p.ops.size() && alone; ++j)
      {
        const Op &o = p.ops[j];
        if (j != i + 1 && reads(o, first.dst)) alone = false;
        if (j != k && reads(o, move.dst)) alone = false;
        if (j != i && o.dst == first.dst) alone = false;
        if (j != i + 1 && o.dst == move.dst) alone = false;
      }
      if (!alone) continue;
      p.chain_first = static_cast<int32_t>(i);
      p.chain_move = static_cast<int32_t>(i + 1);
      p.chain_second = static_cast<int32_t>(k);
      return;
    }
  }

  namespace
  {
    constexpr int kChainTile = 32;  // the tile of an item (kF64TileM x kF64TileN)
    // Four workers of 128 threads per SM, each with one warp on every quarter of the SM: while one
    // worker claims, waits for its operands or sums a partial tile, the others keep the quarters'
    // FP64 units busy.
    constexpr int kChainWorkers = 4, kChainThreads = 128;
    constexpr int kPer = 8;                           // a thread's slots of a tile
    constexpr int kSlots = kChainThreads * kPer;      // a worker's slots

    // The work estimate of an item, in multiply-adds: its live entries in warps of 32 times K, plus
    // the equivalent of a quarter tile over 16 of K per staged step and per item.
    double item_work(double rows, double cols, double k)
    {
      const double lanes = std::ceil(rows * cols / 32.0) * 32.0;
      return lanes * k + 0.25 * kChainTile * kChainTile * 16.0 * (std::ceil(k / kDmmaStepK) + 1.0);
    }

    // The items of one product: the grouped FP64 schedule's 32 x 32 tiles over K ranges (gemm.cu
    // schedule_gemm: about six items per SM, a tile cut along K into partial tiles when it is
    // larger), with their tile extents in ChainItem::pad and ChainReduce::pad0 (rows | cols << 8)
    // and their work for the deal.
    struct ChainCut
    {
      std::vector<ChainItem> items;
      std::vector<double> work;
      std::vector<ChainReduce> reduces;
      int64_t slots = 0;
    };
    void cut_product(const Program &p, const Op &op, int32_t stage, ChainCut &cut)
    {
      const GemmSchedule s = schedule_gemm(p, op, kChainTile, kChainTile, true);
      const int32_t slot0 = static_cast<int32_t>(cut.slots), reduce0 = static_cast<int32_t>(cut.reduces.size());
      constexpr int32_t extents = kChainTile | kChainTile << 8;
      for (const GemmReduce &r : s.reduces)
        cut.reduces.push_back(ChainReduce{stage, r.block, r.m0, r.n0, r.slot0 + slot0, r.nslots, extents, 0});
      for (const GemmItem &g : s.items)
      {
        const GemmBlock &blk = p.gemm_blocks[static_cast<size_t>(g.block)];
        ChainItem it{stage, g.block, g.m0, g.n0, g.k0, g.k1, -1, -1, 0, extents};
        if (g.slot >= 0)
        {
          it.slot = g.slot + slot0;
          it.reduce = g.reduce + reduce0;
        }
        cut.items.push_back(it);
        cut.work.push_back(item_work(std::min(kChainTile, blk.m - g.m0), std::min(kChainTile, blk.n - g.n0), g.k1 - g.k0));
      }
      cut.slots += s.slots;
    }
  } // namespace

  int64_t chain_partial_slots(const Program &p)
  {
    if (p.chain_first < 0) return 0;
    // the partial tiles do not depend on the deal: the schedule's sizing pass counts them
    return schedule_gemm(p, p.ops[static_cast<size_t>(p.chain_first)], kChainTile, kChainTile, false).slots +
           schedule_gemm(p, p.ops[static_cast<size_t>(p.chain_second)], kChainTile, kChainTile, false).slots;
  }

  namespace
  {
    // The items of both products, their work, and one list per SM dealt largest first onto the
    // least loaded, the first product before the second; false when the counters do not fit the
    // ticket region.
    bool build_chain(const Program &p, DeviceTables::ChainTables &ct, TableStaging &staging,
                     std::vector<ChainItem> &items, std::vector<int32_t> &cta_begin, std::vector<ChainReduce> &reduces)
    {
      ChainCut cut;
      cut_product(p, p.ops[static_cast<size_t>(p.chain_first)], 0, cut);
      const size_t first_items = cut.items.size(), first_reduces = cut.reduces.size();
      cut_product(p, p.ops[static_cast<size_t>(p.chain_second)], 1, cut);
      // the workspace holds the partial tiles the plan was sized for
      if (cut.slots > p.chain_slots) return false;
      const int64_t n_reduces = static_cast<int64_t>(cut.reduces.size());
      // tickets of both products, then the first product's done count, the exit count, the error
      // flag and the count of CTAs that zeroed the partial-tile accumulators
      if (n_reduces + 4 > kTicketInts) return false;
      reduces = cut.reduces;
      int64_t first_tiles = static_cast<int64_t>(first_reduces);
      struct Sized
      {
        ChainItem item;
        double work;
      };
      std::vector<Sized> stage[2];
      for (size_t i = 0; i < cut.items.size(); ++i)
      {
        stage[i < first_items ? 0 : 1].push_back(Sized{cut.items[i], cut.work[i]});
        if (i < first_items && cut.items[i].slot < 0) ++first_tiles;
      }
      ct.host_items.clear();
      ct.host_work.clear();
      for (const std::vector<Sized> &st : stage)
        for (const Sized &one : st)
        {
          ct.host_items.push_back(one.item);
          ct.host_work.push_back(one.work);
        }
      const size_t n_items = stage[0].size() + stage[1].size();
      const int ctas = static_cast<int>(std::min<size_t>(static_cast<size_t>(p.ctas), std::max<size_t>(n_items, 1)));
      std::vector<std::pair<double, int>> heap;
      for (int c = 0; c < ctas; ++c) heap.push_back({0.0, c});
      const auto later = [](const std::pair<double, int> &a, const std::pair<double, int> &b)
      { return a.first > b.first || (a.first == b.first && a.second > b.second); };
      std::make_heap(heap.begin(), heap.end(), later);
      std::vector<std::vector<ChainItem>> per_cta(static_cast<size_t>(ctas));
      for (std::vector<Sized> &st : stage)
      {
        // the second product starts on every SM when the first is done everywhere: its items are
        // balanced on their own
        if (&st == &stage[1])
        {
          for (auto &h : heap) h.first = 0.0;
          std::make_heap(heap.begin(), heap.end(), later);
        }
        std::stable_sort(st.begin(), st.end(), [](const Sized &a, const Sized &b) { return a.work > b.work; });
        for (const Sized &one : st)
        {
          std::pop_heap(heap.begin(), heap.end(), later);
          auto &least = heap.back();
          per_cta[static_cast<size_t>(least.second)].push_back(one.item);
          least.first += one.work;
          std::push_heap(heap.begin(), heap.end(), later);
        }
      }
      items.clear();
      cta_begin.assign(1, 0);
      int64_t longest = 0;
      for (const auto &list : per_cta)
      {
        items.insert(items.end(), list.begin(), list.end());
        cta_begin.push_back(static_cast<int32_t>(items.size()));
        longest = std::max<int64_t>(longest, static_cast<int64_t>(list.size()));
      }
      ct.n_ctas = ctas;
      ct.longest = longest;
      ct.n_items = static_cast<int64_t>(items.size());
      ct.n_reduces = n_reduces;
      ct.first_tiles = first_tiles;
      ct.slots = cut.slots;
      staging.add(items, reinterpret_cast<void **>(const_cast<ChainItem **>(&ct.items)));
      staging.add(cta_begin, reinterpret_cast<void **>(const_cast<int32_t **>(&ct.cta_begin)));
      staging.add(reduces, reinterpret_cast<void **>(const_cast<ChainReduce **>(&ct.reduces)));
      return true;
    }

    // relabel[in] = out for every entry a move's tiles copy (one tile chunk per CTA; the offsets
    // are the mixed-radix sums of the tiles kernel, kernels.cu).
    __device__ int64_t mixed_radix(const Tile &t, int32_t first, int32_t last, int32_t index)
    {
      int64_t off = 0;
      for (int32_t l = last; l >= first; --l)
      {
        const int32_t e = t.extent[l];
        off += static_cast<int64_t>(index % e) * t.stride[l];
        index /= e;
      }
      return off;
    }

    __global__ void relabel_kernel(const Tile *__restrict__ tiles, const TileChunk *__restrict__ chunks,
                                   int32_t *__restrict__ relabel, int64_t n_from)
    {
      const TileChunk ch = chunks[blockIdx.x];
      const Tile &t = tiles[ch.tile];
      if (t.in_base < 0) return;  // the zero pad entry of an odd block
      const int32_t n = ch.nrows * t.cols;
      for (int32_t e = threadIdx.x; e < n; e += blockDim.x)
      {
        const int32_t r = e / t.cols, c = e - r * t.cols;
        const int64_t in = t.in_base + mixed_radix(t, 0, t.n_row - 1, ch.row0 + r) + mixed_radix(t, t.n_row, t.n_row + t.n_col - 1, c);
        if (in >= 0 && in < n_from)
          relabel[in] = static_cast<int32_t>(t.out_base + static_cast<int64_t>(ch.row0 + r) * t.out_ld + c);
      }
    }

    // The relabelling table (t.mutex held): filled on the library's own stream and waited for, so
    // that launches on any stream read it complete.
    cudaError_t build_relabel(const Program &p, DeviceTables &t)
    {
      DeviceTables::ChainTables &ct = t.chain;
      if (ct.relabel_tried) return cudaSuccess;
      ct.relabel_tried = true;
      if (p.chain_first < 0) return cudaSuccess;
      const Op &first = p.ops[static_cast<size_t>(p.chain_first)];
      const Op &move = p.ops[static_cast<size_t>(p.chain_move)];
      const Op &second = p.ops[static_cast<size_t>(p.chain_second)];
      // the move writes every entry of X' (the compiler zeroes a destination a move does not cover
      // before it, and such a program is not a chain): check the count of entries at least
      int64_t covered = 0, read = 0;
      for (int64_t c = move.begin; c < move.begin + move.count; ++c)
      {
        const TileChunk &ch = p.tile_chunks[static_cast<size_t>(c)];
        const Tile &tile = p.tiles[static_cast<size_t>(ch.tile)];
        if (tile.in_base >= 0) covered += static_cast<int64_t>(ch.nrows) * tile.cols;
      }
      std::set<int64_t> a_blocks;
      for (int64_t b = second.begin; b < second.begin + second.count; ++b)
      {
        const GemmBlock &blk = p.gemm_blocks[static_cast<size_t>(b)];
        for (int32_t q = 0; q < blk.pair_count; ++q)
        {
          const GemmPair &pr = p.gemm_pairs[static_cast<size_t>(blk.pair_begin + q)];
          if (a_blocks.insert(pr.a).second) read += static_cast<int64_t>(blk.m) * pr.k;
        }
      }
      if (covered < read) return cudaSuccess;
      ct.moved_from = p.buffers[static_cast<size_t>(first.dst)].size;
      cudaStream_t stream = nullptr;
      cudaError_t e = upload_stream(&stream);
      if (e != cudaSuccess) return e;
      void *relabel = nullptr;
      if ((e = cudaMalloc(&relabel, static_cast<size_t>(std::max<int64_t>(ct.moved_from, 1)) * 4)) != cudaSuccess) return e;
      ct.relabel_base = relabel;
      ct.relabel = static_cast<int32_t *>(relabel);
      if ((e = cudaMemsetAsync(relabel, 0xff, static_cast<size_t>(ct.moved_from) * 4, stream)) != cudaSuccess) return e;
      if (move.count > 0)
      {
        relabel_kernel<<<static_cast<unsigned>(move.count), 256, 0, stream>>>(t.tiles, t.tile_chunks + move.begin,
                                                                             static_cast<int32_t *>(relabel), ct.moved_from);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
      }
      if ((e = cudaStreamSynchronize(stream)) != cudaSuccess) return e;
      ct.relabel_ok = true;
      return cudaSuccess;
    }

    cudaError_t ensure_chain(const Program &p, DeviceTables &t)
    {
      std::lock_guard<std::mutex> lock(t.mutex);
      DeviceTables::ChainTables &ct = t.chain;
      if (ct.tried) return cudaSuccess;
      ct.tried = true;
      if (p.chain_first < 0) return cudaSuccess;
      cudaError_t e = build_relabel(p, t);
      if (e != cudaSuccess || !ct.relabel_ok) return e;
      TableStaging staging;
      std::vector<ChainItem> items;
      std::vector<int32_t> cta_begin;
      std::vector<ChainReduce> reduces;
      if (!build_chain(p, ct, staging, items, cta_begin, reduces)) return cudaSuccess;
      if ((e = staging.commit(&ct.base)) != cudaSuccess) return e;
      ct.ok = true;
      return cudaSuccess;
    }
  } // namespace

  // ------------------------------------------------------------------------------------------
  // device
  // ------------------------------------------------------------------------------------------

  namespace
  {
    // One program of a launch: its operands, tables, scratch and counters.
    struct ChainWindow
    {
      const double *a1, *b1, *b2;
      double *moved, *c;
      const int32_t *relabel;
      const DevBlock *blocks;
      const DevPair *pairs;
      const ChainReduce *reduces;
      double *partial;
      int *tickets;         // one per reduce (left zero by the last finisher of the tile)
      int *done;            // first-product tiles done so far (reset by the last CTA out)
      int32_t first_tiles;  // first-product tiles (items that cover their tile, and reductions)
      int32_t accumulators; // partial-tile accumulators (32 x 32 doubles each, one per cut tile)
    };
    // A launch: the dealt items of every program (ChainItem::window names its program) and the
    // programs themselves, passed by value (a kernel parameter of a few KiB).
    struct ChainLaunch
    {
      const ChainItem *items;
      const int32_t *cta_begin;
      int *exit_count;  // CTAs done (reset by the last)
      int *error;       // set when a wait gave up
      int *zeroed;      // CTAs that zeroed their share of the accumulators (reset by the last out)
      int32_t windows;
      ChainWindow w[kChainBatch];
    };

    constexpr unsigned long long kWaitLimitNs = 2000000000ull;  // two seconds

    __device__ __forceinline__ void chain_sync(int worker)
    {
      asm volatile("bar.sync %0, %1;\n" ::"r"(worker + 1), "r"(kChainThreads) : "memory");
    }
    // The next entry of the CTA's own list for a worker.
    __device__ __forceinline__ int64_t chain_claim(int worker, int lt, int *slot, int *taken)
    {
      if (lt == 0) *slot = atomicAdd(taken, 1);
      chain_sync(worker);
      const int64_t idx = *slot;
      chain_sync(worker);
      return idx;
    }

    __device__ __forceinline__ unsigned long long global_ns()
    {
      unsigned long long t;
      asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
      return t;
    }
    __device__ __forceinline__ int load_acquire(const int *p)
    {
      int v;
      asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
      return v;
    }

    // One entry of a finished tile: a first-product entry at its place after the move (nowhere when
    // the move drops it), a second-product entry in its block of C.
    __device__ __forceinline__ void store_entry(const ChainWindow &a, int stage, const DevBlock &blk, int gm, int gn, double v)
    {
      const int64_t at = blk.c + static_cast<int64_t>(gm) * blk.n + gn;
      if (stage == 0)
      {
        const int32_t to = a.relabel[at];
        if (to >= 0) a.moved[to] = v;
      }
      else
        a.c[at] = v;
    }

    // A second-product tile that covers the end of its block (tile extents rows | cols << 8) writes
    // the block's alignment pad.
    __device__ __forceinline__ void store_pad(const ChainWindow &a, int stage, const DevBlock &blk, int m0, int n0, int extents, int lt)
    {
      const int64_t entries = static_cast<int64_t>(blk.m) * blk.n;
      if (stage == 1 && lt == 0 && m0 + (extents & 0xff) >= blk.m && n0 + (extents >> 8) >= blk.n && (entries & 1))
        a.c[blk.c + entries] = 0.0;
    }

    // First-product tiles complete in the moved layout are counted per worker and program in
    // shared memory (`pending`, the worker's row) and published once, before the worker's first
    // wait and at its end: every thread's fence orders its stores before the counts (a
    // second-product item waits for all of its program's first-product tiles, so publishing each
    // tile as it completes would gain nothing).
    __device__ __forceinline__ void publish_done(const ChainLaunch &L, int *pending, int worker, int lt)
    {
      __threadfence();
      chain_sync(worker);
      if (lt == 0)
        for (int w = 0; w < L.windows; ++w)
          if (pending[w] != 0)
          {
            atomicAdd(L.w[w].done, pending[w]);
            pending[w] = 0;
          }
      chain_sync(worker);
    }

    // A worker waits until a counter reaches its target (one thread polls with acquire loads, the
    // worker's barrier releases the rest); after two seconds it raises the error flag and goes on.
    // A second-product item waits until every first-product tile of its program is done.
    __device__ __forceinline__ void wait_count(const int *count, int target, int *error, int worker, int lt)
    {
      if (lt == 0)
      {
        const unsigned long long start = global_ns();
        while (load_acquire(count) < target)
        {
          if (global_ns() - start > kWaitLimitNs)
          {
            atomicExch(error, 1);
            break;
          }
          __nanosleep(128);
        }
      }
      chain_sync(worker);
      __threadfence();
    }
    __device__ __forceinline__ void wait_first(const ChainWindow &a, int *error, int worker, int lt)
    {
      wait_count(a.done, a.first_tiles, error, worker, lt);
    }

    // After a worker added its partial tile into the tile's accumulator (zeroed at the start of
    // the launch): the worker holding the tile's last ticket reads the sum and stores the tile
    // (first-product tiles through the move, counted).  The partial tiles are summed by FP64
    // atomic additions in L2, in the order their items finish: a tile's value is the same up to
    // the rounding of that order (a few units in the last place over its K chunks), while a sum
    // of separate partial tiles by the last finisher would cost it a round trip to L2 per group of
    // partials at the end of the product.  The move's targets of the tile's entries are read
    // before the ticket, to overlap that latency.
    __device__ void finish_chain_partial(const ChainWindow &a, int window, int *pending, int worker, int lt, int *flag, int reduce)
    {
      constexpr int BN = kChainTile, PER = kChainTile * kChainTile / kChainThreads;
      const ChainReduce r = a.reduces[reduce];
      const DevBlock blk = a.blocks[r.block];
      int64_t at[PER];
#pragma unroll
      for (int k = 0; k < PER; ++k)
      {
        const int e = lt + k * kChainThreads, tr = e / BN, tc = e % BN;
        const int gm = r.m0 + tr, gn = r.n0 + tc;
        at[k] = -1;
        if (tr < (r.pad0 & 0xff) && tc < (r.pad0 >> 8) && gm < blk.m && gn < blk.n)
        {
          at[k] = blk.c + static_cast<int64_t>(gm) * blk.n + gn;
          if (r.stage == 0) at[k] = __ldg(a.relabel + at[k]);
        }
      }
      __threadfence();
      chain_sync(worker);
      if (lt == 0) *flag = atomicAdd(a.tickets + reduce, 1) == r.nslots - 1;
      chain_sync(worker);
      const bool last = *flag;
      chain_sync(worker);
      if (!last) return;
      if (lt == 0) a.tickets[reduce] = 0;
      __threadfence();
      double *sum = a.partial + static_cast<int64_t>(reduce) * kChainTile * kChainTile + lt;
      double v[PER];
#pragma unroll
      for (int k = 0; k < PER; ++k) v[k] = __ldcg(sum + k * kChainThreads);
#pragma unroll
      for (int k = 0; k < PER; ++k)
        if (at[k] >= 0) (r.stage == 0 ? a.moved : a.c)[at[k]] = v[k];
      store_pad(a, r.stage, blk, r.m0, r.n0, r.pad0, lt);
      if (r.stage == 0 && lt == 0) ++pending[window];
    }

    // A worker's place in an item: the block pair of its next K step, that step's first K within
    // the pair and the end of the item's range in the pair.
    struct Cursor
    {
      int32_t pi, kbase;  // the pair (index within the block) and its first K in the block's sum
      int32_t k0, hi, K;  // the step's first K within the pair, the range's end there, the pair's K
      int64_t a_off, b_off;
    };

    // The first step at or after pair c.pi (whose first K in the block's sum is c.kbase) that lies
    // in the item's range; false when there is none.
    __device__ __forceinline__ bool seek(const ChainWindow &a, const ChainItem &it, const DevBlock &blk, Cursor &c)
    {
      for (; c.pi < blk.pair_count; ++c.pi)
      {
        const DevPair pr = a.pairs[blk.pair_begin + c.pi];
        const int32_t lo = max(it.k0 - c.kbase, 0), hi = min(it.k1 - c.kbase, pr.k);
        if (lo < hi)
        {
          c.k0 = lo;
          c.hi = hi;
          c.K = pr.k;
          c.a_off = pr.a;
          c.b_off = pr.b;
          return true;
        }
        c.kbase += pr.k;
      }
      return false;
    }
    __device__ __forceinline__ bool first_step(const ChainWindow &a, const ChainItem &it, const DevBlock &blk, Cursor &c)
    {
      c.pi = 0;
      c.kbase = 0;
      return seek(a, it, blk, c);
    }
    __device__ __forceinline__ bool next_step(const ChainWindow &a, const ChainItem &it, const DevBlock &blk, Cursor &c)
    {
      c.k0 += kDmmaStepK;
      if (c.k0 < c.hi) return true;
      c.kbase += c.K;
      ++c.pi;
      return seek(a, it, blk, c);
    }

    constexpr int kStageP = 36;                                      // shared row pitch (doubles)
    constexpr int kXPer = kChainTile * kDmmaStepK / kChainThreads;  // a thread's X' entries of a step

    // One K step's operands into a shared stage: the first product's both sides and the second's B
    // side by cp.async (one group, committed by the caller); the second's A side (X', written during
    // the launch by other SMs) by L2 loads into `xa`, which put_x stores once the stage is free.
    __device__ __forceinline__ void load_step(const ChainWindow &a, const ChainItem &it, const DevBlock &blk, const Cursor &c,
                                              double *as, double *bs, int lt, double (&xa)[kXPer])
    {
      constexpr int BM = kChainTile, BN = kChainTile, BK = kDmmaStepK, P = kStageP;
      const bool second = it.stage == 1;
      const double *pa = (second ? a.moved : a.a1) + c.a_off;
      const double *pb = (second ? a.b2 : a.b1) + c.b_off;
      const int th = it.pad & 0xff, tw = it.pad >> 8;
      if (second)
      {
#pragma unroll
        for (int j = 0; j < kXPer; ++j)
        {
          const int i = lt + j * kChainThreads, r = i / BK, kk = i % BK;
          const int gm = it.m0 + r, gk = c.k0 + kk;
          xa[j] = (r < th && gm < blk.m && gk < c.hi) ? __ldcg(pa + static_cast<int64_t>(gm) * c.K + gk) : 0.0;
        }
      }
      else
        for (int i = lt; i < th * BK; i += kChainThreads)
        {
          const int r = i / BK, kk = i % BK;
          const int gm = it.m0 + r, gk = c.k0 + kk;
          const bool in = gm < blk.m && gk < c.hi;
          copy8(as + kk * P + r, in ? pa + static_cast<int64_t>(gm) * c.K + gk : pa, in);
        }
      for (int i = lt; i < BK * tw; i += kChainThreads)
      {
        const int kk = i / tw, cc = i - kk * tw;
        const int gk = c.k0 + kk, gn = it.n0 + cc;
        const bool in = gk < c.hi && gn < blk.n;
        copy8(bs + kk * P + cc, in ? pb + static_cast<int64_t>(gk) * blk.n + gn : pb, in);
      }
    }
    __device__ __forceinline__ void put_x(double *as, int lt, const double (&xa)[kXPer])
    {
#pragma unroll
      for (int j = 0; j < kXPer; ++j)
      {
        const int i = lt + j * kChainThreads;
        as[(i % kDmmaStepK) * kStageP + i / kDmmaStepK] = xa[j];
      }
    }

    // An item's tile as the worker computes it.  Its live entries (rows x cols of the block) times
    // R phases of K (R a power of two, the most that fit the worker's 2048 slots, at most the 32 K of
    // a step) are the slots: slot v = entry * R + phase sums the products at K = phase, phase + R, ...
    // of every step, so that a small tile still gives each thread up to eight independent chains
    // (the FP64 unit of an SM quarter serves every warp on it in turn: a lone chain of dependent
    // multiply-adds waits behind all of them).  Thread lt holds slots lt, lt + 256, ... (at most
    // kPer, packed row | column << 8 | phase << 16); the phases of an entry are summed in order at
    // the end of the item.
    struct Layout
    {
      int mine, cols, live, shift;
      int at[kPer];
    };
    __device__ __forceinline__ void layout_of(const ChainItem &it, const DevBlock &blk, int lt, Layout &l)
    {
      const int rows = min(it.pad & 0xff, blk.m - it.m0), cols = min(it.pad >> 8, blk.n - it.n0);
      const int live = rows * cols;
      int shift = 0;
      while (shift < 5 && (live << (shift + 1)) <= kSlots) ++shift;
      const int slots = live << shift;
      l.cols = cols;
      l.live = live;
      l.shift = shift;
      l.mine = slots > lt ? (slots - lt + kChainThreads - 1) / kChainThreads : 0;
#pragma unroll
      for (int i = 0; i < kPer; ++i)
      {
        const int v = min(lt + i * kChainThreads, max(slots - 1, 0));
        const int e = v >> shift, r = e / cols;
        l.at[i] = r | (e - r * cols) << 8 | (v & ((1 << shift) - 1)) << 16;
      }
    }

    // The items of both products, each a 32 x 32 tile over a K range: K in steps of 32 through two
    // shared stages per worker, the next step's operands (the next item's first step at the end of
    // an item) in flight while a step is computed, and the tile's live entries computed by FP64
    // fused multiply-adds, eight per thread.  GB300's FP64 pipe is shared by DMMA and DFMA and
    // measured faster for DFMA (1.05 against 1.17 TFLOP/s on register operands, 1.05 against 1.20
    // fed from shared memory), and an entry costs one lane: a 16 x 8 DMMA fragment would spend its
    // whole width on the ragged edges of the small blocks of a two-site matvec (1.16 times the
    // products' multiply-adds at bond 256).  The first product's operands and the second's B side
    // are read-only during the launch and staged with cp.async; the second's A side (X', written
    // during the launch by other SMs) is read with L2 loads, so that no SM reads a stale copy of a
    // line from its L1.  A second-product item is waited for (its program's first-product tiles all
    // done) only once the worker's current item is finished when that item is a first-product one.
    __global__ void __launch_bounds__(kChainWorkers * kChainThreads, 1) chain_fp64_kernel(const __grid_constant__ ChainLaunch L)
    {
      dependent_entry();
      constexpr int BK = kDmmaStepK, P = kStageP, BN = kChainTile, BM = kChainTile;
      extern __shared__ __align__(16) unsigned char smem_raw[];
      const int worker = threadIdx.x / kChainThreads, lt = threadIdx.x % kChainThreads;
      double *stage_base = reinterpret_cast<double *>(smem_raw) + static_cast<size_t>(worker) * (2 * 2 * BK * P + kSlots);
      __shared__ int flags[kChainWorkers];
      __shared__ int next[kChainWorkers];
      __shared__ int taken;
      __shared__ int last_out;
      // first-product tiles done and not yet published, per worker and program
      __shared__ int pending_all[kChainWorkers * kChainBatch];
      int *pending = pending_all + worker * kChainBatch;
      if (threadIdx.x == 0) taken = 0;
      for (int w = threadIdx.x; w < kChainWorkers * kChainBatch; w += blockDim.x) pending_all[w] = 0;
      // the partial-tile accumulators (in the workspace's scratch, which other launches also use)
      // zeroed by all CTAs together before any item adds into them
      for (int w = 0; w < L.windows; ++w)
      {
        const int64_t n = static_cast<int64_t>(L.w[w].accumulators) * kChainTile * kChainTile;
        for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += static_cast<int64_t>(gridDim.x) * blockDim.x)
          __stcg(L.w[w].partial + i, 0.0);
      }
      __threadfence();
      __syncthreads();
      if (threadIdx.x == 0) atomicAdd(L.zeroed, 1);
      const int64_t list_begin = L.cta_begin[blockIdx.x], list_end = L.cta_begin[blockIdx.x + 1];
      const auto stage_a = [&](int buf) { return stage_base + buf * 2 * BK * P; };
      // the phase sums of a finished item (kSlots doubles after the worker's two stages)
      double *scratch = stage_base + 2 * 2 * BK * P;
      bool zero_seen = false;  // set once the partial-tile accumulators are known to be zeroed
      const auto stage_b = [&](int buf) { return stage_base + buf * 2 * BK * P + BK * P; };

      // the epilogue of a finished item (`val` holds its slots, then its entries): the phases of
      // each entry summed (through `scratch` when there are several),
      // then its entries stored (through the move for the first product, and counted) or its
      // partial tile written and, by the tile's last finisher, summed
      const auto finish = [&](const ChainItem &it, const DevBlock &blk, const Layout &l, double (&val)[kPer], double *scratch)
      {
        const ChainWindow &a = L.w[it.window];
        if (l.shift != 0)
        {
#pragma unroll
          for (int i = 0; i < kPer; ++i)
            if (i < l.mine) scratch[lt + i * kChainThreads] = val[i];
          chain_sync(worker);
          const int phases = 1 << l.shift;
#pragma unroll
          for (int j = 0; j < kPer; ++j)
          {
            const int e = lt + j * kChainThreads;
            double sum = 0.0;
            if (e < l.live)
              for (int q = 0; q < phases; ++q) sum += scratch[(e << l.shift) + q];
            val[j] = sum;
          }
          chain_sync(worker);  // the scratch is written again after this
        }
        const int entries = l.live > lt ? (l.live - lt + kChainThreads - 1) / kChainThreads : 0;
        if (it.slot >= 0)
        {
          // added into the tile's accumulator, once every CTA has zeroed its share
          if (!zero_seen)
          {
            wait_count(L.zeroed, static_cast<int>(gridDim.x), L.error, worker, lt);
            zero_seen = true;
          }
          double *out = a.partial + static_cast<int64_t>(it.reduce) * BM * BN;
#pragma unroll
          for (int j = 0; j < kPer; ++j)
            if (j < entries)
            {
              const int e = lt + j * kChainThreads, r = e / l.cols;
              atomicAdd(out + r * BN + (e - r * l.cols), val[j]);
            }
          finish_chain_partial(a, it.window, pending, worker, lt, flags + worker, it.reduce);
          return;
        }
#pragma unroll
        for (int j = 0; j < kPer; ++j)
          if (j < entries)
          {
            const int e = lt + j * kChainThreads, r = e / l.cols;
            store_entry(a, it.stage, blk, it.m0 + r, it.n0 + (e - r * l.cols), val[j]);
          }
        store_pad(a, it.stage, blk, it.m0, it.n0, it.pad, lt);
        if (it.stage == 0 && lt == 0) ++pending[it.window];
      };

      // claim the worker's next item, wait for it when it is a second-product one, and place its
      // first step; items with no K (a block that no pair feeds) are stored as zeros on the way
      ChainItem it{};
      DevBlock blk{};
      Cursor cur{};
      double xa[kXPer];
      // set once the worker's first-product counts are published (the CTA's list holds all its
      // first-product items first)
      bool published = false;
      const auto open = [&]() -> bool
      {
        for (;;)
        {
          const int64_t idx = list_begin + chain_claim(worker, lt, next + worker, &taken);
          if (idx >= list_end) return false;
          it = L.items[idx];
          blk = L.w[it.window].blocks[it.block];
          if (it.stage == 1)
          {
            if (!published) publish_done(L, pending, worker, lt);
            published = true;
            wait_first(L.w[it.window], L.error, worker, lt);
          }
          if (first_step(L.w[it.window], it, blk, cur)) return true;
          Layout l;
          layout_of(it, blk, lt, l);
          l.shift = 0;  // nothing to sum
          double zero[kPer];
#pragma unroll
          for (int i = 0; i < kPer; ++i) zero[i] = 0.0;
          finish(it, blk, l, zero, nullptr);
        }
      };

      int buf = 0;
      bool have = open();
      if (have)
      {
        load_step(L.w[it.window], it, blk, cur, stage_a(0), stage_b(0), lt, xa);
        if (it.stage == 1) put_x(stage_a(0), lt, xa);
      }
      copy_commit();
      while (have)
      {
        Layout l;
        layout_of(it, blk, lt, l);
        double acc[kPer];
#pragma unroll
        for (int i = 0; i < kPer; ++i) acc[i] = 0.0;
        // the steps of the item; `follow` is set when the next item's first step was prefetched
        bool follow = false, have_next = false;
        ChainItem nit{};
        DevBlock nblk{};
        Cursor ncur{};
        for (;;)
        {
          Cursor step = cur;
          const bool more = next_step(L.w[it.window], it, blk, step);
          bool pending_x = false;
          if (more)
          {
            load_step(L.w[it.window], it, blk, step, stage_a(buf ^ 1), stage_b(buf ^ 1), lt, xa);
            pending_x = it.stage == 1;
          }
          else
          {
            // the item's last step: claim the next item now and prefetch its first step unless it
            // would wait on first-product tiles while this worker still holds one
            const int64_t idx = list_begin + chain_claim(worker, lt, next + worker, &taken);
            have_next = idx < list_end;
            if (have_next)
            {
              nit = L.items[idx];
              nblk = L.w[nit.window].blocks[nit.block];
              if ((nit.stage == 0 || it.stage == 1))
              {
                if (nit.stage == 1)
                {
                  if (!published) publish_done(L, pending, worker, lt);
                  published = true;
                  wait_first(L.w[nit.window], L.error, worker, lt);
                }
                if (first_step(L.w[nit.window], nit, nblk, ncur))
                {
                  load_step(L.w[nit.window], nit, nblk, ncur, stage_a(buf ^ 1), stage_b(buf ^ 1), lt, xa);
                  pending_x = nit.stage == 1;
                  follow = true;
                }
              }
            }
          }
          copy_commit();  // an empty group when nothing was issued keeps the count of the wait below
          copy_wait_one();
          chain_sync(worker);
          {
            const double(*as)[P] = reinterpret_cast<const double(*)[P]>(stage_a(buf));
            const double(*bs)[P] = reinterpret_cast<const double(*)[P]>(stage_b(buf));
            const int steps = min(BK, cur.hi - cur.k0);
            if (l.shift == 0 && l.mine == kPer && l.cols == BN)
            {
              // a full tile: the thread's entries share one column
              const int c = (l.at[0] >> 8) & 0xff;
#pragma unroll 4
              for (int kk = 0; kk < steps; ++kk)
              {
                const double b = bs[kk][c];
#pragma unroll
                for (int i = 0; i < kPer; ++i) acc[i] = fma(as[kk][l.at[i] & 0xff], b, acc[i]);
              }
            }
            else
            {
              const int phases = 1 << l.shift;
              for (int kb = 0; kb < steps; kb += phases)
              {
#pragma unroll
                for (int i = 0; i < kPer; ++i)
                {
                  const int kk = kb + (l.at[i] >> 16);
                  if (i < l.mine && kk < steps) acc[i] = fma(as[kk][l.at[i] & 0xff], bs[kk][(l.at[i] >> 8) & 0xff], acc[i]);
                }
              }
            }
          }
          chain_sync(worker);
          if (pending_x) put_x(stage_a(buf ^ 1), lt, xa);
          buf ^= 1;
          if (!more) break;
          cur = step;
        }
        finish(it, blk, l, acc, scratch);
        if (!have_next) break;
        if (follow)
        {
          it = nit;
          blk = nblk;
          cur = ncur;
          continue;
        }
        // the claimed item was not prefetched (a second-product item after a first-product one,
        // or one with no K): wait for it now, then go on from it
        it = nit;
        blk = nblk;
        if (it.stage == 1)
        {
          if (!published) publish_done(L, pending, worker, lt);
          published = true;
          wait_first(L.w[it.window], L.error, worker, lt);
        }
        if (!first_step(L.w[it.window], it, blk, cur))
        {
          Layout z;
          layout_of(it, blk, lt, z);
          z.shift = 0;  // nothing to sum
          double zero[kPer];
#pragma unroll
          for (int i = 0; i < kPer; ++i) zero[i] = 0.0;
          finish(it, blk, z, zero, nullptr);
          have = open();
          if (!have) break;
        }
        load_step(L.w[it.window], it, blk, cur, stage_a(buf), stage_b(buf), lt, xa);
        if (it.stage == 1) put_x(stage_a(buf), lt, xa);
        copy_commit();
      }
      if (!published) publish_done(L, pending, worker, lt);
      // the last CTA to leave resets the done counts and the exit count for the next launch
      __syncthreads();
      if (threadIdx.x == 0)
      {
        __threadfence();
        last_out = atomicAdd(L.exit_count, 1) == static_cast<int>(gridDim.x) - 1;
      }
      __syncthreads();
      if (last_out)
      {
        __threadfence();
        for (int w = threadIdx.x; w < L.windows; w += blockDim.x) *L.w[w].done = 0;
        if (threadIdx.x == 0)
        {
          *L.exit_count = 0;
          *L.zeroed = 0;
        }
      }
    }

    constexpr int kChainPinBytes = 120 * 1024;  // one CTA per SM

    ChainWindow window_of(const Program &p, const DeviceTables &t, const double *A1, const double *B1, double *moved,
                          const double *B2, double *C, void *workspace)
    {
      const DeviceTables::ChainTables &ct = t.chain;
      ChainWindow w{};
      w.a1 = A1;
      w.b1 = B1;
      w.b2 = B2;
      w.moved = moved;
      w.c = C;
      w.relabel = ct.relabel;
      w.blocks = reinterpret_cast<const DevBlock *>(t.blocks);
      w.pairs = reinterpret_cast<const DevPair *>(t.pairs);
      w.reduces = ct.reduces;
      w.partial = reinterpret_cast<double *>(static_cast<char *>(workspace) + p.scratch_offset * 8);
      w.tickets = static_cast<int *>(workspace);
      w.done = w.tickets + ct.n_reduces;
      w.first_tiles = static_cast<int32_t>(ct.first_tiles);
      w.accumulators = static_cast<int32_t>(ct.n_reduces);
      return w;
    }

    cudaError_t launch_chain(const ChainLaunch &launch, int32_t n_ctas, int64_t longest, cudaStream_t stream)
    {
      const int bytes = std::max<int>(kChainWorkers * (2 * 2 * kDmmaStepK * kStageP + kSlots) * 8, kChainPinBytes);
      static std::once_flag once;
      cudaError_t e = cudaSuccess;
      std::call_once(once, [&] { e = cudaFuncSetAttribute(chain_fp64_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes); });
      if (e != cudaSuccess) return e;
      const int workers = static_cast<int>(std::clamp<int64_t>(longest, 1, kChainWorkers));
      return launch_dependent(chain_fp64_kernel, n_ctas, workers * kChainThreads, bytes, stream, launch);
    }

    // The deal of a batch's items, per list of programs.
    struct BatchDeal
    {
      void *base = nullptr;
      const ChainItem *items = nullptr;
      const int32_t *cta_begin = nullptr;
      int32_t n_ctas = 0;
      int64_t longest = 0;
    };
    std::mutex batch_mutex;
    std::map<std::vector<const DeviceTables *>, BatchDeal> batch_deals;
  } // namespace

  // ------------------------------------------------------------------------------------------
  // host: launches
  // ------------------------------------------------------------------------------------------

  cudaError_t chain_relabel(const Program &p, DeviceTables &t, const int32_t **relabel)
  {
    *relabel = nullptr;
    std::lock_guard<std::mutex> lock(t.mutex);
    const cudaError_t e = build_relabel(p, t);
    if (e == cudaSuccess && t.chain.relabel_ok) *relabel = t.chain.relabel;
    return e;
  }

  void clear_chain_batches()
  {
    std::lock_guard<std::mutex> lock(batch_mutex);
    for (auto &entry : batch_deals)
      if (entry.second.base) cudaFree(entry.second.base);
    batch_deals.clear();
  }

  cudaError_t launch_chain_f64(const Program &p, DeviceTables &t, const double *A1, const double *B1, double *moved,
                               const double *B2, double *C, void *workspace, cudaStream_t stream, bool *used)
  {
    *used = false;
    cudaError_t e = ensure_chain(p, t);
    if (e != cudaSuccess) return e;
    const DeviceTables::ChainTables &ct = t.chain;
    if (!ct.ok || ct.n_items == 0) return cudaSuccess;
    ChainLaunch launch{};
    launch.items = ct.items;
    launch.cta_begin = ct.cta_begin;
    launch.windows = 1;
    launch.w[0] = window_of(p, t, A1, B1, moved, B2, C, workspace);
    launch.exit_count = launch.w[0].done + 1;
    launch.error = launch.exit_count + 1;
    launch.zeroed = launch.error + 1;
    e = launch_chain(launch, ct.n_ctas, ct.longest, stream);
    if (e == cudaSuccess) *used = true;
    return e;
  }

  cudaError_t launch_chain_batch(const std::vector<ChainBatchEntry> &entries, cudaStream_t stream, bool *used)
  {
    *used = false;
    if (entries.empty() || entries.size() > static_cast<size_t>(kChainBatch)) return cudaSuccess;
    std::vector<const DeviceTables *> key;
    for (const ChainBatchEntry &en : entries)
    {
      const cudaError_t e = ensure_chain(*en.program, *en.tables);
      if (e != cudaSuccess) return e;
      if (!en.tables->chain.ok) return cudaSuccess;
      key.push_back(en.tables);
    }
    BatchDeal deal;
    {
      std::lock_guard<std::mutex> lock(batch_mutex);
      auto found = batch_deals.find(key);
      if (found == batch_deals.end())
      {
        // every program's first-product items, largest first, each to the least loaded SM; then the
        // second-product items the same way; each SM's list keeps that order
        struct Tagged
        {
          ChainItem item;
          double work;
        };
        std::vector<Tagged> stage[2];
        for (size_t w = 0; w < entries.size(); ++w)
        {
          const DeviceTables::ChainTables &ct = entries[w].tables->chain;
          for (size_t i = 0; i < ct.host_items.size(); ++i)
          {
            ChainItem it = ct.host_items[i];
            it.window = static_cast<int32_t>(w);
            stage[it.stage == 0 ? 0 : 1].push_back({it, ct.host_work[i]});
          }
        }
        const size_t n_items = stage[0].size() + stage[1].size();
        const int ctas = static_cast<int>(
          std::min<size_t>(static_cast<size_t>(entries.front().program->ctas), std::max<size_t>(n_items, 1)));
        std::vector<std::pair<double, int>> heap;
        for (int c = 0; c < ctas; ++c) heap.push_back({0.0, c});
        const auto later = [](const std::pair<double, int> &a, const std::pair<double, int> &b)
        { return a.first > b.first || (a.first == b.first && a.second > b.second); };
        std::make_heap(heap.begin(), heap.end(), later);
        std::vector<std::vector<ChainItem>> per_cta(static_cast<size_t>(ctas));
        for (std::vector<Tagged> &st : stage)
        {
          std::stable_sort(st.begin(), st.end(), [](const Tagged &a, const Tagged &b) { return a.work > b.work; });
          for (const Tagged &one : st)
          {
            std::pop_heap(heap.begin(), heap.end(), later);
            auto &least = heap.back();
            per_cta[static_cast<size_t>(least.second)].push_back(one.item);
            least.first += one.work;
            std::push_heap(heap.begin(), heap.end(), later);
          }
        }
        std::vector<ChainItem> items;
        std::vector<int32_t> cta_begin{0};
        int64_t longest = 0;
        for (const auto &list : per_cta)
        {
          items.insert(items.end(), list.begin(), list.end());
          cta_begin.push_back(static_cast<int32_t>(items.size()));
          longest = std::max<int64_t>(longest, static_cast<int64_t>(list.size()));
        }
        BatchDeal fresh;
        TableStaging staging;
        staging.add(items, reinterpret_cast<void **>(const_cast<ChainItem **>(&fresh.items)));
        staging.add(cta_begin, reinterpret_cast<void **>(const_cast<int32_t **>(&fresh.cta_begin)));
        const cudaError_t e = staging.commit(&fresh.base);
        if (e != cudaSuccess) return e;
        fresh.n_ctas = ctas;
        fresh.longest = longest;
        found = batch_deals.emplace(key, fresh).first;
      }
      deal = found->second;
    }
    ChainLaunch launch{};
    launch.items = deal.items;
    launch.cta_begin = deal.cta_begin;
    launch.windows = static_cast<int32_t>(entries.size());
    for (size_t w = 0; w < entries.size(); ++w)
    {
      const ChainBatchEntry &en = entries[w];
      launch.w[w] = window_of(*en.program, *en.tables, en.a1, en.b1, en.moved, en.b2, en.c, en.workspace);
    }
    // the launch's exit count and error flag after the first program's done count
    launch.exit_count = launch.w[0].done + 1;
    launch.error = launch.exit_count + 1;
    launch.zeroed = launch.error + 1;
    const cudaError_t e = launch_chain(launch, deal.n_ctas, deal.longest, stream);
    if (e == cudaSuccess) *used = true;
    return e;
  }

} // namespace ttg
