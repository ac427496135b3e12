// Grouped block-pair GEMM for sm_103a: balanced work schedules, the persistent FP64 / complex128
// kernel, the persistent split-precision kernel (exact bf16 slices on mma.sync with exact fp32 level
// sums, folded into FP64), and the slicing pass.  See gemm.h for the numerical scheme.
//
// Both GEMM kernels are persistent: one CTA per SM, held there by its shared-memory request, split
// into independent workers of 128 threads that claim work items from a list sorted largest first
// through an atomic counter.  A tile whose K was cut into several items is reduced by the worker that finishes
// its last item (an atomic ticket per tile): the partials are summed in slot order, so the result
// is deterministic, and no thread ever waits on another CTA.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cstdlib>
#include <numeric>
#include <cmath>
#include <map>
#include <mutex>

#include "executor.h"
#include "gemm.h"
#include "gemm_device.cuh"
#include "launch.h"

namespace ttg
{
  // ------------------------------------------------------------------------------------------
  // schedules (host)
  // ------------------------------------------------------------------------------------------

  namespace
  {
    double op_work(const Program &p, const Op &op)
    {
      double total = 0;
      for (int64_t b = op.begin; b < op.begin + op.count; ++b)
      {
        const GemmBlock &blk = p.gemm_blocks[static_cast<size_t>(b)];
        for (int32_t k = 0; k < blk.pair_count; ++k)
          total += static_cast<double>(blk.m) * blk.n * p.gemm_pairs[static_cast<size_t>(blk.pair_begin + k)].k;
      }
      return total;
    }

    int64_t up256(int64_t bytes) { return (bytes + 255) / 256 * 256; }
  } // namespace

  GemmSchedule schedule_gemm(const Program &p, const Op &op, int bm, int bn, bool full)
  {
    GemmSchedule s;
    // The workers of one SM share its FP64 pipe, so what has to balance is the work per SM: items
    // of a few per SM (a matvec's stage has only ~10^5 multiply-adds per SM), each a tile over a
    // K range of at least 16, dealt to the SMs largest first, each to the least loaded (LPT).
    // Cost of an item: the 16 x 8 DMMA fragments it computes (fragments wholly outside the block are
    // skipped) times its K range, plus per staged K step (its copies and barriers) and per item
    // (claim, write or partial tile) a quarter of a full tile over 16 of K.
    const auto cost = [bm, bn](double rows, double cols, double k)
    {
      const double frag = std::ceil(rows / 16.0) * 16.0 * std::ceil(cols / 8.0) * 8.0;
      return frag * k + 0.25 * bm * bn * 16.0 * (std::ceil(k / kDmmaStepK) + 1.0);
    };
    double total = 0;
    for (int64_t b = op.begin; b < op.begin + op.count; ++b)
    {
      const GemmBlock &blk = p.gemm_blocks[static_cast<size_t>(b)];
      int64_t ktotal = 0;
      for (int32_t k = 0; k < blk.pair_count; ++k) ktotal += p.gemm_pairs[static_cast<size_t>(blk.pair_begin + k)].k;
      for (int32_t m0 = 0; m0 < blk.m; m0 += bm)
        for (int32_t n0 = 0; n0 < blk.n; n0 += bn)
          total += cost(std::min(bm, blk.m - m0), std::min(bn, blk.n - n0), static_cast<double>(ktotal));
    }
    const double target = std::max(total / (p.ctas * 6.0), cost(bm, bn, 16.0));
    struct Sized
    {
      GemmItem item;
      double work;
    };
    std::vector<Sized> items;
    int64_t n_items = 0;
    for (int64_t b = op.begin; b < op.begin + op.count; ++b)
    {
      const GemmBlock &blk = p.gemm_blocks[static_cast<size_t>(b)];
      int64_t ktotal = 0;
      for (int32_t k = 0; k < blk.pair_count; ++k) ktotal += p.gemm_pairs[static_cast<size_t>(blk.pair_begin + k)].k;
      for (int32_t m0 = 0; m0 < blk.m; m0 += bm)
        for (int32_t n0 = 0; n0 < blk.n; n0 += bn)
        {
          const double rows = std::min(bm, blk.m - m0), cols = std::min(bn, blk.n - n0);
          const double work = cost(rows, cols, static_cast<double>(ktotal));
          int64_t chunks = std::max<int64_t>(1, static_cast<int64_t>(std::ceil(work / target)));
          int64_t kc = (ktotal + chunks - 1) / std::max<int64_t>(chunks, 1);
          kc = std::max<int64_t>(16, (kc + 15) / 16 * 16);
          chunks = ktotal > 0 ? (ktotal + kc - 1) / kc : 1;
          const int32_t bi = static_cast<int32_t>(b);
          n_items += chunks;
          if (chunks == 1)
          {
            if (full) items.push_back({{bi, m0, n0, 0, static_cast<int32_t>(ktotal), -1, -1, 0}, work});
            continue;
          }
          const int32_t slot0 = static_cast<int32_t>(s.slots), reduce = static_cast<int32_t>(s.reduces.size());
          for (int64_t c = 0; c < chunks; ++c)
          {
            const int64_t k0 = c * kc, k1 = std::min(ktotal, (c + 1) * kc);
            if (full)
              items.push_back({{bi, m0, n0, static_cast<int32_t>(k0), static_cast<int32_t>(k1), static_cast<int32_t>(s.slots),
                                reduce, 0},
                               cost(rows, cols, static_cast<double>(k1 - k0))});
            ++s.slots;
          }
          s.reduces.push_back({bi, m0, n0, slot0, static_cast<int32_t>(chunks), 0});
        }
    }
    s.n_items = n_items;
    if (!full) return s;
    // largest first, equal work in the order made
    std::vector<int32_t> order(items.size());
    std::iota(order.begin(), order.end(), 0);
    std::sort(order.begin(), order.end(), [&items](int32_t a, int32_t b)
              { return items[static_cast<size_t>(a)].work > items[static_cast<size_t>(b)].work ||
                       (items[static_cast<size_t>(a)].work == items[static_cast<size_t>(b)].work && a < b); });
    // LPT: each item to the CTA with the least work so far (ties to the lower index)
    const int ctas = static_cast<int>(std::min<size_t>(static_cast<size_t>(p.ctas), std::max<size_t>(items.size(), 1)));
    std::vector<std::pair<double, int>> heap;
    heap.reserve(static_cast<size_t>(ctas));
    for (int c = 0; c < ctas; ++c) heap.push_back({0.0, c});
    const auto later = [](const std::pair<double, int> &a, const std::pair<double, int> &b)
    { return a.first > b.first || (a.first == b.first && a.second > b.second); };
    std::make_heap(heap.begin(), heap.end(), later);
    std::vector<int32_t> cta_of(items.size());
    s.cta_begin.assign(static_cast<size_t>(ctas) + 1, 0);
    for (const int32_t i : order)
    {
      std::pop_heap(heap.begin(), heap.end(), later);
      auto &least = heap.back();
      cta_of[static_cast<size_t>(i)] = least.second;
      ++s.cta_begin[static_cast<size_t>(least.second) + 1];
      least.first += items[static_cast<size_t>(i)].work;
      std::push_heap(heap.begin(), heap.end(), later);
    }
    // the lists back to back, each in the order its items were dealt
    for (int c = 0; c < ctas; ++c) s.cta_begin[static_cast<size_t>(c) + 1] += s.cta_begin[static_cast<size_t>(c)];
    std::vector<int32_t> fill(s.cta_begin.begin(), s.cta_begin.end() - 1);
    s.items.resize(items.size());
    for (const int32_t i : order)
      s.items[static_cast<size_t>(fill[static_cast<size_t>(cta_of[static_cast<size_t>(i)])]++)] = items[static_cast<size_t>(i)].item;
    return s;
  }

  void gemm_operands(const Program &p, const Op &op, std::vector<OperandBlock> &left, std::vector<OperandBlock> &right)
  {
    std::map<int64_t, int> seen_a, seen_b;
    left.clear();
    right.clear();
    for (int64_t b = op.begin; b < op.begin + op.count; ++b)
    {
      const GemmBlock &blk = p.gemm_blocks[static_cast<size_t>(b)];
      for (int32_t k = 0; k < blk.pair_count; ++k)
      {
        const GemmPair &pr = p.gemm_pairs[static_cast<size_t>(blk.pair_begin + k)];
        if (seen_a.emplace(pr.a, 0).second) left.push_back({pr.a, blk.m, pr.k});
        if (seen_b.emplace(pr.b, 0).second) right.push_back({pr.b, pr.k, blk.n});
      }
    }
  }

  SplitSchedule schedule_split(const Program &p, const Op &op, bool full)
  {
    SplitSchedule s;
    if (full) s.pairs.assign(p.gemm_pairs.size(), SplitPair{0, 0, 0, 0, 0, 0});
    // slices: every distinct left block as rows of K padded to 32, every distinct right block
    // transposed the same way; exponents: one per row of A, one per column of B
    std::map<int64_t, std::pair<int64_t, int32_t>> a_at, b_at;  // arena offset -> (slice offset, exponent base)
    const auto pad32 = [](int64_t k) { return (k + kSplitStepK - 1) / kSplitStepK * kSplitStepK; };
    std::vector<SplitLine> b_lines;
    for (int64_t bi = op.begin; bi < op.begin + op.count; ++bi)
    {
      const GemmBlock &blk = p.gemm_blocks[static_cast<size_t>(bi)];
      for (int32_t k = 0; k < blk.pair_count; ++k)
      {
        const size_t pi = static_cast<size_t>(blk.pair_begin + k);
        const GemmPair &pr = p.gemm_pairs[pi];
        const int64_t kp = pad32(pr.k);
        auto fa = a_at.find(pr.a);
        if (fa == a_at.end())
        {
          fa = a_at.emplace(pr.a, std::make_pair(s.slice_a, static_cast<int32_t>(s.exps_a))).first;
          for (int32_t r = 0; full && r < blk.m; ++r)
            s.lines.push_back({pr.a + static_cast<int64_t>(r) * pr.k, s.slice_a + r * kp, pr.k, 1, static_cast<int32_t>(kp),
                               static_cast<int32_t>(s.exps_a + r)});
          s.slice_a += (blk.m * kp + 63) / 64 * 64;
          s.exps_a += blk.m;
        }
        auto fb = b_at.find(pr.b);
        if (fb == b_at.end())
        {
          fb = b_at.emplace(pr.b, std::make_pair(s.slice_b, static_cast<int32_t>(s.exps_b))).first;
          for (int32_t c = 0; full && c < blk.n; ++c)
            b_lines.push_back({pr.b + c, s.slice_b + c * kp, pr.k, blk.n, static_cast<int32_t>(kp),
                               static_cast<int32_t>(s.exps_b + c)});
          s.slice_b += (blk.n * kp + 63) / 64 * 64;
          s.exps_b += blk.n;
        }
        if (full)
          s.pairs[pi] = SplitPair{fa->second.first, fb->second.first, static_cast<int32_t>(kp), fa->second.second,
                                  fb->second.second, 0};
      }
    }
    s.exps = s.exps_a + s.exps_b;
    s.lines_a = static_cast<int64_t>(s.lines.size());
    s.lines.insert(s.lines.end(), b_lines.begin(), b_lines.end());
    // items: one pair's K range each (a multiple of 32), about two per worker, never below a tile
    // over 256 of K (one exact level chunk: smaller items cost more in folds and partial tiles than
    // they gain in spread; at bond 512 the split matvec took 147 us with 128 and 123 us with 256)
    const double target =
      std::max(op_work(p, op) / (p.ctas * kSplitWorkers * 2.0), static_cast<double>(kSplitTileM) * kSplitTileN * kExactChunk);
    struct Sized
    {
      SplitItem item;
      double work;
    };
    std::vector<Sized> items, tile;
    for (int64_t bi = op.begin; bi < op.begin + op.count; ++bi)
    {
      const GemmBlock &blk = p.gemm_blocks[static_cast<size_t>(bi)];
      for (int32_t m0 = 0; m0 < blk.m; m0 += kSplitTileM)
        for (int32_t n0 = 0; n0 < blk.n; n0 += kSplitTileN)
        {
          const double rows = std::min(kSplitTileM, blk.m - m0), cols = std::min(kSplitTileN, blk.n - n0);
          // a warp's 16 x 16 quarter outside the block skips its products
          const double quarters = std::ceil(rows / 16.0) * std::ceil(cols / 16.0);
          const auto cost = [quarters](double k)
          { return quarters * 256.0 * (std::ceil(k / kSplitStepK) * kSplitStepK + 2.0 * kSplitStepK * (std::ceil(k / kExactChunk) + 1.0)); };
          tile.clear();
          for (int32_t k = 0; k < blk.pair_count; ++k)
          {
            const int32_t pi = blk.pair_begin + k;
            const int64_t K = p.gemm_pairs[static_cast<size_t>(pi)].k;
            const double work = rows * cols * static_cast<double>(K);
            int64_t chunks = std::max<int64_t>(1, static_cast<int64_t>(std::ceil(work / target)));
            const int64_t kc = pad32((K + chunks - 1) / chunks);
            chunks = (K + kc - 1) / kc;
            for (int64_t c = 0; c < chunks; ++c)
            {
              const int64_t k0 = c * kc, k1 = std::min<int64_t>(K, (c + 1) * kc);
              tile.push_back({{static_cast<int32_t>(bi), m0, n0, pi, static_cast<int32_t>(k0), static_cast<int32_t>(k1), 0, -1},
                              cost(static_cast<double>(k1 - k0))});
            }
          }
          if (tile.size() == 1)
          {
            tile[0].item.slot = -1;
            if (full) items.push_back(tile[0]);
          }
          else if (tile.empty())
          {
            if (full) items.push_back({{static_cast<int32_t>(bi), m0, n0, -1, 0, 0, -1, -1}, cost(0.0)});  // no pair: zeros
          }
          else
          {
            const int32_t slot0 = static_cast<int32_t>(s.slots), reduce = static_cast<int32_t>(s.reduces.size());
            for (Sized &t : tile)
            {
              t.item.slot = static_cast<int32_t>(s.slots++);
              t.item.reduce = reduce;
              if (full) items.push_back(t);
            }
            s.reduces.push_back({static_cast<int32_t>(bi), m0, n0, slot0, static_cast<int32_t>(tile.size()), 0});
          }
        }
    }
    if (!full) return s;
    std::stable_sort(items.begin(), items.end(), [](const Sized &a, const Sized &b) { return a.work > b.work; });
    // dealt to the SMs like the FP64 items (largest first onto the least loaded)
    const int ctas = static_cast<int>(std::min<size_t>(static_cast<size_t>(p.ctas), std::max<size_t>(items.size(), 1)));
    std::vector<std::vector<SplitItem>> lists(static_cast<size_t>(ctas));
    std::vector<std::pair<double, int>> heap;
    for (int c = 0; c < ctas; ++c) heap.push_back({0.0, c});
    const auto later = [](const std::pair<double, int> &a, const std::pair<double, int> &b)
    { return a.first > b.first || (a.first == b.first && a.second > b.second); };
    std::make_heap(heap.begin(), heap.end(), later);
    for (const Sized &it : items)
    {
      std::pop_heap(heap.begin(), heap.end(), later);
      auto &least = heap.back();
      lists[static_cast<size_t>(least.second)].push_back(it.item);
      least.first += it.work;
      std::push_heap(heap.begin(), heap.end(), later);
    }
    s.cta_begin.push_back(0);
    for (const auto &list : lists)
    {
      s.items.insert(s.items.end(), list.begin(), list.end());
      s.cta_begin.push_back(static_cast<int32_t>(s.items.size()));
    }
    return s;
  }

  namespace
  {
    // bytes of split scratch: slices of A and of B (bf16), exponents (int16), partial tiles, tickets
    int64_t split_bytes(const SplitSchedule &s, int slices)
    {
      return up256(2 * slices * s.slice_a) + up256(2 * slices * s.slice_b) + up256(2 * s.exps) +
             up256(s.slots * kSplitTileM * kSplitTileN * 8) + up256(4 * (static_cast<int64_t>(s.reduces.size()) + 1));
    }
    // bytes of FP64 scratch: partial tiles (two doubles an entry for complex), tickets
    int64_t f64_bytes(const GemmSchedule &s)
    {
      return up256(s.slots * kF64TileM * kF64TileN * 16) + up256(4 * (static_cast<int64_t>(s.reduces.size()) + 1));
    }
  } // namespace

  int device_sms()
  {
    static std::atomic<int> cached[64] = {};
    int device = 0;
    if (cudaGetDevice(&device) != cudaSuccess || device < 0 || device >= 64)
    {
      cudaGetLastError();
      return 152;
    }
    int n = cached[device].load(std::memory_order_relaxed);
    if (n > 0) return n;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, device) != cudaSuccess || n <= 0)
    {
      cudaGetLastError();
      return 152;
    }
    cached[device].store(n, std::memory_order_relaxed);
    return n;
  }

  int64_t plan_gemms(Program &p)
  {
    p.ctas = device_sms();
    auto plans = std::make_shared<GemmPlans>();
    plans->f64.resize(p.ops.size());
    plans->split.resize(p.ops.size());
    plans->cache_a.assign(p.ops.size(), -1);
    plans->cache_b.assign(p.ops.size(), -1);
    int64_t need = 0;
    for (size_t i = 0; i < p.ops.size(); ++i)
    {
      const Op &op = p.ops[i];
      if (op.kind != OpKind::gemm) continue;
      plans->f64[i] = schedule_gemm(p, op, kF64TileM, kF64TileN, false);
      // the split schedule itself is built on the first split launch (most plans never run one);
      // here only its scratch
      need = std::max(need, (f64_bytes(plans->f64[i]) + 7) / 8);
      // a chain's one launch holds the partial tiles of both its products at once
      if (static_cast<int32_t>(i) == p.chain_second)
      {
        // its items are cut for the FMA kernel (chain.cu)
        p.chain_slots = chain_partial_slots(p);
        need = std::max(need, (up256(p.chain_slots * kF64TileM * kF64TileN * 8) + 7) / 8);
      }
      const SplitSchedule sizes = schedule_split(p, op, false);
      need = std::max(need, (split_bytes(sizes, kMaxSlices) + 7) / 8);
      // the slices of a prepared operand's value go into its arena
      for (int side = 0; side < 2; ++side)
      {
        const int32_t buffer = side == 0 ? op.src : op.src2;
        if (buffer < 0) continue;
        const int32_t operand = p.buffers[static_cast<size_t>(buffer)].prepared_of;
        if (operand < 0) continue;
        if (plans->prepared_bytes.empty())
        {
          plans->prepared_bytes.assign(static_cast<size_t>(p.n_inputs), 0);
          for (int32_t j = 0; j < p.n_inputs; ++j)
            if (p.prepared[static_cast<size_t>(j)] >= 0)
              plans->prepared_bytes[static_cast<size_t>(j)] = up256(p.buffers[static_cast<size_t>(p.prepared[static_cast<size_t>(j)])].size * 8);
        }
        SliceCache c;
        c.op = static_cast<int32_t>(i);
        c.side = side;
        c.operand = operand;
        c.offset = plans->prepared_bytes[static_cast<size_t>(operand)];
        const int64_t slice = side == 0 ? sizes.slice_a : sizes.slice_b, exps = side == 0 ? sizes.exps_a : sizes.exps_b;
        c.exps_offset = c.offset + up256(2 * kMaxSlices * slice);
        c.bytes = up256(2 * kMaxSlices * slice) + up256(2 * exps);
        plans->prepared_bytes[static_cast<size_t>(operand)] += c.bytes;
        (side == 0 ? plans->cache_a : plans->cache_b)[i] = static_cast<int32_t>(plans->caches.size());
        plans->caches.push_back(c);
      }
    }
    p.gemm_plans = std::move(plans);
    return need;
  }

  // ------------------------------------------------------------------------------------------
  // device
  // ------------------------------------------------------------------------------------------

  namespace
  {
    // After a worker has written a partial tile: take the tile's ticket; the worker holding the last
    // ticket sums every partial of the tile in slot order into C.  The fences order the partial
    // writes before the ticket and the ticket before the reads (reads bypass L1).
    template <typename T, int BM, int BN>
    __device__ void finish_partial(int worker, int lt, int *flag, int *tickets, const GemmReduce *reduces, int reduce,
                                   const DevBlock *blocks, const T *partial, T *C, const int32_t *relabel = nullptr)
    {
      __threadfence();
      worker_sync(worker);
      const GemmReduce r = reduces[reduce];
      if (lt == 0) *flag = atomicAdd(tickets + reduce, 1) == r.nslots - 1;
      worker_sync(worker);
      const bool last = *flag;
      worker_sync(worker);
      if (!last) return;
      // every other partial of the tile has taken its ticket: leave the counter zero for the next launch
      if (lt == 0) tickets[reduce] = 0;
      __threadfence();
      const DevBlock blk = blocks[r.block];
      // every entry of the tile sums its slots in slot order; the loads of four slots for all of the
      // thread's entries are issued together, so a deep split costs a few L2 round trips, not one
      // per slot
      constexpr int PER = BM * BN / kWorkerThreads;
      T sum[PER];
#pragma unroll
      for (int k = 0; k < PER; ++k) sum[k] = zero_t<T>();
      const T *base = partial + static_cast<int64_t>(r.slot0) * BM * BN + lt;
      int s = 0;
      for (; s + 4 <= r.nslots; s += 4)
      {
        T v[4][PER];
#pragma unroll
        for (int u = 0; u < 4; ++u)
#pragma unroll
          for (int k = 0; k < PER; ++k) v[u][k] = __ldcg(base + static_cast<int64_t>(s + u) * BM * BN + k * kWorkerThreads);
#pragma unroll
        for (int u = 0; u < 4; ++u)
#pragma unroll
          for (int k = 0; k < PER; ++k) sum[k] = add_t(sum[k], v[u][k]);
      }
      for (; s < r.nslots; ++s)
#pragma unroll
        for (int k = 0; k < PER; ++k) sum[k] = add_t(sum[k], __ldcg(base + static_cast<int64_t>(s) * BM * BN + k * kWorkerThreads));
#pragma unroll
      for (int k = 0; k < PER; ++k)
      {
        const int e = lt + k * kWorkerThreads;
        const int gm = r.m0 + e / BN, gn = r.n0 + e % BN;
        if (gm >= blk.m || gn >= blk.n) continue;
        const int64_t at = blk.c + static_cast<int64_t>(gm) * blk.n + gn;
        if (!relabel)
          C[at] = sum[k];
        else if (relabel[at] >= 0)
          C[relabel[at]] = sum[k];  // straight to its place after the leg move that follows
      }
      const int64_t entries = static_cast<int64_t>(blk.m) * blk.n;
      if (!relabel && lt == 0 && r.m0 + BM >= blk.m && r.n0 + BN >= blk.n && (entries & 1)) C[blk.c + entries] = zero_t<T>();
    }

    // ---------------------------------------------------------------------------------------
    // FP64 / complex128
    // ---------------------------------------------------------------------------------------

    // Persistent: kF64Workers workers of 128 threads, each computing 32 x 32 tiles over a K range
    // with 2 x 4 entries per thread, K staged 16 at a time through its own shared memory (A padded
    // to 33 columns so the k-fast, coalesced stores hit distinct banks).  FP64 retires about 0.44
    // DFMA per clock per SM sub-partition on this part: the workers keep all four busy.
    template <typename T>
    __global__ void __launch_bounds__(kF64Workers * kWorkerThreads, 1)
      gemm_f64_kernel(const T *__restrict__ A, const T *__restrict__ B, T *__restrict__ C,
                      const DevBlock *__restrict__ blocks, const DevPair *__restrict__ pairs,
                      const GemmItem *__restrict__ items, const int32_t *__restrict__ cta_begin, const GemmReduce *__restrict__ reduces,
                      int64_t n_reduces, T *__restrict__ partial, int *__restrict__ tickets)
    {
      dependent_entry();
      constexpr int BM = kF64TileM, BN = kF64TileN, BK = 16, TM = 2, TN = 4;
      extern __shared__ __align__(16) unsigned char smem_raw[];
      const int worker = threadIdx.x / kWorkerThreads, lt = threadIdx.x % kWorkerThreads;
      T(*as)[BM + 1] = reinterpret_cast<T(*)[BM + 1]>(smem_raw + worker * 2 * BK * (BM + 1) * sizeof(T));
      T(*bs)[BN + 1] = reinterpret_cast<T(*)[BN + 1]>(smem_raw + (worker * 2 + 1) * BK * (BM + 1) * sizeof(T));
      __shared__ int flags[kF64Workers];
      const int tx = lt % (BN / TN), ty = lt / (BN / TN);
      // this CTA's list of items (dealt by the host, largest first, to balance the SMs); its
      // workers take them in order through a shared counter
      __shared__ int next[kF64Workers];
      __shared__ int taken;
      if (threadIdx.x == 0) taken = 0;
      __syncthreads();
      const int64_t list_begin = cta_begin[blockIdx.x], list_end = cta_begin[blockIdx.x + 1];
      for (int64_t idx = list_begin + local_claim(worker, lt, next + worker, &taken); idx < list_end;
           idx = list_begin + local_claim(worker, lt, next + worker, &taken))
      {
        const GemmItem it = items[idx];
        const DevBlock blk = blocks[it.block];
        T acc[TM][TN];
#pragma unroll
        for (int i = 0; i < TM; ++i)
#pragma unroll
          for (int j = 0; j < TN; ++j) acc[i][j] = zero_t<T>();
        int32_t kbase = 0;
        for (int32_t pi = 0; pi < blk.pair_count; ++pi)
        {
          const DevPair pr = pairs[blk.pair_begin + pi];
          const int K = pr.k;
          const int lo = max(it.k0 - kbase, 0), hi = min(it.k1 - kbase, K);
          kbase += K;
          if (lo >= hi) continue;
          const T *a = A + pr.a;
          const T *b = B + pr.b;
          for (int k0 = lo; k0 < hi; k0 += BK)
          {
            for (int i = lt; i < BM * BK; i += kWorkerThreads)
            {
              const int r = i / BK, kk = i % BK;
              const int gm = it.m0 + r, gk = k0 + kk;
              as[kk][r] = (gm < blk.m && gk < hi) ? a[static_cast<int64_t>(gm) * K + gk] : zero_t<T>();
            }
            for (int i = lt; i < BK * BN; i += kWorkerThreads)
            {
              const int kk = i / BN, cc = i % BN;
              const int gk = k0 + kk, gn = it.n0 + cc;
              bs[kk][cc] = (gk < hi && gn < blk.n) ? b[static_cast<int64_t>(gk) * blk.n + gn] : zero_t<T>();
            }
            worker_sync(worker);
#pragma unroll
            for (int kk = 0; kk < BK; ++kk)
            {
              T av[TM], bv[TN];
#pragma unroll
              for (int i = 0; i < TM; ++i) av[i] = as[kk][ty * TM + i];
#pragma unroll
              for (int j = 0; j < TN; ++j) bv[j] = bs[kk][tx * TN + j];
#pragma unroll
              for (int i = 0; i < TM; ++i)
#pragma unroll
                for (int j = 0; j < TN; ++j) acc[i][j] = fma_t(av[i], bv[j], acc[i][j]);
            }
            worker_sync(worker);
          }
        }
        if (it.slot >= 0)
        {
          T *out = partial + static_cast<int64_t>(it.slot) * BM * BN;
#pragma unroll
          for (int i = 0; i < TM; ++i)
#pragma unroll
            for (int j = 0; j < TN; ++j) out[(ty * TM + i) * BN + tx * TN + j] = acc[i][j];
          finish_partial<T, BM, BN>(worker, lt, flags + worker, tickets, reduces, it.reduce, blocks, partial, C);
          continue;
        }
#pragma unroll
        for (int i = 0; i < TM; ++i)
        {
          const int gm = it.m0 + ty * TM + i;
          if (gm >= blk.m) continue;
#pragma unroll
          for (int j = 0; j < TN; ++j)
          {
            const int gn = it.n0 + tx * TN + j;
            if (gn < blk.n) C[blk.c + static_cast<int64_t>(gm) * blk.n + gn] = acc[i][j];
          }
        }
        // the alignment pad after an odd-sized block reads as zero in arena-wide sums
        const int64_t entries = static_cast<int64_t>(blk.m) * blk.n;
        if (lt == 0 && it.m0 + BM >= blk.m && it.n0 + BN >= blk.n && (entries & 1)) C[blk.c + entries] = zero_t<T>();
      }
    }

    // The float64 form of gemm_f64_kernel on the FP64 matrix instruction (mma m16n8k8 f64): each of
    // a worker's 4 warps owns a 16 x 16 quarter of the 32 x 32 tile as two m16n8 accumulators; per
    // 8 of K staged in shared memory a warp issues 2 DMMA.
    __global__ void __launch_bounds__(kF64Workers * kWorkerThreads, 1)
      gemm_dmma_kernel(const double *__restrict__ A, const double *__restrict__ B, double *__restrict__ C,
                       const DevBlock *__restrict__ blocks, const DevPair *__restrict__ pairs,
                       const GemmItem *__restrict__ items, const int32_t *__restrict__ cta_begin, const GemmReduce *__restrict__ reduces,
                       int64_t n_reduces, double *__restrict__ partial, int *__restrict__ tickets)
    {
      dependent_entry();
      constexpr int BM = kF64TileM, BN = kF64TileN, BK = kDmmaStepK;
      extern __shared__ __align__(16) unsigned char smem_raw[];
      const int worker = threadIdx.x / kWorkerThreads, lt = threadIdx.x % kWorkerThreads;
      // rows of 36 doubles: a warp's fragment loads (k = lane % 4 (+ 4), row = lane / 4 (+ 8)) then
      // fall on distinct bank pairs within each half warp.  Two stages of A (k-major) and B per worker.
      constexpr int P = 36;
      double *stage_base = reinterpret_cast<double *>(smem_raw) + static_cast<size_t>(worker) * 2 * 2 * BK * P;
      __shared__ int flags[kF64Workers];
      const int warp = lt >> 5, lane = lt & 31;
      const int wm = warp >> 1, wn = warp & 1;
      const int fr = lane >> 2, fk = lane & 3;  // fragment row (or column) and k of this lane
      // this CTA's list of items (dealt by the host, largest first, to balance the SMs); its
      // workers take them in order through a shared counter
      __shared__ int next[kF64Workers];
      __shared__ int taken;
      if (threadIdx.x == 0) taken = 0;
      __syncthreads();
      const int64_t list_begin = cta_begin[blockIdx.x], list_end = cta_begin[blockIdx.x + 1];
      for (int64_t idx = list_begin + local_claim(worker, lt, next + worker, &taken); idx < list_end;
           idx = list_begin + local_claim(worker, lt, next + worker, &taken))
      {
        const GemmItem it = items[idx];
        const DevBlock blk = blocks[it.block];
        double acc[2][4] = {};
        const bool live_i = it.m0 + wm * 16 < blk.m;
        const bool live_j[2] = {it.n0 + wn * 16 < blk.n, it.n0 + wn * 16 + 8 < blk.n};
        int32_t kbase = 0;
        for (int32_t pi = 0; pi < blk.pair_count; ++pi)
        {
          const DevPair pr = pairs[blk.pair_begin + pi];
          const int K = pr.k;
          const int lo = max(it.k0 - kbase, 0), hi = min(it.k1 - kbase, K);
          kbase += K;
          if (lo >= hi) continue;
          const double *a = A + pr.a;
          const double *b = B + pr.b;
          // K in steps of BK through two shared stages: the copies of step s + 1 (cp.async, entries
          // outside the block or past hi filled with zeros) are in flight while step s computes
          const auto load = [&](int stage, int k0)
          {
            double *as = stage_base + stage * 2 * BK * P, *bs = as + BK * P;
            for (int i = lt; i < BM * BK; i += kWorkerThreads)
            {
              const int r = i / BK, kk = i % BK;
              const int gm = it.m0 + r, gk = k0 + kk;
              const bool in = gm < blk.m && gk < hi;
              copy8(as + kk * P + r, in ? a + static_cast<int64_t>(gm) * K + gk : a, in);
            }
            for (int i = lt; i < BK * BN; i += kWorkerThreads)
            {
              const int kk = i / BN, cc = i % BN;
              const int gk = k0 + kk, gn = it.n0 + cc;
              const bool in = gk < hi && gn < blk.n;
              copy8(bs + kk * P + cc, in ? b + static_cast<int64_t>(gk) * blk.n + gn : b, in);
            }
            copy_commit();
          };
          load(0, lo);
          int stage = 0;
          for (int k0 = lo; k0 < hi; k0 += BK, stage ^= 1)
          {
            if (k0 + BK < hi)
              load(stage ^ 1, k0 + BK);
            else
              copy_commit();  // an empty group keeps the count of the wait below
            copy_wait_one();
            worker_sync(worker);
            const double(*as)[P] = reinterpret_cast<const double(*)[P]>(stage_base + stage * 2 * BK * P);
            const double(*bs)[P] = reinterpret_cast<const double(*)[P]>(stage_base + stage * 2 * BK * P + BK * P);
            const int steps = min(BK, hi - k0);
            // a 16 x 8 fragment wholly outside the block costs the FP64 pipe as much as a full one:
            // skip it (warp-uniform); a full step runs unrolled with no bound, so the fragment loads
            // of the next k are issued ahead of the products of this one.  Entries of the stage past
            // `hi` are zeros, so a last step rounded up to 8 adds nothing.
            const auto step_k = [&](int kb)
            {
              double af[4], bf[2][2];
#pragma unroll
              for (int h = 0; h < 4; ++h) af[h] = as[kb + fk + (h >> 1) * 4][wm * 16 + (h & 1) * 8 + fr];
#pragma unroll
              for (int j = 0; j < 2; ++j)
#pragma unroll
                for (int h = 0; h < 2; ++h) bf[j][h] = bs[kb + fk + h * 4][wn * 16 + j * 8 + fr];
#pragma unroll
              for (int j = 0; j < 2; ++j)
                if (live_j[j]) dmma16(acc[j], af, bf[j]);
            };
            if (live_i && live_j[0])  // the warp's 16 x 16 quarter touches the block
            {
              if (steps == BK)
              {
#pragma unroll
                for (int kb = 0; kb < BK; kb += 8) step_k(kb);
              }
              else
                for (int kb = 0; kb < steps; kb += 8) step_k(kb);
            }
            worker_sync(worker);
          }
        }
        if (it.slot >= 0)
        {
          double *out = partial + static_cast<int64_t>(it.slot) * BM * BN;
#pragma unroll
          for (int j = 0; j < 2; ++j)
#pragma unroll
            for (int h = 0; h < 4; ++h) out[(wm * 16 + (h >> 1) * 8 + fr) * BN + wn * 16 + j * 8 + fk * 2 + (h & 1)] = acc[j][h];
          finish_partial<double, BM, BN>(worker, lt, flags + worker, tickets, reduces, it.reduce, blocks, partial, C);
          continue;
        }
#pragma unroll
        for (int j = 0; j < 2; ++j)
#pragma unroll
          for (int h = 0; h < 4; ++h)
          {
            const int gm = it.m0 + wm * 16 + (h >> 1) * 8 + fr, gn = it.n0 + wn * 16 + j * 8 + fk * 2 + (h & 1);
            if (gm < blk.m && gn < blk.n) C[blk.c + static_cast<int64_t>(gm) * blk.n + gn] = acc[j][h];
          }
        const int64_t entries = static_cast<int64_t>(blk.m) * blk.n;
        if (lt == 0 && it.m0 + BM >= blk.m && it.n0 + BN >= blk.n && (entries & 1)) C[blk.c + entries] = 0.0;
      }
    }

    // ---------------------------------------------------------------------------------------
    // split precision
    // ---------------------------------------------------------------------------------------

    // One warp per line (a row of A or a column of B), lines of A from `a` and lines of B from `b`:
    // the power of two 2^e that bounds the line, then each entry as the integer round(x 2^(56-e))
    // cut into `slices` balanced 7-bit digits (|q_1| <= 128, |q_t| <= 64 after it), exact in bf16,
    // written to a row padded with zeros to a multiple of 32.  Loads are issued eight at a time.
    constexpr int kLineHeld = 16;  // entries a lane holds of a line sliced in one pass (lines <= 512)

    __global__ void split_lines_kernel(const double *__restrict__ a, const double *__restrict__ b,
                                       uint16_t *__restrict__ slices_a, uint16_t *__restrict__ slices_b,
                                       int16_t *__restrict__ exps_a, int16_t *__restrict__ exps_b, int64_t stride_a,
                                       int64_t stride_b, const SplitLine *__restrict__ lines, int64_t lines_a,
                                       int64_t line_begin, int64_t line_end, int slices_n)
    {
      dependent_entry();
      const int lane = threadIdx.x & 31;
      const int64_t warp = (static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
      const int64_t warps = (static_cast<int64_t>(gridDim.x) * blockDim.x) >> 5;
      for (int64_t l = line_begin + warp; l < line_end; l += warps)
      {
        const SplitLine line = lines[l];
        const bool left = l < lines_a;
        const double *src = (left ? a : b) + line.src;
        uint16_t *dst = (left ? slices_a : slices_b) + line.dst;
        int16_t *exps = left ? exps_a : exps_b;
        const int64_t stride = left ? stride_a : stride_b;
        const auto cut = [&](int i, long long r)
        {
          for (int t = 0; t < slices_n; ++t)
          {
            const int shift = 49 - 7 * t;  // digit t weighs 2^(49 - 7t) of the 2^56 scale
            long long q;
            if (shift > 0)
            {
              q = (r + (1ll << (shift - 1))) >> shift;  // nearest integer, halves up
              r -= q << shift;
            }
            else
              q = r;
            // |q| <= 128: exact in bf16, converted through int32 and fp32
            dst[t * stride + i] = __bfloat16_as_ushort(__float2bfloat16_rn(__int2float_rn(static_cast<int>(q))));
          }
        };
        if (line.padded <= 32 * kLineHeld)
        {
          // the whole line in registers, all its loads in flight at once: one round trip to memory
          // for the maximum and the digits together
          double v[kLineHeld];
          unsigned long long big = 0;
#pragma unroll
          for (int u = 0; u < kLineHeld; ++u)
          {
            const int i = u * 32 + lane;
            v[u] = i < line.len ? src[static_cast<int64_t>(i) * line.src_stride] : 0.0;
            const unsigned long long bits = static_cast<unsigned long long>(__double_as_longlong(v[u])) & 0x7fffffffffffffffull;
            big = bits > big ? bits : big;
          }
          for (int off = 16; off > 0; off >>= 1)
          {
            const unsigned long long o = __shfl_xor_sync(0xffffffffu, big, off);
            big = o > big ? o : big;
          }
          const int e = frexp_exponent(big);
          if (lane == 0) exps[line.exp] = static_cast<int16_t>(e);
#pragma unroll
          for (int u = 0; u < kLineHeld; ++u)
          {
            const int i = u * 32 + lane;
            if (i < line.padded) cut(i, i < line.len ? scaled_integer(v[u], 56 - e) : 0ll);
          }
          continue;
        }
        // the largest |entry| by its bits (positive doubles order as integers), then its frexp
        // exponent e: every |entry| < 2^e
        unsigned long long big = 0;
        for (int i0 = 0; i0 < line.len; i0 += 256)
        {
          unsigned long long v[8];
#pragma unroll
          for (int u = 0; u < 8; ++u)
          {
            const int i = i0 + u * 32 + lane;
            v[u] = i < line.len ? (static_cast<unsigned long long>(__double_as_longlong(src[static_cast<int64_t>(i) * line.src_stride])) &
                                   0x7fffffffffffffffull)
                                : 0ull;
          }
#pragma unroll
          for (int u = 0; u < 8; ++u) big = v[u] > big ? v[u] : big;
        }
        for (int off = 16; off > 0; off >>= 1)
        {
          const unsigned long long o = __shfl_xor_sync(0xffffffffu, big, off);
          big = o > big ? o : big;
        }
        const int e = frexp_exponent(big);
        if (lane == 0) exps[line.exp] = static_cast<int16_t>(e);
        for (int i0 = 0; i0 < line.padded; i0 += 128)
        {
          long long x[4];
#pragma unroll
          for (int u = 0; u < 4; ++u)
          {
            const int i = i0 + u * 32 + lane;
            x[u] = i < line.len ? scaled_integer(src[static_cast<int64_t>(i) * line.src_stride], 56 - e) : 0ll;
          }
#pragma unroll
          for (int u = 0; u < 4; ++u)
          {
            const int i = i0 + u * 32 + lane;
            if (i < line.padded) cut(i, x[u]);
          }
        }
      }
    }

    template <int S>
    __host__ __device__ constexpr int split_worker_bytes() { return 2 * S * (kSplitTileM + kSplitTileN) * kRow * 2; }

    // Persistent: kSplitWorkers workers of 128 threads (4 warps of 16 x 16), each computing 32 x 32
    // tiles of one pair over a K range.  All S slices of a 32-wide K step are staged in the worker's
    // shared memory with 16-byte cp.async, double buffered; every A and B slice fragment of a k16
    // step is loaded once with ldmatrix and reused for the S(S+1)/2 products.  Level sums stay exact
    // in fp32 for 256 of K and are then folded into FP64 with the pair's row and column scales: the
    // four leading levels exactly, the rest (weights <= 2^-42 of the first) through one fp32 sum.
    template <int S>
    __global__ void __launch_bounds__(kSplitWorkers * kWorkerThreads, 1)
      gemm_split_kernel(const uint16_t *__restrict__ sa_all, const uint16_t *__restrict__ sb_all,
                        const int16_t *__restrict__ exps_a, const int16_t *__restrict__ exps_b, int64_t stride_a,
                        int64_t stride_b, double *__restrict__ C,
                        const DevBlock *__restrict__ blocks, const DevSplitPair *__restrict__ spairs,
                        const SplitItem *__restrict__ items, const int32_t *__restrict__ cta_begin, const GemmReduce *__restrict__ reduces,
                        int64_t n_reduces, double *__restrict__ partial, int *__restrict__ tickets,
                        const int32_t *__restrict__ relabel)
    {
      dependent_entry();
      extern __shared__ __align__(16) unsigned char smem_raw[];
      const int worker = threadIdx.x / kWorkerThreads, lt = threadIdx.x % kWorkerThreads;
      uint16_t *sA = reinterpret_cast<uint16_t *>(smem_raw + worker * split_worker_bytes<S>());  // [2][S][32][kRow]
      uint16_t *sB = sA + 2 * S * kSplitTileM * kRow;                                           // [2][S][32][kRow]
      __shared__ int flags[kSplitWorkers];
      const int warp = lt >> 5, lane = lt & 31;
      const int g = lane >> 2, tig = lane & 3;
      const int wm = warp >> 1, wn = warp & 1;
      __shared__ int next[kSplitWorkers];
      __shared__ int taken;
      if (threadIdx.x == 0) taken = 0;
      __syncthreads();
      const int64_t list_begin = cta_begin[blockIdx.x], list_end = cta_begin[blockIdx.x + 1];
      for (int64_t idx = list_begin + local_claim(worker, lt, next + worker, &taken); idx < list_end;
           idx = list_begin + local_claim(worker, lt, next + worker, &taken))
      {
        const SplitItem it = items[idx];
        const DevBlock blk = blocks[it.block];
        double acc[2][4] = {};
        const int r0 = it.m0 + wm * 16 + g, c0 = it.n0 + wn * 16 + tig * 2;
        // the warp's 16 x 16 quarter of the tile touches the block (warp-uniform)
        const bool live = it.m0 + wm * 16 < blk.m && it.n0 + wn * 16 < blk.n;
        if (it.pair >= 0 && it.k1 > it.k0)
        {
          const DevSplitPair sp = spairs[it.pair];
          const int rows = min(kSplitTileM, blk.m - it.m0), cols = min(kSplitTileN, blk.n - it.n0);
          const uint16_t *ga = sa_all + sp.sa + static_cast<int64_t>(it.m0) * sp.kp;
          const uint16_t *gb = sb_all + sp.sb + static_cast<int64_t>(it.n0) * sp.kp;
          const auto load = [&](int stage, int k) {
            for (int c = lt; c < S * kSplitTileM * 4; c += kWorkerThreads)
            {
              const int t = c / (kSplitTileM * 4), r = (c / 4) % kSplitTileM, q = c % 4;
              const bool ok = r < rows;
              cp_async16(sA + ((stage * S + t) * kSplitTileM + r) * kRow + q * 8,
                         ga + t * stride_a + static_cast<int64_t>(ok ? r : 0) * sp.kp + k + q * 8, ok ? 16 : 0);
            }
            for (int c = lt; c < S * kSplitTileN * 4; c += kWorkerThreads)
            {
              const int u = c / (kSplitTileN * 4), r = (c / 4) % kSplitTileN, q = c % 4;
              const bool ok = r < cols;
              cp_async16(sB + ((stage * S + u) * kSplitTileN + r) * kRow + q * 8,
                         gb + u * stride_b + static_cast<int64_t>(ok ? r : 0) * sp.kp + k + q * 8, ok ? 16 : 0);
            }
            cp_async_commit();
          };
          const int steps = (it.k1 - it.k0 + kSplitStepK - 1) / kSplitStepK;
          long long acc_int[2][4] = {};
          float acc_tail[2][4] = {};
          float lev[S][2][4];
#pragma unroll
          for (int l = 0; l < S; ++l)
#pragma unroll
            for (int ns = 0; ns < 2; ++ns)
#pragma unroll
              for (int q = 0; q < 4; ++q) lev[l][ns][q] = 0.0f;
          const int er0 = r0 < blk.m ? exps_a[sp.ea + r0] : 0, er1 = r0 + 8 < blk.m ? exps_a[sp.ea + r0 + 8] : 0;
          int ec[2][2];
#pragma unroll
          for (int ns = 0; ns < 2; ++ns)
#pragma unroll
            for (int h = 0; h < 2; ++h) ec[ns][h] = c0 + ns * 8 + h < blk.n ? exps_b[sp.eb + c0 + ns * 8 + h] : 0;
          load(0, it.k0);
          for (int step = 0; step < steps; ++step)
          {
            const int stage = step & 1;
            if (step + 1 < steps)
            {
              load(stage ^ 1, it.k0 + (step + 1) * kSplitStepK);
              cp_async_wait<1>();
            }
            else
              cp_async_wait<0>();
            worker_sync(worker);
#pragma unroll
            for (int kk = 0; kk < kSplitStepK; kk += 16)
            {
              if (!live) break;
              uint32_t af[S][4], bf[S][4];
#pragma unroll
              for (int t = 0; t < S; ++t)
              {
                ldmatrix_x4(af[t], sA + ((stage * S + t) * kSplitTileM + wm * 16 + (lane & 15)) * kRow + kk + (lane >> 4) * 8);
                ldmatrix_x4(bf[t], sB + ((stage * S + t) * kSplitTileN + wn * 16 + (lane & 7) + ((lane >> 4) << 3)) * kRow +
                                     kk + ((lane >> 3) & 1) * 8);
              }
#pragma unroll
              for (int t = 0; t < S; ++t)
#pragma unroll
                for (int u = 0; u + t < S; ++u)
                {
                  mma_bf16(lev[t + u][0], af[t], bf[u][0], bf[u][1]);
                  mma_bf16(lev[t + u][1], af[t], bf[u][2], bf[u][3]);
                }
            }
            worker_sync(worker);
            if ((step + 1) % (kExactChunk / kSplitStepK) == 0 || step + 1 == steps)
            {
              // the four leading levels are exact integers (below 2^24 over a chunk of <= 256 of K):
              // combined exactly in int64 as sum_l lev_l 2^(7 (3 - l)); the rest in fp32
#pragma unroll
              for (int ns = 0; ns < 2; ++ns)
#pragma unroll
                for (int q = 0; q < 4; ++q)
                {
                  float tail = 0.0f;
#pragma unroll
                  for (int l = S - 1; l >= 4; --l) tail = fmaf(lev[l][ns][q], ldexpf(1.0f, -7 * (l - 4)), tail);
                  long long head = 0;
#pragma unroll
                  for (int l = 0; l < 4; ++l)
                    head = head * 128 + (l < S ? static_cast<long long>(__float2int_rn(lev[l][ns][q])) : 0ll);
                  acc_int[ns][q] += head;
                  acc_tail[ns][q] += tail;
#pragma unroll
                  for (int l = 0; l < S; ++l) lev[l][ns][q] = 0.0f;
                }
            }
          }
          // one FP64 step per entry: head 2^-35 + tail 2^-42, times the row and column scales
#pragma unroll
          for (int ns = 0; ns < 2; ++ns)
#pragma unroll
            for (int q = 0; q < 4; ++q)
            {
              const int ex = (q < 2 ? er0 : er1) + ec[ns][q & 1];
              acc[ns][q] = fma(static_cast<double>(acc_int[ns][q]), pow2(ex - 35),
                               static_cast<double>(acc_tail[ns][q]) * pow2(ex - 42));
            }
        }
        if (it.slot >= 0)
        {
          double *out = partial + static_cast<int64_t>(it.slot) * kSplitTileM * kSplitTileN;
#pragma unroll
          for (int ns = 0; ns < 2; ++ns)
#pragma unroll
            for (int q = 0; q < 4; ++q)
              out[(wm * 16 + g + (q >= 2 ? 8 : 0)) * kSplitTileN + wn * 16 + ns * 8 + tig * 2 + (q & 1)] = acc[ns][q];
          finish_partial<double, kSplitTileM, kSplitTileN>(worker, lt, flags + worker, tickets, reduces, it.reduce, blocks,
                                                           partial, C, relabel);
          continue;
        }
#pragma unroll
        for (int ns = 0; ns < 2; ++ns)
#pragma unroll
          for (int q = 0; q < 4; ++q)
          {
            const int gm = r0 + (q >= 2 ? 8 : 0), gn = c0 + ns * 8 + (q & 1);
            if (gm >= blk.m || gn >= blk.n) continue;
            const int64_t at = blk.c + static_cast<int64_t>(gm) * blk.n + gn;
            if (!relabel)
              C[at] = acc[ns][q];
            else if (relabel[at] >= 0)
              C[relabel[at]] = acc[ns][q];  // straight to its place after the leg move that follows
          }
        const int64_t entries = static_cast<int64_t>(blk.m) * blk.n;
        if (!relabel && lt == 0 && it.m0 + kSplitTileM >= blk.m && it.n0 + kSplitTileN >= blk.n && (entries & 1))
          C[blk.c + entries] = 0.0;
      }
    }


    // Shared memory that holds one CTA per SM: at least 120 KiB, so a second never fits beside it.
    constexpr int kPinBytes = 120 * 1024;

    template <typename K>
    cudaError_t configure(K kernel, int bytes, std::once_flag &once)
    {
      cudaError_t e = cudaSuccess;
      std::call_once(once, [&] { e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes); });
      return e;
    }

    template <int S>
    cudaError_t launch_split_s(const uint16_t *sa, const uint16_t *sb, const int16_t *exps_a, const int16_t *exps_b,
                               int64_t stride_a, int64_t stride_b, double *C, const DevBlock *blocks, const DevSplitPair *spairs,
                               const SplitItem *items, const int32_t *cta_begin, int32_t n_ctas, int64_t longest,
                               const GemmReduce *reduces, int64_t n_reduces, double *partial, int *tickets,
                               const int32_t *relabel, cudaStream_t stream)
    {
      const int bytes = std::max(kSplitWorkers * split_worker_bytes<S>(), kPinBytes);
      static std::once_flag once;
      cudaError_t e = configure(gemm_split_kernel<S>, bytes, once);
      if (e != cudaSuccess) return e;
      // one CTA per list the schedule dealt, as many workers as its longest list needs
      const int workers = static_cast<int>(std::clamp<int64_t>(longest, 1, kSplitWorkers));
      return launch_dependent(gemm_split_kernel<S>, n_ctas, workers * kWorkerThreads, bytes, stream, sa, sb, exps_a, exps_b,
                              stride_a, stride_b, C, blocks, spairs, items, cta_begin, reduces, n_reduces, partial, tickets,
                              relabel);
    }
  } // namespace

  // ------------------------------------------------------------------------------------------
  // launchers
  // ------------------------------------------------------------------------------------------

  namespace
  {
    // The FP64 tables of a GEMM op, built on its first FP64 launch.
    cudaError_t ensure_f64(const Program &p, DeviceTables &t, size_t op_index)
    {
      std::lock_guard<std::mutex> lock(t.mutex);
      DeviceTables::GemmTables &dst = t.gemm[op_index];
      if (dst.ready) return cudaSuccess;
      const GemmSchedule s = schedule_gemm(p, p.ops[op_index], kF64TileM, kF64TileN, true);
      dst.n_items = static_cast<int64_t>(s.items.size());
      dst.n_reduces = static_cast<int64_t>(s.reduces.size());
      dst.slots = s.slots;
      dst.n_ctas = static_cast<int32_t>(s.cta_begin.size()) - 1;
      dst.longest = 0;
      for (size_t c = 0; c + 1 < s.cta_begin.size(); ++c)
        dst.longest = std::max<int64_t>(dst.longest, s.cta_begin[c + 1] - s.cta_begin[c]);
      TableStaging staging;
      staging.add(s.items, reinterpret_cast<void **>(&dst.items));
      staging.add(s.reduces, reinterpret_cast<void **>(&dst.reduces));
      staging.add(s.cta_begin, reinterpret_cast<void **>(&dst.cta_begin));
      const cudaError_t e = staging.commit(&dst.base);
      if (e != cudaSuccess) return e;
      dst.ready = true;
      return cudaSuccess;
    }
  } // namespace

  cudaError_t launch_gemm_f64(const Program &p, DeviceTables &t, size_t op_index, const void *A, const void *B, void *C,
                              bool complex, void *scratch, int *ticket_region, cudaStream_t stream)
  {
    if (const cudaError_t built = ensure_f64(p, t, op_index); built != cudaSuccess) return built;
    const auto &sched = t.gemm[op_index];
    if (sched.n_items == 0) return cudaSuccess;
    const auto *blocks = reinterpret_cast<const DevBlock *>(t.blocks);
    const auto *pairs = reinterpret_cast<const DevPair *>(t.pairs);
    char *base = static_cast<char *>(scratch);
    void *partial = base;
    // the workspace's ticket region (zero, and left zero by the kernel) when it holds them all,
    // else tickets of our own in the scratch, cleared first
    int *tickets = ticket_region;
    cudaError_t e = cudaSuccess;
    if (sched.n_reduces > kTicketInts)
    {
      tickets = reinterpret_cast<int *>(base + up256(sched.slots * kF64TileM * kF64TileN * 16));
      if ((e = cudaMemsetAsync(tickets, 0, static_cast<size_t>(sched.n_reduces) * 4, stream)) != cudaSuccess) return e;
    }
    // one CTA per list the schedule dealt, as many workers as its longest list needs (at most four)
    const int grid = sched.n_ctas;
    const int workers = static_cast<int>(std::clamp<int64_t>(sched.longest, 1, kF64Workers));
    if (complex)
    {
      const int bytes = std::max<int>(kF64Workers * 2 * 16 * (kF64TileM + 1) * 16, kPinBytes);
      static std::once_flag once;
      if ((e = configure(gemm_f64_kernel<double2>, bytes, once)) != cudaSuccess) return e;
      e = launch_dependent(gemm_f64_kernel<double2>, grid, workers * kWorkerThreads, bytes, stream,
                           static_cast<const double2 *>(A), static_cast<const double2 *>(B), static_cast<double2 *>(C), blocks,
                           pairs, static_cast<const GemmItem *>(sched.items), static_cast<const int32_t *>(sched.cta_begin),
                           static_cast<const GemmReduce *>(sched.reduces), sched.n_reduces, static_cast<double2 *>(partial),
                           tickets);
    }
    else
    {
      const int bytes = std::max<int>(kF64Workers * 2 * 2 * kDmmaStepK * 36 * 8, kPinBytes);
      static std::once_flag once;
      if ((e = configure(gemm_dmma_kernel, bytes, once)) != cudaSuccess) return e;
      e = launch_dependent(gemm_dmma_kernel, grid, workers * kWorkerThreads, bytes, stream, static_cast<const double *>(A),
                           static_cast<const double *>(B), static_cast<double *>(C), blocks, pairs,
                           static_cast<const GemmItem *>(sched.items), static_cast<const int32_t *>(sched.cta_begin),
                           static_cast<const GemmReduce *>(sched.reduces), sched.n_reduces, static_cast<double *>(partial),
                           tickets);
    }
    return e;
  }

  namespace
  {
    // The split tables of a GEMM op, built on its first split use.
    cudaError_t ensure_split(const Program &p, const Op &op, DeviceTables &t, size_t op_index)
    {
      std::lock_guard<std::mutex> lock(t.mutex);
      DeviceTables::SplitTables &dst = t.split[op_index];
      if (dst.ready) return cudaSuccess;
      const SplitSchedule s = schedule_split(p, op, true);
      dst.n_items = static_cast<int64_t>(s.items.size());
      dst.n_reduces = static_cast<int64_t>(s.reduces.size());
      dst.n_lines_a = s.lines_a;
      dst.n_lines_b = static_cast<int64_t>(s.lines.size()) - s.lines_a;
      dst.slice_a = s.slice_a;
      dst.slice_b = s.slice_b;
      dst.exps_a = s.exps_a;
      dst.exps = s.exps;
      dst.slots = s.slots;
      dst.n_ctas = static_cast<int32_t>(s.cta_begin.size()) - 1;
      dst.longest = 0;
      for (size_t c = 0; c + 1 < s.cta_begin.size(); ++c)
        dst.longest = std::max<int64_t>(dst.longest, s.cta_begin[c + 1] - s.cta_begin[c]);
      TableStaging staging;
      staging.add(s.cta_begin, reinterpret_cast<void **>(&dst.cta_begin));
      staging.add(s.items, &dst.items);
      staging.add(s.reduces, reinterpret_cast<void **>(&dst.reduces));
      staging.add(s.pairs, &dst.pairs);
      staging.add(s.lines, &dst.lines);
      const cudaError_t e = staging.commit(&dst.base);
      if (e != cudaSuccess) return e;
      dst.ready = true;
      return cudaSuccess;
    }

    cudaError_t launch_lines(const DeviceTables::SplitTables &sched, const double *A, const double *B, uint16_t *sa,
                             uint16_t *sb, int16_t *exps_a, int16_t *exps_b, int64_t begin, int64_t end, int slices,
                             cudaStream_t stream)
    {
      if (begin >= end) return cudaSuccess;
      const auto *lines = reinterpret_cast<const SplitLine *>(sched.lines);
      // a warp per line, two warps per CTA so that the lines spread over every SM
      return launch_dependent(split_lines_kernel,
                              static_cast<unsigned>(std::max<int64_t>(1, std::min<int64_t>((end - begin + 1) / 2, device_sms() * 32))),
                              64, 0, stream, A, B, sa, sb, exps_a, exps_b, sched.slice_a, sched.slice_b, lines,
                              sched.n_lines_a, begin, end, slices);
    }
  } // namespace

  cudaError_t fill_slice_caches(const Program &p, DeviceTables &t, int32_t operand, const void *arena, cudaStream_t stream)
  {
    if (!p.gemm_plans) return cudaSuccess;
    for (const SliceCache &c : p.gemm_plans->caches)
    {
      if (c.operand != operand) continue;
      const Op &op = p.ops[static_cast<size_t>(c.op)];
      cudaError_t e = ensure_split(p, op, t, static_cast<size_t>(c.op));
      if (e != cudaSuccess) return e;
      const auto &sched = t.split[static_cast<size_t>(c.op)];
      if (sched.n_items == 0) continue;
      char *base = static_cast<char *>(const_cast<void *>(arena));
      auto *slices = reinterpret_cast<uint16_t *>(base + c.offset);
      auto *exps = reinterpret_cast<int16_t *>(base + c.exps_offset);
      const auto *value = static_cast<const double *>(arena);
      e = c.side == 0 ? launch_lines(sched, value, nullptr, slices, nullptr, exps, nullptr, 0, sched.n_lines_a, kMaxSlices, stream)
                      : launch_lines(sched, nullptr, value, nullptr, slices, nullptr, exps, sched.n_lines_a,
                                     sched.n_lines_a + sched.n_lines_b, kMaxSlices, stream);
      if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
  }

  cudaError_t launch_gemm_split(const Program &p, const Op &op, DeviceTables &t, size_t op_index, const double *A,
                                const double *B, double *C, int32_t slices, void *scratch, int *ticket_region,
                                const void *const *prepared, cudaStream_t stream, const int32_t *relabel, bool tensor_cores)
  {
    cudaError_t e = ensure_split(p, op, t, op_index);
    if (e != cudaSuccess) return e;
    const auto &sched = t.split[op_index];
    if (sched.n_items == 0) return cudaSuccess;
    char *base = static_cast<char *>(scratch);
    auto *sa = reinterpret_cast<uint16_t *>(base);
    base += up256(2 * kMaxSlices * sched.slice_a);
    auto *sb = reinterpret_cast<uint16_t *>(base);
    base += up256(2 * kMaxSlices * sched.slice_b);
    auto *exps_a = reinterpret_cast<int16_t *>(base);
    auto *exps_b = exps_a + sched.exps_a;
    base += up256(2 * sched.exps);
    auto *partial = reinterpret_cast<double *>(base);
    base += up256(sched.slots * kSplitTileM * kSplitTileN * 8);
    int *tickets = ticket_region;
    if (sched.n_reduces > kTicketInts)
    {
      tickets = reinterpret_cast<int *>(base);
      if ((e = cudaMemsetAsync(tickets, 0, static_cast<size_t>(sched.n_reduces) * 4, stream)) != cudaSuccess) return e;
    }
    // a side whose operand's prepared arena the caller holds was cut when the arena was prepared
    int64_t begin = 0, end = sched.n_lines_a + sched.n_lines_b;
    if (p.gemm_plans && prepared)
    {
      const int32_t ca = p.gemm_plans->cache_a[op_index], cb = p.gemm_plans->cache_b[op_index];
      if (ca >= 0 && prepared[p.gemm_plans->caches[static_cast<size_t>(ca)].operand])
      {
        const SliceCache &c = p.gemm_plans->caches[static_cast<size_t>(ca)];
        char *arena = static_cast<char *>(const_cast<void *>(prepared[c.operand]));
        sa = reinterpret_cast<uint16_t *>(arena + c.offset);
        exps_a = reinterpret_cast<int16_t *>(arena + c.exps_offset);
        begin = sched.n_lines_a;
      }
      if (cb >= 0 && prepared[p.gemm_plans->caches[static_cast<size_t>(cb)].operand])
      {
        const SliceCache &c = p.gemm_plans->caches[static_cast<size_t>(cb)];
        char *arena = static_cast<char *>(const_cast<void *>(prepared[c.operand]));
        sb = reinterpret_cast<uint16_t *>(arena + c.offset);
        exps_b = reinterpret_cast<int16_t *>(arena + c.exps_offset);
        end = sched.n_lines_a;
      }
    }
    if ((e = launch_lines(sched, A, B, sa, sb, exps_a, exps_b, begin, end, slices, stream)) != cudaSuccess) return e;
    // large blocks: whole 128 x 64 tiles on the tensor cores (tcgen05), no partial tiles
    static const bool tc_enabled = []
    {
      const char *v = std::getenv("TENTORCH_GB300_TCGEN05");
      return !(v && v[0] == '0');
    }();
    if (tc_enabled && tensor_cores && !relabel && split_tc_suits(p, op, slices))
      return launch_split_tc(p, op, t, op_index, slices, sa, sb, exps_a, exps_b, sched.slice_a, sched.slice_b, sched.pairs,
                             C, ticket_region + kTicketInts - 1, stream);
    const auto *blocks = reinterpret_cast<const DevBlock *>(t.blocks);
    const auto *spairs = reinterpret_cast<const DevSplitPair *>(sched.pairs);
    const auto *items = reinterpret_cast<const SplitItem *>(sched.items);
    switch (slices)
    {
#define TTG_SPLIT(S)                                                                                                    \
  case S:                                                                                                               \
    e = launch_split_s<S>(sa, sb, exps_a, exps_b, sched.slice_a, sched.slice_b, C, blocks, spairs, items,              \
                          sched.cta_begin, sched.n_ctas, sched.longest, sched.reduces, sched.n_reduces, partial, tickets,  \
                          relabel, stream);                                                                             \
    break;
      TTG_SPLIT(1) TTG_SPLIT(2) TTG_SPLIT(3) TTG_SPLIT(4) TTG_SPLIT(5) TTG_SPLIT(6) TTG_SPLIT(7) TTG_SPLIT(8)
#undef TTG_SPLIT
    default: return cudaErrorInvalidValue;
    }
    return e;
  }

  // The device copies of every GEMM op's schedules and slicing lines, staged into the program's
  // one table allocation.
  void stage_gemm(const Program &p, DeviceTables &t, TableStaging &staging)
  {
    t.gemm.assign(p.ops.size(), {});
    t.split.assign(p.ops.size(), {});
    t.tc.assign(p.ops.size(), {});
    if (!p.gemm_plans) return;
    for (size_t i = 0; i < p.ops.size(); ++i)
    {
      if (p.ops[i].kind != OpKind::gemm) continue;
      // the FP64 tables are built on the op's first FP64 launch (ensure_f64)
    }
  }

} // namespace ttg
