// One launch for a block product whose result is moved and multiplied again: the two-site
// effective-Hamiltonian matvec of DMRG, head' theta -> X, X -> X' (a leg move with unit
// coefficients, a relabelling of entries for abelian symmetries), X' tail'' -> image
// (tentorch/linalg/graded/einsum.cpp:351-376 folds it as two contractions with a recoupling between
// them, tentorch/linalg/graded/contract.cpp:148-163 one product per block pair).
//
// The persistent FP64 kernel runs the work items of both products from one list per SM:
//   - a first-product tile writes its entries straight to their places after the move (a table of
//     one int32 per entry of X, built on the device once per plan from the move's tile
//     descriptors, replaces the move's own pass), then counts itself done;
//   - a second-product item waits until every first-product tile is done, then runs like any other
//     tile.
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
    constexpr int kChainTile = 32;  // the DMMA tile (kF64TileM x kF64TileN)

    // The work estimate the FP64 schedules deal by (gemm.cu schedule_gemm): 16 x 8 fragments
    // touching the block times K, plus a quarter tile over 16 of K per staged step and per item.
    double item_work(double rows, double cols, double k)
    {
      const double frag = std::ceil(rows / 16.0) * 16.0 * std::ceil(cols / 8.0) * 8.0;
      return frag * k + 0.25 * kChainTile * kChainTile * 16.0 * (std::ceil(k / kDmmaStepK) + 1.0);
    }

    // The items of both products (cut as their separate launches cut them, first product first),
    // their work, and one list per SM dealt largest first onto the least loaded, the first product
    // before the second; false when the counters do not fit the ticket region.
    bool build_chain(const Program &p, DeviceTables::ChainTables &ct, TableStaging &staging,
                     std::vector<ChainItem> &items, std::vector<int32_t> &cta_begin, std::vector<ChainReduce> &reduces)
    {
      const Op &first = p.ops[static_cast<size_t>(p.chain_first)];
      const Op &second = p.ops[static_cast<size_t>(p.chain_second)];
      const GemmSchedule s1 = schedule_gemm(p, first, kChainTile, kChainTile, true);
      const GemmSchedule s2 = schedule_gemm(p, second, kChainTile, kChainTile, true);
      const int64_t n_reduces = static_cast<int64_t>(s1.reduces.size() + s2.reduces.size());
      // tickets of both products, then the first product's done count, the exit count, the error flag
      if (n_reduces + 3 > kTicketInts) return false;
      reduces.clear();
      for (const GemmReduce &r : s1.reduces) reduces.push_back(ChainReduce{0, r.block, r.m0, r.n0, r.slot0, r.nslots, 0, 0});
      for (const GemmReduce &r : s2.reduces)
        reduces.push_back(ChainReduce{1, r.block, r.m0, r.n0, static_cast<int32_t>(r.slot0 + s1.slots), r.nslots, 0, 0});
      int64_t first_tiles = static_cast<int64_t>(s1.reduces.size());
      struct Sized
      {
        ChainItem item;
        double work;
      };
      std::vector<Sized> stage[2];
      const auto sized = [&](const GemmItem &g, int32_t which) -> Sized
      {
        const GemmBlock &blk = p.gemm_blocks[static_cast<size_t>(g.block)];
        ChainItem it{which, g.block, g.m0, g.n0, g.k0, g.k1, -1, -1, 0, 0};
        if (g.slot >= 0)
        {
          it.slot = static_cast<int32_t>(g.slot + (which ? s1.slots : 0));
          it.reduce = g.reduce + (which ? static_cast<int32_t>(s1.reduces.size()) : 0);
        }
        const double rows = std::min(kChainTile, blk.m - g.m0), cols = std::min(kChainTile, blk.n - g.n0);
        return Sized{it, item_work(rows, cols, static_cast<double>(g.k1 - g.k0))};
      };
      for (const GemmItem &g : s1.items)
      {
        stage[0].push_back(sized(g, 0));
        if (g.slot < 0) ++first_tiles;
      }
      for (const GemmItem &g : s2.items) stage[1].push_back(sized(g, 1));
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
      ct.slots = s1.slots + s2.slots;
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
    };
    // A launch: the dealt items of every program (ChainItem::window names its program) and the
    // programs themselves, passed by value (a kernel parameter of a few KiB).
    struct ChainLaunch
    {
      const ChainItem *items;
      const int32_t *cta_begin;
      int *exit_count;  // CTAs done (reset by the last)
      int *error;       // set when a wait gave up
      int32_t windows;
      ChainWindow w[kChainBatch];
    };

    constexpr unsigned long long kWaitLimitNs = 2000000000ull;  // two seconds

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

    // A second-product tile that covers the end of its block writes the block's alignment pad.
    __device__ __forceinline__ void store_pad(const ChainWindow &a, int stage, const DevBlock &blk, int m0, int n0, int lt)
    {
      const int64_t entries = static_cast<int64_t>(blk.m) * blk.n;
      if (stage == 1 && lt == 0 && m0 + kChainTile >= blk.m && n0 + kChainTile >= blk.n && (entries & 1))
        a.c[blk.c + entries] = 0.0;
    }

    // A first-product tile is complete in the moved layout: count it done.  Every thread's fence
    // orders its stores before the count.
    __device__ __forceinline__ void signal_done(const ChainWindow &a, int worker, int lt)
    {
      __threadfence();
      worker_sync(worker);
      if (lt == 0) atomicAdd(a.done, 1);
    }

    // A second-product item waits until every first-product tile of its program is done (one thread
    // polls with acquire loads, the worker's barrier releases the rest); after two seconds it raises
    // the error flag and goes on.
    __device__ __forceinline__ void wait_first(const ChainWindow &a, int *error, int worker, int lt)
    {
      if (lt == 0)
      {
        const unsigned long long start = global_ns();
        while (load_acquire(a.done) < a.first_tiles)
        {
          if (global_ns() - start > kWaitLimitNs)
          {
            atomicExch(error, 1);
            break;
          }
          __nanosleep(128);
        }
      }
      worker_sync(worker);
      __threadfence();
    }

    // After a worker wrote a partial tile: the worker holding the tile's last ticket sums the
    // partials in slot order (deterministic) and stores the tile; first-product tiles then signal.
    __device__ void finish_chain_partial(const ChainWindow &a, int worker, int lt, int *flag, int reduce)
    {
      constexpr int BM = kChainTile, BN = kChainTile, PER = BM * BN / kWorkerThreads;
      __threadfence();
      worker_sync(worker);
      const ChainReduce r = a.reduces[reduce];
      if (lt == 0) *flag = atomicAdd(a.tickets + reduce, 1) == r.nslots - 1;
      worker_sync(worker);
      const bool last = *flag;
      worker_sync(worker);
      if (!last) return;
      if (lt == 0) a.tickets[reduce] = 0;
      __threadfence();
      const DevBlock blk = a.blocks[r.block];
      double sum[PER];
#pragma unroll
      for (int k = 0; k < PER; ++k) sum[k] = 0.0;
      const double *base = a.partial + static_cast<int64_t>(r.slot0) * BM * BN + lt;
      int s = 0;
      for (; s + 4 <= r.nslots; s += 4)
      {
        double v[4][PER];
#pragma unroll
        for (int u = 0; u < 4; ++u)
#pragma unroll
          for (int k = 0; k < PER; ++k) v[u][k] = __ldcg(base + static_cast<int64_t>(s + u) * BM * BN + k * kWorkerThreads);
#pragma unroll
        for (int u = 0; u < 4; ++u)
#pragma unroll
          for (int k = 0; k < PER; ++k) sum[k] += v[u][k];
      }
      for (; s < r.nslots; ++s)
#pragma unroll
        for (int k = 0; k < PER; ++k) sum[k] += __ldcg(base + static_cast<int64_t>(s) * BM * BN + k * kWorkerThreads);
#pragma unroll
      for (int k = 0; k < PER; ++k)
      {
        const int e = lt + k * kWorkerThreads;
        const int gm = r.m0 + e / BN, gn = r.n0 + e % BN;
        if (gm < blk.m && gn < blk.n) store_entry(a, r.stage, blk, gm, gn, sum[k]);
      }
      store_pad(a, r.stage, blk, r.m0, r.n0, lt);
      if (r.stage == 0) signal_done(a, worker, lt);
    }

    // The DMMA tile machinery of gemm_dmma_kernel (gemm.cu) over the items of both products: K in
    // steps of 32 through two shared stages per worker, a 16 x 16 quarter of the 32 x 32 tile per
    // warp.  The first product's operands and the second's B side are read-only during
    // the launch and staged with cp.async; the second's A side (X', written during the launch by
    // other SMs) is read with L2 loads, so that no SM reads a stale copy of a line from its L1.
    __global__ void __launch_bounds__(kF64Workers * kWorkerThreads, 1) chain_dmma_kernel(const __grid_constant__ ChainLaunch L)
    {
      dependent_entry();
      constexpr int BM = kChainTile, BN = kChainTile, BK = kDmmaStepK, P = 36;
      extern __shared__ __align__(16) unsigned char smem_raw[];
      const int worker = threadIdx.x / kWorkerThreads, lt = threadIdx.x % kWorkerThreads;
      double *stage_base = reinterpret_cast<double *>(smem_raw) + static_cast<size_t>(worker) * 2 * 2 * BK * P;
      __shared__ int flags[kF64Workers];
      __shared__ int next[kF64Workers];
      __shared__ int taken;
      __shared__ int last_out;
      const int warp = lt >> 5, lane = lt & 31;
      const int wm = warp >> 1, wn = warp & 1;
      const int fr = lane >> 2, fk = lane & 3;
      if (threadIdx.x == 0) taken = 0;
      __syncthreads();
      const int64_t list_begin = L.cta_begin[blockIdx.x], list_end = L.cta_begin[blockIdx.x + 1];
      for (int64_t idx = list_begin + local_claim(worker, lt, next + worker, &taken); idx < list_end;
           idx = list_begin + local_claim(worker, lt, next + worker, &taken))
      {
        const ChainItem it = L.items[idx];
        const ChainWindow &a = L.w[it.window];
        const bool second = it.stage == 1;
        const DevBlock blk = a.blocks[it.block];
        if (second) wait_first(a, L.error, worker, lt);
        const double *A = second ? a.moved : a.a1;
        const double *B = second ? a.b2 : a.b1;
        double acc[2][4] = {};
        const bool live_i = it.m0 + wm * 16 < blk.m;
        const bool live_j[2] = {it.n0 + wn * 16 < blk.n, it.n0 + wn * 16 + 8 < blk.n};
        int32_t kbase = 0;
        for (int32_t pi = 0; pi < blk.pair_count; ++pi)
        {
          const DevPair pr = a.pairs[blk.pair_begin + pi];
          const int K = pr.k;
          const int lo = max(it.k0 - kbase, 0), hi = min(it.k1 - kbase, K);
          kbase += K;
          if (lo >= hi) continue;
          const double *pa = A + pr.a;
          const double *pb = B + pr.b;
          const auto load = [&](int stage, int k0)
          {
            double *as = stage_base + stage * 2 * BK * P, *bs = as + BK * P;
            if (second)
            {
              // X': plain L2 loads into shared memory
              for (int i = lt; i < BM * BK; i += kWorkerThreads)
              {
                const int r = i / BK, kk = i % BK;
                const int gm = it.m0 + r, gk = k0 + kk;
                as[kk * P + r] = (gm < blk.m && gk < hi) ? __ldcg(pa + static_cast<int64_t>(gm) * K + gk) : 0.0;
              }
            }
            else
              for (int i = lt; i < BM * BK; i += kWorkerThreads)
              {
                const int r = i / BK, kk = i % BK;
                const int gm = it.m0 + r, gk = k0 + kk;
                const bool in = gm < blk.m && gk < hi;
                copy8(as + kk * P + r, in ? pa + static_cast<int64_t>(gm) * K + gk : pa, in);
              }
            for (int i = lt; i < BK * BN; i += kWorkerThreads)
            {
              const int kk = i / BN, cc = i % BN;
              const int gk = k0 + kk, gn = it.n0 + cc;
              const bool in = gk < hi && gn < blk.n;
              copy8(bs + kk * P + cc, in ? pb + static_cast<int64_t>(gk) * blk.n + gn : pb, in);
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
            const auto step_k = [&](int kb, double (&into)[2][4])
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
                if (live_j[j]) dmma16(into[j], af, bf[j]);
            };
            if (live_i && live_j[0])
            {
              if (steps == BK)
              {
#pragma unroll
                for (int kb = 0; kb < BK; kb += 8) step_k(kb, acc);
              }
              else
                for (int kb = 0; kb < steps; kb += 8) step_k(kb, acc);
            }
            worker_sync(worker);
          }
        }
        if (it.slot >= 0)
        {
          double *out = a.partial + static_cast<int64_t>(it.slot) * BM * BN;
#pragma unroll
          for (int j = 0; j < 2; ++j)
#pragma unroll
            for (int h = 0; h < 4; ++h) out[(wm * 16 + (h >> 1) * 8 + fr) * BN + wn * 16 + j * 8 + fk * 2 + (h & 1)] = acc[j][h];
          finish_chain_partial(a, worker, lt, flags + worker, it.reduce);
          continue;
        }
#pragma unroll
        for (int j = 0; j < 2; ++j)
#pragma unroll
          for (int h = 0; h < 4; ++h)
          {
            const int gm = it.m0 + wm * 16 + (h >> 1) * 8 + fr, gn = it.n0 + wn * 16 + j * 8 + fk * 2 + (h & 1);
            if (gm < blk.m && gn < blk.n) store_entry(a, it.stage, blk, gm, gn, acc[j][h]);
          }
        store_pad(a, it.stage, blk, it.m0, it.n0, lt);
        if (!second) signal_done(a, worker, lt);
      }
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
        if (threadIdx.x == 0) *L.exit_count = 0;
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
      return w;
    }

    cudaError_t launch_chain(const ChainLaunch &launch, int32_t n_ctas, int64_t longest, cudaStream_t stream)
    {
      const int bytes = std::max<int>(kF64Workers * 2 * 2 * kDmmaStepK * 36 * 8, kChainPinBytes);
      static std::once_flag once;
      cudaError_t e = cudaSuccess;
      std::call_once(once, [&] { e = cudaFuncSetAttribute(chain_dmma_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes); });
      if (e != cudaSuccess) return e;
      const int workers = static_cast<int>(std::clamp<int64_t>(longest, 1, kF64Workers));
      return launch_dependent(chain_dmma_kernel, n_ctas, workers * kWorkerThreads, bytes, stream, launch);
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
    const cudaError_t e = launch_chain(launch, deal.n_ctas, deal.longest, stream);
    if (e == cudaSuccess) *used = true;
    return e;
  }

} // namespace ttg
