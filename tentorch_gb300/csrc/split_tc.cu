// Split-precision block products on the 5th-generation tensor cores (tcgen05) for GEMM ops whose
// blocks are large enough to fill 128 x 64 output tiles (the SU(2) and Fibonacci recouplings, large
// bonds).  The numerical scheme is the one of gemm.cu (Ozaki's error-free splitting: every row of A
// and column of B cut into S exact 7-bit bf16 slices, cut once by the slicing pass); what changes is
// where the slice products run:
//
//   - a CTA (16 warps, one per SM) owns a 128 x 64 output tile and runs every pair of its block over
//     the whole K, so no tile is split into partial sums;
//   - K advances 32 at a time through a ring of three shared-memory stages, each holding the S
//     slices of A (128 x 32) and of B (64 x 32) in the K-major core-matrix layout (8 rows x 16 bytes
//     per core matrix, no swizzle), filled with 16-byte cp.async;
//   - one thread issues tcgen05.mma kind::f16 (bf16 x bf16 -> fp32, M = 128, N = 64, K = 16) for
//     every slice pair (t, u) with t + u < S, into the accumulator of level t + u in tensor memory
//     (S accumulators of 64 columns: at most 6 x 64 = 384 of the SM's 512 columns); tcgen05.commit
//     on the stage's mbarrier tells when the stage may be refilled;
//   - every 256 of K (the level sums are integers below 2^24 that far, so fp32 holds them exactly)
//     the warps read the levels back with tcgen05.ld (warp w reads lanes 32 (w % 4) .. + 31, the rows
//     of its quarter, columns 16 (w / 4) .. + 15) and fold them exactly: the four leading levels as
//     an int64 sum_l lev_l 2^(7 (3 - l)), the rest through one fp32 sum; at the end of a pair one FP64
//     step per entry applies the row and column scales and adds into the tile's FP64 value.
// Every wait on an mbarrier gives up after two seconds and raises an error flag; the outcome of every
// wait is made the same for the whole CTA before anything depends on it, and the CTA frees its
// tensor memory on every path out.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <mutex>
#include <vector>

#include "executor.h"
#include "gemm.h"
#include "gemm_device.cuh"
#include "launch.h"

namespace ttg
{
  namespace
  {
    constexpr int kTcM = 128, kTcN = 64, kTcK = 32;  // output tile, K per stage
    constexpr int kTcStages = 3;
    constexpr int kTcThreads = 512;
    constexpr int kTcCols = kTcN / (kTcThreads / 128);  // columns of a tile each thread folds and stores
    constexpr int kTcMaxSlices = 6;
    constexpr int kTcChunkSteps = kExactChunk / kTcK;  // stages between drains of the level sums
    // core-matrix layout of one operand slice in a stage: 16 bytes per (row, 8 of K); the 4 groups of
    // 8 of K of a row group follow one another (LBO), row groups after them (SBO)
    constexpr int kTcLbo = 128, kTcSbo = (kTcK / 8) * 128;
    constexpr int kTcSliceA = kTcM * kTcK * 2, kTcSliceB = kTcN * kTcK * 2;  // bytes
    constexpr unsigned long long kTcWaitNs = 2000000000ull;

    template <int S>
    __host__ __device__ constexpr int tc_stage_bytes() { return S * (kTcSliceA + kTcSliceB); }
    template <int S>
    __host__ __device__ constexpr int tc_smem_bytes() { return kTcStages * tc_stage_bytes<S>(); }
    // at least 120 KiB, so that a second CTA never shares the SM (each holds all 512 columns of its
    // tensor memory)
    template <int S>
    constexpr int tc_launch_bytes() { return tc_smem_bytes<S>() > 120 * 1024 ? tc_smem_bytes<S>() : 120 * 1024; }

    struct TcItem
    {
      int32_t block, m0, n0, pad;
    };

    struct TcArgs
    {
      const uint16_t *sa, *sb;  // slices of A rows and of B columns (gemm.cu's scratch layout)
      const int16_t *exps_a, *exps_b;
      int64_t stride_a, stride_b;  // elements between two slices of all A rows (B columns)
      double *c;
      const DevBlock *blocks;
      const DevPair *pairs;
      const DevSplitPair *spairs;
      const TcItem *items;
      const int32_t *cta_begin;
      int *error;
    };

    __device__ __forceinline__ uint32_t smem_addr(const void *p) { return static_cast<uint32_t>(__cvta_generic_to_shared(p)); }

    __device__ __forceinline__ uint64_t tc_desc(uint32_t addr)
    {
      // start address, leading (K) and stride (row group) byte offsets in 16-byte units, version 1,
      // base offset 0, no swizzle
      return static_cast<uint64_t>((addr >> 4) & 0x3FFF) | (static_cast<uint64_t>((kTcLbo >> 4) & 0x3FFF) << 16) |
             (static_cast<uint64_t>((kTcSbo >> 4) & 0x3FFF) << 32) | (static_cast<uint64_t>(1) << 46);
    }

    // kind::f16 instruction descriptor: D fp32, A and B bf16, both K-major, N >> 3 at bit 17, M >> 4
    // at bit 24
    constexpr uint32_t kTcInstr = (1u << 4) | (1u << 7) | (1u << 10) | (static_cast<uint32_t>(kTcN >> 3) << 17) |
                                  (static_cast<uint32_t>(kTcM >> 4) << 24);

    __device__ __forceinline__ void tc_mma(uint32_t tmem, uint64_t a, uint64_t b, uint32_t accumulate)
    {
      asm volatile("{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                   "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem),
                   "l"(a), "l"(b), "r"(kTcInstr), "r"(accumulate));
    }

    __device__ __forceinline__ unsigned long long tc_now()
    {
      unsigned long long t;
      asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
      return t;
    }

    // Wait for the phase of `bar` with parity `parity`; false when two seconds passed first.
    __device__ __forceinline__ bool tc_wait(uint64_t *bar, uint32_t parity)
    {
      const uint32_t at = smem_addr(bar);
      const unsigned long long start = tc_now();
      while (true)
      {
        uint32_t done;
        asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}\n"
                     : "=r"(done)
                     : "r"(at), "r"(parity)
                     : "memory");
        if (done) return true;
        if (tc_now() - start > kTcWaitNs) return false;
      }
    }

    // 16 columns of one lane of tensor memory
    __device__ __forceinline__ void tc_load16(uint32_t addr, uint32_t (&r)[16])
    {
      asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
                   : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                     "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
                   : "r"(addr));
    }

    template <int S>
    __global__ void __launch_bounds__(kTcThreads, 1) gemm_split_tc_kernel(TcArgs a)
    {
      dependent_entry();
      extern __shared__ __align__(1024) unsigned char smem[];
      __shared__ __align__(8) uint64_t stage_done[kTcStages];
      __shared__ uint32_t tmem_base;
      __shared__ int col_exp[kTcN];
      __shared__ int failed;
      const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
      // tensor-memory lanes 32 quarter .. + 31 (the quarter a warp may access), columns kTcCols part ..
      const int quarter = warp & 3, part = warp >> 2;
      if (warp == 0)
      {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;" ::"r"(smem_addr(&tmem_base)));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
      }
      if (tid == 0)
      {
        for (int s = 0; s < kTcStages; ++s) asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&stage_done[s])));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        failed = 0;
      }
      __syncthreads();
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t tmem = tmem_base;
      // per stage: whether a commit is outstanding, and the parity of the phase it completes (the
      // same for every thread: control flow is uniform)
      bool pending[kTcStages] = {};
      uint32_t parity[kTcStages] = {};
      const auto settle = [&](int s) -> bool
      {
        if (!pending[s]) return true;
        pending[s] = false;
        const bool ok = tc_wait(&stage_done[s], parity[s]);
        parity[s] ^= 1u;
        return ok;
      };
      const int64_t list_begin = a.cta_begin[blockIdx.x], list_end = a.cta_begin[blockIdx.x + 1];
      for (int64_t idx = list_begin; idx < list_end && !failed; ++idx)
      {
        const TcItem it = a.items[idx];
        const DevBlock blk = a.blocks[it.block];
        const int row = it.m0 + 32 * quarter + lane;
        const int col0 = kTcCols * part;
        double value[kTcCols];
#pragma unroll
        for (int j = 0; j < kTcCols; ++j) value[j] = 0.0;
        for (int32_t pi = 0; pi < blk.pair_count && !failed; ++pi)
        {
          const DevPair pr = a.pairs[blk.pair_begin + pi];
          const DevSplitPair sp = a.spairs[blk.pair_begin + pi];
          if (pr.k <= 0) continue;
          const int steps = (pr.k + kTcK - 1) / kTcK;
          const uint16_t *ga = a.sa + sp.sa + static_cast<int64_t>(it.m0) * sp.kp;
          const uint16_t *gb = a.sb + sp.sb + static_cast<int64_t>(it.n0) * sp.kp;
          const int rows = min(kTcM, blk.m - it.m0), cols = min(kTcN, blk.n - it.n0);
          // the stage of step `step`: S slices of A then of B, zeros outside the block
          const auto load = [&](int step)
          {
            unsigned char *base = smem + (step % kTcStages) * tc_stage_bytes<S>();
            const int k = step * kTcK;
            for (int c = tid; c < S * kTcM * 4; c += kTcThreads)
            {
              const int t = c / (kTcM * 4), r = (c >> 2) % kTcM, q = c & 3;
              const bool in = r < rows;
              const uint32_t dst = smem_addr(base + t * kTcSliceA + (r >> 3) * kTcSbo + q * kTcLbo + (r & 7) * 16);
              const uint16_t *src = ga + t * a.stride_a + static_cast<int64_t>(in ? r : 0) * sp.kp + k + q * 8;
              asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(dst), "l"(src), "r"(in ? 16 : 0));
            }
            for (int c = tid; c < S * kTcN * 4; c += kTcThreads)
            {
              const int u = c / (kTcN * 4), r = (c >> 2) % kTcN, q = c & 3;
              const bool in = r < cols;
              const uint32_t dst =
                smem_addr(base + S * kTcSliceA + u * kTcSliceB + (r >> 3) * kTcSbo + q * kTcLbo + (r & 7) * 16);
              const uint16_t *src = gb + u * a.stride_b + static_cast<int64_t>(in ? r : 0) * sp.kp + k + q * 8;
              asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(dst), "l"(src), "r"(in ? 16 : 0));
            }
            asm volatile("cp.async.commit_group;\n" ::: "memory");
          };
          if (tid < kTcN) col_exp[tid] = tid < cols ? a.exps_b[sp.eb + it.n0 + tid] : 0;
          const int row_exp = row < blk.m ? a.exps_a[sp.ea + row] : 0;
          long long head[kTcCols];
          float tail[kTcCols];
#pragma unroll
          for (int j = 0; j < kTcCols; ++j)
          {
            head[j] = 0;
            tail[j] = 0.0f;
          }
          // the ring: steps 0 and 1 in flight before the first products
          bool ok = settle(0);
          ok = settle(1) && ok;
          ok = __syncthreads_and(ok);
          if (ok)
          {
            load(0);
            if (steps > 1) load(1);
          }
          for (int step = 0; step < steps && ok; ++step)
          {
            const int s = step % kTcStages;
            bool good = true;
            if (step + 2 < steps)
            {
              good = settle((step + 2) % kTcStages);  // the products of step - 1 read it
              load(step + 2);
              asm volatile("cp.async.wait_group 2;\n" ::: "memory");
            }
            else if (step + 1 < steps)
              asm volatile("cp.async.wait_group 1;\n" ::: "memory");
            else
              asm volatile("cp.async.wait_group 0;\n" ::: "memory");
            // the stage's bytes, written through the generic proxy, become visible to the tensor cores
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            if (!__syncthreads_and(good))
            {
              ok = false;
              break;
            }
            const bool chunk_first = step % kTcChunkSteps == 0;
            if (tid == 0)
            {
              asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
              const uint32_t a_base = smem_addr(smem + s * tc_stage_bytes<S>());
              const uint32_t b_base = a_base + S * kTcSliceA;
#pragma unroll 1
              for (int kk = 0; kk < kTcK; kk += 16)
#pragma unroll 1
                for (int t = 0; t < S; ++t)
#pragma unroll 1
                  for (int u = 0; u + t < S; ++u)
                  {
                    // level t + u is first reached at t = 0: that product starts the chunk's sum
                    const uint32_t accumulate = (chunk_first && kk == 0 && t == 0) ? 0u : 1u;
                    tc_mma(tmem + static_cast<uint32_t>((t + u) * kTcN), tc_desc(a_base + t * kTcSliceA + (kk / 8) * kTcLbo),
                           tc_desc(b_base + u * kTcSliceB + (kk / 8) * kTcLbo), accumulate);
                  }
              asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                smem_addr(&stage_done[s])));
            }
            pending[s] = true;
            if ((step + 1) % kTcChunkSteps == 0 || step + 1 == steps)
            {
              // the chunk's level sums: wait for its products, read them back, fold them exactly
              good = settle(s);
              asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
              uint32_t lev[kTcCols];
              const uint32_t lane_addr = tmem + (static_cast<uint32_t>(32 * quarter) << 16) + static_cast<uint32_t>(col0);
#pragma unroll
              for (int l = 0; l < S; ++l)
              {
                tc_load16(lane_addr + static_cast<uint32_t>(l * kTcN), lev);
                asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
                for (int j = 0; j < kTcCols; ++j)
                {
                  const float x = __uint_as_float(lev[j]);
                  if (l < 4)
                    head[j] += static_cast<long long>(__float2int_rn(x)) << (7 * (3 - l));
                  else
                    tail[j] = fmaf(x, ldexpf(1.0f, -7 * (l - 4)), tail[j]);
                }
              }
              asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
              if (!__syncthreads_and(good))
              {
                ok = false;
                break;
              }
            }
          }
          if (!ok)
          {
            if (tid == 0) atomicExch(a.error, 1);
            failed = 1;
          }
          __syncthreads();
          // one FP64 step per entry: head 2^-35 + tail 2^-42 times the row and column scales
#pragma unroll
          for (int j = 0; j < kTcCols; ++j)
          {
            const int ex = row_exp + col_exp[col0 + j];
            value[j] += fma(static_cast<double>(head[j]), pow2(ex - 35), static_cast<double>(tail[j]) * pow2(ex - 42));
          }
          __syncthreads();  // col_exp is rewritten by the next pair
        }
        if (row < blk.m)
        {
          double *out = a.c + blk.c + static_cast<int64_t>(row) * blk.n + it.n0 + col0;
#pragma unroll
          for (int j = 0; j < kTcCols; ++j)
            if (it.n0 + col0 + j < blk.n) out[j] = value[j];
        }
        const int64_t entries = static_cast<int64_t>(blk.m) * blk.n;
        if (tid == 0 && it.m0 + kTcM >= blk.m && it.n0 + kTcN >= blk.n && (entries & 1)) a.c[blk.c + entries] = 0.0;
      }
      // no copy or product may still write shared or tensor memory when the CTA leaves
      asm volatile("cp.async.wait_all;\n" ::: "memory");
      for (int s = 0; s < kTcStages; ++s)
        if (!settle(s) && lane == 0) atomicExch(a.error, 1);
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncthreads();
      if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;" ::"r"(tmem));
    }
  } // namespace

  // ------------------------------------------------------------------------------------------
  // host
  // ------------------------------------------------------------------------------------------

  bool split_tc_suits(const Program &p, const Op &op, int32_t slices)
  {
    if (slices < 1 || slices > kTcMaxSlices) return false;
    // enough whole tiles to give every SM several, and most of the work in them
    double work = 0, tiled = 0;
    int64_t tiles = 0;
    for (int64_t b = op.begin; b < op.begin + op.count; ++b)
    {
      const GemmBlock &blk = p.gemm_blocks[static_cast<size_t>(b)];
      int64_t k = 0;
      for (int32_t q = 0; q < blk.pair_count; ++q) k += p.gemm_pairs[static_cast<size_t>(blk.pair_begin + q)].k;
      const double w = static_cast<double>(blk.m) * blk.n * k;
      work += w;
      tiles += static_cast<int64_t>((blk.m + kTcM - 1) / kTcM) * ((blk.n + kTcN - 1) / kTcN);
      if (blk.m >= kTcM / 2 && blk.n >= kTcN / 2) tiled += w;
    }
    return tiles >= 4 * static_cast<int64_t>(p.ctas) && tiled >= 0.9 * work;
  }

  cudaError_t launch_split_tc(const Program &p, const Op &op, DeviceTables &t, size_t op_index, int32_t slices,
                              const uint16_t *sa, const uint16_t *sb, const int16_t *exps_a, const int16_t *exps_b,
                              int64_t stride_a, int64_t stride_b, const void *spairs, double *C, int *error,
                              cudaStream_t stream)
  {
    DeviceTables::TcTables &tc = t.tc[op_index];
    {
      std::lock_guard<std::mutex> lock(t.mutex);
      if (!tc.ready)
      {
        // tiles largest first (K of the block), each to the least loaded SM
        struct Sized
        {
          TcItem item;
          double work;
        };
        std::vector<Sized> all;
        for (int64_t b = op.begin; b < op.begin + op.count; ++b)
        {
          const GemmBlock &blk = p.gemm_blocks[static_cast<size_t>(b)];
          int64_t k = 0;
          for (int32_t q = 0; q < blk.pair_count; ++q) k += p.gemm_pairs[static_cast<size_t>(blk.pair_begin + q)].k;
          for (int32_t m0 = 0; m0 < blk.m; m0 += kTcM)
            for (int32_t n0 = 0; n0 < blk.n; n0 += kTcN)
              all.push_back({{static_cast<int32_t>(b), m0, n0, 0}, static_cast<double>(kTcK) * (1 + (k + kTcK - 1) / kTcK)});
        }
        std::stable_sort(all.begin(), all.end(), [](const Sized &x, const Sized &y) { return x.work > y.work; });
        const int ctas = static_cast<int>(std::min<size_t>(static_cast<size_t>(p.ctas), std::max<size_t>(all.size(), 1)));
        std::vector<std::vector<TcItem>> lists(static_cast<size_t>(ctas));
        std::vector<std::pair<double, int>> heap;
        for (int c = 0; c < ctas; ++c) heap.push_back({0.0, c});
        const auto later = [](const std::pair<double, int> &x, const std::pair<double, int> &y)
        { return x.first > y.first || (x.first == y.first && x.second > y.second); };
        std::make_heap(heap.begin(), heap.end(), later);
        for (const Sized &s : all)
        {
          std::pop_heap(heap.begin(), heap.end(), later);
          auto &least = heap.back();
          lists[static_cast<size_t>(least.second)].push_back(s.item);
          least.first += s.work;
          std::push_heap(heap.begin(), heap.end(), later);
        }
        std::vector<TcItem> items;
        std::vector<int32_t> begin{0};
        for (const auto &list : lists)
        {
          items.insert(items.end(), list.begin(), list.end());
          begin.push_back(static_cast<int32_t>(items.size()));
        }
        TableStaging staging;
        staging.add(items, &tc.items);
        staging.add(begin, reinterpret_cast<void **>(&tc.cta_begin));
        const cudaError_t e = staging.commit(&tc.base);
        if (e != cudaSuccess) return e;
        tc.n_ctas = ctas;
        tc.ready = true;
      }
    }
    TcArgs args{sa, sb, exps_a, exps_b, stride_a, stride_b, C, reinterpret_cast<const DevBlock *>(t.blocks),
                reinterpret_cast<const DevPair *>(t.pairs), static_cast<const DevSplitPair *>(spairs),
                static_cast<const TcItem *>(tc.items), tc.cta_begin, error};
    cudaError_t e = cudaSuccess;
    switch (slices)
    {
#define TTG_TC(S)                                                                                                          \
  case S:                                                                                                                  \
  {                                                                                                                        \
    static std::once_flag once;                                                                                            \
    std::call_once(once, [&] {                                                                                             \
      e = cudaFuncSetAttribute(gemm_split_tc_kernel<S>, cudaFuncAttributeMaxDynamicSharedMemorySize, tc_launch_bytes<S>()); \
    });                                                                                                                    \
    if (e != cudaSuccess) return e;                                                                                        \
    e = launch_dependent(gemm_split_tc_kernel<S>, tc.n_ctas, kTcThreads, tc_launch_bytes<S>(), stream, args);             \
    break;                                                                                                                 \
  }
      TTG_TC(1) TTG_TC(2) TTG_TC(3) TTG_TC(4) TTG_TC(5) TTG_TC(6)
#undef TTG_TC
    default: return cudaErrorInvalidValue;
    }
    return e;
  }

} // namespace ttg
