// Grouped block-pair GEMM for sm_103a: the balanced work schedule, the FP64 / complex128 item
// kernel, the deterministic partial-tile reduction, and the split-precision path (row / column
// slicing into exact bf16 integers, mma.sync bf16 products with exact fp32 accumulation per
// K-chunk, FP64 combination).  See gemm.h for the numerical scheme.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <set>

#include "executor.h"
#include "gemm.h"

namespace ttg
{
  // ------------------------------------------------------------------------------------------
  // schedules (host)
  // ------------------------------------------------------------------------------------------

  GemmSchedule schedule_gemm(const Program &p, const Op &op, int bm, int bn)
  {
    GemmSchedule s;
    double total = 0;
    for (int64_t b = op.begin; b < op.begin + op.count; ++b)
    {
      const GemmBlock &blk = p.gemm_blocks[static_cast<size_t>(b)];
      for (int32_t k = 0; k < blk.pair_count; ++k)
        total += static_cast<double>(blk.m) * blk.n * p.gemm_pairs[static_cast<size_t>(blk.pair_begin + k)].k;
    }
    // about four items per SM of the 152, never smaller than a tile over 64 of K
    const double target = std::max(total / (152.0 * 4.0), static_cast<double>(bm) * bn * 64.0);
    struct Sized
    {
      GemmItem item;
      double work;
    };
    std::vector<Sized> items;
    for (int64_t b = op.begin; b < op.begin + op.count; ++b)
    {
      const GemmBlock &blk = p.gemm_blocks[static_cast<size_t>(b)];
      int64_t ktotal = 0;
      for (int32_t k = 0; k < blk.pair_count; ++k) ktotal += p.gemm_pairs[static_cast<size_t>(blk.pair_begin + k)].k;
      for (int32_t m0 = 0; m0 < blk.m; m0 += bm)
        for (int32_t n0 = 0; n0 < blk.n; n0 += bn)
        {
          const double rows = std::min(bm, blk.m - m0), cols = std::min(bn, blk.n - n0);
          const double work = rows * cols * static_cast<double>(ktotal);
          int64_t chunks = std::max<int64_t>(1, static_cast<int64_t>(std::ceil(work / target)));
          int64_t kc = (ktotal + chunks - 1) / std::max<int64_t>(chunks, 1);
          kc = std::max<int64_t>(16, (kc + 15) / 16 * 16);
          chunks = ktotal > 0 ? (ktotal + kc - 1) / kc : 1;
          const int32_t bi = static_cast<int32_t>(b);
          if (chunks == 1)
          {
            items.push_back({{bi, m0, n0, 0, static_cast<int32_t>(ktotal), -1}, work});
            continue;
          }
          const int32_t slot0 = static_cast<int32_t>(s.slots);
          for (int64_t c = 0; c < chunks; ++c)
          {
            const int64_t k0 = c * kc, k1 = std::min(ktotal, (c + 1) * kc);
            items.push_back({{bi, m0, n0, static_cast<int32_t>(k0), static_cast<int32_t>(k1), static_cast<int32_t>(s.slots++)},
                             rows * cols * static_cast<double>(k1 - k0)});
          }
          s.reduces.push_back({bi, m0, n0, slot0, static_cast<int32_t>(chunks), 0});
        }
    }
    // the largest items launch first, so the tail of the grid is made of small ones
    std::stable_sort(items.begin(), items.end(), [](const Sized &a, const Sized &b) { return a.work > b.work; });
    for (const Sized &it : items) s.items.push_back(it.item);
    return s;
  }

  void gemm_operands(const Program &p, const Op &op, std::vector<OperandBlock> &left, std::vector<OperandBlock> &right)
  {
    std::set<int64_t> seen_a, seen_b;
    left.clear();
    right.clear();
    for (int64_t b = op.begin; b < op.begin + op.count; ++b)
    {
      const GemmBlock &blk = p.gemm_blocks[static_cast<size_t>(b)];
      for (int32_t k = 0; k < blk.pair_count; ++k)
      {
        const GemmPair &pr = p.gemm_pairs[static_cast<size_t>(blk.pair_begin + k)];
        if (seen_a.insert(pr.a).second) left.push_back({pr.a, blk.m, pr.k});
        if (seen_b.insert(pr.b).second) right.push_back({pr.b, pr.k, blk.n});
      }
    }
  }

  namespace
  {
    int64_t split_scratch(int64_t size_a, int64_t size_b, int64_t slots)
    {
      // bf16 slices and int16 exponents of both operands, then the FP64 partial tiles, all in
      // doubles and each part rounded up to 256 bytes
      const auto up = [](int64_t bytes) { return (bytes + 255) / 256 * 32; };
      return up(2 * kMaxSlices * size_a) + up(2 * kMaxSlices * size_b) + up(2 * size_a) + up(2 * size_b) +
             slots * kSplitTileM * kSplitTileN;
    }
  } // namespace

  int64_t gemm_scratch(const Program &p)
  {
    int64_t need = 0;
    for (const Op &op : p.ops)
    {
      if (op.kind != OpKind::gemm) continue;
      const GemmSchedule f = schedule_gemm(p, op, kF64TileM, kF64TileN);
      const GemmSchedule s = schedule_gemm(p, op, kSplitTileM, kSplitTileN);
      const int64_t size_a = p.buffers[static_cast<size_t>(op.src)].size;
      const int64_t size_b = p.buffers[static_cast<size_t>(op.src2)].size;
      // complex partials take two doubles an entry
      need = std::max(need, 2 * f.slots * kF64TileM * kF64TileN);
      need = std::max(need, split_scratch(size_a, size_b, s.slots));
    }
    return need;
  }

  // ------------------------------------------------------------------------------------------
  // device
  // ------------------------------------------------------------------------------------------

  namespace
  {
    struct DevBlock
    {
      int64_t c;
      int32_t m, n, pair_begin, pair_count;
    };
    struct DevPair
    {
      int64_t a, b;
      int32_t k, pad;
    };

    __device__ __forceinline__ double2 cfma(double2 a, double2 b, double2 c)
    {
      c.x = fma(a.x, b.x, fma(-a.y, b.y, c.x));
      c.y = fma(a.x, b.y, fma(a.y, b.x, c.y));
      return c;
    }
    __device__ __forceinline__ double fma_t(double a, double b, double c) { return fma(a, b, c); }
    __device__ __forceinline__ double2 fma_t(double2 a, double2 b, double2 c) { return cfma(a, b, c); }
    template <typename T>
    __device__ __forceinline__ T zero_t();
    template <>
    __device__ __forceinline__ double zero_t<double>() { return 0.0; }
    template <>
    __device__ __forceinline__ double2 zero_t<double2>() { return make_double2(0.0, 0.0); }
    __device__ __forceinline__ double add_t(double a, double b) { return a + b; }
    __device__ __forceinline__ double2 add_t(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }

    // One work item: a 32x32 output tile over a K range, 64 threads of 4x4 entries, K staged 16 at
    // a time through shared memory.  FP64 on this part issues about two DFMA per SM clock, which
    // small balanced items keep busy on every SM.
    template <typename T>
    __global__ void __launch_bounds__(64) gemm_items_kernel(const T *__restrict__ A, const T *__restrict__ B,
                                                            T *__restrict__ C, const DevBlock *__restrict__ blocks,
                                                            const DevPair *__restrict__ pairs,
                                                            const GemmItem *__restrict__ items, T *__restrict__ partial)
    {
      constexpr int BM = kF64TileM, BN = kF64TileN, BK = 16, TM = 4, TN = 4, THREADS = 64;
      __shared__ T as[BK][BM];
      __shared__ T bs[BK][BN + 1];
      const GemmItem it = items[blockIdx.x];
      const DevBlock blk = blocks[it.block];
      const int tx = threadIdx.x % (BN / TN), ty = threadIdx.x / (BN / TN);
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
          for (int i = threadIdx.x; i < BM * BK; i += THREADS)
          {
            const int r = i / BK, kk = i % BK;
            const int gm = it.m0 + r, gk = k0 + kk;
            as[kk][r] = (gm < blk.m && gk < hi) ? a[static_cast<int64_t>(gm) * K + gk] : zero_t<T>();
          }
          for (int i = threadIdx.x; i < BK * BN; i += THREADS)
          {
            const int kk = i / BN, cc = i % BN;
            const int gk = k0 + kk, gn = it.n0 + cc;
            bs[kk][cc] = (gk < hi && gn < blk.n) ? b[static_cast<int64_t>(gk) * blk.n + gn] : zero_t<T>();
          }
          __syncthreads();
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
          __syncthreads();
        }
      }
      if (it.slot >= 0)
      {
        T *out = partial + static_cast<int64_t>(it.slot) * BM * BN;
#pragma unroll
        for (int i = 0; i < TM; ++i)
#pragma unroll
          for (int j = 0; j < TN; ++j) out[(ty * TM + i) * BN + tx * TN + j] = acc[i][j];
        return;
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
      if (threadIdx.x == 0 && it.m0 + BM >= blk.m && it.n0 + BN >= blk.n && (entries & 1)) C[blk.c + entries] = zero_t<T>();
    }

    // The partial tiles of one split tile, summed in slot order into C.
    template <typename T>
    __global__ void reduce_kernel(T *__restrict__ C, const DevBlock *__restrict__ blocks,
                                  const GemmReduce *__restrict__ reduces, const T *__restrict__ partial, int bm, int bn)
    {
      const GemmReduce r = reduces[blockIdx.x];
      const DevBlock blk = blocks[r.block];
      for (int e = threadIdx.x; e < bm * bn; e += blockDim.x)
      {
        const int i = e / bn, j = e % bn;
        const int gm = r.m0 + i, gn = r.n0 + j;
        if (gm >= blk.m || gn >= blk.n) continue;
        T sum = zero_t<T>();
        for (int s = 0; s < r.nslots; ++s) sum = add_t(sum, partial[static_cast<int64_t>(r.slot0 + s) * bm * bn + e]);
        C[blk.c + static_cast<int64_t>(gm) * blk.n + gn] = sum;
      }
      const int64_t entries = static_cast<int64_t>(blk.m) * blk.n;
      if (threadIdx.x == 0 && r.m0 + bm >= blk.m && r.n0 + bn >= blk.n && (entries & 1)) C[blk.c + entries] = zero_t<T>();
    }

    // ---------------------------------------------------------------------------------------
    // split precision
    // ---------------------------------------------------------------------------------------

    struct SplitLine
    {
      int64_t src, dst, exp;
      int32_t len, src_stride;
    };

    // One warp per line (a row of A or a column of B): the power of two that bounds the line,
    // then `slices` 7-bit integer slices of every entry, exact in bf16.
    __global__ void split_lines_kernel(const double *__restrict__ src, uint16_t *__restrict__ slices,
                                       int16_t *__restrict__ exps, int64_t slice_stride,
                                       const SplitLine *__restrict__ lines, int64_t n_lines, int slices_n)
    {
      const int lane = threadIdx.x & 31;
      const int64_t warp = (static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
      const int64_t warps = (static_cast<int64_t>(gridDim.x) * blockDim.x) >> 5;
      for (int64_t l = warp; l < n_lines; l += warps)
      {
        const SplitLine line = lines[l];
        double big = 0.0;
        for (int i = lane; i < line.len; i += 32) big = fmax(big, fabs(src[line.src + static_cast<int64_t>(i) * line.src_stride]));
        for (int off = 16; off > 0; off >>= 1) big = fmax(big, __shfl_xor_sync(0xffffffffu, big, off));
        int e = 0;
        if (big > 0.0) frexp(big, &e);  // big = f 2^e with f in [0.5, 1): every |entry| / 2^e < 1
        if (lane == 0) exps[line.exp] = static_cast<int16_t>(e);
        for (int i = lane; i < line.len; i += 32)
        {
          double x = ldexp(src[line.src + static_cast<int64_t>(i) * line.src_stride], -e);
          for (int t = 0; t < slices_n; ++t)
          {
            x *= 128.0;
            const double q = rint(x);
            x -= q;  // exact: q is the nearest integer to x
            slices[t * slice_stride + line.dst + i] = __bfloat16_as_ushort(__double2bfloat16(q));
          }
        }
      }
    }

    __device__ __forceinline__ uint32_t pack2(uint16_t lo, uint16_t hi)
    {
      return static_cast<uint32_t>(lo) | (static_cast<uint32_t>(hi) << 16);
    }

    __device__ __forceinline__ void mma_bf16(float (&c)[4], const uint32_t (&a)[4], const uint32_t (&b)[2])
    {
      asm volatile("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
                   "{%0,%1,%2,%3};\n"
                   : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
                   : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
    }

    // One work item: a 64x32 tile over a K range, 8 warps of 16x16 (one m16 x two n8 MMA tiles).
    // For every K-chunk of <= 256, the products of slices t and u are summed exactly in fp32 per
    // level t + u, then folded into FP64 with the weight 2^-7(t+u+2) and the pair's row and column
    // scales.  S slices keep the levels t + u <= S - 1.
    template <int S>
    __global__ void __launch_bounds__(256, 1) gemm_split_kernel(const uint16_t *__restrict__ sa, const int16_t *__restrict__ ea,
                                                             int64_t stride_a, const uint16_t *__restrict__ sb,
                                                             const int16_t *__restrict__ eb, int64_t stride_b,
                                                             double *__restrict__ C, const DevBlock *__restrict__ blocks,
                                                             const DevPair *__restrict__ pairs,
                                                             const GemmItem *__restrict__ items, double *__restrict__ partial)
    {
      const GemmItem it = items[blockIdx.x];
      const DevBlock blk = blocks[it.block];
      const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
      const int g = lane >> 2, tig = lane & 3;
      const int wm = warp >> 1, wn = warp & 1;        // 4 x 2 warps of 16 x 16
      const int row0 = it.m0 + wm * 16 + g;           // and row0 + 8
      const int colb = it.n0 + wn * 16 + tig * 2;     // + nsub * 8 + {0, 1}
      double acc[2][4] = {};                          // [nsub][c0..c3]
      int32_t kbase = 0;
      for (int32_t pi = 0; pi < blk.pair_count; ++pi)
      {
        const DevPair pr = pairs[blk.pair_begin + pi];
        const int K = pr.k;
        const int lo = max(it.k0 - kbase, 0), hi = min(it.k1 - kbase, K);
        kbase += K;
        if (lo >= hi) continue;
        // the pair's scales of this thread's two rows and four columns
        const bool r0ok = row0 < blk.m, r1ok = row0 + 8 < blk.m;
        const int er0 = r0ok ? ea[pr.a + static_cast<int64_t>(row0) * K] : 0;
        const int er1 = r1ok ? ea[pr.a + static_cast<int64_t>(row0 + 8) * K] : 0;
        int ec[2][2];
#pragma unroll
        for (int ns = 0; ns < 2; ++ns)
#pragma unroll
          for (int h = 0; h < 2; ++h)
          {
            const int col = colb + ns * 8 + h;
            ec[ns][h] = col < blk.n ? eb[pr.b + col] : 0;
          }
        for (int kc = lo; kc < hi; kc += kExactChunk)
        {
          const int kend = min(kc + kExactChunk, hi);
          float lev[S][2][4];
#pragma unroll
          for (int l = 0; l < S; ++l)
#pragma unroll
            for (int ns = 0; ns < 2; ++ns)
#pragma unroll
              for (int q = 0; q < 4; ++q) lev[l][ns][q] = 0.0f;
          for (int k = kc; k < kend; k += 16)
          {
            const int ka = k + tig * 2;  // this thread's first k in each half of the step
#pragma unroll
            for (int t = 0; t < S; ++t)
            {
              const uint16_t *at = sa + t * stride_a + pr.a;
              uint32_t afrag[4];
              const auto ld_a = [&](int row, int kk) -> uint16_t {
                return (row < blk.m && kk < kend) ? at[static_cast<int64_t>(row) * K + kk] : uint16_t(0);
              };
              afrag[0] = pack2(ld_a(row0, ka), ld_a(row0, ka + 1));
              afrag[1] = pack2(ld_a(row0 + 8, ka), ld_a(row0 + 8, ka + 1));
              afrag[2] = pack2(ld_a(row0, ka + 8), ld_a(row0, ka + 9));
              afrag[3] = pack2(ld_a(row0 + 8, ka + 8), ld_a(row0 + 8, ka + 9));
#pragma unroll
              for (int u = 0; u + t < S; ++u)
              {
                const uint16_t *bt = sb + u * stride_b + pr.b;
#pragma unroll
                for (int ns = 0; ns < 2; ++ns)
                {
                  const int col = it.n0 + wn * 16 + ns * 8 + g;
                  const auto ld_b = [&](int kk) -> uint16_t {
                    return (col < blk.n && kk < kend) ? bt[static_cast<int64_t>(col) * K + kk] : uint16_t(0);
                  };
                  uint32_t bfrag[2] = {pack2(ld_b(ka), ld_b(ka + 1)), pack2(ld_b(ka + 8), ld_b(ka + 9))};
                  mma_bf16(lev[t + u][ns], afrag, bfrag);
                }
              }
            }
          }
          // fold the exact level sums into FP64
#pragma unroll
          for (int ns = 0; ns < 2; ++ns)
#pragma unroll
            for (int q = 0; q < 4; ++q)
            {
              double s = 0.0;
#pragma unroll
              for (int l = S - 1; l >= 0; --l) s = fma(static_cast<double>(lev[l][ns][q]), ldexp(1.0, -7 * (l + 2)), s);
              const int er = q < 2 ? er0 : er1;
              acc[ns][q] = fma(s, ldexp(1.0, er + ec[ns][q & 1]), acc[ns][q]);
            }
        }
      }
      if (it.slot >= 0)
      {
        double *out = partial + static_cast<int64_t>(it.slot) * kSplitTileM * kSplitTileN;
#pragma unroll
        for (int ns = 0; ns < 2; ++ns)
#pragma unroll
          for (int q = 0; q < 4; ++q)
          {
            const int r = wm * 16 + g + (q >= 2 ? 8 : 0), c = wn * 16 + ns * 8 + tig * 2 + (q & 1);
            out[r * kSplitTileN + c] = acc[ns][q];
          }
        return;
      }
#pragma unroll
      for (int ns = 0; ns < 2; ++ns)
#pragma unroll
        for (int q = 0; q < 4; ++q)
        {
          const int gm = row0 + (q >= 2 ? 8 : 0), gn = colb + ns * 8 + (q & 1);
          if (gm < blk.m && gn < blk.n) C[blk.c + static_cast<int64_t>(gm) * blk.n + gn] = acc[ns][q];
        }
      const int64_t entries = static_cast<int64_t>(blk.m) * blk.n;
      if (threadIdx.x == 0 && it.m0 + kSplitTileM >= blk.m && it.n0 + kSplitTileN >= blk.n && (entries & 1))
        C[blk.c + entries] = 0.0;
    }

    template <int S>
    cudaError_t launch_split_s(const uint16_t *sa, const int16_t *ea, int64_t stride_a, const uint16_t *sb,
                               const int16_t *eb, int64_t stride_b, double *C, const DevBlock *blocks,
                               const DevPair *pairs, const GemmItem *items, int64_t n_items, double *partial,
                               cudaStream_t stream)
    {
      gemm_split_kernel<S><<<static_cast<unsigned>(n_items), 256, 0, stream>>>(sa, ea, stride_a, sb, eb, stride_b, C,
                                                                              blocks, pairs, items, partial);
      return cudaGetLastError();
    }
  } // namespace

  // ------------------------------------------------------------------------------------------
  // launchers
  // ------------------------------------------------------------------------------------------

  cudaError_t launch_gemm_f64(const Program &p, DeviceTables &t, size_t op_index, const void *A, const void *B, void *C,
                              bool complex, void *scratch, cudaStream_t stream)
  {
    const auto &sched = t.gemm[op_index];
    if (sched.n_items == 0) return cudaSuccess;
    const auto *blocks = reinterpret_cast<const DevBlock *>(t.blocks);
    const auto *pairs = reinterpret_cast<const DevPair *>(t.pairs);
    if (complex)
    {
      gemm_items_kernel<double2><<<static_cast<unsigned>(sched.n_items), 64, 0, stream>>>(
        static_cast<const double2 *>(A), static_cast<const double2 *>(B), static_cast<double2 *>(C), blocks, pairs,
        sched.items, static_cast<double2 *>(scratch));
      if (sched.n_reduces)
        reduce_kernel<double2><<<static_cast<unsigned>(sched.n_reduces), 256, 0, stream>>>(
          static_cast<double2 *>(C), blocks, sched.reduces, static_cast<const double2 *>(scratch), kF64TileM, kF64TileN);
    }
    else
    {
      gemm_items_kernel<double><<<static_cast<unsigned>(sched.n_items), 64, 0, stream>>>(
        static_cast<const double *>(A), static_cast<const double *>(B), static_cast<double *>(C), blocks, pairs,
        sched.items, static_cast<double *>(scratch));
      if (sched.n_reduces)
        reduce_kernel<double><<<static_cast<unsigned>(sched.n_reduces), 256, 0, stream>>>(
          static_cast<double *>(C), blocks, sched.reduces, static_cast<const double *>(scratch), kF64TileM, kF64TileN);
    }
    (void)p;
    return cudaGetLastError();
  }

  cudaError_t launch_gemm_split(const Program &p, const Op &op, DeviceTables &t, size_t op_index, const double *A,
                                const double *B, double *C, int32_t slices, void *scratch, cudaStream_t stream)
  {
    const auto &sched = t.split[op_index];
    if (sched.n_items == 0) return cudaSuccess;
    const int64_t size_a = p.buffers[static_cast<size_t>(op.src)].size;
    const int64_t size_b = p.buffers[static_cast<size_t>(op.src2)].size;
    const auto up = [](int64_t bytes) { return (bytes + 255) / 256 * 256; };
    char *base = static_cast<char *>(scratch);
    auto *sa = reinterpret_cast<uint16_t *>(base);
    base += up(2 * kMaxSlices * size_a);
    auto *sb = reinterpret_cast<uint16_t *>(base);
    base += up(2 * kMaxSlices * size_b);
    auto *ea = reinterpret_cast<int16_t *>(base);
    base += up(2 * size_a);
    auto *eb = reinterpret_cast<int16_t *>(base);
    base += up(2 * size_b);
    auto *partial = reinterpret_cast<double *>(base);
    const auto *lines = reinterpret_cast<const SplitLine *>(sched.lines);
    if (sched.n_lines_a)
      split_lines_kernel<<<static_cast<unsigned>(std::min<int64_t>((sched.n_lines_a + 7) / 8, 152 * 16)), 256, 0, stream>>>(
        A, sa, ea, size_a, lines, sched.n_lines_a, slices);
    if (sched.n_lines_b)
      split_lines_kernel<<<static_cast<unsigned>(std::min<int64_t>((sched.n_lines_b + 7) / 8, 152 * 16)), 256, 0, stream>>>(
        B, sb, eb, size_b, lines + sched.n_lines_a, sched.n_lines_b, slices);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    const auto *blocks = reinterpret_cast<const DevBlock *>(t.blocks);
    const auto *pairs = reinterpret_cast<const DevPair *>(t.pairs);
    switch (slices)
    {
    case 1: e = launch_split_s<1>(sa, ea, size_a, sb, eb, size_b, C, blocks, pairs, sched.items, sched.n_items, partial, stream); break;
    case 2: e = launch_split_s<2>(sa, ea, size_a, sb, eb, size_b, C, blocks, pairs, sched.items, sched.n_items, partial, stream); break;
    case 3: e = launch_split_s<3>(sa, ea, size_a, sb, eb, size_b, C, blocks, pairs, sched.items, sched.n_items, partial, stream); break;
    case 4: e = launch_split_s<4>(sa, ea, size_a, sb, eb, size_b, C, blocks, pairs, sched.items, sched.n_items, partial, stream); break;
    case 5: e = launch_split_s<5>(sa, ea, size_a, sb, eb, size_b, C, blocks, pairs, sched.items, sched.n_items, partial, stream); break;
    case 6: e = launch_split_s<6>(sa, ea, size_a, sb, eb, size_b, C, blocks, pairs, sched.items, sched.n_items, partial, stream); break;
    case 7: e = launch_split_s<7>(sa, ea, size_a, sb, eb, size_b, C, blocks, pairs, sched.items, sched.n_items, partial, stream); break;
    case 8: e = launch_split_s<8>(sa, ea, size_a, sb, eb, size_b, C, blocks, pairs, sched.items, sched.n_items, partial, stream); break;
    default: return cudaErrorInvalidValue;
    }
    if (e != cudaSuccess) return e;
    if (sched.n_reduces)
      reduce_kernel<double><<<static_cast<unsigned>(sched.n_reduces), 256, 0, stream>>>(C, blocks, sched.reduces, partial,
                                                                                       kSplitTileM, kSplitTileN);
    return cudaGetLastError();
  }

  // The device copies of every GEMM op's schedules and slicing lines.
  cudaError_t upload_gemm(const Program &p, DeviceTables &t)
  {
    t.gemm.assign(p.ops.size(), {});
    t.split.assign(p.ops.size(), {});
    for (size_t i = 0; i < p.ops.size(); ++i)
    {
      const Op &op = p.ops[i];
      if (op.kind != OpKind::gemm) continue;
      for (int which = 0; which < 2; ++which)
      {
        const GemmSchedule s = schedule_gemm(p, op, which ? kSplitTileM : kF64TileM, which ? kSplitTileN : kF64TileN);
        DeviceTables::GemmTables &dst = which ? t.split[i] : t.gemm[i];
        dst.n_items = static_cast<int64_t>(s.items.size());
        dst.n_reduces = static_cast<int64_t>(s.reduces.size());
        cudaError_t e = cudaSuccess;
        if (!s.items.empty())
        {
          e = cudaMalloc(&dst.items, s.items.size() * sizeof(GemmItem));
          if (e == cudaSuccess) e = cudaMemcpy(dst.items, s.items.data(), s.items.size() * sizeof(GemmItem), cudaMemcpyHostToDevice);
        }
        if (e == cudaSuccess && !s.reduces.empty())
        {
          e = cudaMalloc(&dst.reduces, s.reduces.size() * sizeof(GemmReduce));
          if (e == cudaSuccess)
            e = cudaMemcpy(dst.reduces, s.reduces.data(), s.reduces.size() * sizeof(GemmReduce), cudaMemcpyHostToDevice);
        }
        if (e != cudaSuccess) return e;
        if (!which) continue;
        // slicing lines: every row of every left block, every column of every right block
        std::vector<OperandBlock> left, right;
        gemm_operands(p, op, left, right);
        std::vector<SplitLine> lines;
        for (const OperandBlock &a : left)
          for (int32_t r = 0; r < a.rows; ++r)
            lines.push_back({a.offset + static_cast<int64_t>(r) * a.cols, a.offset + static_cast<int64_t>(r) * a.cols,
                             a.offset + static_cast<int64_t>(r) * a.cols, a.cols, 1});
        dst.n_lines_a = static_cast<int64_t>(lines.size());
        for (const OperandBlock &b : right)
          for (int32_t c = 0; c < b.cols; ++c)
            lines.push_back({b.offset + c, b.offset + static_cast<int64_t>(c) * b.rows, b.offset + c, b.rows, b.cols});
        dst.n_lines_b = static_cast<int64_t>(lines.size()) - dst.n_lines_a;
        if (!lines.empty())
        {
          e = cudaMalloc(&dst.lines, lines.size() * sizeof(SplitLine));
          if (e == cudaSuccess) e = cudaMemcpy(dst.lines, lines.data(), lines.size() * sizeof(SplitLine), cudaMemcpyHostToDevice);
          if (e != cudaSuccess) return e;
        }
      }
    }
    return cudaSuccess;
  }

} // namespace ttg
