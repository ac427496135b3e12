// Device side of the engine for sm_103a: the executor of a compiled program (program.h) and the
// kernels it launches.
//
//   gather_kernel      a composed chain of leg moves with unit coefficients: one coalesced write
//                      and one gathered read per entry (HBM/L2 bound; index 4 B per entry)
//   runs_kernel        a leg-move step with F/R coefficients: one destination run per warp slice,
//                      sum over the run's terms in registers, no atomics
//   gemm_f64_kernel    grouped block-pair products in FP64 (one CTA per 32x32 output tile, all
//                      tiles of all output blocks of a contraction in one launch)
//   gemm_c128_kernel   the same for complex128
//   add_kernel         dst += src over an arena
//
// The split-precision GEMM lives in gemm_split.cu.
#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include "executor.h"

namespace ttg
{
  namespace
  {
    // ------------------------------------------------------------------------------------------
    // elementwise
    // ------------------------------------------------------------------------------------------

    template <typename T>
    __global__ void gather_kernel(const T *__restrict__ src, T *__restrict__ dst, const int32_t *__restrict__ index,
                                  int64_t n)
    {
      for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
           i += static_cast<int64_t>(gridDim.x) * blockDim.x)
      {
        const int32_t s = __ldg(index + i);
        T v{};
        if (s >= 0) v = src[s];
        dst[i] = v;
      }
    }

    __global__ void add_f64_kernel(const double *__restrict__ src, double *__restrict__ dst, int64_t n)
    {
      for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
           i += static_cast<int64_t>(gridDim.x) * blockDim.x)
        dst[i] += src[i];
    }

    // ------------------------------------------------------------------------------------------
    // runs: dst[d + t*ds] = sum_k c_k * src[s_k + t*ss_k], one chunk (<= 128 entries) per 128 threads
    // ------------------------------------------------------------------------------------------

    struct DevChunk
    {
      int64_t dst;
      int32_t len, dst_step, term_begin, term_count;
    };
    struct DevTerm
    {
      int64_t src, src_step;
      double re, im;
    };
    static_assert(sizeof(DevChunk) == sizeof(Chunk), "chunk layout");
    static_assert(sizeof(DevTerm) == sizeof(Term), "term layout");

    template <bool Complex>
    __global__ void runs_kernel(const double *__restrict__ src, double *__restrict__ dst,
                                const DevChunk *__restrict__ chunks, const DevTerm *__restrict__ terms, int64_t n_chunks)
    {
      for (int64_t c = blockIdx.x; c < n_chunks; c += gridDim.x)
      {
        const DevChunk ch = chunks[c];
        const int t = threadIdx.x;
        if (t >= ch.len) continue;
        if constexpr (Complex)
        {
          double re = 0.0, im = 0.0;
          for (int32_t k = 0; k < ch.term_count; ++k)
          {
            const DevTerm term = terms[ch.term_begin + k];
            const int64_t at = term.src + t * term.src_step;
            const double xr = src[2 * at], xi = src[2 * at + 1];
            re = fma(term.re, xr, fma(-term.im, xi, re));
            im = fma(term.re, xi, fma(term.im, xr, im));
          }
          const int64_t d = ch.dst + static_cast<int64_t>(t) * ch.dst_step;
          dst[2 * d] = re;
          dst[2 * d + 1] = im;
        }
        else
        {
          // a float64 tensor takes the real part of every coefficient (tentorch/tensors/cache.cpp:84-92)
          double acc = 0.0;
          for (int32_t k = 0; k < ch.term_count; ++k)
          {
            const DevTerm term = terms[ch.term_begin + k];
            acc = fma(term.re, src[term.src + t * term.src_step], acc);
          }
          dst[ch.dst + static_cast<int64_t>(t) * ch.dst_step] = acc;
        }
      }
    }

    // ------------------------------------------------------------------------------------------
    // grouped GEMM, FP64 / complex128
    // ------------------------------------------------------------------------------------------

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
    static_assert(sizeof(DevBlock) == sizeof(GemmBlock), "block layout");
    static_assert(sizeof(DevPair) == sizeof(GemmPair), "pair layout");

    // 32x32 output tile per CTA, 64 threads, 4x4 per thread, K staged 16 at a time through shared
    // memory.  FP64 on this part issues about two DFMA per SM clock, so the tile is small to spread
    // the uneven blocks of a contraction over all SMs.
    constexpr int BM = 32, BN = 32, BK = 16, TM = 4, TN = 4;
    constexpr int GEMM_THREADS = (BM / TM) * (BN / TN);

    __global__ void __launch_bounds__(GEMM_THREADS) gemm_f64_kernel(const double *__restrict__ A,
                                                                    const double *__restrict__ B, double *__restrict__ C,
                                                                    const DevBlock *__restrict__ blocks,
                                                                    const DevPair *__restrict__ pairs,
                                                                    const int4 *__restrict__ tiles)
    {
      __shared__ double as[BK][BM];
      __shared__ double bs[BK][BN + 1];
      const int4 tile = tiles[blockIdx.x];  // (block, m0, n0, 0)
      const DevBlock blk = blocks[tile.x];
      const int m0 = tile.y, n0 = tile.z;
      const int tx = threadIdx.x % (BN / TN), ty = threadIdx.x / (BN / TN);
      double acc[TM][TN] = {};
      for (int32_t pi = 0; pi < blk.pair_count; ++pi)
      {
        const DevPair pr = pairs[blk.pair_begin + pi];
        const double *a = A + pr.a;
        const double *b = B + pr.b;
        const int K = pr.k;
        for (int k0 = 0; k0 < K; k0 += BK)
        {
          for (int i = threadIdx.x; i < BM * BK; i += GEMM_THREADS)
          {
            const int r = i / BK, kk = i % BK;
            const int gm = m0 + r, gk = k0 + kk;
            as[kk][r] = (gm < blk.m && gk < K) ? a[static_cast<int64_t>(gm) * K + gk] : 0.0;
          }
          for (int i = threadIdx.x; i < BK * BN; i += GEMM_THREADS)
          {
            const int kk = i / BN, cc = i % BN;
            const int gk = k0 + kk, gn = n0 + cc;
            bs[kk][cc] = (gk < K && gn < blk.n) ? b[static_cast<int64_t>(gk) * blk.n + gn] : 0.0;
          }
          __syncthreads();
#pragma unroll
          for (int kk = 0; kk < BK; ++kk)
          {
            double av[TM], bv[TN];
#pragma unroll
            for (int i = 0; i < TM; ++i) av[i] = as[kk][ty * TM + i];
#pragma unroll
            for (int j = 0; j < TN; ++j) bv[j] = bs[kk][tx * TN + j];
#pragma unroll
            for (int i = 0; i < TM; ++i)
#pragma unroll
              for (int j = 0; j < TN; ++j) acc[i][j] = fma(av[i], bv[j], acc[i][j]);
          }
          __syncthreads();
        }
      }
#pragma unroll
      for (int i = 0; i < TM; ++i)
      {
        const int gm = m0 + ty * TM + i;
        if (gm >= blk.m) continue;
#pragma unroll
        for (int j = 0; j < TN; ++j)
        {
          const int gn = n0 + tx * TN + j;
          if (gn < blk.n) C[blk.c + static_cast<int64_t>(gm) * blk.n + gn] = acc[i][j];
        }
      }
      // the block's alignment pad (one entry after an odd-sized block) reads as zero in arena sums
      const int64_t entries = static_cast<int64_t>(blk.m) * blk.n;
      if (threadIdx.x == 0 && m0 + BM >= blk.m && n0 + BN >= blk.n && (entries & 1)) C[blk.c + entries] = 0.0;
    }

    constexpr int CBM = 32, CBN = 32, CBK = 8, CTM = 4, CTN = 4;
    constexpr int CGEMM_THREADS = (CBM / CTM) * (CBN / CTN);

    __global__ void __launch_bounds__(CGEMM_THREADS) gemm_c128_kernel(const double2 *__restrict__ A,
                                                                      const double2 *__restrict__ B,
                                                                      double2 *__restrict__ C,
                                                                      const DevBlock *__restrict__ blocks,
                                                                      const DevPair *__restrict__ pairs,
                                                                      const int4 *__restrict__ tiles)
    {
      __shared__ double2 as[CBK][CBM];
      __shared__ double2 bs[CBK][CBN + 1];
      const int4 tile = tiles[blockIdx.x];
      const DevBlock blk = blocks[tile.x];
      const int m0 = tile.y, n0 = tile.z;
      const int tx = threadIdx.x % (CBN / CTN), ty = threadIdx.x / (CBN / CTN);
      double2 acc[CTM][CTN];
#pragma unroll
      for (int i = 0; i < CTM; ++i)
#pragma unroll
        for (int j = 0; j < CTN; ++j) acc[i][j] = make_double2(0.0, 0.0);
      for (int32_t pi = 0; pi < blk.pair_count; ++pi)
      {
        const DevPair pr = pairs[blk.pair_begin + pi];
        const double2 *a = A + pr.a;
        const double2 *b = B + pr.b;
        const int K = pr.k;
        for (int k0 = 0; k0 < K; k0 += CBK)
        {
          for (int i = threadIdx.x; i < CBM * CBK; i += CGEMM_THREADS)
          {
            const int r = i / CBK, kk = i % CBK;
            const int gm = m0 + r, gk = k0 + kk;
            as[kk][r] = (gm < blk.m && gk < K) ? a[static_cast<int64_t>(gm) * K + gk] : make_double2(0.0, 0.0);
          }
          for (int i = threadIdx.x; i < CBK * CBN; i += CGEMM_THREADS)
          {
            const int kk = i / CBN, cc = i % CBN;
            const int gk = k0 + kk, gn = n0 + cc;
            bs[kk][cc] = (gk < K && gn < blk.n) ? b[static_cast<int64_t>(gk) * blk.n + gn] : make_double2(0.0, 0.0);
          }
          __syncthreads();
#pragma unroll
          for (int kk = 0; kk < CBK; ++kk)
          {
            double2 av[CTM], bv[CTN];
#pragma unroll
            for (int i = 0; i < CTM; ++i) av[i] = as[kk][ty * CTM + i];
#pragma unroll
            for (int j = 0; j < CTN; ++j) bv[j] = bs[kk][tx * CTN + j];
#pragma unroll
            for (int i = 0; i < CTM; ++i)
#pragma unroll
              for (int j = 0; j < CTN; ++j)
              {
                acc[i][j].x = fma(av[i].x, bv[j].x, fma(-av[i].y, bv[j].y, acc[i][j].x));
                acc[i][j].y = fma(av[i].x, bv[j].y, fma(av[i].y, bv[j].x, acc[i][j].y));
              }
          }
          __syncthreads();
        }
      }
#pragma unroll
      for (int i = 0; i < CTM; ++i)
      {
        const int gm = m0 + ty * CTM + i;
        if (gm >= blk.m) continue;
#pragma unroll
        for (int j = 0; j < CTN; ++j)
        {
          const int gn = n0 + tx * CTN + j;
          if (gn < blk.n) C[blk.c + static_cast<int64_t>(gm) * blk.n + gn] = acc[i][j];
        }
      }
      const int64_t entries = static_cast<int64_t>(blk.m) * blk.n;
      if (threadIdx.x == 0 && m0 + CBM >= blk.m && n0 + CBN >= blk.n && (entries & 1))
        C[blk.c + entries] = make_double2(0.0, 0.0);
    }

    int grid_for(int64_t n, int threads)
    {
      // enough CTAs to cover the arena, capped at 8 waves of the 152 SMs
      const int64_t want = (n + threads - 1) / threads;
      return static_cast<int>(std::max<int64_t>(1, std::min<int64_t>(want, 152 * 8)));
    }

    cudaError_t check_launch() { return cudaGetLastError(); }
  } // namespace

  // --------------------------------------------------------------------------------------------
  // device tables
  // --------------------------------------------------------------------------------------------

  DeviceTables::~DeviceTables()
  {
    for (void *p : {static_cast<void *>(gather), static_cast<void *>(chunks), static_cast<void *>(terms),
                    static_cast<void *>(blocks), static_cast<void *>(pairs), static_cast<void *>(tiles)})
      if (p) cudaFree(p);
  }

  namespace
  {
    template <typename T>
    cudaError_t upload(const std::vector<T> &host, T **dev)
    {
      *dev = nullptr;
      if (host.empty()) return cudaSuccess;
      cudaError_t e = cudaMalloc(reinterpret_cast<void **>(dev), host.size() * sizeof(T));
      if (e != cudaSuccess) return e;
      return cudaMemcpy(*dev, host.data(), host.size() * sizeof(T), cudaMemcpyHostToDevice);
    }
  } // namespace

  // The output tiles of every GEMM op, in op order; tile_begin of op i is recorded per op.
  void build_tiles(const Program &p, std::vector<int32_t> &host_tiles, std::vector<int64_t> &tile_begin,
                   std::vector<int64_t> &tile_count)
  {
    host_tiles.clear();
    tile_begin.assign(p.ops.size(), 0);
    tile_count.assign(p.ops.size(), 0);
    for (size_t i = 0; i < p.ops.size(); ++i)
    {
      const Op &op = p.ops[i];
      if (op.kind != OpKind::gemm) continue;
      tile_begin[i] = static_cast<int64_t>(host_tiles.size() / 4);
      for (int64_t b = op.begin; b < op.begin + op.count; ++b)
      {
        const GemmBlock &blk = p.gemm_blocks[static_cast<size_t>(b)];
        for (int32_t m0 = 0; m0 < blk.m; m0 += BM)
          for (int32_t n0 = 0; n0 < blk.n; n0 += BN)
          {
            host_tiles.push_back(static_cast<int32_t>(b));
            host_tiles.push_back(m0);
            host_tiles.push_back(n0);
            host_tiles.push_back(0);
          }
      }
      tile_count[i] = static_cast<int64_t>(host_tiles.size() / 4) - tile_begin[i];
    }
  }

  cudaError_t DeviceTables::ensure(const Program &p)
  {
    std::lock_guard<std::mutex> lock(mutex);
    if (ready) return cudaSuccess;
    cudaError_t e;
    if ((e = upload(p.gather_index, &gather)) != cudaSuccess) return e;
    if ((e = upload(p.chunks, &chunks)) != cudaSuccess) return e;
    if ((e = upload(p.terms, &terms)) != cudaSuccess) return e;
    if ((e = upload(p.gemm_blocks, &blocks)) != cudaSuccess) return e;
    if ((e = upload(p.gemm_pairs, &pairs)) != cudaSuccess) return e;
    std::vector<int32_t> host_tiles;
    build_tiles(p, host_tiles, tile_begin, tile_count);
    if ((e = upload(host_tiles, &tiles)) != cudaSuccess) return e;
    ready = true;
    return cudaSuccess;
  }

  // --------------------------------------------------------------------------------------------
  // executor
  // --------------------------------------------------------------------------------------------

  cudaError_t execute(const Program &p, DeviceTables &t, const ExecArgs &args)
  {
    cudaError_t e = t.ensure(p);
    if (e != cudaSuccess) return e;
    const size_t esize = args.complex ? 16 : 8;
    std::vector<char *> ptr(p.buffers.size(), nullptr);
    for (size_t i = 0; i < p.buffers.size(); ++i)
    {
      const Buffer &b = p.buffers[i];
      if (b.kind == BufferKind::input)
        ptr[i] = static_cast<char *>(const_cast<void *>(args.inputs[b.index]));
      else if (b.kind == BufferKind::output)
        ptr[i] = static_cast<char *>(args.output);
      else if (b.prepared_of >= 0 && args.prepared && args.prepared[b.prepared_of])
        ptr[i] = static_cast<char *>(const_cast<void *>(args.prepared[b.prepared_of]));
      else
        ptr[i] = static_cast<char *>(args.workspace) + b.offset * esize;
    }
    if (args.only_phase >= 0 && args.prepared_out)
      ptr[static_cast<size_t>(p.prepared[static_cast<size_t>(args.only_phase)])] = static_cast<char *>(args.prepared_out);
    for (size_t i = 0; i < p.ops.size(); ++i)
    {
      const Op &op = p.ops[i];
      if (args.only_phase >= 0)
      {
        if (op.phase != args.only_phase) continue;
      }
      else if (op.phase >= 0 && args.prepared && args.prepared[op.phase])
        continue;  // the caller holds this operand's prepared arena
      if (args.events)
      {
        e = cudaEventRecord(args.events[2 * i], args.stream);
        if (e != cudaSuccess) return e;
      }
      char *dst = ptr[static_cast<size_t>(op.dst)];
      const char *src = op.src >= 0 ? ptr[static_cast<size_t>(op.src)] : nullptr;
      const char *src2 = op.src2 >= 0 ? ptr[static_cast<size_t>(op.src2)] : nullptr;
      switch (op.kind)
      {
      case OpKind::zero:
        e = cudaMemsetAsync(dst, 0, static_cast<size_t>(op.elements) * esize, args.stream);
        break;
      case OpKind::copy:
        e = cudaMemcpyAsync(dst, src, static_cast<size_t>(op.elements) * esize, cudaMemcpyDeviceToDevice, args.stream);
        break;
      case OpKind::add:
      {
        const int64_t n = op.elements * (args.complex ? 2 : 1);
        add_f64_kernel<<<grid_for(n, 256), 256, 0, args.stream>>>(reinterpret_cast<const double *>(src),
                                                                 reinterpret_cast<double *>(dst), n);
        e = check_launch();
        break;
      }
      case OpKind::gather:
        if (args.complex)
          gather_kernel<double2><<<grid_for(op.elements, 256), 256, 0, args.stream>>>(
            reinterpret_cast<const double2 *>(src), reinterpret_cast<double2 *>(dst), t.gather + op.begin, op.elements);
        else
          gather_kernel<double><<<grid_for(op.elements, 256), 256, 0, args.stream>>>(
            reinterpret_cast<const double *>(src), reinterpret_cast<double *>(dst), t.gather + op.begin, op.elements);
        e = check_launch();
        break;
      case OpKind::runs:
        if (op.count > 0)
        {
          const int grid = static_cast<int>(std::min<int64_t>(op.count, 152 * 16));
          const auto *ch = reinterpret_cast<const DevChunk *>(t.chunks) + op.begin;
          const auto *te = reinterpret_cast<const DevTerm *>(t.terms);
          if (args.complex)
            runs_kernel<true><<<grid, kChunk, 0, args.stream>>>(reinterpret_cast<const double *>(src),
                                                                 reinterpret_cast<double *>(dst), ch, te, op.count);
          else
            runs_kernel<false><<<grid, kChunk, 0, args.stream>>>(reinterpret_cast<const double *>(src),
                                                                  reinterpret_cast<double *>(dst), ch, te, op.count);
          e = check_launch();
        }
        break;
      case OpKind::gemm:
      {
        const int64_t ntiles = t.tile_count[i];
        if (ntiles == 0) break;
        const auto *blk = reinterpret_cast<const DevBlock *>(t.blocks);
        const auto *prs = reinterpret_cast<const DevPair *>(t.pairs);
        const int4 *tl = reinterpret_cast<const int4 *>(t.tiles) + t.tile_begin[i];
        if (args.complex)
          gemm_c128_kernel<<<static_cast<unsigned>(ntiles), CGEMM_THREADS, 0, args.stream>>>(
            reinterpret_cast<const double2 *>(src), reinterpret_cast<const double2 *>(src2),
            reinterpret_cast<double2 *>(dst), blk, prs, tl);
        else if (args.precision > 0)
          e = launch_gemm_split(p, op, t, i, reinterpret_cast<const double *>(src), reinterpret_cast<const double *>(src2),
                                reinterpret_cast<double *>(dst), args.precision, args.stream);
        else
          gemm_f64_kernel<<<static_cast<unsigned>(ntiles), GEMM_THREADS, 0, args.stream>>>(
            reinterpret_cast<const double *>(src), reinterpret_cast<const double *>(src2), reinterpret_cast<double *>(dst),
            blk, prs, tl);
        if (e == cudaSuccess) e = check_launch();
        break;
      }
      }
      if (e != cudaSuccess) return e;
      if (args.events)
      {
        e = cudaEventRecord(args.events[2 * i + 1], args.stream);
        if (e != cudaSuccess) return e;
      }
    }
    return cudaSuccess;
  }

  // ------------------------------------------------------------------------------------------
  // arena arithmetic for the Krylov solver: dot products without a host sync, axpy, scale
  // ------------------------------------------------------------------------------------------

  namespace
  {
    // out[j] = sum_i conj(a_j[i]) b[i] for j < count, one block of partial sums per CTA, then a
    // second pass; n counts doubles (complex arenas interleave re, im).
    template <bool Complex>
    __global__ void dot_partial_kernel(const double *const *__restrict__ as, const double *__restrict__ b, int64_t n,
                                       double *__restrict__ partial)
    {
      const double *a = as[blockIdx.y];
      double re = 0.0, im = 0.0;
      if constexpr (Complex)
      {
        for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; 2 * i < n;
             i += static_cast<int64_t>(gridDim.x) * blockDim.x)
        {
          const double ar = a[2 * i], ai = a[2 * i + 1], br = b[2 * i], bi = b[2 * i + 1];
          re = fma(ar, br, fma(ai, bi, re));
          im = fma(ar, bi, fma(-ai, br, im));
        }
      }
      else
      {
        for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
             i += static_cast<int64_t>(gridDim.x) * blockDim.x)
          re = fma(a[i], b[i], re);
      }
      __shared__ double sr[32], si[32];
      for (int off = 16; off > 0; off >>= 1)
      {
        re += __shfl_down_sync(0xffffffffu, re, off);
        im += __shfl_down_sync(0xffffffffu, im, off);
      }
      const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
      if (lane == 0)
      {
        sr[warp] = re;
        si[warp] = im;
      }
      __syncthreads();
      if (warp == 0)
      {
        const int warps = blockDim.x >> 5;
        re = lane < warps ? sr[lane] : 0.0;
        im = lane < warps ? si[lane] : 0.0;
        for (int off = 16; off > 0; off >>= 1)
        {
          re += __shfl_down_sync(0xffffffffu, re, off);
          im += __shfl_down_sync(0xffffffffu, im, off);
        }
        if (lane == 0)
        {
          partial[2 * (static_cast<int64_t>(blockIdx.y) * gridDim.x + blockIdx.x)] = re;
          partial[2 * (static_cast<int64_t>(blockIdx.y) * gridDim.x + blockIdx.x) + 1] = im;
        }
      }
    }

    __global__ void dot_final_kernel(const double *__restrict__ partial, int parts, double *__restrict__ out)
    {
      // one warp per result, fixed summation order
      const int j = blockIdx.x;
      double re = 0.0, im = 0.0;
      for (int i = threadIdx.x; i < parts; i += 32)
      {
        re += partial[2 * (static_cast<int64_t>(j) * parts + i)];
        im += partial[2 * (static_cast<int64_t>(j) * parts + i) + 1];
      }
      for (int off = 16; off > 0; off >>= 1)
      {
        re += __shfl_down_sync(0xffffffffu, re, off);
        im += __shfl_down_sync(0xffffffffu, im, off);
      }
      if (threadIdx.x == 0)
      {
        out[2 * j] = re;
        out[2 * j + 1] = im;
      }
    }
  } // namespace

  cudaError_t arena_dots(const double *const *dev_as, int32_t count, const double *b, int64_t n_doubles, bool complex,
                         double *partial, double *out, cudaStream_t stream)
  {
    const int parts = kDotParts;
    dim3 grid(parts, static_cast<unsigned>(count));
    if (complex)
      dot_partial_kernel<true><<<grid, 256, 0, stream>>>(dev_as, b, n_doubles, partial);
    else
      dot_partial_kernel<false><<<grid, 256, 0, stream>>>(dev_as, b, n_doubles, partial);
    dot_final_kernel<<<static_cast<unsigned>(count), 32, 0, stream>>>(partial, parts, out);
    return cudaGetLastError();
  }

} // namespace ttg
