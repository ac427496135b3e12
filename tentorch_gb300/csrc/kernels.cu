// Device side of the engine for sm_103a: the executor of a compiled program (program.h) and the
// kernels it launches.
//
//   gather_kernel      a composed chain of leg moves with unit coefficients: one coalesced write
//                      and one gathered read per entry (HBM/L2 bound; index 4 B per entry)
//   runs_kernel        a leg-move step with F/R coefficients: one destination run per warp slice,
//                      sum over the run's terms in registers, no atomics
//   add_kernel         dst += src over an arena
//
// The grouped GEMMs live in gemm.cu.
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include "executor.h"
#include "tentorch_gb300.h"
#include "launch.h"

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
      dependent_entry();
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
      dependent_entry();
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
      dependent_entry();
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

    // One chunk of a tile per CTA.  The input offset of an entry is the sum of its row's part
    // (mixed radix over the copies of the output codomain legs) and its column's part (the same
    // over the domain legs, the last fastest): both are computed once per chunk into shared
    // memory, then the chunk's entries are dealt to the threads in output order (coalesced
    // writes, one division per entry).  A chunk wider than the tables falls back to computing the
    // column part per entry.
    __device__ __forceinline__ double conj_of(double x) { return x; }
    __device__ __forceinline__ double2 conj_of(double2 x) { return make_double2(x.x, -x.y); }

    constexpr int kTileTable = 2048;  // rows and columns of a chunk with precomputed offsets

    __device__ __forceinline__ int64_t radix_offset(const Tile &t, int32_t first, int32_t last, int32_t index)
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

    template <typename T, bool Conj>
    __global__ void __launch_bounds__(256) tiles_kernel(const T *__restrict__ src, T *__restrict__ dst,
                                                        const Tile *__restrict__ tiles,
                                                        const TileChunk *__restrict__ chunks)
    {
      dependent_entry();
      __shared__ Tile t;
      __shared__ int64_t row_off[kTileTable];
      __shared__ int64_t col_off[kTileTable];
      const TileChunk ch = chunks[blockIdx.x];
      if (threadIdx.x == 0) t = tiles[ch.tile];
      __syncthreads();
      if (t.in_base < 0)
      {
        // the zero pad entry of an odd block
        if (threadIdx.x == 0) dst[t.out_base] = T{};
        return;
      }
      const int32_t n_row = t.n_row, n_col = t.n_col, cols = t.cols, rows = ch.nrows;
      if (cols <= kTileTable && rows <= kTileTable)
      {
        for (int32_t c = threadIdx.x; c < cols; c += blockDim.x) col_off[c] = radix_offset(t, n_row, n_row + n_col - 1, c);
        for (int32_t r = threadIdx.x; r < rows; r += blockDim.x)
          row_off[r] = t.in_base + radix_offset(t, 0, n_row - 1, ch.row0 + r);
        __syncthreads();
        T *out = dst + t.out_base + static_cast<int64_t>(ch.row0) * t.out_ld;
        const int32_t n = rows * cols;
        for (int32_t e = threadIdx.x; e < n; e += blockDim.x)
        {
          const int32_t r = e / cols, c = e - r * cols;
          const T x = src[row_off[r] + col_off[c]];
          out[static_cast<int64_t>(r) * t.out_ld + c] = Conj ? conj_of(x) : x;
        }
        return;
      }
      const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
      for (int32_t r = ch.row0 + warp; r < ch.row0 + rows; r += 8)
      {
        const int64_t row_in = t.in_base + radix_offset(t, 0, n_row - 1, r);
        T *out = dst + t.out_base + static_cast<int64_t>(r) * t.out_ld;
        for (int32_t c = lane; c < cols; c += 32)
        {
          const T x = src[row_in + radix_offset(t, n_row, n_row + n_col - 1, c)];
          out[c] = Conj ? conj_of(x) : x;
        }
      }
    }

    int grid_for(int64_t n, int threads)
    {
      // enough CTAs to cover the arena, capped at 8 waves of the device's SMs
      const int64_t want = (n + threads - 1) / threads;
      return static_cast<int>(std::max<int64_t>(1, std::min<int64_t>(want, device_sms() * 8)));
    }

  } // namespace

  // --------------------------------------------------------------------------------------------
  // device tables
  // --------------------------------------------------------------------------------------------

  DeviceTables::~DeviceTables()
  {
    if (base) cudaFree(base);
    if (chain.base) cudaFree(chain.base);
    if (chain.relabel_base) cudaFree(chain.relabel_base);
    for (TcTables &g : tc)
      if (g.base) cudaFree(g.base);
    for (GemmTables &g : gemm)
      if (g.base) cudaFree(g.base);
    for (SplitTables &g : split)
      if (g.base) cudaFree(g.base);
  }

  // A non-blocking stream per device for table uploads.
  cudaError_t upload_stream(cudaStream_t *stream)
    {
      static std::mutex mutex;
      static std::map<int, cudaStream_t> streams;
      int device = 0;
      cudaError_t e = cudaGetDevice(&device);
      if (e != cudaSuccess) return e;
      std::lock_guard<std::mutex> lock(mutex);
      auto found = streams.find(device);
      if (found == streams.end())
      {
        cudaStream_t created = nullptr;
        if ((e = cudaStreamCreateWithFlags(&created, cudaStreamNonBlocking)) != cudaSuccess) return e;
        found = streams.emplace(device, created).first;
      }
      *stream = found->second;
      return cudaSuccess;
    }

  cudaError_t TableStaging::commit(void **base)
  {
    *base = nullptr;
    if (host.empty()) return cudaSuccess;
    // The copy runs on a stream of its own and is waited for here, so the tables are in device
    // memory before any stream launches a kernel that reads them: a plain copy from pageable
    // memory may still be in flight when it returns, ordered only against the legacy stream.
    cudaStream_t stream = nullptr;
    cudaError_t e = upload_stream(&stream);
    if (e != cudaSuccess) return e;
    void *device = nullptr;
    if ((e = cudaMalloc(&device, host.size())) != cudaSuccess) return e;
    e = cudaMemcpyAsync(device, host.data(), host.size(), cudaMemcpyHostToDevice, stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    if (e != cudaSuccess)
    {
      cudaFree(device);
      return e;
    }
    *base = device;
    for (const auto &[at, slot] : slots) *slot = static_cast<char *>(device) + at;
    return cudaSuccess;
  }

  cudaError_t DeviceTables::ensure(const Program &p)
  {
    std::lock_guard<std::mutex> lock(mutex);
    if (ready) return cudaSuccess;
    TableStaging staging;
    staging.add(p.gather_index, reinterpret_cast<void **>(&gather));
    staging.add(p.tiles, reinterpret_cast<void **>(&tiles));
    staging.add(p.tile_chunks, reinterpret_cast<void **>(&tile_chunks));
    staging.add(p.chunks, reinterpret_cast<void **>(&chunks));
    staging.add(p.terms, reinterpret_cast<void **>(&terms));
    staging.add(p.gemm_blocks, reinterpret_cast<void **>(&blocks));
    staging.add(p.gemm_pairs, reinterpret_cast<void **>(&pairs));
    stage_gemm(p, *this, staging);
    const cudaError_t e = staging.commit(&base);
    if (e != cudaSuccess) return e;
    ready = true;
    return cudaSuccess;
  }

  // --------------------------------------------------------------------------------------------
  // executor
  // --------------------------------------------------------------------------------------------

  std::vector<char *> buffer_pointers(const Program &p, const ExecArgs &args)
  {
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
    return ptr;
  }

  cudaError_t execute(const Program &p, DeviceTables &t, const ExecArgs &args)
  {
    cudaError_t e = t.ensure(p);
    if (e != cudaSuccess) return e;
    const size_t esize = args.complex ? 16 : 8;
    const std::vector<char *> ptr = buffer_pointers(p, args);
    // whether op i runs in this execution: a prepare-only call runs its operand's phase; otherwise
    // the ops of a phase whose prepared arena the caller holds are skipped (and with phases_only
    // only the phases run)
    const auto runs_now = [&](size_t i)
    {
      const Op &op = p.ops[i];
      if (args.only_phase >= 0) return op.phase == args.only_phase;
      if (args.phases_only && op.phase < 0) return false;
      return !(op.phase >= 0 && args.prepared && args.prepared[op.phase]);
    };
    // the forms the caller asked for, else those the autotuner chose for this histogram
    int32_t forms = args.forms;
    if (forms < 0) forms = std::max(tuned_forms(p.tune_key, args.complex, args.precision), 0);
    const bool tensor_cores = (forms & kFormNoTensorCores) == 0;
    const auto run_op = [&](size_t i) -> cudaError_t
    {
      const Op &op = p.ops[i];
      cudaError_t e = cudaSuccess;
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
        e = launch_dependent(add_f64_kernel, grid_for(n, 256), 256, 0, args.stream, reinterpret_cast<const double *>(src),
                             reinterpret_cast<double *>(dst), n);
        break;
      }
      case OpKind::gather:
        if (args.complex)
          e = launch_dependent(gather_kernel<double2>, grid_for(op.elements, 256), 256, 0, args.stream,
                               reinterpret_cast<const double2 *>(src), reinterpret_cast<double2 *>(dst),
                               static_cast<const int32_t *>(t.gather + op.begin), op.elements);
        else
          e = launch_dependent(gather_kernel<double>, grid_for(op.elements, 256), 256, 0, args.stream,
                               reinterpret_cast<const double *>(src), reinterpret_cast<double *>(dst),
                               static_cast<const int32_t *>(t.gather + op.begin), op.elements);
        break;
      case OpKind::tiles:
        if (op.count > 0)
        {
          const dim3 grid(static_cast<unsigned>(op.count));
          const Tile *tiles = t.tiles;
          const TileChunk *chunks = t.tile_chunks + op.begin;
          if (args.complex && (op.flags & 1))
            e = launch_dependent(tiles_kernel<double2, true>, grid, 256, 0, args.stream, reinterpret_cast<const double2 *>(src),
                                 reinterpret_cast<double2 *>(dst), tiles, chunks);
          else if (args.complex)
            e = launch_dependent(tiles_kernel<double2, false>, grid, 256, 0, args.stream, reinterpret_cast<const double2 *>(src),
                                 reinterpret_cast<double2 *>(dst), tiles, chunks);
          else
            e = launch_dependent(tiles_kernel<double, false>, grid, 256, 0, args.stream, reinterpret_cast<const double *>(src),
                                 reinterpret_cast<double *>(dst), tiles, chunks);
        }
        break;
      case OpKind::runs:
        if (op.count > 0)
        {
          const int grid = static_cast<int>(std::min<int64_t>(op.count, device_sms() * 16));
          const auto *ch = reinterpret_cast<const DevChunk *>(t.chunks) + op.begin;
          const auto *te = reinterpret_cast<const DevTerm *>(t.terms);
          if (args.complex)
            e = launch_dependent(runs_kernel<true>, grid, kChunk, 0, args.stream, reinterpret_cast<const double *>(src),
                                 reinterpret_cast<double *>(dst), ch, te, op.count);
          else
            e = launch_dependent(runs_kernel<false>, grid, kChunk, 0, args.stream, reinterpret_cast<const double *>(src),
                                 reinterpret_cast<double *>(dst), ch, te, op.count);
        }
        break;
      case OpKind::gemm:
      {
        void *scratch = static_cast<char *>(args.workspace) + p.scratch_offset * esize;
        int *tickets = static_cast<int *>(args.workspace);
        if (args.precision < 0)
          e = launch_gemm_per_block(p, op, src, src2, dst, args.complex, args.stream);
        else if (args.precision > 0 && !args.complex)
          e = launch_gemm_split(p, op, t, i, reinterpret_cast<const double *>(src), reinterpret_cast<const double *>(src2),
                                reinterpret_cast<double *>(dst), args.precision, scratch, tickets, args.prepared,
                                args.stream, nullptr, tensor_cores);
        else
          e = launch_gemm_f64(p, t, i, src, src2, dst, args.complex, scratch, tickets, args.stream);
        break;
      }
      }
      if (e != cudaSuccess) return e;
      if (args.events) e = cudaEventRecord(args.events[2 * i + 1], args.stream);
      return e;
    };
    // the product chain (chain.cu): in FP64 one launch for both products and the move between them;
    // in split precision the first product stores through the move's relabelling (float64 arenas,
    // full executions only)
    static const bool chain_enabled = []
    {
      const char *v = std::getenv("TENTORCH_GB300_CHAIN");
      return !(v && v[0] == '0');
    }();
    const bool chain = chain_enabled && (forms & kFormSeparate) == 0 && p.chain_first >= 0 && args.only_phase < 0 &&
                       !args.phases_only && !args.complex && args.precision >= 0;
    std::vector<char> done(p.ops.size(), 0);
    if (args.chain_ran) *args.chain_ran = false;
    for (size_t i = 0; i < p.ops.size(); ++i)
    {
      if (done[i] || !runs_now(i)) continue;
      if (chain && static_cast<int32_t>(i) == p.chain_first)
      {
        // ops between the move and the second product prepare other operands: run them first
        for (size_t j = static_cast<size_t>(p.chain_move) + 1; j < static_cast<size_t>(p.chain_second); ++j)
          if (runs_now(j))
          {
            if ((e = run_op(j)) != cudaSuccess) return e;
            done[j] = 1;
          }
        const Op &first = p.ops[i], &move = p.ops[static_cast<size_t>(p.chain_move)],
                 &second = p.ops[static_cast<size_t>(p.chain_second)];
        if (args.precision > 0)
        {
          // split products: the first one stores its result at its places after the move, which
          // then does not run; the second product runs in its turn
          const int32_t *relabel = nullptr;
          if ((e = chain_relabel(p, t, &relabel)) != cudaSuccess) return e;
          if (relabel)
          {
            if (args.events && (e = cudaEventRecord(args.events[2 * i], args.stream)) != cudaSuccess) return e;
            e = launch_gemm_split(p, first, t, i, reinterpret_cast<const double *>(ptr[static_cast<size_t>(first.src)]),
                                  reinterpret_cast<const double *>(ptr[static_cast<size_t>(first.src2)]),
                                  reinterpret_cast<double *>(ptr[static_cast<size_t>(move.dst)]), args.precision,
                                  static_cast<char *>(args.workspace) + p.scratch_offset * esize,
                                  static_cast<int *>(args.workspace), args.prepared, args.stream, relabel);
            if (e != cudaSuccess) return e;
            if (args.events && (e = cudaEventRecord(args.events[2 * i + 1], args.stream)) != cudaSuccess) return e;
            done[static_cast<size_t>(p.chain_move)] = 1;
            continue;
          }
          if ((e = run_op(i)) != cudaSuccess) return e;
          continue;
        }
        if (args.events && (e = cudaEventRecord(args.events[2 * i], args.stream)) != cudaSuccess) return e;
        bool used = false;
        e = launch_chain_f64(p, t, reinterpret_cast<const double *>(ptr[static_cast<size_t>(first.src)]),
                             reinterpret_cast<const double *>(ptr[static_cast<size_t>(first.src2)]),
                             reinterpret_cast<double *>(ptr[static_cast<size_t>(move.dst)]),
                             reinterpret_cast<const double *>(ptr[static_cast<size_t>(second.src2)]),
                             reinterpret_cast<double *>(ptr[static_cast<size_t>(second.dst)]), args.workspace,
                             args.stream, &used);
        if (e != cudaSuccess) return e;
        if (used)
        {
          if (args.events && (e = cudaEventRecord(args.events[2 * i + 1], args.stream)) != cudaSuccess) return e;
          done[static_cast<size_t>(p.chain_move)] = done[static_cast<size_t>(p.chain_second)] = 1;
          if (args.chain_ran) *args.chain_ran = true;
          continue;
        }
      }
      if ((e = run_op(i)) != cudaSuccess) return e;
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
      dependent_entry();
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
      dependent_entry();
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
    cudaError_t e = complex ? launch_dependent(dot_partial_kernel<true>, grid, 256, 0, stream, dev_as, b, n_doubles, partial)
                            : launch_dependent(dot_partial_kernel<false>, grid, 256, 0, stream, dev_as, b, n_doubles, partial);
    if (e != cudaSuccess) return e;
    return launch_dependent(dot_final_kernel, static_cast<unsigned>(count), 32, 0, stream, static_cast<const double *>(partial),
                            parts, out);
  }

} // namespace ttg

// ---------------------------------------------------------------------------------------------
// tt_dots_noalloc: the dot products of tt_dots with their partial sums in a static device array
// ---------------------------------------------------------------------------------------------
//
// For callers that cannot allocate device memory at the point they need a Krylov dot product:
// a solver step running under a host framework that forbids allocation in its inner loop (a
// real-time or embedded host, or one whose memory pool is owned by another runtime and exposes
// no allocator through the FFI), or code that must not touch the allocator between a warm-up and
// a timed or replayed sequence.  tt_dots needs `scratch` from the caller; this variant keeps the
// partial sums in the array below, which every GPU that loads this library holds until the
// process exits.

namespace
{
  // At most this many vectors per call: 2 doubles per (vector, CTA) and kDotParts CTAs per vector
  // (64 * 120 * 16 bytes = 120 KiB per device).
  constexpr int32_t kNoAllocMaxVectors = 64;
  constexpr int kNoAllocMaxDevices = 64;
}

static __device__ __align__(256) double tt_dots_noalloc_scratch[2 * ttg::kDotParts * kNoAllocMaxVectors];

namespace
{
  std::mutex noalloc_mutex;
  double *noalloc_scratch[kNoAllocMaxDevices] = {};
}

extern "C" int32_t tt_dots_noalloc(int32_t dtype, int32_t count, const void *const *as, const void *b, int64_t n,
                                   double *out, void *stream)
{
  if (count <= 0) return TT_OK;
  if (count > kNoAllocMaxVectors)
    return ttg::report(TT_EINVAL, "tt_dots_noalloc takes at most " + std::to_string(kNoAllocMaxVectors) + " vectors, got " +
                            std::to_string(count) + "; call tt_dots with caller-provided scratch instead");
  if (dtype != TT_DTYPE_FLOAT64 && dtype != TT_DTYPE_COMPLEX128)
    return ttg::report(TT_EINVAL, "unknown dtype " + std::to_string(dtype));
  int device = 0;
  cudaError_t e = cudaGetDevice(&device);
  if (e != cudaSuccess) return ttg::report(TT_ECUDA, std::string("CUDA: ") + cudaGetErrorString(e));
  if (device < 0 || device >= kNoAllocMaxDevices) return ttg::report(TT_EINVAL, "device index beyond the static table");
  double *scratch = nullptr;
  {
    // set-up, once per device, with that device current: the device address of the array (host
    // code only knows a host-side stand-in for it)
    std::lock_guard<std::mutex> lock(noalloc_mutex);
    if (!noalloc_scratch[device])
    {
      void *address = nullptr;
      e = cudaGetSymbolAddress(&address, tt_dots_noalloc_scratch);
      if (e != cudaSuccess) return ttg::report(TT_ECUDA, std::string("CUDA: ") + cudaGetErrorString(e));
      noalloc_scratch[device] = static_cast<double *>(address);
    }
    scratch = noalloc_scratch[device];
  }
  // Every partial sum a call reads is written earlier in the same call, so nothing has to start at
  // zero; two calls whose work overlaps on the GPU share the array and race.
  const bool complex = dtype == 1;
  e = ttg::arena_dots(reinterpret_cast<const double *const *>(as), count, static_cast<const double *>(b),
                      n * (complex ? 2 : 1), complex, scratch, out, static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return ttg::report(TT_ECUDA, std::string("CUDA: ") + cudaGetErrorString(e));
  return TT_OK;
}


// ------------------------------------------------------------------------------------------
// host <-> device transfers by a kernel over the coherent host link
// ------------------------------------------------------------------------------------------

namespace
{
  // 16-byte words while both ends are 16-byte aligned, then the rest one byte at a time.
  __global__ void link_copy_kernel(unsigned char *__restrict__ dst, const unsigned char *__restrict__ src, int64_t bytes)
  {
    const int64_t thread = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    const int64_t threads = static_cast<int64_t>(gridDim.x) * blockDim.x;
    const bool aligned = ((reinterpret_cast<uintptr_t>(dst) | reinterpret_cast<uintptr_t>(src)) & 15) == 0;
    const int64_t words = aligned ? bytes / 16 : 0;
    for (int64_t i = thread; i < words; i += threads)
      reinterpret_cast<uint4 *>(dst)[i] = reinterpret_cast<const uint4 *>(src)[i];
    for (int64_t i = words * 16 + thread; i < bytes; i += threads) dst[i] = src[i];
  }

  // The device address of page-locked host memory allocated mapped (cudaHostAlloc; every
  // allocation is mapped where the device has unified addressing), or an error when it is not.
  cudaError_t mapped(const void *host, void **device)
  {
    cudaPointerAttributes attributes{};
    cudaError_t e = cudaPointerGetAttributes(&attributes, host);
    if (e != cudaSuccess) return e;
    if (attributes.type != cudaMemoryTypeHost || attributes.devicePointer == nullptr) return cudaErrorInvalidValue;
    return cudaHostGetDevicePointer(device, const_cast<void *>(host), 0);
  }
}

extern "C" int32_t tt_link_copy(void *dst, const void *src, int64_t bytes, int32_t direction, void *stream)
{
  if (bytes < 0 || (bytes > 0 && (!dst || !src))) return ttg::report(TT_EINVAL, "tt_link_copy needs both ends");
  if (direction != 0 && direction != 1) return ttg::report(TT_EINVAL, "direction is 0 (host to device) or 1 (device to host)");
  if (bytes == 0) return TT_OK;
  void *host = direction == 0 ? const_cast<void *>(src) : dst, *through = nullptr;
  cudaError_t e = mapped(host, &through);
  if (e != cudaSuccess)
  {
    cudaGetLastError();
    return ttg::report(TT_EINVAL, "the host end of tt_link_copy is not mapped page-locked memory (cudaHostAlloc)");
  }
  unsigned char *d = static_cast<unsigned char *>(direction == 0 ? dst : through);
  const unsigned char *s = static_cast<const unsigned char *>(direction == 0 ? through : src);
  const int64_t words = (bytes + 15) / 16;
  const unsigned grid = static_cast<unsigned>(std::max<int64_t>(1, std::min<int64_t>((words + 255) / 256, ttg::device_sms() * 4)));
  link_copy_kernel<<<grid, 256, 0, static_cast<cudaStream_t>(stream)>>>(d, s, bytes);
  e = cudaGetLastError();
  if (e != cudaSuccess) return ttg::report(TT_ECUDA, std::string("CUDA: ") + cudaGetErrorString(e));
  return TT_OK;
}
