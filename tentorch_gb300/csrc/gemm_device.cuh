// Device helpers shared by the grouped GEMM kernels (gemm.cu), the chained matvec kernel
// (chain.cu) and the tensor-core split products (split_tc.cu): the device copies of the block and
// pair tables, the barriers and work claims of a worker (128 threads), asynchronous copies, the FP64
// and bf16 matrix instructions, and the bit arithmetic of the split-precision slicing.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "gemm.h"

namespace ttg
{
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
    struct DevSplitPair
    {
      int64_t sa, sb;
      int32_t kp, ea, eb, pad;
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

    // a barrier over one worker's 128 threads (named barrier 1 + worker)
    __device__ __forceinline__ void worker_sync(int worker)
    {
      asm volatile("bar.sync %0, %1;\n" ::"r"(worker + 1), "r"(kWorkerThreads) : "memory");
    }

    // 8-byte asynchronous copy global -> shared; `in` false fills the destination with zeros and
    // reads nothing
    __device__ __forceinline__ void copy8(double *dst, const double *src, bool in)
    {
      const unsigned d = static_cast<unsigned>(__cvta_generic_to_shared(dst));
      asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(d), "l"(src), "r"(in ? 8 : 0) : "memory");
    }
    __device__ __forceinline__ void copy_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
    __device__ __forceinline__ void copy_wait_one() { asm volatile("cp.async.wait_group 1;\n" ::: "memory"); }

    // The next entry of the CTA's own list for a worker.
    __device__ __forceinline__ int64_t local_claim(int worker, int lt, int *slot, int *taken)
    {
      if (lt == 0) *slot = atomicAdd(taken, 1);
      worker_sync(worker);
      const int64_t idx = *slot;
      worker_sync(worker);
      return idx;
    }


    // D = A B + D on a 16 x 8 x 8 FP64 fragment.  Lane l (g = l / 4, t = l % 4) holds A at rows
    // g, g + 8 and columns t, t + 4 (a0: (g, t), a1: (g + 8, t), a2: (g, t + 4), a3: (g + 8, t + 4)),
    // B at rows t, t + 4 of column g, and D at rows g (c0, c1) and g + 8 (c2, c3) of columns 2t, 2t + 1.
    __device__ __forceinline__ void dmma16(double (&c)[4], const double (&a)[4], const double (&b)[2])
    {
      asm volatile("mma.sync.aligned.m16n8k8.row.col.f64.f64.f64.f64 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
                   "{%0,%1,%2,%3};\n"
                   : "+d"(c[0]), "+d"(c[1]), "+d"(c[2]), "+d"(c[3])
                   : "d"(a[0]), "d"(a[1]), "d"(a[2]), "d"(a[3]), "d"(b[0]), "d"(b[1]));
    }


    // FP64 runs at a sixty-fourth of the FP32 rate on this GPU, so the slicing works on the bits of
    // the doubles with integer instructions.
    //
    // frexp's exponent of a non-negative double given by its bits: x = f 2^e with f in [0.5, 1)
    // (0 for zero).
    __device__ __forceinline__ int frexp_exponent(unsigned long long bits)
    {
      if (bits == 0) return 0;
      const int field = static_cast<int>(bits >> 52);
      if (field != 0) return field - 1022;
      return (64 - __clzll(static_cast<long long>(bits))) - 1074;  // subnormal: bits * 2^-1074
    }

    // __double2ll_rn(ldexp(x, k)) for |x| < 2^(63 - k) on the bits of x: the significand shifted by
    // the exponent, rounded to nearest with ties to even.
    __device__ __forceinline__ long long scaled_integer(double x, int k)
    {
      const unsigned long long bits = static_cast<unsigned long long>(__double_as_longlong(x));
      const int field = static_cast<int>((bits >> 52) & 0x7ff);
      unsigned long long mant = bits & 0xfffffffffffffull;
      if (field != 0) mant |= 1ull << 52;
      const int shift = (field != 0 ? field : 1) - 1075 + k;  // x 2^k = mant 2^shift
      unsigned long long q;
      if (mant == 0)
        q = 0;
      else if (shift >= 0)
        q = mant << shift;
      else if (shift < -62)
        q = 0;
      else
      {
        const int down = -shift;
        q = mant >> down;
        const unsigned long long rem = mant & ((1ull << down) - 1), half = 1ull << (down - 1);
        if (rem > half || (rem == half && (q & 1ull))) ++q;
      }
      const long long v = static_cast<long long>(q);
      return (bits >> 63) ? -v : v;
    }

    // 2^k as a double built from its bits (k in the normal range), else through ldexp
    __device__ __forceinline__ double pow2(int k)
    {
      if (k > -1023 && k < 1024) return __longlong_as_double(static_cast<long long>(k + 1023) << 52);
      return ldexp(1.0, k);
    }


    __device__ __forceinline__ void mma_bf16(float (&c)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1)
    {
      asm volatile("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
                   "{%0,%1,%2,%3};\n"
                   : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
                   : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
    }

    __device__ __forceinline__ void ldmatrix_x4(uint32_t (&r)[4], const void *smem)
    {
      const uint32_t at = static_cast<uint32_t>(__cvta_generic_to_shared(smem));
      asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                   : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                   : "r"(at));
    }

    // 16 bytes global -> shared; `bytes` 0 writes zeros and reads nothing
    __device__ __forceinline__ void cp_async16(void *smem, const void *gmem, int bytes)
    {
      const uint32_t at = static_cast<uint32_t>(__cvta_generic_to_shared(smem));
      asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(at), "l"(gmem), "r"(bytes));
    }
    __device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
    template <int N>
    __device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N)); }

    constexpr int kRow = kSplitStepK + 8;  // shared row of 32 slice entries plus 8 of padding (80 bytes)

  } // namespace
} // namespace ttg
