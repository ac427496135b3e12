// Thin SVDs of the blocks of a tensor in one launch, for the truncating splittings
// (tentorch/linalg/graded/svd.cpp:41-177, which calls at::linalg_svd once per block).
//
// Method: one-sided Jacobi (Hestenes 1958; the rotation of Rutishauser as in Demmel & Veselic,
// "Jacobi's method is more accurate than QR", SIAM J. Matrix Anal. Appl. 13 (1992)).  The columns
// of W (the block, or its transpose when it is wider than tall, so that W has k = min(m, n)
// columns) are rotated in pairs until every pair is orthogonal to working precision; then the
// column norms are the singular values, the normalised columns one set of singular vectors and
// the accumulated rotations V the other.  U and V come out orthonormal to round-off, which a
// truncating DMRG needs for the kept vectors however small their values.
//
// FP64 on this GPU runs at about 1/64 of the FP32 rate, so the sweeps are mixed precision:
//   1. FP32 sweeps on a scaled copy of the block until its columns are orthogonal to ~1e-5; they
//      give a rotation V32 close to the right singular vectors.
//   2. V = V32 in FP64, made orthonormal to FP64 precision by two Newton-Schulz steps
//      V <- V (3 I - V^T V) / 2 (quadratic: 1e-7 -> 1e-14 -> round-off).
//   3. W = A V in FP64 (columns already orthogonal to ~1e-6).
//   4. FP64 sweeps on W with V accumulated: from a start that close, Jacobi's quadratic
//      convergence needs two sweeps and a third that finds nothing to rotate.
// In the FP64 sweeps only the dot product of the pair is taken (the squared column norms are
// carried along with the exact update of a rotation and recomputed at each sweep's start), and the
// angle is found in FP32 and then made exactly orthogonal in FP64 (c^2 + s^2 = 1 by two Newton
// steps): an angle good to 1e-7 still shrinks the pair's cosine by that factor each rotation.
//
// One CTA of 1024 threads per block; each sweep runs the pairs in the round-robin (circle) order,
// k - 1 rounds of disjoint pairs, a warp per pair.  Everything sits in shared memory when it fits
// (227 KB), else in a global workspace (L2 resident).  At most kMaxSweeps sweeps per phase; a
// block whose FP64 phase did not converge reports -1 in `info` (the host raises).  All loops are
// bounded: no waits.
//
// A second kernel writes the kept part of each block's factors into the two output arenas, with
// the singular values absorbed as the caller asks, so that a whole truncating split is two
// launches and one read of the singular values.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <mutex>

#include "executor.h"

namespace ttg
{
  namespace
  {
    constexpr int kSvdThreads = 1024;
    constexpr int kMaxSweeps = 40;
    constexpr int kSvdSmemBytes = 227 * 1024;
    constexpr int kStaticBytes = 12 * 1024;  // the ranks and values below
    constexpr int64_t kDynamicBytes = kSvdSmemBytes - kStaticBytes - 1024;

    // per block: a_off, rows, cols, u_off, s_off, vh_off, ws_off (doubles; ws_off -1: no workspace)
    struct SvdEntry
    {
      int64_t a_off, rows, cols, u_off, s_off, vh_off, ws_off;
    };

    // bytes of one block's working set: W (len x k) FP64, V and the Newton-Schulz product (k x k)
    // FP64, W and V in FP32, the squared norms in FP64 and FP32
    __host__ __device__ inline int64_t svd_bytes(int64_t len, int64_t k)
    {
      return (len * k + 2 * k * k + k) * 8 + (len * k + k * k + k) * 4 + 256;
    }

    template <typename T>
    __device__ __forceinline__ T warp_sum(T v)
    {
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
      return v;
    }

    // The rotation that makes the pair (alpha = |w_p|^2, beta = |w_q|^2, gamma = w_p . w_q)
    // orthogonal: w_p' = c w_p - s w_q, w_q' = s w_p + c w_q with t = s / c the smaller root of
    // t^2 + 2 zeta t - 1 = 0, zeta = (beta - alpha) / (2 gamma).  Found in FP32 on values scaled
    // by a power of two; false when gamma is negligible at that scale.
    __device__ __forceinline__ bool angle_of(float a, float b, float g, float &c, float &s)
    {
      if (g == 0.0f) return false;
      const float zeta = (b - a) / (2.0f * g);
      const float t = fabsf(zeta) > 1e15f ? 0.5f / zeta : copysignf(1.0f, zeta) / (fabsf(zeta) + sqrtf(1.0f + zeta * zeta));
      c = rsqrtf(1.0f + t * t);
      s = c * t;
      return true;
    }

    // FP32 columns are scaled to |entries| <= 1, so their squared norms neither overflow nor lose
    // the angle; FP64 ones are brought to that scale by a power of two first
    __device__ __forceinline__ bool angle(float alpha, float beta, float gamma, float &c, float &s)
    {
      return angle_of(alpha, beta, gamma, c, s);
    }
    __device__ __forceinline__ bool angle(double alpha, double beta, double gamma, float &c, float &s)
    {
      int ex;
      frexp(fmax(alpha, beta), &ex);
      return angle_of(static_cast<float>(ldexp(alpha, -ex)), static_cast<float>(ldexp(beta, -ex)),
                      static_cast<float>(ldexp(gamma, -ex)), c, s);
    }

    // One Jacobi phase over W (len x k, column-major) with the rotations accumulated into V (k x k).
    // FP32: everything in FP32.  FP64: the dot products, updates and norms in FP64, the angle in
    // FP32 made exactly orthogonal.  Returns the sweeps taken, -1 when kMaxSweeps did not do.
    template <typename T, int G>
    __device__ __forceinline__ T group_sum(T v)
    {
#pragma unroll
      for (int o = G / 2; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o, G);
      return v;
    }

    // One Jacobi phase over W (len x k, column-major) with the rotations accumulated into V (k x k).
    // FP32: everything in FP32.  FP64: the dot products, updates and norms in FP64, the angle in
    // FP32 made exactly orthogonal.  A group of G lanes takes a pair (G = 8 for columns of up to 128
    // entries, so a warp rotates four pairs at once and a dot product needs three shuffle steps, not
    // five: FP64 instructions cost the same however few lanes they serve).  Returns the sweeps taken,
    // -1 when kMaxSweeps did not do.
    template <typename T, int G>
    __device__ int jacobi_phase(T *w, T *v, T *norms, int64_t len, int64_t k, double tol, int *rotated)
    {
      const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, warps = blockDim.x >> 5;
      const int group = lane / G, gl = lane % G;
      constexpr int per_warp = 32 / G;
      const int64_t players = k + (k & 1);  // a dummy column pairs with the odd one out
      const T tol2 = static_cast<T>(tol * tol);
      for (int sweep = 0; sweep < kMaxSweeps; ++sweep)
      {
        // exact squared norms at the start of every sweep
        for (int64_t j = warp; j < k; j += warps)
        {
          const T *wj = w + j * len;
          T sum = 0;
          for (int64_t i = lane; i < len; i += 32) sum = fma(wj[i], wj[i], sum);
          sum = warp_sum(sum);
          if (lane == 0) norms[j] = sum;
        }
        if (threadIdx.x == 0) *rotated = 0;
        __syncthreads();
        for (int64_t round = 0; round + 1 < players; ++round)
        {
          // every group of the warp walks the same number of turns, so the shuffles stay converged
          for (int64_t t0 = static_cast<int64_t>(warp) * per_warp; t0 < players / 2; t0 += static_cast<int64_t>(warps) * per_warp)
          {
            const int64_t t = t0 + group;
            // circle method: player players-1 stays, the others turn
            int64_t p = 0, q = 0;
            if (t == 0)
            {
              p = round;
              q = players - 1;
            }
            else
            {
              p = (round + t) % (players - 1);
              q = (round - t + players - 1) % (players - 1);
            }
            if (p > q)
            {
              const int64_t lower = q;
              q = p;
              p = lower;
            }
            const bool pair = t < players / 2 && q < k;  // not past the round, not the dummy
            T *wp = w + (pair ? p : 0) * len, *wq = w + (pair ? q : 0) * len;
            T gamma = 0;
            if (pair)
              for (int64_t i = gl; i < len; i += G) gamma = fma(wp[i], wq[i], gamma);
            gamma = group_sum<T, G>(gamma);
            if (!pair) continue;
            const T alpha = norms[p], beta = norms[q];
            // orthogonal to working precision: cos^2 of the pair's angle below tol^2
            if (gamma * gamma <= tol2 * alpha * beta) continue;
            float cf, sf;
            if (!angle(alpha, beta, gamma, cf, sf)) continue;
            T c = cf, sn = sf;
            if (sizeof(T) == 8)
            {
              // c^2 + s^2 = 1 to FP64 precision: two Newton steps on 1 / sqrt(c^2 + s^2)
#pragma unroll
              for (int it = 0; it < 2; ++it)
              {
                const T f = static_cast<T>(1.5) - static_cast<T>(0.5) * fma(c, c, sn * sn);
                c *= f;
                sn *= f;
              }
            }
            for (int64_t i = gl; i < len; i += G)
            {
              const T x = wp[i], y = wq[i];
              wp[i] = fma(c, x, -sn * y);
              wq[i] = fma(sn, x, c * y);
            }
            T *vp = v + p * k, *vq = v + q * k;
            for (int64_t i = gl; i < k; i += G)
            {
              const T x = vp[i], y = vq[i];
              vp[i] = fma(c, x, -sn * y);
              vq[i] = fma(sn, x, c * y);
            }
            if (gl == 0)
            {
              const T cc = c * c, ss = sn * sn, cs2 = 2 * c * sn * gamma;
              norms[p] = cc * alpha - cs2 + ss * beta;
              norms[q] = ss * alpha + cs2 + cc * beta;
              *rotated = 1;
            }
          }
          __syncthreads();
        }
        const int any = *rotated;
        __syncthreads();
        if (!any) return sweep + 1;
      }
      return -1;
    }

    template <typename T>
    __device__ int jacobi_phase(T *w, T *v, T *norms, int64_t len, int64_t k, double tol, int *rotated)
    {
      if (len <= 128) return jacobi_phase<T, 8>(w, v, norms, len, k, tol, rotated);
      return jacobi_phase<T, 32>(w, v, norms, len, k, tol, rotated);
    }

    __global__ void __launch_bounds__(kSvdThreads, 1)
      jacobi_svd_kernel(const SvdEntry *__restrict__ table, const double *__restrict__ a, double *__restrict__ u,
                        double *__restrict__ s, double *__restrict__ vh, unsigned char *__restrict__ workspace,
                        int32_t *__restrict__ info)
    {
      extern __shared__ __align__(16) unsigned char dynamic[];
      __shared__ int rotated;
      __shared__ int rank_of[1024];
      __shared__ double sigma[1024];
      __shared__ double big;
      const SvdEntry e = table[blockIdx.x];
      const int64_t m = e.rows, n = e.cols;
      const bool wide = n > m;
      const int64_t len = wide ? n : m, k = wide ? m : n;  // W is len x k, column-major
      if (k == 0)
      {
        if (threadIdx.x == 0) info[blockIdx.x] = 0;
        return;
      }
      unsigned char *base = svd_bytes(len, k) <= kDynamicBytes ? dynamic : workspace + e.ws_off * 8;
      double *w = reinterpret_cast<double *>(base);
      double *v = w + len * k;
      double *g = v + k * k;
      double *norms = g + k * k;
      float *w32 = reinterpret_cast<float *>(norms + k);
      float *v32 = w32 + len * k;
      float *norms32 = v32 + k * k;
      const double *src = a + e.a_off;
      const auto entry = [&](int64_t row, int64_t col) -> double
      { return wide ? src[col * n + row] : src[row * n + col]; };  // row < len, col < k

      // 1. FP32 sweeps on the block scaled to |entries| <= 1
      if (threadIdx.x == 0) big = 0.0;
      __syncthreads();
      {
        double local = 0.0;
        for (int64_t i = threadIdx.x; i < len * k; i += blockDim.x) local = fmax(local, fabs(entry(i % len, i / len)));
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) local = fmax(local, __shfl_xor_sync(0xffffffffu, local, o));
        if ((threadIdx.x & 31) == 0) atomicMax(reinterpret_cast<unsigned long long *>(&big), __double_as_longlong(local));
      }
      __syncthreads();
      const double scale = big > 0.0 ? 1.0 / big : 1.0;
      for (int64_t i = threadIdx.x; i < len * k; i += blockDim.x)
        w32[i] = static_cast<float>(entry(i % len, i / len) * scale);
      for (int64_t i = threadIdx.x; i < k * k; i += blockDim.x) v32[i] = (i / k == i % k) ? 1.0f : 0.0f;
      __syncthreads();
      jacobi_phase<float>(w32, v32, norms32, len, k, 1e-5, &rotated);

      // 2. V = V32 in FP64, orthonormal by two Newton-Schulz steps: G = V^T V, V <- V (3 I - G) / 2
      for (int64_t i = threadIdx.x; i < k * k; i += blockDim.x) v[i] = static_cast<double>(v32[i]);
      __syncthreads();
      for (int step = 0; step < 2; ++step)
      {
        for (int64_t i = threadIdx.x; i < k * k; i += blockDim.x)
        {
          const int64_t r = i % k, c = i / k;  // G[r][c] = v_r . v_c (columns of V)
          const double *vr = v + r * k, *vc = v + c * k;
          double sum = 0.0;
          for (int64_t x = 0; x < k; ++x) sum = fma(vr[x], vc[x], sum);
          g[i] = sum;
        }
        __syncthreads();
        // the new V into W's space (free until step 3): V'[:, c] = sum_r V[:, r] (1.5 d_rc - 0.5 G[r][c])
        for (int64_t i = threadIdx.x; i < k * k; i += blockDim.x)
        {
          const int64_t row = i % k, c = i / k;
          double sum = 1.5 * v[c * k + row];
          for (int64_t r = 0; r < k; ++r) sum = fma(-0.5 * g[c * k + r], v[r * k + row], sum);
          w[i] = sum;
        }
        __syncthreads();
        for (int64_t i = threadIdx.x; i < k * k; i += blockDim.x) v[i] = w[i];
        __syncthreads();
      }

      // 3. W = A V in FP64
      for (int64_t i = threadIdx.x; i < len * k; i += blockDim.x)
      {
        const int64_t row = i % len, j = i / len;
        const double *vj = v + j * k;
        double sum = 0.0;
        for (int64_t c = 0; c < k; ++c) sum = fma(entry(row, c), vj[c], sum);
        w[i] = sum;
      }
      __syncthreads();

      // 4. FP64 sweeps
      const int sweeps = jacobi_phase<double>(w, v, norms, len, k, 2.220446049250313e-16 * sqrt(static_cast<double>(len)),
                                             &rotated);

      // singular values (column norms), their ranks, and the factors in descending order
      const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, warps = blockDim.x >> 5;
      for (int64_t j = warp; j < k; j += warps)
      {
        const double *wj = w + j * len;
        double sum = 0;
        for (int64_t i = lane; i < len; i += 32) sum = fma(wj[i], wj[i], sum);
        sum = warp_sum(sum);
        if (lane == 0) sigma[j] = sqrt(sum);
      }
      __syncthreads();
      for (int64_t j = threadIdx.x; j < k; j += blockDim.x)
      {
        int r = 0;
        const double sj = sigma[j];
        for (int64_t i = 0; i < k; ++i) r += (sigma[i] > sj || (sigma[i] == sj && i < j)) ? 1 : 0;
        rank_of[j] = r;
        s[e.s_off + r] = sj;
      }
      __syncthreads();
      // tall: U = W / sigma (m x k), Vh = V^T; wide: U = V (m x m), Vh = (W / sigma)^T
      double *uo = u + e.u_off, *vo = vh + e.vh_off;
      for (int64_t i = threadIdx.x; i < len * k; i += blockDim.x)
      {
        const int64_t j = i / len, row = i % len;
        const double sj = sigma[j];
        const double x = sj > 0 ? w[i] / sj : 0.0;
        if (wide)
          vo[static_cast<int64_t>(rank_of[j]) * n + row] = x;
        else
          uo[row * k + rank_of[j]] = x;
      }
      for (int64_t i = threadIdx.x; i < k * k; i += blockDim.x)
      {
        const int64_t j = i / k, row = i % k;  // entry row of column j of V
        if (wide)
          uo[row * k + rank_of[j]] = v[i];
        else
          vo[static_cast<int64_t>(rank_of[j]) * n + row] = v[i];
      }
      if (threadIdx.x == 0) info[blockIdx.x] = sweeps;
    }

    // per kept block: where its factors sit in the packed output of the SVD and where their kept
    // part lands in the two arenas
    struct KeepEntry
    {
      int64_t u_off, s_off, vh_off;      // packed factors: U rows x k, s k, Vh k x cols
      int64_t first_off, second_off;     // output blocks: first (rows x first_ld), second (second_rows x cols)
      int64_t values_off;                // where the kept values go in the bond array
      int32_t rows, cols, k, kept, first_ld, column, row, absorb;
    };

    // one CTA per kept block: first[:, column:column+kept] = U[:, :kept] (times s or sqrt(s)),
    // second[row:row+kept, :] = Vh[:kept, :] (times s or sqrt(s)), values[...] = s[:kept]
    __global__ void keep_kernel(const KeepEntry *__restrict__ table, const double *__restrict__ u,
                                const double *__restrict__ s, const double *__restrict__ vh,
                                double *__restrict__ first, double *__restrict__ second, double *__restrict__ values)
    {
      const KeepEntry e = table[blockIdx.x];
      const double *sv = s + e.s_off;
      for (int64_t i = threadIdx.x; i < static_cast<int64_t>(e.rows) * e.kept; i += blockDim.x)
      {
        const int64_t r = i / e.kept, j = i % e.kept;
        double x = u[e.u_off + r * e.k + j];
        if (e.absorb == 1) x *= sv[j];
        else if (e.absorb == 3) x *= sqrt(sv[j]);
        first[e.first_off + r * e.first_ld + e.column + j] = x;
      }
      for (int64_t i = threadIdx.x; i < static_cast<int64_t>(e.kept) * e.cols; i += blockDim.x)
      {
        const int64_t j = i / e.cols, c = i % e.cols;
        double x = vh[e.vh_off + j * e.cols + c];
        if (e.absorb == 2) x *= sv[j];
        else if (e.absorb == 3) x *= sqrt(sv[j]);
        second[e.second_off + (e.row + j) * static_cast<int64_t>(e.cols) + c] = x;
      }
      for (int64_t j = threadIdx.x; j < e.kept; j += blockDim.x) values[e.values_off + j] = sv[j];
    }
  } // namespace

  cudaError_t svd_blocks(int32_t count, const void *table, const double *a, double *u, double *s, double *vh,
                         void *workspace, int32_t *info, cudaStream_t stream)
  {
    if (count <= 0) return cudaSuccess;
    static std::once_flag once;
    static cudaError_t configured = cudaSuccess;
    std::call_once(once, [] {
      configured = cudaFuncSetAttribute(jacobi_svd_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        static_cast<int>(kDynamicBytes));
    });
    if (configured != cudaSuccess) return configured;
    jacobi_svd_kernel<<<count, kSvdThreads, kDynamicBytes, stream>>>(static_cast<const SvdEntry *>(table), a, u, s, vh,
                                                                      static_cast<unsigned char *>(workspace), info);
    return cudaGetLastError();
  }

  int64_t svd_workspace_doubles(int64_t rows, int64_t cols)
  {
    const int64_t len = std::max(rows, cols), k = std::min(rows, cols);
    const int64_t bytes = svd_bytes(len, k);
    return bytes <= kDynamicBytes ? 0 : (bytes + 7) / 8;
  }

  cudaError_t svd_keep(int32_t count, const void *table, const double *u, const double *s, const double *vh,
                       double *first, double *second, double *values, cudaStream_t stream)
  {
    if (count <= 0) return cudaSuccess;
    keep_kernel<<<count, 256, 0, stream>>>(static_cast<const KeepEntry *>(table), u, s, vh, first, second, values);
    return cudaGetLastError();
  }

} // namespace ttg
