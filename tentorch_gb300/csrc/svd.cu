// Thin SVDs of the blocks of a tensor in one launch, for the truncating splittings
// (tentorch/linalg/graded/svd.cpp:41-177, which calls at::linalg_svd once per block).
//
// Method: one-sided Jacobi (Hestenes 1958; the rotation of Rutishauser as in Demmel & Veselic,
// "Jacobi's method is more accurate than QR", SIAM J. Matrix Anal. Appl. 13 (1992)).  The columns
// of W (the block, or its transpose when it is wider than tall, so that W has min(m, n) columns)
// are rotated in pairs until every pair is orthogonal to working precision; then the column norms
// are the singular values, the normalised columns one set of singular vectors and the accumulated
// rotations V the other.  The method is accurate in the relative sense for every singular value,
// and U and V come out orthonormal to round-off, which a truncating DMRG needs for the kept
// vectors however small their values.
//
// One CTA of 1024 threads per block: each sweep runs the pairs in the round-robin (circle) order,
// min(m, n) - 1 rounds of disjoint pairs, a warp per pair: three dot products over the column
// length reduced with shuffles, the rotation, and the update of both columns of W and of V.  W and
// V sit in shared memory when they fit (227 KB), else in a global workspace (L2 resident).  The
// sweeps stop when a sweep rotates nothing, at most kMaxSweeps; a block that did not converge
// reports -1 in `info` (the host raises).  The loops are all bounded: no waits.
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

    // per block: a_off, rows, cols, u_off, s_off, vh_off, ws_off (doubles; ws_off -1: no workspace)
    struct SvdEntry
    {
      int64_t a_off, rows, cols, u_off, s_off, vh_off, ws_off;
    };

    __device__ __forceinline__ double warp_sum(double v)
    {
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
      return v;
    }

    __global__ void __launch_bounds__(kSvdThreads, 1)
      jacobi_svd_kernel(const SvdEntry *__restrict__ table, const double *__restrict__ a, double *__restrict__ u,
                        double *__restrict__ s, double *__restrict__ vh, double *__restrict__ workspace,
                        int32_t *__restrict__ info, int64_t smem_doubles)
    {
      extern __shared__ double shared[];
      __shared__ int rotated;
      __shared__ int rank_of[1024];
      const SvdEntry e = table[blockIdx.x];
      const int64_t m = e.rows, n = e.cols;
      const bool wide = n > m;
      const int64_t len = wide ? n : m, k = wide ? m : n;  // W is len x k, column-major
      if (k == 0)
      {
        if (threadIdx.x == 0) info[blockIdx.x] = 0;
        return;
      }
      double *w, *v;
      if ((len * k + k * k) <= smem_doubles)
      {
        w = shared;
        v = shared + len * k;
      }
      else if (len * k <= smem_doubles)
      {
        w = shared;
        v = workspace + e.ws_off;
      }
      else
      {
        w = workspace + e.ws_off;
        v = w + len * k;
      }
      const double *src = a + e.a_off;
      // W: column j of the block (tall) or row j of the block (wide); V = identity
      for (int64_t i = threadIdx.x; i < len * k; i += blockDim.x)
      {
        const int64_t col = i / len, row = i % len;
        w[i] = wide ? src[col * n + row] : src[row * n + col];
      }
      for (int64_t i = threadIdx.x; i < k * k; i += blockDim.x) v[i] = (i / k == i % k) ? 1.0 : 0.0;
      __syncthreads();

      const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, warps = blockDim.x >> 5;
      const double tolerance = 2.220446049250313e-16 * sqrt(static_cast<double>(len));
      const int64_t players = k + (k & 1);  // a dummy column pairs with the odd one out
      int sweeps = -1;
      for (int sweep = 0; sweep < kMaxSweeps; ++sweep)
      {
        if (threadIdx.x == 0) rotated = 0;
        __syncthreads();
        for (int64_t round = 0; round + 1 < players; ++round)
        {
          for (int64_t t = warp; t < players / 2; t += warps)
          {
            // circle method: player players-1 stays, the others turn
            int64_t p, q;
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
            if (q >= k) continue;  // the dummy
            double *wp = w + p * len, *wq = w + q * len;
            double alpha = 0, beta = 0, gamma = 0;
            for (int64_t i = lane; i < len; i += 32)
            {
              const double x = wp[i], y = wq[i];
              alpha = fma(x, x, alpha);
              beta = fma(y, y, beta);
              gamma = fma(x, y, gamma);
            }
            alpha = warp_sum(alpha);
            beta = warp_sum(beta);
            gamma = warp_sum(gamma);
            // orthogonal to working precision: the cosine of the pair's angle below sqrt(len) eps
            if (gamma == 0.0 || fabs(gamma) <= tolerance * sqrt(alpha) * sqrt(beta)) continue;
            const double zeta = (beta - alpha) / (2.0 * gamma);
            const double tan = copysign(1.0, zeta) / (fabs(zeta) + hypot(1.0, zeta));
            const double cs = 1.0 / hypot(1.0, tan), sn = cs * tan;
            for (int64_t i = lane; i < len; i += 32)
            {
              const double x = wp[i], y = wq[i];
              wp[i] = cs * x - sn * y;
              wq[i] = sn * x + cs * y;
            }
            double *vp = v + p * k, *vq = v + q * k;
            for (int64_t i = lane; i < k; i += 32)
            {
              const double x = vp[i], y = vq[i];
              vp[i] = cs * x - sn * y;
              vq[i] = sn * x + cs * y;
            }
            if (lane == 0) rotated = 1;
          }
          __syncthreads();
        }
        const int any = rotated;
        __syncthreads();
        if (!any)
        {
          sweeps = sweep + 1;
          break;
        }
      }
      // singular values (column norms) into the shared tail of the ranks, then the ranks
      __shared__ double sigma[1024];
      for (int64_t j = warp; j < k; j += warps)
      {
        const double *wj = w + j * len;
        double norm = 0;
        for (int64_t i = lane; i < len; i += 32) norm = fma(wj[i], wj[i], norm);
        norm = warp_sum(norm);
        if (lane == 0) sigma[j] = sqrt(norm);
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
                         double *workspace, int32_t *info, cudaStream_t stream)
  {
    if (count <= 0) return cudaSuccess;
    static std::once_flag once;
    static cudaError_t configured = cudaSuccess;
    std::call_once(once, [] {
      configured = cudaFuncSetAttribute(jacobi_svd_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        kSvdSmemBytes - 16 * 1024);
    });
    if (configured != cudaSuccess) return configured;
    const int64_t smem = kSvdSmemBytes - 16 * 1024;  // the static arrays take 12 KB
    jacobi_svd_kernel<<<count, kSvdThreads, smem, stream>>>(static_cast<const SvdEntry *>(table), a, u, s, vh,
                                                            workspace, info, smem / 8);
    return cudaGetLastError();
  }

  int64_t svd_shared_doubles() { return (kSvdSmemBytes - 16 * 1024) / 8; }

  cudaError_t svd_keep(int32_t count, const void *table, const double *u, const double *s, const double *vh,
                       double *first, double *second, double *values, cudaStream_t stream)
  {
    if (count <= 0) return cudaSuccess;
    keep_kernel<<<count, 256, 0, stream>>>(static_cast<const KeepEntry *>(table), u, s, vh, first, second, values);
    return cudaGetLastError();
  }

} // namespace ttg
