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
// FP64 on this GPU runs at about 1/64 of the FP32 rate (about two FP64 multiply-adds per clock
// per SM), so the sweeps are mixed precision and the FP64 part is spread over several SMs:
//   1. FP32 sweeps on a scaled copy of the block until its columns are orthogonal to ~1e-5; they
//      give a rotation V32 close to the right singular vectors.
//   2. V = V32 in FP64, made orthonormal to FP64 precision by two Newton-Schulz steps
//      V <- V + V (I - V^T V) / 2 (quadratic: 1e-6 -> 1e-12 -> round-off).
//   3. W = A V in FP64 (columns already orthogonal to ~1e-6).
//   4. FP64 sweeps on W with V accumulated: from a start that close, Jacobi's quadratic
//      convergence needs two sweeps and a third that finds nothing to rotate.
// In the FP64 sweeps only the dot product of the pair is taken (the squared column norms are
// carried along with the exact update of a rotation and recomputed at each sweep's start), and the
// angle is found in FP32 and then made exactly orthogonal in FP64 (c^2 + s^2 = 1 by two Newton
// steps): an angle good to 1e-7 still shrinks the pair's cosine by that factor each rotation.
//
// A thread-block cluster of up to 8 CTAs (1024 threads each) per block.  Rank 0 runs step 1 alone;
// steps 2-4 run on the whole cluster, step 4 with the rows of W and V dealt to the ranks and the
// dot products of each round summed over the cluster through distributed shared memory.  Each
// sweep runs the pairs in the round-robin (circle) order, k - 1 rounds of disjoint pairs, a group
// of lanes per pair.  Working sets sit in shared memory when they fit (227 KB per CTA), else in
// the global workspace (L2 resident).  At most kMaxSweeps sweeps per phase; a block whose FP64
// phase did not converge reports -1 in `info` (the host raises).  All loops are bounded and every
// CTA of a cluster passes the same sequence of cluster barriers: the number of sweeps is decided
// by rank 0's flag, read by all.
//
// A second kernel writes the kept part of each block's factors into the two output arenas, with
// the singular values absorbed as the caller asks, so that a whole truncating split is two
// launches and one read of the singular values.
#include <cooperative_groups.h>
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
    namespace cg = cooperative_groups;

    constexpr int kSvdThreads = 1024;
    constexpr int kMaxSweeps = 40;
    constexpr int kMaxCols = 1024;              // k = min(rows, cols) of a block
    constexpr int kMaxPairs = kMaxCols / 2;     // pairs of a round
    constexpr int kSvdSmemBytes = 227 * 1024;
    constexpr int kStaticBytes = 29 * 1024;     // the shares, norms, ranks and flags of the kernel
    constexpr int64_t kDynamicBytes = kSvdSmemBytes - kStaticBytes - 1024;
    constexpr int kMaxCluster = 8;

    // per block: a_off, rows, cols, u_off, s_off, vh_off, ws_off (doubles)
    struct SvdEntry
    {
      int64_t a_off, rows, cols, u_off, s_off, vh_off, ws_off;
    };

    // One block's global workspace, in doubles: V and its next iterate (k x k each) and G = V^T V
    // for the Newton-Schulz steps; W (len x k) and V by rank for clusters whose rows do not fit in
    // shared memory (up to kMaxCluster - 1 padding rows each); rank 0's FP32 working set (W, V,
    // norms) when it does not fit in shared memory.
    struct SvdLayout
    {
      int64_t v0, v1, g, w_slices, v_slices, leader, total;
      bool leader_in_smem;
    };
    __host__ __device__ inline SvdLayout svd_layout(int64_t len, int64_t k)
    {
      SvdLayout l;
      const int64_t leader_bytes = (len * k + k * k + k) * 4 + 256;
      l.leader_in_smem = leader_bytes <= kDynamicBytes;
      l.v0 = 0;
      l.v1 = k * k;
      l.g = 2 * k * k;
      l.w_slices = 3 * k * k;
      l.v_slices = l.w_slices + (len + kMaxCluster) * k;
      l.leader = l.v_slices + (k + kMaxCluster) * k;
      l.total = l.leader + (l.leader_in_smem ? 0 : (leader_bytes + 7) / 8);
      l.total = (l.total + 31) / 32 * 32;
      return l;
    }

    // The circle method's pair t of a round (players even): player players - 1 stays, the others
    // turn; p < q.
    __device__ __forceinline__ void circle_pair(int64_t round, int64_t t, int64_t players, int64_t &p, int64_t &q)
    {
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
            int64_t p, q;
            circle_pair(round, t, players, p, q);
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

    // The sweeps of a phase distributed over the CTAs of a cluster by rows: rank r holds `rows`
    // rows of W (column-major, leading dimension `rows`) and `vrows` rows of V (leading dimension
    // `vrows`).  Per round every CTA takes its rows' share of each pair's dot product, the shares
    // cross the cluster through distributed shared memory, and every CTA adds them in the same
    // order, so that all hold the same dot products, angles and norms; each then rotates its own
    // rows.  One cluster barrier per round (shares double-buffered) and two per sweep.  Whether a
    // sweep rotated anything is read from rank 0 so that every CTA leaves the loop together.
    template <int G>
    __device__ int cluster_sweeps(const cg::cluster_group &cluster, double *w, int64_t rows, double *v, int64_t vrows,
                                  int64_t k, double tol, double *norms, double *shares, double *partial, int *flags)
    {
      const unsigned ranks = cluster.num_blocks();
      const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, warps = blockDim.x >> 5;
      const int group = lane / G, gl = lane % G;
      constexpr int per_warp = 32 / G;
      const int64_t players = k + (k & 1), pairs = players / 2;
      const double tol2 = tol * tol;
      for (int sweep = 0; sweep < kMaxSweeps; ++sweep)
      {
        // exact squared norms: this CTA's share of each, summed over the cluster in rank order
        for (int64_t j = warp; j < k; j += warps)
        {
          const double *wj = w + j * rows;
          double sum = 0;
          for (int64_t i = lane; i < rows; i += 32) sum = fma(wj[i], wj[i], sum);
          sum = warp_sum(sum);
          if (lane == 0) partial[j] = sum;
        }
        if (threadIdx.x == 0) flags[sweep & 1] = 0;
        cluster.sync();
        for (int64_t j = threadIdx.x; j < k; j += blockDim.x)
        {
          double sum = 0;
          for (unsigned r = 0; r < ranks; ++r) sum += cluster.map_shared_rank(partial, r)[j];
          norms[j] = sum;
        }
        __syncthreads();
        for (int64_t round = 0; round + 1 < players; ++round)
        {
          double *share = shares + (round & 1) * kMaxPairs;
          // this CTA's share of the dot product of every pair of the round
          for (int64_t t0 = static_cast<int64_t>(warp) * per_warp; t0 < pairs; t0 += static_cast<int64_t>(warps) * per_warp)
          {
            const int64_t t = t0 + group;
            int64_t p, q;
            circle_pair(round, t, players, p, q);
            const bool pair = t < pairs && q < k;
            const double *wp = w + (pair ? p : 0) * rows, *wq = w + (pair ? q : 0) * rows;
            double gamma = 0;
            if (pair)
              for (int64_t i = gl; i < rows; i += G) gamma = fma(wp[i], wq[i], gamma);
            gamma = group_sum<double, G>(gamma);
            if (t < pairs && gl == 0) share[t] = gamma;
          }
          cluster.sync();
          for (int64_t t0 = static_cast<int64_t>(warp) * per_warp; t0 < pairs; t0 += static_cast<int64_t>(warps) * per_warp)
          {
            const int64_t t = t0 + group;
            int64_t p, q;
            circle_pair(round, t, players, p, q);
            const bool pair = t < pairs && q < k;
            // the shares of the cluster: lane gl adds ranks gl, gl + G, ...; the group's butterfly
            // sum then gives every lane of every CTA the same value
            double gamma = 0;
            if (pair)
              for (unsigned r = gl; r < ranks; r += G) gamma += cluster.map_shared_rank(share, r)[t];
            gamma = group_sum<double, G>(gamma);
            if (!pair) continue;
            const double alpha = norms[p], beta = norms[q];
            if (gamma * gamma <= tol2 * alpha * beta) continue;
            float cf, sf;
            if (!angle(alpha, beta, gamma, cf, sf)) continue;
            double c = cf, sn = sf;
#pragma unroll
            for (int it = 0; it < 2; ++it)
            {
              const double f = 1.5 - 0.5 * fma(c, c, sn * sn);
              c *= f;
              sn *= f;
            }
            double *wp = w + p * rows, *wq = w + q * rows;
            for (int64_t i = gl; i < rows; i += G)
            {
              const double x = wp[i], y = wq[i];
              wp[i] = fma(c, x, -sn * y);
              wq[i] = fma(sn, x, c * y);
            }
            double *vp = v + p * vrows, *vq = v + q * vrows;
            for (int64_t i = gl; i < vrows; i += G)
            {
              const double x = vp[i], y = vq[i];
              vp[i] = fma(c, x, -sn * y);
              vq[i] = fma(sn, x, c * y);
            }
            if (gl == 0)
            {
              const double cc = c * c, ss = sn * sn, cs2 = 2 * c * sn * gamma;
              norms[p] = cc * alpha - cs2 + ss * beta;
              norms[q] = ss * alpha + cs2 + cc * beta;
              flags[sweep & 1] = 1;
            }
          }
          __syncthreads();
        }
        cluster.sync();
        const int any = cluster.map_shared_rank(flags, 0)[sweep & 1];
        if (!any) return sweep + 1;
      }
      return -1;
    }

    // A cluster of CTAs per block (grid = blocks x cluster size).  Rank 0 runs the FP32 sweeps alone
    // (they are cheap and latency-bound: a cluster barrier per round would cost more than it
    // saves); the cluster then shares the Newton-Schulz steps, forms its rows of W = A V, and runs
    // the FP64 sweeps on rows dealt to the ranks.  Per block, the global workspace holds V twice
    // and G = V^T V for the exchange, W and V by rank when a rank's rows do not fit in shared
    // memory, and rank 0's FP32 working set when that does not fit.
    __global__ void __launch_bounds__(kSvdThreads, 1)
      jacobi_svd_kernel(const SvdEntry *__restrict__ table, const double *__restrict__ a, double *__restrict__ u,
                        double *__restrict__ s, double *__restrict__ vh, double *__restrict__ workspace,
                        int32_t *__restrict__ info)
    {
      extern __shared__ __align__(16) unsigned char dynamic[];
      __shared__ double shares[2 * kMaxPairs];
      __shared__ double norms[kMaxCols];
      __shared__ double partial[kMaxCols];
      __shared__ int rank_of[kMaxCols];
      __shared__ int flags[2];
      __shared__ double big;
      const cg::cluster_group cluster = cg::this_cluster();
      const unsigned ranks = cluster.num_blocks(), rank = cluster.block_rank();
      const int64_t block = blockIdx.x / ranks;
      const SvdEntry e = table[block];
      const int64_t m = e.rows, n = e.cols;
      const bool wide = n > m;
      const int64_t len = wide ? n : m, k = wide ? m : n;  // W is len x k, column-major
      if (k == 0)
      {
        if (threadIdx.x == 0 && rank == 0) info[block] = 0;
        return;
      }
      const SvdLayout lay = svd_layout(len, k);
      double *ws = workspace + e.ws_off;
      double *v_cur = ws + lay.v0, *v_next = ws + lay.v1, *g = ws + lay.g;
      const double *src = a + e.a_off;
      const auto entry = [&](int64_t row, int64_t col) -> double
      { return wide ? src[col * n + row] : src[row * n + col]; };  // row < len, col < k

      // 1. rank 0: FP32 sweeps on the block scaled to |entries| <= 1; V32 goes out as V in FP64
      if (rank == 0)
      {
        unsigned char *base = lay.leader_in_smem ? dynamic : reinterpret_cast<unsigned char *>(ws + lay.leader);
        float *w32 = reinterpret_cast<float *>(base);
        float *v32 = w32 + len * k;
        float *norms32 = v32 + k * k;
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
        jacobi_phase<float>(w32, v32, norms32, len, k, 1e-5, flags);
        for (int64_t i = threadIdx.x; i < k * k; i += blockDim.x) v_cur[i] = static_cast<double>(v32[i]);
      }
      cluster.sync();

      // 2. V orthonormal to FP64 precision by two Newton-Schulz steps V <- V + V (I - V^T V) / 2.
      // G = V^T V in FP64 (the symmetric half, by the whole cluster); the correction V E, E = I - G
      // of size ~1e-6 and then ~1e-12, in FP32 accumulation: its rounding (~1e-7 of E) is below
      // FP64 precision of V after the second step.  V and G pass between the CTAs through the
      // workspace, read past L1 (__ldcg) so that no CTA sees an earlier iterate.
      const int64_t lane_all = static_cast<int64_t>(rank) * blockDim.x + threadIdx.x;
      const int64_t lanes_all = static_cast<int64_t>(ranks) * blockDim.x;
      for (int step = 0; step < 2; ++step)
      {
        for (int64_t i = lane_all; i < k * k; i += lanes_all)
        {
          const int64_t r = i % k, c = i / k;  // G[r][c] = v_r . v_c (columns of V)
          if (r > c) continue;
          const double *vr = v_cur + r * k, *vc = v_cur + c * k;
          double sum = 0.0;
          for (int64_t x = 0; x < k; ++x) sum = fma(__ldcg(vr + x), __ldcg(vc + x), sum);
          g[c * k + r] = sum;
          g[r * k + c] = sum;
        }
        cluster.sync();
        for (int64_t i = lane_all; i < k * k; i += lanes_all)
        {
          const int64_t row = i % k, c = i / k;
          const double *gc = g + c * k;
          float sum = 0.0f;
          for (int64_t r = 0; r < k; ++r)
            sum = fmaf(static_cast<float>(__ldcg(v_cur + r * k + row)), static_cast<float>((r == c ? 1.0 : 0.0) - __ldcg(gc + r)), sum);
          v_next[i] = fma(0.5, static_cast<double>(sum), __ldcg(v_cur + i));
        }
        cluster.sync();
        double *t = v_cur;
        v_cur = v_next;
        v_next = t;
      }

      // 3. this rank's rows of W = A V (FP64) and of V
      const int64_t rows = (len + ranks - 1) / ranks, vrows = (k + ranks - 1) / ranks;
      const int64_t r0 = min(len, static_cast<int64_t>(rank) * rows), r1 = min(len, r0 + rows);
      const int64_t c0 = min(k, static_cast<int64_t>(rank) * vrows), c1 = min(k, c0 + vrows);
      const bool slices_in_smem = (rows + vrows) * k * 8 <= kDynamicBytes;
      double *w = slices_in_smem ? reinterpret_cast<double *>(dynamic) : ws + lay.w_slices + rank * rows * k;
      double *v = slices_in_smem ? w + rows * k : ws + lay.v_slices + rank * vrows * k;
      for (int64_t i = threadIdx.x; i < rows * k; i += blockDim.x)
      {
        const int64_t row = r0 + i % rows, j = i / rows;
        double sum = 0.0;
        if (row < r1)
        {
          const double *vj = v_cur + j * k;
          for (int64_t c = 0; c < k; ++c) sum = fma(entry(row, c), __ldcg(vj + c), sum);
        }
        w[i] = sum;
      }
      for (int64_t i = threadIdx.x; i < vrows * k; i += blockDim.x)
      {
        const int64_t row = c0 + i % vrows, j = i / vrows;
        v[i] = row < c1 ? __ldcg(v_cur + j * k + row) : 0.0;
      }
      __syncthreads();

      // 4. FP64 sweeps over the cluster
      const double tol = 2.220446049250313e-16 * sqrt(static_cast<double>(len));
      const int sweeps = rows <= 32 ? cluster_sweeps<4>(cluster, w, rows, v, vrows, k, tol, norms, shares, partial, flags)
                                    : rows <= 128 ? cluster_sweeps<8>(cluster, w, rows, v, vrows, k, tol, norms, shares, partial, flags)
                                                  : cluster_sweeps<32>(cluster, w, rows, v, vrows, k, tol, norms, shares, partial, flags);

      // singular values (column norms over the cluster), their ranks, and this rank's rows of the
      // factors in descending order
      const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, warps = blockDim.x >> 5;
      for (int64_t j = warp; j < k; j += warps)
      {
        const double *wj = w + j * rows;
        double sum = 0;
        for (int64_t i = lane; i < rows; i += 32) sum = fma(wj[i], wj[i], sum);
        sum = warp_sum(sum);
        if (lane == 0) partial[j] = sum;
      }
      cluster.sync();
      for (int64_t j = threadIdx.x; j < k; j += blockDim.x)
      {
        double sum = 0;
        for (unsigned r = 0; r < ranks; ++r) sum += cluster.map_shared_rank(partial, r)[j];
        norms[j] = sqrt(sum);
      }
      __syncthreads();
      for (int64_t j = threadIdx.x; j < k; j += blockDim.x)
      {
        int r = 0;
        const double sj = norms[j];
        for (int64_t i = 0; i < k; ++i) r += (norms[i] > sj || (norms[i] == sj && i < j)) ? 1 : 0;
        rank_of[j] = r;
        if (rank == 0) s[e.s_off + r] = sj;
      }
      __syncthreads();
      // tall: U = W / sigma (m x k), Vh = V^T; wide: U = V (m x m), Vh = (W / sigma)^T
      double *uo = u + e.u_off, *vo = vh + e.vh_off;
      for (int64_t i = threadIdx.x; i < rows * k; i += blockDim.x)
      {
        const int64_t j = i / rows, row = r0 + i % rows;
        if (row >= r1) continue;
        const double sj = norms[j];
        const double x = sj > 0 ? w[i] / sj : 0.0;
        if (wide)
          vo[static_cast<int64_t>(rank_of[j]) * n + row] = x;
        else
          uo[row * k + rank_of[j]] = x;
      }
      for (int64_t i = threadIdx.x; i < vrows * k; i += blockDim.x)
      {
        const int64_t j = i / vrows, row = c0 + i % vrows;  // entry row of column j of V
        if (row >= c1) continue;
        if (wide)
          uo[row * k + rank_of[j]] = v[i];
        else
          vo[static_cast<int64_t>(rank_of[j]) * n + row] = v[i];
      }
      if (threadIdx.x == 0 && rank == 0) info[block] = sweeps;
      // no CTA leaves while another may still read its shared memory
      cluster.sync();
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
    static int cluster_for[kMaxCluster + 1] = {};  // clusters of each size that fit on the GPU at once
    std::call_once(once, [] {
      configured = cudaFuncSetAttribute(jacobi_svd_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        static_cast<int>(kDynamicBytes));
      for (int size = 1; size <= kMaxCluster && configured == cudaSuccess; size *= 2)
      {
        cudaLaunchConfig_t config = {};
        cudaLaunchAttribute attribute[1];
        attribute[0].id = cudaLaunchAttributeClusterDimension;
        attribute[0].val.clusterDim.x = static_cast<unsigned>(size);
        attribute[0].val.clusterDim.y = 1;
        attribute[0].val.clusterDim.z = 1;
        config.gridDim = dim3(static_cast<unsigned>(size));
        config.blockDim = dim3(kSvdThreads);
        config.dynamicSmemBytes = kDynamicBytes;
        config.attrs = attribute;
        config.numAttrs = 1;
        int clusters = 0;
        if (cudaOccupancyMaxActiveClusters(&clusters, jacobi_svd_kernel, &config) != cudaSuccess)
        {
          cudaGetLastError();
          clusters = 0;
        }
        cluster_for[size] = clusters;
      }
    });
    if (configured != cudaSuccess) return configured;
    // the largest cluster with which every block's cluster is resident at once (one CTA per block
    // when even that does not hold)
    int size = 1;
    for (int c = kMaxCluster; c > 1; c /= 2)
      if (cluster_for[c] >= count)
      {
        size = c;
        break;
      }
    cudaLaunchConfig_t config = {};
    cudaLaunchAttribute attribute[1];
    attribute[0].id = cudaLaunchAttributeClusterDimension;
    attribute[0].val.clusterDim.x = static_cast<unsigned>(size);
    attribute[0].val.clusterDim.y = 1;
    attribute[0].val.clusterDim.z = 1;
    config.gridDim = dim3(static_cast<unsigned>(count) * static_cast<unsigned>(size));
    config.blockDim = dim3(kSvdThreads);
    config.dynamicSmemBytes = kDynamicBytes;
    config.stream = stream;
    config.attrs = attribute;
    config.numAttrs = 1;
    return cudaLaunchKernelEx(&config, jacobi_svd_kernel, static_cast<const SvdEntry *>(table), a, u, s, vh,
                              static_cast<double *>(workspace), info);
  }

  int64_t svd_workspace_doubles(int64_t rows, int64_t cols)
  {
    const int64_t len = std::max(rows, cols), k = std::min(rows, cols);
    return k == 0 ? 0 : svd_layout(len, k).total;
  }

  cudaError_t svd_keep(int32_t count, const void *table, const double *u, const double *s, const double *vh,
                       double *first, double *second, double *values, cudaStream_t stream)
  {
    if (count <= 0) return cudaSuccess;
    keep_kernel<<<count, 256, 0, stream>>>(static_cast<const KeepEntry *>(table), u, s, vh, first, second, values);
    return cudaGetLastError();
  }

} // namespace ttg
