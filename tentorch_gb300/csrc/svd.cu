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
//   0. (blocks of 32 columns or more) the columns sorted by norm and factored A P = Q R; steps 1-4
//      then work on the graded X = R^T, and U = Q J at the end (Drmac & Veselic 2008).
//   1. FP32 sweeps on a scaled copy of the block until its columns are orthogonal to ~1e-5; they
//      give a rotation V32 close to the right singular vectors.
//   2. V = V32 in FP64, made orthonormal to FP64 precision by two Newton-Schulz steps
//      V <- V + V (I - V^T V) / 2 (quadratic: 1e-6 -> 1e-12 -> round-off).
//   3. W = A V in FP64 (columns already orthogonal to ~1e-6).
//   4. FP64 sweeps on W with V accumulated: from a start that close, Jacobi's quadratic
//      convergence needs two or three sweeps; a sweep whose cosines were all below sqrt(tol) is
//      the last (the cosines it leaves are below ~tol).
// In the FP64 sweeps only the dot product of the pair is taken (the squared column norms are
// carried along with the exact update of a rotation and recomputed at each sweep's start), and the
// angle is found in FP32 and then made exactly orthogonal in FP64 (c^2 + s^2 = 1 by a second-order
// correction): an angle good to 1e-7 still shrinks the pair's cosine by that factor each rotation.
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

    constexpr int kSvdThreads = 512;
    constexpr int kMaxSweeps = 40;
    constexpr int kMaxCols = 1024;              // k = min(rows, cols) of a block
    constexpr int kSvdSmemBytes = 227 * 1024;
    constexpr int kStaticBytes = 21 * 1024;     // the norms, their shares, ranks and flags of the kernel
    constexpr int64_t kDynamicBytes = kSvdSmemBytes - kStaticBytes - 1024;
    constexpr int kTile = 32;                   // tiles of the Newton-Schulz and W = A V products
    constexpr int64_t kStageBytes = 2 * kTile * (kTile + 1) * 8;
    // the end of the dynamic shared memory holds the tile stages (Newton-Schulz, W = A V) or, during
    // sweeps over a cluster, the dot-product shares every rank pushes to every rank
    __host__ __device__ inline int64_t exchange_bytes(int64_t k, int64_t ranks, int64_t size)
    {
      const int64_t pairs = (k + (k & 1)) / 2;
      return ranks > 1 ? (2 * ranks * pairs * size + 15) / 16 * 16 : 0;
    }
    constexpr int kMaxCluster = 16;
    constexpr int kNper = 12;                   // entries of a column each lane of a pair holds

    // per block: a_off, rows, cols, u_off, s_off, vh_off, ws_off (doubles)
    struct SvdEntry
    {
      int64_t a_off, rows, cols, u_off, s_off, vh_off, ws_off;
    };

    // One block's global workspace, in doubles: V and its next iterate (k x k each) and G = V^T V
    // for the Newton-Schulz steps; W (len x k) and V (k x k) by rank for working sets that do not
    // fit in shared memory (up to kMaxCluster - 1 padding rows each), in FP64 and again in FP32.
    // For a block preconditioned by QR: its columns in their sorted order factored in place (R on
    // and above the diagonal, the Householder vectors below it; len x k, column-major), the
    // Householder scalars, the sorted order (k indices), and the product Q [J; 0] (len x k).
    struct SvdLayout
    {
      int64_t v0, v1, g, w_slices, v_slices, w32_slices, v32_slices, f, tau, order, b, total;
    };
    __host__ __device__ inline SvdLayout svd_layout(int64_t len, int64_t k)
    {
      SvdLayout l;
      l.v0 = 0;
      l.v1 = k * k;
      l.g = 2 * k * k;
      l.w_slices = 3 * k * k;
      l.v_slices = l.w_slices + (len + kMaxCluster) * k;
      l.w32_slices = l.v_slices + (k + kMaxCluster) * k;
      l.v32_slices = l.w32_slices + ((len + kMaxCluster) * k + 1) / 2;
      l.f = l.v32_slices + ((k + kMaxCluster) * k + 1) / 2;
      l.tau = l.f + len * k;
      l.order = l.tau + k;
      l.b = l.order + k;
      l.total = l.b + len * k;
      l.total = (l.total + 31) / 32 * 32;
      return l;
    }
    // Blocks of at least this many columns (swept over a cluster) are preconditioned by QR.
    constexpr int64_t kQrMinCols = 32;

    // The circle method's pair t of a round (players even, round < players - 1, t < players / 2):
    // player players - 1 stays, the others turn; p < q.  In 32-bit arithmetic with one conditional
    // subtraction each instead of a 64-bit remainder, which costs a long instruction sequence.
    __device__ __forceinline__ void circle_pair(int64_t round, int64_t t, int64_t players, int64_t &p, int64_t &q)
    {
      const int32_t n = static_cast<int32_t>(players - 1), r = static_cast<int32_t>(round), u = static_cast<int32_t>(t);
      int32_t a, b;
      if (u == 0)
      {
        a = r;
        b = n;
      }
      else
      {
        a = r + u;
        if (a >= n) a -= n;
        b = r - u + n;
        if (b >= n) b -= n;
      }
      p = a < b ? a : b;
      q = a < b ? b : a;
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

    template <typename T, int G>
    __device__ __forceinline__ T group_sum(T v)
    {
      if constexpr (G > 1)
      {
#pragma unroll
        for (int o = G / 2; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o, G);
      }
      return v;
    }

    // A pair's columns as a group of G lanes holds them: lane gl has entries gl, gl + G, ... of
    // each, the first kNper in registers (loads issued together, one latency), any further ones
    // read again where needed.  Register slots past the column's length are skipped whole (the
    // count is the same for every lane), so no FP64 instruction is spent on padding.
    template <typename T, int G>
    __device__ __forceinline__ T pair_dot(const T *wp, const T *wq, int64_t n, int gl, T (&x)[kNper], T (&y)[kNper])
    {
      const int64_t slots = (n + G - 1) / G;
#pragma unroll
      for (int u = 0; u < kNper; ++u)
      {
        const int64_t i = gl + static_cast<int64_t>(u) * G;
        x[u] = u < slots && i < n ? wp[i] : T(0);
        y[u] = u < slots && i < n ? wq[i] : T(0);
      }
      T sum = 0;
#pragma unroll
      for (int u = 0; u < kNper; ++u)
        if (u < slots) sum = fma(x[u], y[u], sum);
      for (int64_t i = static_cast<int64_t>(G) * kNper + gl; i < n; i += G) sum = fma(wp[i], wq[i], sum);
      return sum;
    }

    template <typename T, int G>
    __device__ __forceinline__ void pair_rotate(T *wp, T *wq, int64_t n, int gl, const T (&x)[kNper], const T (&y)[kNper],
                                                T c, T sn)
    {
      const int64_t slots = (n + G - 1) / G;
#pragma unroll
      for (int u = 0; u < kNper; ++u)
      {
        const int64_t i = gl + static_cast<int64_t>(u) * G;
        if (u < slots && i < n)
        {
          wp[i] = fma(c, x[u], -sn * y[u]);
          wq[i] = fma(sn, x[u], c * y[u]);
        }
      }
      for (int64_t i = static_cast<int64_t>(G) * kNper + gl; i < n; i += G)
      {
        const T a = wp[i], b = wq[i];
        wp[i] = fma(c, a, -sn * b);
        wq[i] = fma(sn, a, c * b);
      }
    }

    // rotate two columns in chunks of kNper entries per lane (each chunk's loads issued together)
    template <typename T, int G>
    __device__ __forceinline__ void cols_rotate(T *vp, T *vq, int64_t n, int gl, T c, T sn)
    {
      for (int64_t base = 0; base < n; base += static_cast<int64_t>(G) * kNper)
      {
        const int64_t slots = (n - base + G - 1) / G;
        T x[kNper], y[kNper];
#pragma unroll
        for (int u = 0; u < kNper; ++u)
        {
          const int64_t i = base + gl + static_cast<int64_t>(u) * G;
          x[u] = u < slots && i < n ? vp[i] : T(0);
          y[u] = u < slots && i < n ? vq[i] : T(0);
        }
#pragma unroll
        for (int u = 0; u < kNper; ++u)
        {
          const int64_t i = base + gl + static_cast<int64_t>(u) * G;
          if (u < slots && i < n)
          {
            vp[i] = fma(c, x[u], -sn * y[u]);
            vq[i] = fma(sn, x[u], c * y[u]);
          }
        }
      }
    }

    // The rotation of a pair as FP64 values with c^2 + s^2 = 1 to FP64 precision, from the FP32
    // angle: with c, s exact in FP64, d = c^2 + s^2 - 1 (~1e-7) is exact to FP64 rounding and
    // 1 / sqrt(1 + d) = 1 - d/2 + 3 d^2/8 to below 1e-20.
    __device__ __forceinline__ void exact_rotation(float cf, float sf, double &c, double &sn)
    {
      c = cf;
      sn = sf;
      const double d = fma(sn, sn, fma(c, c, -1.0));
      const double f = fma(d, fma(0.375, d, -0.5), 1.0);
      c *= f;
      sn *= f;
    }
    __device__ __forceinline__ void exact_rotation(float cf, float sf, float &c, float &sn)
    {
      c = cf;
      sn = sf;
    }

    // Jacobi sweeps over W (column-major, `rows` rows) with the rotations accumulated into V
    // (`vrows` rows), until a sweep rotates no pair whose cosine is above sqrt(tol) (or
    // kMaxSweeps); pairs below tol are not rotated.  Alone, one CTA holds every
    // row; otherwise the rows are dealt to the CTAs of the cluster: per round each CTA takes its
    // rows' share of every pair's dot product, the shares cross the cluster through distributed
    // shared memory and every CTA adds them in the same order, so that all hold the same dot
    // products, angles and norms, and rotates its own rows.  One cluster barrier per round (shares
    // double-buffered) and two per sweep; whether a sweep ended the phase is read from rank 0, so
    // every CTA leaves the loop together.  FP32: everything in FP32; FP64: the angle in FP32 made
    // exactly orthogonal in FP64 (exact_rotation; an angle good to 1e-7 still shrinks the pair's
    // cosine by that factor each rotation).  Only the pair's dot product is taken: the squared norms are
    // recomputed at each sweep's start and carried with each rotation's exact update.
    template <typename T, int G>
    __device__ int sweeps(const cg::cluster_group &cluster, bool alone, T *w, int64_t rows, T *v, int64_t vrows, int64_t k,
                          double tol, T *norms, T *exchange, T *partial, int *flags, int *list)
    {
      const unsigned ranks = alone ? 1u : cluster.num_blocks(), me = alone ? 0u : cluster.block_rank();
      const auto sync = [&] {
        if (alone) __syncthreads();
        else cluster.sync();
      };
      const auto at_rank = [&](T *local, unsigned r) -> const T * { return alone ? local : cluster.map_shared_rank(local, r); };
      const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, warps = blockDim.x >> 5;
      const int group = lane / G, gl = lane % G;
      constexpr int per_warp = 32 / G;
      const int64_t players = k + (k & 1), pairs = players / 2;
      const T tol2 = static_cast<T>(tol * tol);
      // a sweep whose rotations all had cosines below sqrt(tol) ends the phase: Jacobi converges
      // quadratically there, so the cosines it leaves are below ~tol and a further sweep (which
      // would find nothing above tol to rotate) is not run
      const T settled2 = static_cast<T>(tol);
      // FP64 over a cluster: after the barrier a group of lanes per pair finds the rotation (the
      // scalar part) and lists it, then the whole CTA rotates the listed pairs' entries, so that
      // the FP64 instructions of the rotations spread over every warp instead of the few that hold
      // the pairs (FP64 issue is the bound of a round).  The rotations of a round are listed in
      // `list` and `partial` (free during the rounds: the other ranks read `partial` only at the
      // sweep's start, before the first round's barrier); flags[4] counts them.
      constexpr bool kSpread = std::is_same_v<T, double>;
      for (int sweep = 0; sweep < kMaxSweeps; ++sweep)
      {
        for (int64_t j = warp; j < k; j += warps)
        {
          const T *wj = w + j * rows;
          T sum = 0;
          for (int64_t i = lane; i < rows; i += 32) sum = fma(wj[i], wj[i], sum);
          sum = warp_sum(sum);
          if (lane == 0) partial[j] = sum;
        }
        if (threadIdx.x == 0) flags[sweep & 1] = 0;
        sync();
        for (int64_t j = threadIdx.x; j < k; j += blockDim.x)
        {
          T sum = 0;
          for (unsigned r = 0; r < ranks; ++r) sum += at_rank(partial, r)[j];
          norms[j] = sum;
        }
        __syncthreads();
        for (int64_t round = 0; round + 1 < players; ++round)
        {
          // this round's shares: [rank][pair], double-buffered by rounds
          T *share = exchange + (round & 1) * static_cast<int64_t>(ranks) * pairs;
          // every group of a warp walks the same number of turns, so the shuffles stay converged
          for (int64_t t0 = static_cast<int64_t>(warp) * per_warp; t0 < pairs; t0 += static_cast<int64_t>(warps) * per_warp)
          {
            const int64_t t = t0 + group;
            int64_t p, q;
            circle_pair(round, t, players, p, q);
            const bool pair = t < pairs && q < k;
            T x[kNper], y[kNper];
            T *wp = w + (pair ? p : 0) * rows, *wq = w + (pair ? q : 0) * rows;
            T gamma = pair_dot<T, G>(wp, wq, pair ? rows : 0, gl, x, y);
            gamma = group_sum<T, G>(gamma);
            if (!alone && t < pairs)
            {
              // this CTA's share goes to every rank (remote stores do not wait); after the barrier
              // each rank holds every share in its own memory
              for (unsigned r = gl; r < ranks; r += G) cluster.map_shared_rank(share + static_cast<int64_t>(me) * pairs + t, r)[0] = gamma;
            }
            if (alone)
            {
              if (!pair) continue;
              const T alpha = norms[p], beta = norms[q];
              if (gamma * gamma <= tol2 * alpha * beta) continue;
              float cf, sf;
              if (!angle(alpha, beta, gamma, cf, sf)) continue;
              T c, sn;
              exact_rotation(cf, sf, c, sn);
              pair_rotate<T, G>(wp, wq, rows, gl, x, y, c, sn);
              cols_rotate<T, G>(v + p * vrows, v + q * vrows, vrows, gl, c, sn);
              if (gl == 0)
              {
                const T cc = c * c, ss = sn * sn, cs2 = 2 * c * sn * gamma;
                norms[p] = cc * alpha - cs2 + ss * beta;
                norms[q] = ss * alpha + cs2 + cc * beta;
                if (gamma * gamma > settled2 * alpha * beta) flags[sweep & 1] = 1;
              }
            }
          }
          if (!alone)
          {
            cluster.sync();
            if constexpr (kSpread)
            {
              T *lc = partial, *ls = partial + pairs;
              if (threadIdx.x == 0) flags[4] = 0;
              __syncthreads();
              for (int64_t t0 = static_cast<int64_t>(warp) * per_warp; t0 < pairs; t0 += static_cast<int64_t>(warps) * per_warp)
              {
                const int64_t t = t0 + group;
                int64_t p, q;
                circle_pair(round, t, players, p, q);
                const bool pair = t < pairs && q < k;
                T gamma = 0;
                if (pair)
                  for (unsigned r = gl; r < ranks; r += G) gamma += share[static_cast<int64_t>(r) * pairs + t];
                gamma = group_sum<T, G>(gamma);
                if (!pair || gl != 0) continue;
                const T alpha = norms[p], beta = norms[q];
                if (gamma * gamma <= tol2 * alpha * beta) continue;
                float cf, sf;
                if (!angle(alpha, beta, gamma, cf, sf)) continue;
                T c, sn;
                exact_rotation(cf, sf, c, sn);
                const T cc = c * c, ss = sn * sn, cs2 = 2 * c * sn * gamma;
                norms[p] = cc * alpha - cs2 + ss * beta;
                norms[q] = ss * alpha + cs2 + cc * beta;
                if (gamma * gamma > settled2 * alpha * beta) flags[sweep & 1] = 1;
                const int at = atomicAdd(flags + 4, 1);
                list[at] = static_cast<int>(t);
                lc[at] = c;
                ls[at] = sn;
              }
              __syncthreads();
              // entry i of a listed pair: row i of W (i < rows), else row i - rows of V
              const int span = static_cast<int>(rows + vrows), items = flags[4] * span;
              for (int it = threadIdx.x; it < items; it += blockDim.x)
              {
                const int at = it / span, i = it - at * span;
                int64_t p, q;
                circle_pair(round, list[at], players, p, q);
                const T c = lc[at], sn = ls[at];
                T *x = i < rows ? w + p * rows + i : v + p * vrows + (i - rows);
                T *y = i < rows ? w + q * rows + i : v + q * vrows + (i - rows);
                const T a = *x, b = *y;
                *x = fma(c, a, -sn * b);
                *y = fma(sn, a, c * b);
              }
            }
            else
            {
              for (int64_t t0 = static_cast<int64_t>(warp) * per_warp; t0 < pairs; t0 += static_cast<int64_t>(warps) * per_warp)
              {
                const int64_t t = t0 + group;
                int64_t p, q;
                circle_pair(round, t, players, p, q);
                const bool pair = t < pairs && q < k;
                // lane gl adds ranks gl, gl + G, ...; the group's butterfly sum then gives every lane
                // of every CTA the same value
                T gamma = 0;
                if (pair)
                  for (unsigned r = gl; r < ranks; r += G) gamma += share[static_cast<int64_t>(r) * pairs + t];
                gamma = group_sum<T, G>(gamma);
                if (!pair) continue;
                const T alpha = norms[p], beta = norms[q];
                if (gamma * gamma <= tol2 * alpha * beta) continue;
                float cf, sf;
                if (!angle(alpha, beta, gamma, cf, sf)) continue;
                T c, sn;
                exact_rotation(cf, sf, c, sn);
                cols_rotate<T, G>(w + p * rows, w + q * rows, rows, gl, c, sn);
                cols_rotate<T, G>(v + p * vrows, v + q * vrows, vrows, gl, c, sn);
                if (gl == 0)
                {
                  const T cc = c * c, ss = sn * sn, cs2 = 2 * c * sn * gamma;
                  norms[p] = cc * alpha - cs2 + ss * beta;
                  norms[q] = ss * alpha + cs2 + cc * beta;
                  if (gamma * gamma > settled2 * alpha * beta) flags[sweep & 1] = 1;
                }
              }
            }
          }
          __syncthreads();
        }
        sync();
        const int any = alone ? flags[sweep & 1] : cluster.map_shared_rank(flags, 0)[sweep & 1];
        if (!any) return sweep + 1;
      }
      return -1;
    }

    template <typename T>
    __device__ int sweeps(const cg::cluster_group &cluster, bool alone, T *w, int64_t rows, T *v, int64_t vrows, int64_t k,
                          double tol, T *norms, T *exchange, T *partial, int *flags, int *list)
    {
      const int64_t most = rows > vrows ? rows : vrows;
      // the fewest lanes per pair that hold its rows in registers (measured faster than more lanes
      // with shorter chains, in FP32 as in FP64, where the per-pair scalar work also runs once per
      // lane of the group on the narrow FP64 pipe)
      if (most <= kNper) return sweeps<T, 1>(cluster, alone, w, rows, v, vrows, k, tol, norms, exchange, partial, flags, list);
      if (most <= 2 * kNper) return sweeps<T, 2>(cluster, alone, w, rows, v, vrows, k, tol, norms, exchange, partial, flags, list);
      if (most <= 4 * kNper) return sweeps<T, 4>(cluster, alone, w, rows, v, vrows, k, tol, norms, exchange, partial, flags, list);
      if (most <= 8 * kNper) return sweeps<T, 8>(cluster, alone, w, rows, v, vrows, k, tol, norms, exchange, partial, flags, list);
      if (most <= 16 * kNper) return sweeps<T, 16>(cluster, alone, w, rows, v, vrows, k, tol, norms, exchange, partial, flags, list);
      return sweeps<T, 32>(cluster, alone, w, rows, v, vrows, k, tol, norms, exchange, partial, flags, list);
    }

    // out(i, j) = sum_x a(x, i) b(x, j) + c(i, j) over a kTile x kTile tile, x < depth, staged
    // kTile at a time in shared memory (a(x, i) from fa(x, i), b from fb; zero outside), with Acc
    // accumulation; each of the 512 threads takes two entries (i, j) and (i, j + 16).  The loaders
    // are called with x fastest across the threads when `x_fast`, else i (or j) fastest, to follow
    // the memory order of the operand.
    template <typename Acc, typename FA, typename FB, typename Out>
    __device__ void tile_product(int64_t depth, FA fa, bool a_x_fast, FB fb, bool b_x_fast, Acc *sa, Acc *sb, Out out)
    {
      constexpr int P = kTile + 1;
      const int t = threadIdx.x, i = t % kTile, j = t / kTile;
      Acc acc0 = 0, acc1 = 0;
      for (int64_t x0 = 0; x0 < depth; x0 += kTile)
      {
        for (int e = t; e < kTile * kTile; e += blockDim.x)
        {
          const int fast = e % kTile, slow = e / kTile;
          const int xa = a_x_fast ? fast : slow, ia = a_x_fast ? slow : fast;
          sa[xa * P + ia] = x0 + xa < depth ? static_cast<Acc>(fa(x0 + xa, ia)) : Acc(0);
          const int xb = b_x_fast ? fast : slow, jb = b_x_fast ? slow : fast;
          sb[xb * P + jb] = x0 + xb < depth ? static_cast<Acc>(fb(x0 + xb, jb)) : Acc(0);
        }
        __syncthreads();
#pragma unroll 8
        for (int x = 0; x < kTile; ++x)
        {
          const Acc ax = sa[x * P + i];
          acc0 = fma(ax, sb[x * P + j], acc0);
          acc1 = fma(ax, sb[x * P + j + 16], acc1);
        }
        __syncthreads();
      }
      out(i, j, acc0);
      out(i, j + 16, acc1);
    }

    // A thread-block cluster of up to 16 CTAs per block (grid = blocks x cluster size, the largest
    // blocks first).  The FP32 sweeps run on rank 0 alone when its working set fits in shared
    // memory (a cluster barrier per round would cost more than it saves), else over the cluster;
    // the cluster shares the Newton-Schulz steps and W = A V as 32 x 32 tiles; the FP64 sweeps run
    // over the cluster for blocks of 32 columns or more, on rank 0 alone for smaller ones.
    __global__ void __launch_bounds__(kSvdThreads, 1)
      jacobi_svd_kernel(const SvdEntry *__restrict__ table, const double *__restrict__ a, double *__restrict__ u,
                        double *__restrict__ s, double *__restrict__ vh, double *__restrict__ workspace,
                        int32_t *__restrict__ info)
    {
      extern __shared__ __align__(16) unsigned char dynamic[];
      __shared__ double norms_raw[kMaxCols];
      __shared__ double partial_raw[kMaxCols];
      __shared__ int rank_of[kMaxCols];
      __shared__ int flags[5];  // [0], [1]: a sweep rotated above sqrt(tol), by sweep parity; [4]: the rotations listed in a round
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
      double *stage = reinterpret_cast<double *>(dynamic + kDynamicBytes - kStageBytes);
      const double *src = a + e.a_off;
      const auto entry_a = [&](int64_t row, int64_t col) -> double
      { return wide ? src[col * n + row] : src[row * n + col]; };  // row < len, col < k

      // 0. Preconditioning (blocks swept over a cluster): the columns sorted by norm, largest
      // first, and factored A P = Q R by Householder reflections; the sweeps then run on X = R^T
      // (k x k), whose graded columns the FP32 sweeps orthogonalise in about a third of the
      // sweeps the block itself takes (Drmac & Veselic, "New fast and accurate Jacobi SVD
      // algorithm", SIAM J. Matrix Anal. Appl. 29 (2008), with the pivoting of their QR replaced by
      // the one sort).  The factors of X give those of A: A P = (Q J) S (U_x)^T with X J = U_x S.
      // Rank r owns the factored columns [q0, q1) (and so the rows [q0, q1) of X, which are its
      // rows of the sweeps).
      const bool precond = ranks > 1 && k >= kQrMinCols;
      double *qf = ws + lay.f, *qtau = ws + lay.tau, *qb = ws + lay.b;
      int64_t *qorder = reinterpret_cast<int64_t *>(ws + lay.order);
      const int64_t cpr = (k + ranks - 1) / ranks;
      const int64_t q0 = min(k, static_cast<int64_t>(rank) * cpr), q1 = min(k, q0 + cpr);
      if (precond)
      {
        const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, warps = blockDim.x >> 5;
        // squared column norms in FP32 (the same on every rank) and the order they give
        float *cn = reinterpret_cast<float *>(partial_raw);
        for (int64_t j = threadIdx.x; j < k; j += blockDim.x)
        {
          float sum = 0.0f;
          for (int64_t i = 0; i < len; ++i)
          {
            const float x = static_cast<float>(entry_a(i, j));
            sum = fmaf(x, x, sum);
          }
          cn[j] = sum;
        }
        __syncthreads();
        for (int64_t j = threadIdx.x; j < k; j += blockDim.x)
        {
          const float nj = cn[j];
          int r = 0;
          for (int64_t i = 0; i < k; ++i) r += (cn[i] > nj || (cn[i] == nj && i < j)) ? 1 : 0;
          rank_of[r] = static_cast<int>(j);
        }
        __syncthreads();
        // this rank's columns in shared memory while they are factored when they fit (else in the
        // global factored matrix); each reflector goes to the global one as it is made
        const bool qr_smem = (cpr + 1) * len * 8 <= kDynamicBytes;
        double *own = reinterpret_cast<double *>(dynamic);
        double *vst = qr_smem ? own + cpr * len : own;  // the reflector of the step, staged
        const auto colp = [&](int64_t c) -> double * { return qr_smem ? own + (c - q0) * len : qf + c * len; };
        for (int64_t c = q0; c < q1; ++c)
        {
          const int64_t from = rank_of[c];
          double *to = colp(c);
          for (int64_t i = threadIdx.x; i < len; i += blockDim.x) to[i] = entry_a(i, from);
          if (threadIdx.x == 0) qorder[c] = from;
        }
        __syncthreads();
        // step j: the owner of column j makes its reflector (as LAPACK's dlarfg: H = I - tau v v^T,
        // v_0 = 1, R_jj = beta) and publishes it, the cluster waits for it, and every rank applies
        // it to its own columns right of j, a warp per column, with v staged in shared memory
        for (int64_t j = 0; j < k; ++j)
        {
          if (j >= q0 && j < q1)
          {
            double *col = colp(j);
            double part = 0.0;
            for (int64_t i = j + 1 + threadIdx.x; i < len; i += blockDim.x) part = fma(col[i], col[i], part);
            part = warp_sum(part);
            if (lane == 0) norms_raw[warp] = part;
            __syncthreads();
            if (threadIdx.x == 0)
            {
              double xn = 0.0;
              for (int w = 0; w < warps; ++w) xn += norms_raw[w];
              const double alpha = col[j];
              double beta = alpha, tau = 0.0, scale = 0.0;
              if (xn > 0.0)
              {
                const double norm = sqrt(fma(alpha, alpha, xn));
                const double d = alpha + copysign(norm, alpha);  // alpha - beta, without cancellation
                beta = -copysign(norm, alpha);
                tau = -d / beta;                                 // (beta - alpha) / beta
                scale = 1.0 / d;
              }
              col[j] = beta;
              qf[j * len + j] = beta;
              qtau[j] = tau;
              big = scale;
            }
            __syncthreads();
            const double scale = big;
            for (int64_t i = j + 1 + threadIdx.x; i < len; i += blockDim.x)
            {
              const double x = col[i] * scale;
              col[i] = x;
              qf[j * len + i] = x;
            }
          }
          cluster.sync();
          for (int64_t i = j + 1 + threadIdx.x; i < len; i += blockDim.x) vst[i] = __ldcg(qf + j * len + i);
          __syncthreads();
          const double tau = __ldcg(qtau + j);
          if (tau != 0.0)
            for (int64_t c = max(q0, j + 1) + warp; c < q1; c += warps)
            {
              double *fc = colp(c);
              double dot = 0.0;
              for (int64_t i = j + 1 + lane; i < len; i += 32) dot = fma(vst[i], fc[i], dot);
              dot = warp_sum(dot);
              const double w = tau * (fc[j] + dot);
              for (int64_t i = j + 1 + lane; i < len; i += 32) fc[i] = fma(-w, vst[i], fc[i]);
              if (lane == 0) fc[j] -= w;
            }
          __syncthreads();
        }
        // R's part of this rank's columns to the global factored matrix
        if (qr_smem)
          for (int64_t c = q0; c < q1; ++c)
            for (int64_t i = threadIdx.x; i <= c && i < len; i += blockDim.x) qf[c * len + i] = colp(c)[i];
        cluster.sync();
      }
      // rows of the swept matrix, and its entries: the block (W orientation) or X = R^T
      const int64_t xl = precond ? k : len;
      const auto entry = [&](int64_t row, int64_t col) -> double
      { return precond ? (col <= row ? __ldcg(qf + row * len + col) : 0.0) : entry_a(row, col); };  // row < xl

      // 1. FP32 sweeps on the block scaled to |entries| <= 1, from V = I; V goes out in FP64.
      // Rank 0 alone when W and V fit in its shared memory, else rows dealt over the cluster.
      {
        const bool alone = ranks == 1 || (k < 32 && (xl * k + k * k) * 4 <= kDynamicBytes);
        const int64_t rows = alone ? xl : (xl + ranks - 1) / ranks, vrows = alone ? k : (k + ranks - 1) / ranks;
        const int64_t r0 = alone ? 0 : min(xl, static_cast<int64_t>(rank) * rows), r1 = alone ? xl : min(xl, r0 + rows);
        const int64_t c0 = alone ? 0 : min(k, static_cast<int64_t>(rank) * vrows), c1 = alone ? k : min(k, c0 + vrows);
        const int64_t swap32 = exchange_bytes(k, alone ? 1 : ranks, 4);
        const bool in_smem = (rows + vrows) * k * 4 + swap32 <= kDynamicBytes;
        float *w32 = in_smem ? reinterpret_cast<float *>(dynamic)
                             : reinterpret_cast<float *>(ws + lay.w32_slices) + static_cast<int64_t>(rank) * rows * k;
        float *v32 = in_smem ? w32 + rows * k : reinterpret_cast<float *>(ws + lay.v32_slices) + static_cast<int64_t>(rank) * vrows * k;
        if (alone ? rank == 0 : true)
        {
          // the largest |entry| of the block (of this rank's rows, then over the cluster)
          if (threadIdx.x == 0) big = 0.0;
          __syncthreads();
          double local = 0.0;
          for (int64_t i = threadIdx.x; i < (r1 - r0) * k; i += blockDim.x)
            local = fmax(local, fabs(entry(r0 + i % (r1 - r0), i / (r1 - r0))));
#pragma unroll
          for (int o = 16; o > 0; o >>= 1) local = fmax(local, __shfl_xor_sync(0xffffffffu, local, o));
          if ((threadIdx.x & 31) == 0) atomicMax(reinterpret_cast<unsigned long long *>(&big), __double_as_longlong(local));
          __syncthreads();
        }
        if (!alone)
        {
          if (threadIdx.x == 0) partial_raw[0] = big;
          cluster.sync();
          if (threadIdx.x == 0)
          {
            double most = 0.0;
            for (unsigned r = 0; r < ranks; ++r) most = fmax(most, cluster.map_shared_rank(partial_raw, r)[0]);
            big = most;
          }
          __syncthreads();
        }
        if (alone ? rank == 0 : true)
        {
          const double scale = big > 0.0 ? 1.0 / big : 1.0;
          for (int64_t i = threadIdx.x; i < rows * k; i += blockDim.x)
          {
            const int64_t row = r0 + i % rows;
            w32[i] = row < r1 ? static_cast<float>(entry(row, i / rows) * scale) : 0.0f;
          }
          for (int64_t i = threadIdx.x; i < vrows * k; i += blockDim.x)
            v32[i] = (c0 + i % vrows == i / vrows && c0 + i % vrows < c1) ? 1.0f : 0.0f;
          __syncthreads();
        }
        if (!alone) cluster.sync();  // every rank's partial_raw read before it holds norms
        if (alone ? rank == 0 : true)
        {
          sweeps<float>(cluster, alone, w32, rows, v32, vrows, k, 1e-5, reinterpret_cast<float *>(norms_raw),
                        reinterpret_cast<float *>(dynamic + kDynamicBytes - swap32), reinterpret_cast<float *>(partial_raw),
                        flags, rank_of);
          for (int64_t i = threadIdx.x; i < vrows * k; i += blockDim.x)
          {
            const int64_t row = c0 + i % vrows;
            if (row < c1) v_cur[(i / vrows) * k + row] = static_cast<double>(v32[i]);
          }
        }
      }
      cluster.sync();

      // 2. V orthonormal to FP64 precision by two Newton-Schulz steps V <- V + V (I - V^T V) / 2:
      // G = V^T V in FP64 (the tiles on and above the diagonal), the correction V E, E = I - G of
      // size ~1e-6 and then ~1e-12, in FP32 accumulation (its rounding, ~1e-7 of E, is below FP64
      // precision of V after the second step).  Tiles are dealt to the ranks; V and G pass between
      // the CTAs through the workspace, read past L1 (__ldcg) so that no CTA sees an earlier value.
      const int64_t nt = (k + kTile - 1) / kTile;
      for (int step = 0; step < 2; ++step)
      {
        for (int64_t tile = rank; tile < nt * nt; tile += ranks)
        {
          const int64_t tr = tile % nt, tc = tile / nt;
          if (tr > tc) continue;
          const double *vc = v_cur;
          tile_product<double>(
            k, [&](int64_t x, int i) { return tr * kTile + i < k ? __ldcg(vc + (tr * kTile + i) * k + x) : 0.0; }, true,
            [&](int64_t x, int j) { return tc * kTile + j < k ? __ldcg(vc + (tc * kTile + j) * k + x) : 0.0; }, true,
            stage, stage + kTile * (kTile + 1),
            [&](int i, int j, double sum) {
              const int64_t r = tr * kTile + i, c = tc * kTile + j;
              if (r < k && c < k)
              {
                g[c * k + r] = sum;
                g[r * k + c] = sum;
              }
            });
        }
        cluster.sync();
        for (int64_t tile = rank; tile < nt * nt; tile += ranks)
        {
          const int64_t tr = tile % nt, tc = tile / nt;  // rows tr, columns tc of V'
          const double *vc = v_cur, *gc = g;
          float *sa = reinterpret_cast<float *>(stage), *sb = sa + kTile * (kTile + 1);
          tile_product<float>(
            k, [&](int64_t x, int i) { return tr * kTile + i < k ? static_cast<float>(__ldcg(vc + x * k + tr * kTile + i)) : 0.0f; },
            false,
            [&](int64_t x, int j) {
              const int64_t c = tc * kTile + j;
              return c < k ? static_cast<float>((x == c ? 1.0 : 0.0) - __ldcg(gc + c * k + x)) : 0.0f;
            },
            true, sa, sb,
            [&](int i, int j, float sum) {
              const int64_t row = tr * kTile + i, c = tc * kTile + j;
              if (row < k && c < k) v_next[c * k + row] = fma(0.5, static_cast<double>(sum), __ldcg(vc + c * k + row));
            });
        }
        cluster.sync();
        double *t = v_cur;
        v_cur = v_next;
        v_next = t;
      }

      // 3. this rank's rows of W = A V (FP64) and of V.  FP64 sweeps over the cluster for 32
      // columns or more, on rank 0 alone below that.
      const bool alone = ranks == 1 || k < 32;
      const int64_t rows = alone ? (rank == 0 ? xl : 0) : (xl + ranks - 1) / ranks;
      const int64_t vrows = alone ? (rank == 0 ? k : 0) : (k + ranks - 1) / ranks;
      const int64_t r0 = alone ? 0 : min(xl, static_cast<int64_t>(rank) * rows), r1 = min(xl, r0 + rows);
      const int64_t c0 = alone ? 0 : min(k, static_cast<int64_t>(rank) * vrows), c1 = min(k, c0 + vrows);
      const int64_t swap64 = exchange_bytes(k, alone ? 1 : ranks, 8);
      const bool slices_in_smem = (rows + vrows) * k * 8 + (swap64 > kStageBytes ? swap64 : kStageBytes) <= kDynamicBytes;
      double *w = slices_in_smem ? reinterpret_cast<double *>(dynamic) : ws + lay.w_slices + static_cast<int64_t>(rank) * rows * k;
      double *v = slices_in_smem ? w + rows * k : ws + lay.v_slices + static_cast<int64_t>(rank) * vrows * k;
      {
        const double *vc = v_cur;
        const int64_t nr = (rows + kTile - 1) / kTile;
        for (int64_t tile = 0; tile < nr * nt; ++tile)
        {
          const int64_t tr = tile % nr, tc = tile / nr;
          tile_product<double>(
            k, [&](int64_t x, int i) { const int64_t row = r0 + tr * kTile + i; return row < r1 ? entry(row, x) : 0.0; }, precond || !wide,
            [&](int64_t x, int j) { return tc * kTile + j < k ? __ldcg(vc + (tc * kTile + j) * k + x) : 0.0; }, true,
            stage, stage + kTile * (kTile + 1),
            [&](int i, int j, double sum) {
              const int64_t row = tr * kTile + i, c = tc * kTile + j;
              if (row < rows && c < k) w[c * rows + row] = r0 + row < r1 ? sum : 0.0;
            });
        }
        for (int64_t i = threadIdx.x; i < vrows * k; i += blockDim.x)
        {
          const int64_t row = c0 + i % vrows, j = i / vrows;
          v[i] = row < c1 ? __ldcg(vc + j * k + row) : 0.0;
        }
        __syncthreads();
      }

      // 4. FP64 sweeps
      const double tol = 2.220446049250313e-16 * sqrt(static_cast<double>(xl));
      int sweeps_taken = 0;
      if (!alone || rank == 0)
        sweeps_taken = sweeps<double>(cluster, alone, w, rows, v, vrows, k, tol, norms_raw,
                                      reinterpret_cast<double *>(dynamic + kDynamicBytes - swap64), partial_raw, flags, rank_of);

      // singular values (column norms over the cluster), their ranks, and this rank's rows of the
      // factors in descending order
      double *norms = norms_raw, *partial = partial_raw;
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
      double *uo = u + e.u_off, *vo = vh + e.vh_off;
      if (!precond)
      {
        // tall: U = W / sigma (m x k), Vh = V^T; wide: U = V (m x m), Vh = (W / sigma)^T
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
      }
      else
      {
        // the right factor P (W / sigma): row `row` of W is row order[row] of it (tall: Vh is its
        // transpose; wide: U is it)
        for (int64_t i = threadIdx.x; i < rows * k; i += blockDim.x)
        {
          const int64_t j = i / rows, row = r0 + i % rows;
          if (row >= r1) continue;
          const double sj = norms[j];
          const double x = sj > 0 ? w[i] / sj : 0.0;
          const int64_t to = __ldcg(qorder + row);
          if (wide)
            uo[to * k + rank_of[j]] = x;
          else
            vo[static_cast<int64_t>(rank_of[j]) * n + to] = x;
        }
        // the left factor Q [J; 0], J = V: V's rows to the workspace (column-major), then each rank
        // applies the reflectors, the last first, to its columns [q0, q1), a warp per column (tall:
        // U is it; wide: Vh is its transpose)
        for (int64_t i = threadIdx.x; i < vrows * k; i += blockDim.x)
        {
          const int64_t j = i / vrows, row = c0 + i % vrows;
          if (row < c1) g[j * k + row] = v[i];
        }
        cluster.sync();
        // the reflectors pass through shared memory in batches, and this rank's columns of B stay
        // there while they are transformed, when both fit (W and V there are no longer read)
        constexpr int64_t kBatch = 16;
        if (((cpr + kBatch) * len + kBatch) * 8 <= kDynamicBytes)
        {
          double *bcols = reinterpret_cast<double *>(dynamic), *stage = bcols + cpr * len, *stau = stage + kBatch * len;
          for (int64_t i = threadIdx.x; i < (q1 - q0) * len; i += blockDim.x)
          {
            const int64_t c = q0 + i / len, r = i % len;
            bcols[i] = r < k ? __ldcg(g + c * k + r) : 0.0;
          }
          for (int64_t top = k - 1; top >= 0; top -= kBatch)
          {
            const int64_t low = max(top - kBatch + 1, static_cast<int64_t>(0));  // reflectors top down to low
            __syncthreads();
            for (int64_t i = threadIdx.x; i < (top - low + 1) * len; i += blockDim.x)
            {
              const int64_t t = top - i / len, r = i % len;
              stage[i] = r > t ? __ldcg(qf + t * len + r) : 0.0;
            }
            if (threadIdx.x < top - low + 1) stau[threadIdx.x] = __ldcg(qtau + top - threadIdx.x);
            __syncthreads();
            for (int64_t c = q0 + warp; c < q1; c += warps)
            {
              double *bc = bcols + (c - q0) * len;
              for (int64_t t = top; t >= low; --t)
              {
                const double tau = stau[top - t];
                if (tau == 0.0) continue;
                const double *vt = stage + (top - t) * len;
                double dot = 0.0;
                for (int64_t i = t + 1 + lane; i < len; i += 32) dot = fma(vt[i], bc[i], dot);
                dot = warp_sum(dot);
                const double wt = tau * (bc[t] + dot);
                for (int64_t i = t + 1 + lane; i < len; i += 32) bc[i] = fma(-wt, vt[i], bc[i]);
                __syncwarp();
                if (lane == 0) bc[t] -= wt;
                __syncwarp();
              }
            }
          }
          __syncthreads();
          for (int64_t i = threadIdx.x; i < (q1 - q0) * len; i += blockDim.x)
          {
            const int64_t c = q0 + i / len, r = i % len;
            const int64_t to = rank_of[c];
            if (wide)
              vo[to * n + r] = bcols[i];
            else
              uo[r * k + to] = bcols[i];
          }
        }
        else
        {
          for (int64_t c = q0 + warp; c < q1; c += warps)
          {
            double *bc = qb + c * len;
            for (int64_t i = lane; i < len; i += 32) bc[i] = i < k ? __ldcg(g + c * k + i) : 0.0;
            __syncwarp();
            for (int64_t t = k - 1; t >= 0; --t)
            {
              const double tau = __ldcg(qtau + t);
              if (tau == 0.0) continue;
              const double *vt = qf + t * len;
              double dot = 0.0;
              for (int64_t i = t + 1 + lane; i < len; i += 32) dot = fma(__ldcg(vt + i), bc[i], dot);
              dot = warp_sum(dot);
              const double wt = tau * (bc[t] + dot);
              for (int64_t i = t + 1 + lane; i < len; i += 32) bc[i] = fma(-wt, __ldcg(vt + i), bc[i]);
              __syncwarp();
              if (lane == 0) bc[t] -= wt;
              __syncwarp();
            }
            const int64_t to = rank_of[c];
            for (int64_t i = lane; i < len; i += 32)
            {
              if (wide)
                vo[to * n + i] = bc[i];
              else
                uo[i * k + to] = bc[i];
            }
          }
        }
      }
      if (threadIdx.x == 0 && rank == 0) info[block] = sweeps_taken;
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

  cudaError_t svd_blocks(int32_t count, int64_t largest, const void *table, const double *a, double *u, double *s,
                         double *vh, void *workspace, int32_t *info, cudaStream_t stream)
  {
    if (count <= 0) return cudaSuccess;
    static std::once_flag once;
    static cudaError_t configured = cudaSuccess;
    static int cluster_for[kMaxCluster + 1] = {};  // clusters of each size that fit on the GPU at once
    std::call_once(once, [] {
      configured = cudaFuncSetAttribute(jacobi_svd_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        static_cast<int>(kDynamicBytes));
      if (configured == cudaSuccess)
        configured = cudaFuncSetAttribute(jacobi_svd_kernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
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
    // the cluster the largest block wants (16 CTAs from 128 columns, 8 from 32, below that the
    // sweeps run on one CTA), or the largest the GPU can hold; blocks come largest first, so a
    // second wave of clusters only holds small blocks
    const int want = largest >= 128 ? 16 : largest >= 32 ? 8 : 1;
    int size = 1;
    for (int c = want; c > 1; c /= 2)
      if (cluster_for[c] >= 1)
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

// ------------------------------------------------------------------------------------------
// the ranking of a split's singular values on the device
// ------------------------------------------------------------------------------------------

namespace ttg
{
  namespace
  {
    // Every singular value of a split (block after block, each block's in descending order) sorted
    // by (value descending, position ascending) — the order of the host's stable sort — by a bitonic
    // sort in shared memory; then one thread walks the sorted values: the cut (values above `tol`,
    // at most `max_bond`), the values each block keeps, and the +-q pairing of the bond (a domain
    // sector keeps at most as many as its dual, the first ones in the sorted order; a sector whose
    // dual keeps nothing drops out), as tentorch/linalg/graded/svd.cpp:68-118 ranks them on the host.
    __global__ void rank_kernel(const double *__restrict__ values, int32_t n_values, const int32_t *__restrict__ block_k,
                                const int32_t *__restrict__ block_sector, int32_t n_blocks, const int32_t *__restrict__ dual,
                                int32_t n_sectors, double tol, int64_t max_bond, int32_t *__restrict__ kept_out)
    {
      extern __shared__ __align__(16) unsigned char smem_raw[];
      int n = 1;
      while (n < n_values) n <<= 1;
      unsigned long long *key = reinterpret_cast<unsigned long long *>(smem_raw);  // [n]
      int32_t *pos = reinterpret_cast<int32_t *>(key + n);                          // [n]
      int32_t *block_of = pos + n;                                                  // [n_values]
      int32_t *kept = block_of + n_values;                                          // [n_blocks]
      int32_t *mult = kept + n_blocks;                                              // [n_sectors] x 3
      int32_t *paired = mult + n_sectors, *used = paired + n_sectors;
      // keys: the complement of |value|'s bits (ascending keys = descending values); padding last
      for (int i = threadIdx.x; i < n; i += blockDim.x)
      {
        if (i < n_values)
        {
          key[i] = ~(static_cast<unsigned long long>(__double_as_longlong(values[i])) & 0x7fffffffffffffffull);
          pos[i] = i;
        }
        else
        {
          key[i] = ~0ull;
          pos[i] = 0x7fffffff;
        }
      }
      if (threadIdx.x == 0)
      {
        int32_t at = 0;
        for (int32_t b = 0; b < n_blocks; ++b)
        {
          for (int32_t j = 0; j < block_k[b]; ++j) block_of[at + j] = b;
          at += block_k[b];
        }
      }
      __syncthreads();
      for (int size = 2; size <= n; size <<= 1)
        for (int stride = size >> 1; stride > 0; stride >>= 1)
        {
          for (int i = threadIdx.x; i < n; i += blockDim.x)
          {
            const int j = i ^ stride;
            if (j > i)
            {
              const bool ascending = (i & size) == 0;
              const bool greater = key[i] > key[j] || (key[i] == key[j] && pos[i] > pos[j]);
              if (greater == ascending)
              {
                const unsigned long long tk = key[i];
                key[i] = key[j];
                key[j] = tk;
                const int32_t tp = pos[i];
                pos[i] = pos[j];
                pos[j] = tp;
              }
            }
          }
          __syncthreads();
        }
      if (threadIdx.x != 0) return;
      int32_t cut = 0;
      while (cut < n_values && values[pos[cut]] > tol) ++cut;
      if (max_bond >= 0 && cut > max_bond) cut = static_cast<int32_t>(max_bond);
      for (int32_t b = 0; b < n_blocks; ++b) kept[b] = 0;
      for (int32_t s = 0; s < n_sectors; ++s) mult[s] = used[s] = 0;
      for (int32_t r = 0; r < cut; ++r) ++kept[block_of[pos[r]]];
      for (int32_t b = 0; b < n_blocks; ++b) mult[block_sector[b]] += kept[b];
      bool any = false, differs = false;
      for (int32_t s = 0; s < n_sectors; ++s)
      {
        paired[s] = -1;
        if (mult[s] == 0) continue;
        if (mult[dual[s]] > 0)
        {
          paired[s] = min(mult[s], mult[dual[s]]);
          any = true;
          if (paired[s] != mult[s]) differs = true;
        }
        else
          differs = true;
      }
      if (any && differs)
      {
        for (int32_t b = 0; b < n_blocks; ++b) kept[b] = 0;
        for (int32_t r = 0; r < cut; ++r)
        {
          const int32_t b = block_of[pos[r]], s = block_sector[b];
          if (paired[s] < 0 || used[s] >= paired[s]) continue;
          ++used[s];
          ++kept[b];
        }
      }
      for (int32_t b = 0; b < n_blocks; ++b) kept_out[b] = kept[b];
    }
  } // namespace

  int64_t rank_bytes(int32_t n_values, int32_t n_blocks, int32_t n_sectors)
  {
    int64_t n = 1;
    while (n < n_values) n <<= 1;
    return n * 12 + static_cast<int64_t>(n_values) * 4 + static_cast<int64_t>(n_blocks) * 4 + static_cast<int64_t>(n_sectors) * 12;
  }

  cudaError_t svd_rank(const double *values, int32_t n_values, const int32_t *block_k, const int32_t *block_sector,
                       int32_t n_blocks, const int32_t *dual, int32_t n_sectors, double tol, int64_t max_bond, int32_t *kept,
                       cudaStream_t stream)
  {
    const int64_t bytes = rank_bytes(n_values, n_blocks, n_sectors);
    cudaError_t e = cudaFuncSetAttribute(rank_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(bytes));
    if (e != cudaSuccess) return e;
    rank_kernel<<<1, 1024, bytes, stream>>>(values, n_values, block_k, block_sector, n_blocks, dual, n_sectors, tol, max_bond,
                                            kept);
    return cudaGetLastError();
  }
} // namespace ttg
