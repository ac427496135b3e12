// The Lanczos eigensolver of a DMRG window (tentorch/linalg/lanczos.py:8-64) as one host loop over
// device work: every Krylov step executes the window's compiled einsum on the current basis vector,
// projects the image against the whole basis three times (the first projection holds alpha and
// replaces the three-term step; then the reference's two full reorthogonalisation passes), takes
// its norm and scales it into the next basis vector, with no host synchronisation.  The device
// then applies the reference's early stop (a beta below `tol` ends the space), solves the small
// eigenproblem and forms the normalised Ritz vector: the whole call is stream-ordered work with no
// host wait, and its energy and Krylov size stay in device memory until the caller reads them.
//
// Per step that is the plan's launches plus ten small ones issued from C++, so the CPU stays ahead
// of the GPU; the same loop driven from Python spends more time launching than the GPU computing.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <vector>

#include "executor.h"
#include "launch.h"

namespace ttg
{
  namespace
  {
    // table[j] = basis + j * n_doubles for j < count, then the image, the start vector and the result
    __global__ void rows_kernel(const double **table, const double *basis, int64_t n_doubles, int32_t count,
                                const double *image, const double *start, const double *result)
    {
      dependent_entry();
      const int32_t j = blockIdx.x * blockDim.x + threadIdx.x;
      if (j < count) table[j] = basis + j * n_doubles;
      if (j == count) table[j] = image;
      if (j == count + 1) table[j] = start;
      if (j == count + 2) table[j] = result;
    }

    // dst = src / sqrt(norm2[0]) (norm2 the real part of <src, src>); beta_out (optional) = sqrt
    __global__ void scale_kernel(double *dst, const double *src, int64_t n_doubles, const double *norm2, double *beta_out)
    {
      dependent_entry();
      const double norm = sqrt(fmax(norm2[0], 0.0));
      const double inv = 1.0 / fmax(norm, 1e-300);
      if (beta_out && blockIdx.x == 0 && threadIdx.x == 0) *beta_out = norm;
      for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n_doubles;
           i += static_cast<int64_t>(gridDim.x) * blockDim.x)
        dst[i] = src[i] * inv;
    }

    // y -= sum_j c_j basis_j (c_j = coeffs[2j] + i coeffs[2j+1] for complex arenas)
    template <bool Complex>
    __global__ void project_kernel(double *y, const double *basis, int64_t n_doubles, int32_t count,
                                   const double *coeffs)
    {
      dependent_entry();
      const int64_t step = static_cast<int64_t>(gridDim.x) * blockDim.x * (Complex ? 2 : 1);
      for (int64_t i = (blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x) * (Complex ? 2 : 1); i < n_doubles;
           i += step)
      {
        if (Complex)
        {
          double re = y[i], im = y[i + 1];
          for (int32_t j = 0; j < count; ++j)
          {
            const double br = basis[j * n_doubles + i], bi = basis[j * n_doubles + i + 1];
            const double cr = coeffs[2 * j], ci = coeffs[2 * j + 1];
            re -= cr * br - ci * bi;
            im -= cr * bi + ci * br;
          }
          y[i] = re;
          y[i + 1] = im;
        }
        else
        {
          double v = y[i];
          for (int32_t j = 0; j < count; ++j) v = fma(-coeffs[2 * j], basis[j * n_doubles + i], v);
          y[i] = v;
        }
      }
    }

    __global__ void save_kernel(double *dst, const double *src)
    {
      dependent_entry();
      *dst = *src;
    }

    // out = sum_j c_j basis_j with real c_j, j < *count
    __global__ void combine_kernel(double *out, const double *basis, int64_t n_doubles, const int32_t *count, const double *c)
    {
      dependent_entry();
      const int32_t used = *count;
      for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n_doubles;
           i += static_cast<int64_t>(gridDim.x) * blockDim.x)
      {
        double v = 0.0;
        for (int32_t j = 0; j < used; ++j) v = fma(c[j], basis[j * n_doubles + i], v);
        out[i] = v;
      }
    }

    // The number of eigenvalues of the symmetric tridiagonal (diagonal a, off-diagonal b) below x: the
    // negative pivots of the LDL^T factorisation of T - x I (Sturm's sequence); a zero pivot is taken
    // as a tiny negative one.
    __device__ int below(const double *a, const double *b, int n, double x, double pivmin)
    {
      int count = 0;
      double d = a[0] - x;
      for (int i = 0;; ++i)
      {
        if (fabs(d) < pivmin) d = -pivmin;
        if (d < 0.0) ++count;
        if (i + 1 == n) break;
        d = (a[i + 1] - x) - b[i] * b[i] / d;
      }
      return count;
    }

    // The Krylov space's lowest Ritz pair on the device, one warp: the size of the space (the steps
    // before the first beta below `tol`, as the reference stops), the tridiagonal's lowest eigenvalue
    // by multisection of its Sturm count (each round the 32 lanes count below 32 points of the
    // bracket, which shrinks it 33-fold, from Gershgorin's bounds down to a few units in the last
    // place) and its eigenvector by inverse iteration (Gaussian elimination with partial pivoting
    // of T - lambda I, three solves from a vector of ones, normalised; W. Kahan, "Accurate
    // eigenvalues of a symmetric tri-diagonal matrix", 1966, and J. H. Wilkinson, "The Algebraic
    // Eigenvalue Problem", 1965, for inverse iteration).
    __global__ void ritz_kernel(const double *tri, int32_t n_iter, double tol, double *ritz, double *energy,
                                int32_t *size_out)
    {
      dependent_entry();
      extern __shared__ double work[];
      __shared__ double bracket[2];
      __shared__ int32_t shared_size;
      const int lane = threadIdx.x;
      if (lane == 0)
      {
        int32_t size = n_iter;
        for (int32_t k = 0; k < n_iter; ++k)
          if (tri[n_iter + k] < tol)
          {
            size = k + 1;
            break;
          }
        shared_size = size;
      }
      __syncwarp();
      const int n = shared_size;
      double *a = work, *b = work + n, *v = work + 2 * n;
      for (int i = lane; i < n; i += 32)
      {
        a[i] = tri[i];
        b[i] = i + 1 < n ? tri[n_iter + i] : 0.0;
      }
      __syncwarp();
      if (lane == 0)
      {
        double lo = a[0], hi = a[0], scale = 0.0;
        for (int i = 0; i < n; ++i)
        {
          const double r = (i > 0 ? fabs(b[i - 1]) : 0.0) + (i + 1 < n ? fabs(b[i]) : 0.0);
          lo = fmin(lo, a[i] - r);
          hi = fmax(hi, a[i] + r);
          scale = fmax(scale, fabs(a[i]) + r);
        }
        bracket[0] = lo;
        bracket[1] = hi;
        work[3 * n] = fmax(scale, 1.0) * 1e-290;  // pivmin
      }
      __syncwarp();
      const double pivmin = work[3 * n];
      for (int round = 0; round < 64; ++round)
      {
        const double lo = bracket[0], hi = bracket[1];
        if (!(hi - lo > 4.0 * 2.220446049250313e-16 * fmax(fabs(lo), fabs(hi))) || !(hi > lo)) break;
        const double x = lo + (hi - lo) * static_cast<double>(lane + 1) / 33.0;
        const bool any = below(a, b, n, x, pivmin) >= 1;
        const unsigned hits = __ballot_sync(0xffffffffu, any);
        __syncwarp();
        if (lane == 0)
        {
          // the first point with an eigenvalue below it closes the bracket of the lowest one
          const int first = hits ? __ffs(hits) - 1 : 32;
          const double step = (hi - lo) / 33.0;
          bracket[0] = first == 0 ? lo : lo + step * first;
          bracket[1] = first == 32 ? hi : lo + step * (first + 1);
        }
        __syncwarp();
      }
      const double lambda = 0.5 * (bracket[0] + bracket[1]);
      if (lane == 0)
      {
        // inverse iteration: (T - lambda I) y = v by elimination with partial pivoting (the
        // tridiagonal's upper factor has two superdiagonals)
        double *d = work + 3 * n + 1, *du = d + n, *du2 = du + n, *dl = du2 + n;
        for (int i = 0; i < n; ++i) v[i] = 1.0;
        for (int it = 0; it < 3; ++it)
        {
          for (int i = 0; i < n; ++i)
          {
            d[i] = a[i] - lambda;
            du[i] = i + 1 < n ? b[i] : 0.0;
            du2[i] = 0.0;
            dl[i] = i + 1 < n ? b[i] : 0.0;
          }
          for (int i = 0; i + 1 < n; ++i)
          {
            if (fabs(d[i]) >= fabs(dl[i]))
            {
              const double piv = d[i] != 0.0 ? d[i] : pivmin;
              const double f = dl[i] / piv;
              d[i] = piv;
              d[i + 1] -= f * du[i];
              v[i + 1] -= f * v[i];
            }
            else
            {
              // swap rows i and i + 1
              const double f = d[i] / dl[i];
              d[i] = dl[i];
              const double t = d[i + 1];
              d[i + 1] = du[i] - f * t;
              du[i] = t;
              du2[i] = i + 2 < n ? du[i + 1] : 0.0;
              if (i + 2 < n) du[i + 1] = -f * du2[i];
              const double vt = v[i];
              v[i] = v[i + 1];
              v[i + 1] = vt - f * v[i + 1];
            }
          }
          if (d[n - 1] == 0.0) d[n - 1] = pivmin;
          for (int i = n - 1; i >= 0; --i)
          {
            double x = v[i];
            if (i + 1 < n) x -= du[i] * v[i + 1];
            if (i + 2 < n) x -= du2[i] * v[i + 2];
            v[i] = x / d[i];
          }
          // scaled by the largest component first (a shift at an eigenvalue makes the solve huge),
          // then normalised with that component positive
          int big = 0;
          for (int i = 1; i < n; ++i)
            if (fabs(v[i]) > fabs(v[big])) big = i;
          const double top = v[big];
          double norm2 = 0.0;
          for (int i = 0; i < n; ++i)
          {
            v[i] /= top;
            norm2 += v[i] * v[i];
          }
          const double inv = 1.0 / sqrt(norm2);
          for (int i = 0; i < n; ++i) v[i] *= inv;
        }
        *energy = lambda;
        *size_out = n;
      }
      __syncwarp();
      for (int k = lane; k < n; k += 32) ritz[k] = v[k];
    }

    int grid_of(int64_t n_doubles) { return static_cast<int>(std::clamp<int64_t>((n_doubles + 255) / 256, 1, device_sms() * 8)); }
  } // namespace

  namespace
  {
    int64_t up32(int64_t x) { return (x + 31) / 32 * 32; }
  }

  int64_t lanczos_scratch_doubles(int64_t n_doubles, int32_t n_iter)
  {
    const int64_t rows = n_iter + 1;
    // basis, image, dot partials, coefficients, alpha and beta, Ritz coefficients with the energy and
    // the size after them, pointer table
    return up32(rows * n_doubles) + up32(n_doubles) + up32(2 * kDotParts * rows) + up32(2 * rows) + up32(2 * rows) +
           up32(rows + 2) + up32(rows + 3);
  }

  cudaError_t lanczos(const Program &p, DeviceTables &t, const ExecArgs &base, int32_t vector_operand,
                      const double *start, int64_t n_doubles, int32_t n_iter, double tol, double *scratch,
                      double *result, double *energy_dev, int32_t *size_dev)
  {
    const bool complex = base.complex;
    const int64_t rows = n_iter + 1;
    double *basis = scratch;
    double *image = basis + up32(rows * n_doubles);
    double *partial = image + up32(n_doubles);
    double *coeffs = partial + up32(2 * kDotParts * rows);
    double *tri = coeffs + up32(2 * rows);  // alpha[0..n_iter), beta[n_iter..2 n_iter)
    double *ritz = tri + up32(2 * rows);
    const double **table = reinterpret_cast<const double **>(ritz + up32(rows + 2));
    // table[j] = basis row j (j < rows), then the image, the start vector and the result
    const double *const *image_slot = table + rows, *const *start_slot = table + rows + 1,
                        *const *result_slot = table + rows + 2;
    cudaStream_t stream = base.stream;
    const int grid = grid_of(n_doubles);
    cudaError_t e;
    if ((e = launch_dependent(rows_kernel, 1, 128, 0, stream, table, basis, n_doubles, static_cast<int32_t>(rows), image, start,
                              result)) != cudaSuccess)
      return e;
    // basis[0] = start / |start|
    if ((e = arena_dots(start_slot, 1, start, n_doubles, complex, partial, coeffs, stream)) != cudaSuccess) return e;
    if ((e = launch_dependent(scale_kernel, grid, 256, 0, stream, basis, start, n_doubles, static_cast<const double *>(coeffs),
                              static_cast<double *>(nullptr))) != cudaSuccess)
      return e;
    std::vector<const void *> inputs(base.inputs, base.inputs + p.n_inputs);
    for (int32_t k = 0; k < n_iter; ++k)
    {
      double *row = basis + static_cast<int64_t>(k) * n_doubles;
      ExecArgs args = base;
      inputs[static_cast<size_t>(vector_operand)] = row;
      args.inputs = inputs.data();
      args.output = image;
      if ((e = execute(p, t, args)) != cudaSuccess) return e;
      for (int pass = 0; pass < 3; ++pass)
      {
        if ((e = arena_dots(table, k + 1, image, n_doubles, complex, partial, coeffs, stream)) != cudaSuccess) return e;
        if (pass == 0 && (e = launch_dependent(save_kernel, 1, 1, 0, stream, tri + k, static_cast<const double *>(coeffs + 2 * k))) != cudaSuccess)
          return e;
        if (complex)
          e = launch_dependent(project_kernel<true>, grid, 256, 0, stream, image, static_cast<const double *>(basis), n_doubles, k + 1,
                               static_cast<const double *>(coeffs));
        else
          e = launch_dependent(project_kernel<false>, grid, 256, 0, stream, image, static_cast<const double *>(basis), n_doubles, k + 1,
                               static_cast<const double *>(coeffs));
        if (e != cudaSuccess) return e;
      }
      if ((e = arena_dots(image_slot, 1, image, n_doubles, complex, partial, coeffs, stream)) != cudaSuccess) return e;
      if ((e = launch_dependent(scale_kernel, grid, 256, 0, stream, row + n_doubles, static_cast<const double *>(image), n_doubles,
                                static_cast<const double *>(coeffs), tri + n_iter + k)) != cudaSuccess)
        return e;
      if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    // the lowest Ritz pair of the tridiagonal (the steps after the first beta below tol dropped, as
    // the reference stops there), then the normalised Ritz vector; complex arenas take the real
    // coefficients on both parts alike
    const int smem = static_cast<int>((7 * n_iter + 1) * sizeof(double));
    if (smem > 48 * 1024 && (e = cudaFuncSetAttribute(ritz_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem)) != cudaSuccess)
      return e;
    if ((e = launch_dependent(ritz_kernel, 1, 32, smem, stream, static_cast<const double *>(tri), n_iter, tol, ritz, energy_dev,
                              size_dev)) != cudaSuccess)
      return e;
    if ((e = launch_dependent(combine_kernel, grid, 256, 0, stream, result, static_cast<const double *>(basis), n_doubles,
                              static_cast<const int32_t *>(size_dev), static_cast<const double *>(ritz))) != cudaSuccess)
      return e;
    if ((e = arena_dots(result_slot, 1, result, n_doubles, complex, partial, coeffs, stream)) != cudaSuccess) return e;
    if ((e = launch_dependent(scale_kernel, grid, 256, 0, stream, result, static_cast<const double *>(result), n_doubles,
                              static_cast<const double *>(coeffs), static_cast<double *>(nullptr))) != cudaSuccess)
      return e;
    return cudaGetLastError();
  }

  double *lanczos_energy_slot(double *scratch, int64_t n_doubles, int32_t n_iter)
  {
    const int64_t rows = n_iter + 1;
    return scratch + up32(rows * n_doubles) + up32(n_doubles) + up32(2 * kDotParts * rows) + up32(2 * rows) +
           up32(2 * rows) + rows;
  }

} // namespace ttg
