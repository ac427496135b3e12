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

namespace ttg
{
  namespace
  {
    // table[j] = basis + j * n_doubles for j < count, then the image, the start vector and the result
    __global__ void rows_kernel(const double **table, const double *basis, int64_t n_doubles, int32_t count,
                                const double *image, const double *start, const double *result)
    {
      const int32_t j = blockIdx.x * blockDim.x + threadIdx.x;
      if (j < count) table[j] = basis + j * n_doubles;
      if (j == count) table[j] = image;
      if (j == count + 1) table[j] = start;
      if (j == count + 2) table[j] = result;
    }

    // dst = src / sqrt(norm2[0]) (norm2 the real part of <src, src>); beta_out (optional) = sqrt
    __global__ void scale_kernel(double *dst, const double *src, int64_t n_doubles, const double *norm2, double *beta_out)
    {
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

    __global__ void save_kernel(double *dst, const double *src) { *dst = *src; }

    // out = sum_j c_j basis_j with real c_j, j < *count
    __global__ void combine_kernel(double *out, const double *basis, int64_t n_doubles, const int32_t *count, const double *c)
    {
      const int32_t used = *count;
      for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n_doubles;
           i += static_cast<int64_t>(gridDim.x) * blockDim.x)
      {
        double v = 0.0;
        for (int32_t j = 0; j < used; ++j) v = fma(c[j], basis[j * n_doubles + i], v);
        out[i] = v;
      }
    }

    // The Krylov space's lowest Ritz pair on the device, one warp: the size of the space (the steps
    // before the first beta below `tol`, as the reference stops), the tridiagonal's eigenpairs by
    // cyclic Jacobi rotations (C. G. J. Jacobi, 1846; the rotation as in Golub & Van Loan, "Matrix
    // Computations", the symmetric Schur decomposition; each rotation's parameters by one lane, its
    // row and column updates over the lanes), the lowest eigenvalue and its eigenvector.  Products
    // and sums are rounded one by one (no fused multiply-add), as the host arithmetic of x86 does.
    __global__ void ritz_kernel(const double *tri, int32_t n_iter, double tol, double *ritz, double *energy,
                                int32_t *size_out)
    {
      extern __shared__ double work[];
      __shared__ double rot[2];
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
      double *a = work, *v = work + n * n;
      for (int i = lane; i < n * n; i += 32)
      {
        const int r = i / n, c = i % n;
        a[i] = r == c ? tri[r] : (c == r + 1 ? tri[n_iter + r] : (r == c + 1 ? tri[n_iter + c] : 0.0));
        v[i] = r == c ? 1.0 : 0.0;
      }
      __syncwarp();
      for (int sweep = 0; sweep < 100; ++sweep)
      {
        if (lane == 0)
        {
          double off = 0.0;
          for (int p = 0; p < n; ++p)
            for (int q = p + 1; q < n; ++q) off = __dadd_rn(off, __dmul_rn(a[p * n + q], a[p * n + q]));
          rot[0] = off;
        }
        __syncwarp();
        if (rot[0] == 0.0) break;
        for (int p = 0; p < n; ++p)
          for (int q = p + 1; q < n; ++q)
          {
            const double apq = a[p * n + q];
            __syncwarp();
            if (apq == 0.0) continue;
            if (lane == 0)
            {
              const double app = a[p * n + p], aqq = a[q * n + q];
              const double tau = __ddiv_rn(__dsub_rn(aqq, app), __dmul_rn(2.0, apq));
              const double t = __ddiv_rn(tau >= 0 ? 1.0 : -1.0, __dadd_rn(fabs(tau), __dsqrt_rn(__dadd_rn(1.0, __dmul_rn(tau, tau)))));
              const double c = __ddiv_rn(1.0, __dsqrt_rn(__dadd_rn(1.0, __dmul_rn(t, t))));
              rot[0] = c;
              rot[1] = __dmul_rn(t, c);
            }
            __syncwarp();
            const double c = rot[0], s = rot[1];
            for (int k = lane; k < n; k += 32)
            {
              const double akp = a[k * n + p], akq = a[k * n + q];
              a[k * n + p] = __dsub_rn(__dmul_rn(c, akp), __dmul_rn(s, akq));
              a[k * n + q] = __dadd_rn(__dmul_rn(s, akp), __dmul_rn(c, akq));
            }
            __syncwarp();
            for (int k = lane; k < n; k += 32)
            {
              const double apk = a[p * n + k], aqk = a[q * n + k];
              a[p * n + k] = __dsub_rn(__dmul_rn(c, apk), __dmul_rn(s, aqk));
              a[q * n + k] = __dadd_rn(__dmul_rn(s, apk), __dmul_rn(c, aqk));
            }
            for (int k = lane; k < n; k += 32)
            {
              const double vkp = v[k * n + p], vkq = v[k * n + q];
              v[k * n + p] = __dsub_rn(__dmul_rn(c, vkp), __dmul_rn(s, vkq));
              v[k * n + q] = __dadd_rn(__dmul_rn(s, vkp), __dmul_rn(c, vkq));
            }
            __syncwarp();
          }
      }
      if (lane == 0)
      {
        int lowest = 0;
        for (int k = 1; k < n; ++k)
          if (a[k * n + k] < a[lowest * n + lowest]) lowest = k;
        *energy = a[lowest * n + lowest];
        *size_out = n;
        shared_size = lowest;
      }
      __syncwarp();
      for (int k = lane; k < n; k += 32) ritz[k] = v[k * n + shared_size];
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
    rows_kernel<<<1, 128, 0, stream>>>(table, basis, n_doubles, static_cast<int32_t>(rows), image, start, result);
    // basis[0] = start / |start|
    if ((e = arena_dots(start_slot, 1, start, n_doubles, complex, partial, coeffs, stream)) != cudaSuccess) return e;
    scale_kernel<<<grid, 256, 0, stream>>>(basis, start, n_doubles, coeffs, nullptr);
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
        if (pass == 0) save_kernel<<<1, 1, 0, stream>>>(tri + k, coeffs + 2 * k);
        if (complex)
          project_kernel<true><<<grid, 256, 0, stream>>>(image, basis, n_doubles, k + 1, coeffs);
        else
          project_kernel<false><<<grid, 256, 0, stream>>>(image, basis, n_doubles, k + 1, coeffs);
      }
      if ((e = arena_dots(image_slot, 1, image, n_doubles, complex, partial, coeffs, stream)) != cudaSuccess) return e;
      scale_kernel<<<grid, 256, 0, stream>>>(row + n_doubles, image, n_doubles, coeffs, tri + n_iter + k);
      if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    // the lowest Ritz pair of the tridiagonal (the steps after the first beta below tol dropped, as
    // the reference stops there), then the normalised Ritz vector; complex arenas take the real
    // coefficients on both parts alike
    const int smem = static_cast<int>(2 * n_iter * n_iter * sizeof(double));
    if (smem > 48 * 1024 && (e = cudaFuncSetAttribute(ritz_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem)) != cudaSuccess)
      return e;
    ritz_kernel<<<1, 32, smem, stream>>>(tri, n_iter, tol, ritz, energy_dev, size_dev);
    combine_kernel<<<grid, 256, 0, stream>>>(result, basis, n_doubles, size_dev, ritz);
    if ((e = arena_dots(result_slot, 1, result, n_doubles, complex, partial, coeffs, stream)) != cudaSuccess) return e;
    scale_kernel<<<grid, 256, 0, stream>>>(result, result, n_doubles, coeffs, nullptr);
    return cudaGetLastError();
  }

  double *lanczos_energy_slot(double *scratch, int64_t n_doubles, int32_t n_iter)
  {
    const int64_t rows = n_iter + 1;
    return scratch + up32(rows * n_doubles) + up32(n_doubles) + up32(2 * kDotParts * rows) + up32(2 * rows) +
           up32(2 * rows) + rows;
  }

} // namespace ttg
