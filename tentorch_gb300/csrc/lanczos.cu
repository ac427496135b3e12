// The Lanczos eigensolver of a DMRG window (tentorch/linalg/lanczos.py:8-64) as one host loop over
// device work: every Krylov step executes the window's compiled einsum on the current basis vector,
// projects the image against the whole basis three times (the first projection holds alpha and
// replaces the three-term step; then the reference's two full reorthogonalisation passes), takes
// its norm and scales it into the next basis vector, with no host synchronisation.  The host reads
// the tridiagonal once at the end, applies the reference's early stop (a beta below `tol` ends the
// space), solves the small eigenproblem and the device forms the normalised Ritz vector.
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
    // table[j] = basis + j * n_doubles
    __global__ void rows_kernel(const double **table, const double *basis, int64_t n_doubles, int32_t count)
    {
      const int32_t j = blockIdx.x * blockDim.x + threadIdx.x;
      if (j < count) table[j] = basis + j * n_doubles;
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

    // out = sum_j c_j basis_j with real c_j
    __global__ void combine_kernel(double *out, const double *basis, int64_t n_doubles, int32_t count, const double *c)
    {
      for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n_doubles;
           i += static_cast<int64_t>(gridDim.x) * blockDim.x)
      {
        double v = 0.0;
        for (int32_t j = 0; j < count; ++j) v = fma(c[j], basis[j * n_doubles + i], v);
        out[i] = v;
      }
    }

    int grid_of(int64_t n_doubles) { return static_cast<int>(std::clamp<int64_t>((n_doubles + 255) / 256, 1, device_sms() * 8)); }

    // Eigenpairs of a small symmetric matrix by cyclic Jacobi rotations (C. G. J. Jacobi, 1846; the
    // rotation as in Golub & Van Loan, "Matrix Computations", the symmetric Schur decomposition):
    // `a` (n x n, row-major) is overwritten, `v` receives the eigenvectors as columns.
    void jacobi_eigen(std::vector<double> &a, std::vector<double> &v, int n)
    {
      v.assign(static_cast<size_t>(n) * n, 0.0);
      for (int i = 0; i < n; ++i) v[static_cast<size_t>(i) * n + i] = 1.0;
      for (int sweep = 0; sweep < 100; ++sweep)
      {
        double off = 0.0;
        for (int p = 0; p < n; ++p)
          for (int q = p + 1; q < n; ++q) off += a[static_cast<size_t>(p) * n + q] * a[static_cast<size_t>(p) * n + q];
        if (off == 0.0) break;
        for (int p = 0; p < n; ++p)
          for (int q = p + 1; q < n; ++q)
          {
            const double apq = a[static_cast<size_t>(p) * n + q];
            if (apq == 0.0) continue;
            const double app = a[static_cast<size_t>(p) * n + p], aqq = a[static_cast<size_t>(q) * n + q];
            const double tau = (aqq - app) / (2.0 * apq);
            const double t = (tau >= 0 ? 1.0 : -1.0) / (std::fabs(tau) + std::sqrt(1.0 + tau * tau));
            const double c = 1.0 / std::sqrt(1.0 + t * t), s = t * c;
            for (int k = 0; k < n; ++k)
            {
              const double akp = a[static_cast<size_t>(k) * n + p], akq = a[static_cast<size_t>(k) * n + q];
              a[static_cast<size_t>(k) * n + p] = c * akp - s * akq;
              a[static_cast<size_t>(k) * n + q] = s * akp + c * akq;
            }
            for (int k = 0; k < n; ++k)
            {
              const double apk = a[static_cast<size_t>(p) * n + k], aqk = a[static_cast<size_t>(q) * n + k];
              a[static_cast<size_t>(p) * n + k] = c * apk - s * aqk;
              a[static_cast<size_t>(q) * n + k] = s * apk + c * aqk;
            }
            for (int k = 0; k < n; ++k)
            {
              const double vkp = v[static_cast<size_t>(k) * n + p], vkq = v[static_cast<size_t>(k) * n + q];
              v[static_cast<size_t>(k) * n + p] = c * vkp - s * vkq;
              v[static_cast<size_t>(k) * n + q] = s * vkp + c * vkq;
            }
          }
      }
    }
  } // namespace

  namespace
  {
    int64_t up32(int64_t x) { return (x + 31) / 32 * 32; }
  }

  int64_t lanczos_scratch_doubles(int64_t n_doubles, int32_t n_iter)
  {
    const int64_t rows = n_iter + 1;
    // basis, image, dot partials, coefficients, alpha and beta, Ritz coefficients, pointer table
    return up32(rows * n_doubles) + up32(n_doubles) + up32(2 * kDotParts * rows) + up32(2 * rows) + up32(2 * rows) +
           up32(rows) + up32(rows + 3);
  }

  cudaError_t lanczos(const Program &p, DeviceTables &t, const ExecArgs &base, int32_t vector_operand,
                      const double *start, int64_t n_doubles, int32_t n_iter, double tol, double *scratch,
                      double *result, double *energy, int32_t *size_out)
  {
    const bool complex = base.complex;
    const int64_t rows = n_iter + 1;
    double *basis = scratch;
    double *image = basis + up32(rows * n_doubles);
    double *partial = image + up32(n_doubles);
    double *coeffs = partial + up32(2 * kDotParts * rows);
    double *tri = coeffs + up32(2 * rows);  // alpha[0..n_iter), beta[n_iter..2 n_iter)
    double *ritz = tri + up32(2 * rows);
    const double **table = reinterpret_cast<const double **>(ritz + up32(rows));
    // table[j] = basis row j (j < rows), then the image, the start vector and the result
    const double *const *image_slot = table + rows, *const *start_slot = table + rows + 1,
                        *const *result_slot = table + rows + 2;
    cudaStream_t stream = base.stream;
    const int grid = grid_of(n_doubles);
    cudaError_t e;
    rows_kernel<<<1, 64, 0, stream>>>(table, basis, n_doubles, static_cast<int32_t>(rows));
    const double *extra[3] = {image, start, result};
    if ((e = cudaMemcpyAsync(table + rows, extra, sizeof(extra), cudaMemcpyHostToDevice, stream)) != cudaSuccess) return e;
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
    std::vector<double> host(static_cast<size_t>(2 * n_iter));
    if ((e = cudaMemcpyAsync(host.data(), tri, host.size() * 8, cudaMemcpyDeviceToHost, stream)) != cudaSuccess) return e;
    if ((e = cudaStreamSynchronize(stream)) != cudaSuccess) return e;
    // the reference stops at the first beta below tol; the steps computed after it are dropped
    int size = n_iter;
    for (int k = 0; k < n_iter; ++k)
      if (host[static_cast<size_t>(n_iter + k)] < tol)
      {
        size = k + 1;
        break;
      }
    std::vector<double> m(static_cast<size_t>(size) * size, 0.0), v;
    for (int k = 0; k < size; ++k) m[static_cast<size_t>(k) * size + k] = host[static_cast<size_t>(k)];
    for (int k = 0; k + 1 < size; ++k)
      m[static_cast<size_t>(k) * size + k + 1] = m[static_cast<size_t>(k + 1) * size + k] = host[static_cast<size_t>(n_iter + k)];
    jacobi_eigen(m, v, size);
    int lowest = 0;
    for (int k = 1; k < size; ++k)
      if (m[static_cast<size_t>(k) * size + k] < m[static_cast<size_t>(lowest) * size + lowest]) lowest = k;
    *energy = m[static_cast<size_t>(lowest) * size + lowest];
    *size_out = size;
    std::vector<double> c(static_cast<size_t>(size));
    for (int k = 0; k < size; ++k) c[static_cast<size_t>(k)] = v[static_cast<size_t>(k) * size + lowest];
    if ((e = cudaMemcpyAsync(ritz, c.data(), c.size() * 8, cudaMemcpyHostToDevice, stream)) != cudaSuccess) return e;
    // the Ritz vector, normalised (complex arenas: real coefficients act on both parts alike)
    combine_kernel<<<grid, 256, 0, stream>>>(result, basis, n_doubles, size, ritz);
    if ((e = arena_dots(result_slot, 1, result, n_doubles, complex, partial, coeffs, stream)) != cudaSuccess) return e;
    scale_kernel<<<grid, 256, 0, stream>>>(result, result, n_doubles, coeffs, nullptr);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    // the host vectors above are read by copies already issued; wait for them before they go
    return cudaStreamSynchronize(stream);
  }

} // namespace ttg
