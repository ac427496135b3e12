// The engine's autotuner: which form a plan's block products run in, chosen by timing the forms on
// the plan's own operands and cached by the plan's block-size histogram, so that every later plan
// with the same histogram (the windows of a DMRG sweep at one bond dimension, the matvec steps of a
// Lanczos loop) runs the chosen form without being timed again.
//
// The forms (ExecArgs::forms bits): kFormSeparate runs a product chain (two products with a leg
// move between them) as separate launches instead of one; kFormNoTensorCores keeps split-precision
// products of large blocks on the mma.sync kernel instead of the tcgen05 one.  The tile shapes and
// schedules inside each form are fixed by the form's kernel (32 x 32 FP64 tiles with K cut to about
// six items per SM, 32 x 32 split tiles, 128 x 64 tcgen05 tiles).
//
// The histogram: per block product of the plan, in order, the multiply-adds of its block pairs
// binned by (log2 m, log2 n, log2 K), each bin's sum kept to a quarter octave; plus whether the plan
// has a chain.  Its 64-bit FNV-1a hash is the key.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include "executor.h"
#include "gemm.h"
#include "program.h"

namespace ttg
{
  namespace
  {
    struct FormKey
    {
      uint64_t histogram;
      bool complex;
      int32_t precision;
      bool operator<(const FormKey &o) const
      {
        return std::tie(histogram, complex, precision) < std::tie(o.histogram, o.complex, o.precision);
      }
    };
    std::mutex forms_mutex;
    std::map<FormKey, int32_t> forms_cache;

    void fnv(uint64_t &h, uint64_t v)
    {
      for (int i = 0; i < 8; ++i)
      {
        h ^= (v >> (8 * i)) & 0xff;
        h *= 1099511628211ull;
      }
    }
    int octave(double x) { return x <= 1.0 ? 0 : static_cast<int>(std::floor(std::log2(x))); }
  } // namespace

  uint64_t tune_key(const Program &p)
  {
    uint64_t h = 14695981039346656037ull;
    fnv(h, p.chain_first >= 0 ? 1 : 0);
    for (const Op &op : p.ops)
    {
      if (op.kind != OpKind::gemm) continue;
      std::map<std::tuple<int, int, int>, double> bins;
      for (int64_t b = op.begin; b < op.begin + op.count; ++b)
      {
        const GemmBlock &blk = p.gemm_blocks[static_cast<size_t>(b)];
        for (int32_t k = 0; k < blk.pair_count; ++k)
        {
          const GemmPair &pr = p.gemm_pairs[static_cast<size_t>(blk.pair_begin + k)];
          bins[{octave(blk.m), octave(blk.n), octave(pr.k)}] += static_cast<double>(blk.m) * blk.n * pr.k;
        }
      }
      fnv(h, 0x9e3779b97f4a7c15ull);
      for (const auto &[bin, macs] : bins)
      {
        fnv(h, static_cast<uint64_t>(std::get<0>(bin)) | static_cast<uint64_t>(std::get<1>(bin)) << 16 |
                 static_cast<uint64_t>(std::get<2>(bin)) << 32);
        fnv(h, static_cast<uint64_t>(std::llround(4.0 * std::log2(std::max(macs, 1.0)))));
      }
    }
    return h;
  }

  int32_t tuned_forms(uint64_t key, bool complex, int32_t precision)
  {
    std::lock_guard<std::mutex> lock(forms_mutex);
    const auto found = forms_cache.find(FormKey{key, complex, precision});
    return found == forms_cache.end() ? -1 : found->second;
  }

  void store_forms(uint64_t key, bool complex, int32_t precision, int32_t forms)
  {
    std::lock_guard<std::mutex> lock(forms_mutex);
    forms_cache[FormKey{key, complex, precision}] = forms;
  }

  void clear_forms()
  {
    std::lock_guard<std::mutex> lock(forms_mutex);
    forms_cache.clear();
  }

  std::vector<int32_t> candidate_forms(const Program &p, bool complex, int32_t precision)
  {
    std::vector<int32_t> out{0};
    if (precision < 0) return out;
    if (p.chain_first >= 0 && !complex) out.push_back(kFormSeparate);
    bool tensor = false;
    if (precision > 0 && !complex)
      for (const Op &op : p.ops)
        if (op.kind == OpKind::gemm && split_tc_suits(p, op, precision)) tensor = true;
    if (tensor)
    {
      const size_t n = out.size();
      for (size_t i = 0; i < n; ++i) out.push_back(out[i] | kFormNoTensorCores);
    }
    return out;
  }

  cudaError_t autotune(const Program &p, DeviceTables &t, const ExecArgs &base, int32_t *best, float *best_ms)
  {
    const std::vector<int32_t> forms = candidate_forms(p, base.complex, base.precision);
    cudaEvent_t start = nullptr, stop = nullptr;
    cudaError_t e = cudaEventCreate(&start);
    if (e == cudaSuccess) e = cudaEventCreate(&stop);
    float best_time = -1.0f;
    int32_t chosen = 0;
    for (const int32_t f : forms)
    {
      if (e != cudaSuccess) break;
      ExecArgs args = base;
      args.forms = f;
      // two untimed runs (tables, relabelling and schedules built on first use), then the median of
      // five timed ones
      for (int i = 0; i < 2 && e == cudaSuccess; ++i) e = execute(p, t, args);
      std::vector<float> times;
      for (int i = 0; i < 5 && e == cudaSuccess; ++i)
      {
        if ((e = cudaEventRecord(start, args.stream)) != cudaSuccess) break;
        if ((e = execute(p, t, args)) != cudaSuccess) break;
        if ((e = cudaEventRecord(stop, args.stream)) != cudaSuccess) break;
        if ((e = cudaEventSynchronize(stop)) != cudaSuccess) break;
        float ms = 0.0f;
        if ((e = cudaEventElapsedTime(&ms, start, stop)) != cudaSuccess) break;
        times.push_back(ms);
      }
      if (e != cudaSuccess) break;
      std::sort(times.begin(), times.end());
      const float median = times[times.size() / 2];
      if (best_time < 0.0f || median < best_time)
      {
        best_time = median;
        chosen = f;
      }
    }
    if (start) cudaEventDestroy(start);
    if (stop) cudaEventDestroy(stop);
    if (e != cudaSuccess) return e;
    store_forms(p.tune_key, base.complex, base.precision, chosen);
    *best = chosen;
    *best_ms = best_time;
    return cudaSuccess;
  }
} // namespace ttg
