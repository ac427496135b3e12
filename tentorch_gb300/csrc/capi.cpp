// The C ABI (include/tentorch_gb300.h): integer handles over the interned categories, legs and
// spaces, cached plans, and status codes instead of exceptions.
#include "../../include/tentorch_gb300.h"

#include <cuda_runtime.h>

#include <cstring>
#include <functional>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "engine.h"
#include "executor.h"
#include "gemm.h"
#include "program.h"

struct tt_plan
{
  std::shared_ptr<ttg::Program> program;
  std::unique_ptr<ttg::DeviceTables> tables;
};

namespace
{
  thread_local std::string last_error;
  std::recursive_mutex registry_mutex;  // categories, legs, spaces, plan caches

  int32_t fail(int32_t code, const std::string &message)
  {
    last_error = message;
    return code;
  }

  template <typename F>
  int32_t guarded(F &&body)
  {
    try
    {
      std::lock_guard<std::recursive_mutex> lock(registry_mutex);
      body();
      return TT_OK;
    }
    catch (const ttg::OutOfRange &e)
    {
      return fail(TT_ERANGE, e.what());
    }
    catch (const ttg::InvalidArgument &e)
    {
      return fail(TT_EINVAL, e.what());
    }
    catch (const std::invalid_argument &e)
    {
      return fail(TT_EINVAL, e.what());
    }
    catch (const std::out_of_range &e)
    {
      return fail(TT_ERANGE, e.what());
    }
    catch (const std::exception &e)
    {
      return fail(TT_ELOGIC, e.what());
    }
  }

  std::vector<const ttg::Category *> &categories()
  {
    static std::vector<const ttg::Category *> held;
    return held;
  }

  const ttg::Category *cat_of(int32_t id)
  {
    auto &held = categories();
    if (id < 0 || static_cast<size_t>(id) >= held.size()) throw ttg::InvalidArgument("no category " + std::to_string(id));
    return held[static_cast<size_t>(id)];
  }

  ttg::Sector S(int64_t v) { return ttg::Sector{v}; }

  void write_matrix(const ttg::Matrix &m, int32_t cap, double *values, int32_t *rows, int32_t *cols)
  {
    *rows = m.rows;
    *cols = m.cols;
    const int32_t n = std::min<int32_t>(cap, m.rows * m.cols);
    for (int32_t i = 0; i < n; ++i)
    {
      values[2 * i] = m.v[static_cast<size_t>(i)].real();
      values[2 * i + 1] = m.v[static_cast<size_t>(i)].imag();
    }
  }

  std::vector<ttg::Leg> legs_of(int32_t n, const int32_t *ids)
  {
    std::vector<ttg::Leg> out;
    for (int32_t i = 0; i < n; ++i) out.push_back(ttg::leg_by_id(ids[i]));
    return out;
  }

  tt_plan *keep(std::map<std::string, std::unique_ptr<tt_plan>> &cache, const std::string &name,
                const std::function<std::shared_ptr<ttg::Program>()> &build)
  {
    auto found = cache.find(name);
    if (found != cache.end()) return found->second.get();
    auto plan = std::make_unique<tt_plan>();
    plan->program = build();
    plan->tables = std::make_unique<ttg::DeviceTables>();
    return cache.emplace(name, std::move(plan)).first->second.get();
  }

  std::map<std::string, std::unique_ptr<tt_plan>> &plan_cache()
  {
    static std::map<std::string, std::unique_ptr<tt_plan>> cache;
    return cache;
  }

  std::string ints(const int32_t *v, int32_t n)
  {
    std::string out;
    for (int32_t i = 0; i < n; ++i) out += std::to_string(v[i]) + ",";
    return out;
  }
} // namespace

namespace ttg
{
  int32_t report(int32_t code, const std::string &message) { return fail(code, message); }
} // namespace ttg

extern "C"
{
  const char *tt_last_error(void) { return last_error.c_str(); }

  int32_t tt_version(void) { return 1; }

  int32_t tt_category(int32_t kind, int64_t param, int32_t *out)
  {
    return guarded([&] {
      if (kind < 0 || kind > 5) throw ttg::InvalidArgument("unknown category kind " + std::to_string(kind));
      const ttg::Category *c = ttg::category(static_cast<ttg::CategoryKind>(kind), param);
      auto &held = categories();
      for (size_t i = 0; i < held.size(); ++i)
        if (held[i] == c)
        {
          *out = static_cast<int32_t>(i);
          return;
        }
      held.push_back(c);
      *out = static_cast<int32_t>(held.size() - 1);
    });
  }

  int32_t tt_outcomes(int32_t cat, int64_t a, int64_t b, int32_t cap, int64_t *sectors, int32_t *mult, int32_t *n)
  {
    return guarded([&] {
      const auto &o = cat_of(cat)->outcomes(S(a), S(b));
      *n = static_cast<int32_t>(o.size());
      for (int32_t i = 0; i < std::min<int32_t>(cap, *n); ++i)
      {
        sectors[i] = o[static_cast<size_t>(i)].sector[0];
        mult[i] = o[static_cast<size_t>(i)].multiplicity;
      }
    });
  }

  int32_t tt_dual(int32_t cat, int64_t a, int64_t *out)
  {
    return guarded([&] { *out = cat_of(cat)->dual(S(a))[0]; });
  }

  int32_t tt_q_dim(int32_t cat, int64_t a, double *out)
  {
    return guarded([&] { *out = cat_of(cat)->q_dim(S(a)); });
  }

  int32_t tt_F_symbol(int32_t cat, int64_t a, int64_t b, int64_t c, int64_t d, int32_t cap, double *values,
                      int32_t *rows, int32_t *cols)
  {
    return guarded([&] { write_matrix(cat_of(cat)->F(S(a), S(b), S(c), S(d)), cap, values, rows, cols); });
  }

  int32_t tt_R_symbol(int32_t cat, int64_t b, int64_t c, int32_t cap, double *values, int32_t *rows, int32_t *cols)
  {
    return guarded([&] { write_matrix(cat_of(cat)->R(S(b), S(c)), cap, values, rows, cols); });
  }

  int32_t tt_leg(int32_t cat, int32_t n, const int64_t *sectors, const int64_t *mult, int32_t *out)
  {
    return guarded([&] {
      std::vector<ttg::Sector> s;
      std::vector<int64_t> m;
      for (int32_t i = 0; i < n; ++i)
      {
        s.push_back(S(sectors[i]));
        m.push_back(mult[i]);
      }
      *out = ttg::make_leg(cat_of(cat), std::move(s), std::move(m))->id;
    });
  }

  int32_t tt_leg_blocks(int32_t leg, int32_t cap, int64_t *sectors, int64_t *mult, int32_t *n)
  {
    return guarded([&] {
      ttg::Leg l = ttg::leg_by_id(leg);
      *n = static_cast<int32_t>(l->sectors.size());
      for (int32_t i = 0; i < std::min<int32_t>(cap, *n); ++i)
      {
        sectors[i] = l->sectors[static_cast<size_t>(i)][0];
        mult[i] = l->mult[static_cast<size_t>(i)];
      }
    });
  }

  int32_t tt_reachable_charges(int32_t cat, int32_t nlegs, const int32_t *legs, int32_t cap, int64_t *out, int32_t *n)
  {
    return guarded([&] {
      const auto charges = ttg::reachable_charges(*cat_of(cat), legs_of(nlegs, legs));
      *n = static_cast<int32_t>(charges.size());
      for (int32_t i = 0; i < std::min<int32_t>(cap, *n); ++i) out[i] = charges[static_cast<size_t>(i)][0];
    });
  }

  int32_t tt_fusion_trees(int32_t cat, int32_t nlegs, const int32_t *legs, int64_t coupled, int64_t cap, int64_t *out,
                          int64_t *n_trees, int32_t *stride)
  {
    return guarded([&] {
      const auto trees = ttg::fusion_trees(*cat_of(cat), legs_of(nlegs, legs), S(coupled));
      const int32_t per = nlegs + std::max(nlegs - 2, 0) + std::max(nlegs - 1, 0) + 1;
      *stride = per;
      *n_trees = static_cast<int64_t>(trees.size());
      int64_t at = 0;
      for (const ttg::Tree &t : trees)
      {
        if (at + per > cap) break;
        for (const auto &s : t.sectors) out[at++] = s[0];
        for (const auto &s : t.inner) out[at++] = s[0];
        for (int32_t c : t.copies) out[at++] = c;
        out[at++] = t.coupled[0];
      }
    });
  }

  int32_t tt_space(int32_t cat, int32_t ncod, const int32_t *cod, int32_t ndom, const int32_t *dom, int64_t qtotal,
                   int32_t *out)
  {
    return guarded([&] { *out = ttg::make_space(cat_of(cat), legs_of(ncod, cod), legs_of(ndom, dom), S(qtotal))->id; });
  }

  int32_t tt_space_size(int32_t space, int64_t *nblocks, int64_t *elements)
  {
    return guarded([&] {
      ttg::Space s = ttg::space_by_id(space);
      *nblocks = static_cast<int64_t>(s->blocks.size());
      *elements = s->size;
    });
  }

  int32_t tt_space_blocks(int32_t space, int64_t cap, int64_t *keys, int64_t *shapes)
  {
    return guarded([&] {
      ttg::Space s = ttg::space_by_id(space);
      for (int64_t i = 0; i < std::min<int64_t>(cap, static_cast<int64_t>(s->blocks.size())); ++i)
      {
        const ttg::Block &b = s->blocks[static_cast<size_t>(i)];
        keys[3 * i] = b.key.codomain[0];
        keys[3 * i + 1] = b.key.domain[0];
        keys[3 * i + 2] = b.key.copy;
        shapes[3 * i] = b.rows;
        shapes[3 * i + 1] = b.cols;
        shapes[3 * i + 2] = b.offset;
      }
    });
  }

  int32_t tt_space_legs(int32_t space, int32_t cap, int32_t *legs, int32_t *ncod, int32_t *ndom, int64_t *qtotal)
  {
    return guarded([&] {
      ttg::Space s = ttg::space_by_id(space);
      *ncod = static_cast<int32_t>(s->codomain.size());
      *ndom = static_cast<int32_t>(s->domain.size());
      *qtotal = s->qtotal[0];
      int32_t at = 0;
      for (ttg::Leg l : s->legs())
        if (at < cap) legs[at++] = l->id;
    });
  }

  int32_t tt_plan_place(int32_t space, int32_t nabove, const int32_t *above, int32_t nbelow, const int32_t *below,
                        tt_plan **out)
  {
    return guarded([&] {
      const std::string name = "place|" + std::to_string(space) + "|" + ints(above, nabove) + "|" + ints(below, nbelow);
      *out = keep(plan_cache(), name, [&] {
        return ttg::compile_place(ttg::space_by_id(space), std::vector<int32_t>(above, above + nabove),
                                  std::vector<int32_t>(below, below + nbelow));
      });
    });
  }

  int32_t tt_plan_conj(int32_t space, tt_plan **out)
  {
    return guarded([&] {
      const std::string name = "conj|" + std::to_string(space);
      *out = keep(plan_cache(), name, [&] { return ttg::compile_conj(ttg::space_by_id(space)); });
    });
  }

  int32_t tt_plan_contract(int32_t left, int32_t right, int32_t n, const int32_t *left_legs, const int32_t *right_legs,
                           int32_t has_charge, int64_t charge, tt_plan **out)
  {
    return guarded([&] {
      const std::string name = "contract|" + std::to_string(left) + "|" + std::to_string(right) + "|" +
                               ints(left_legs, n) + "|" + ints(right_legs, n) + "|" + std::to_string(has_charge) + "|" +
                               std::to_string(charge);
      *out = keep(plan_cache(), name, [&] {
        return ttg::compile_contract(ttg::space_by_id(left), ttg::space_by_id(right),
                                     std::vector<int32_t>(left_legs, left_legs + n),
                                     std::vector<int32_t>(right_legs, right_legs + n), has_charge != 0, S(charge));
      });
    });
  }

  int32_t tt_plan_einsum(const char *spec, int32_t n, const int32_t *spaces, int32_t has_charge, int64_t charge,
                         tt_plan **out)
  {
    return guarded([&] {
      const std::string name = std::string("einsum|") + spec + "|" + ints(spaces, n) + "|" + std::to_string(has_charge) +
                               "|" + std::to_string(charge);
      *out = keep(plan_cache(), name, [&] {
        std::vector<ttg::Space> ops;
        for (int32_t i = 0; i < n; ++i) ops.push_back(ttg::space_by_id(spaces[i]));
        return ttg::compile_einsum(spec, ops, has_charge != 0, S(charge));
      });
    });
  }

  int32_t tt_plan_info(const tt_plan *plan, int32_t *out_space, int64_t *workspace, double *gemm_flops,
                       int64_t *moved_elements, int32_t *n_ops)
  {
    return guarded([&] {
      if (!plan) throw ttg::InvalidArgument("no plan");
      const ttg::Program &p = *plan->program;
      *out_space = p.output_space->id;
      *workspace = p.workspace;
      *gemm_flops = p.gemm_flops;
      *moved_elements = p.moved_elements;
      *n_ops = static_cast<int32_t>(p.ops.size());
    });
  }

  int32_t tt_plan_gather(const tt_plan *plan, int32_t op, int64_t cap, int32_t *index, int64_t *count)
  {
    return guarded([&] {
      if (!plan) throw ttg::InvalidArgument("no plan");
      const ttg::Program &p = *plan->program;
      if (op < 0 || static_cast<size_t>(op) >= p.ops.size())
        throw ttg::OutOfRange("the plan has no operation " + std::to_string(op));
      const ttg::Op &o = p.ops[static_cast<size_t>(op)];
      if (o.kind == ttg::OpKind::gather)
      {
        *count = o.count;
        if (cap >= o.count && o.count > 0)
          std::memcpy(index, p.gather_index.data() + o.begin, static_cast<size_t>(o.count) * sizeof(int32_t));
        return;
      }
      if (o.kind != ttg::OpKind::tiles)
        throw ttg::InvalidArgument("operation " + std::to_string(op) + " is neither a gather nor tiles");
      // the index the tiles amount to, entry by entry
      *count = o.elements;
      if (cap < o.elements) return;
      const std::vector<int32_t> expanded = ttg::expand_move(p, o);
      std::copy(expanded.begin(), expanded.end(), index);
    });
  }

  int32_t tt_plan_cache_clear(void)
  {
    return guarded([&] {
      std::lock_guard<std::recursive_mutex> lock(registry_mutex);
      ttg::clear_chain_batches();
      plan_cache().clear();
    });
  }

  int32_t tt_plan_describe(const tt_plan *plan, int64_t cap, char *text, int64_t *length)
  {
    return guarded([&] {
      const ttg::Program &p = *plan->program;
      static const char *kinds[] = {"zero", "gather", "runs", "gemm", "add", "copy", "tiles"};
      std::string out;
      if (p.chain_first >= 0)
        out += "chain ops " + std::to_string(p.chain_first) + " " + std::to_string(p.chain_move) + " " +
               std::to_string(p.chain_second) + "\n";
      if (!p.fold.empty())
      {
        out += "fold order";
        for (const int32_t o : p.fold) out += " " + std::to_string(o);
        out += "\n";
      }
      for (size_t i = 0; i < p.ops.size(); ++i)
      {
        const ttg::Op &op = p.ops[i];
        out += "op " + std::to_string(i) + " " + kinds[static_cast<int>(op.kind)] + " src " + std::to_string(op.src) +
               " src2 " + std::to_string(op.src2) + " dst " + std::to_string(op.dst) + " phase " + std::to_string(op.phase) +
               " elements " + std::to_string(op.elements) + " count " + std::to_string(op.count) + "\n";
        if (op.kind == ttg::OpKind::gemm && p.gemm_plans && i < p.gemm_plans->f64.size())
        {
          // the FP64 schedule: items dealt to the SMs, K-split tiles and the longest list
          const ttg::GemmSchedule s = ttg::schedule_gemm(p, op, ttg::kF64TileM, ttg::kF64TileN, true);
          int64_t longest = 0;
          for (size_t c = 0; c + 1 < s.cta_begin.size(); ++c) longest = std::max<int64_t>(longest, s.cta_begin[c + 1] - s.cta_begin[c]);
          out += "  fp64 schedule: items " + std::to_string(s.items.size()) + " split tiles " + std::to_string(s.reduces.size()) +
                 " partial slots " + std::to_string(s.slots) + " ctas " +
                 std::to_string(s.cta_begin.empty() ? 0 : s.cta_begin.size() - 1) + " longest list " + std::to_string(longest) + "\n";
        }
        if (op.kind == ttg::OpKind::gemm)
          for (int64_t b = op.begin; b < op.begin + op.count; ++b)
          {
            const ttg::GemmBlock &blk = p.gemm_blocks[static_cast<size_t>(b)];
            out += "  block m " + std::to_string(blk.m) + " n " + std::to_string(blk.n) + " k";
            for (int32_t k = 0; k < blk.pair_count; ++k)
              out += " " + std::to_string(p.gemm_pairs[static_cast<size_t>(blk.pair_begin + k)].k);
            out += "\n";
          }
      }
      *length = static_cast<int64_t>(out.size());
      if (cap > 0)
      {
        const int64_t n = std::min<int64_t>(cap - 1, static_cast<int64_t>(out.size()));
        std::memcpy(text, out.data(), static_cast<size_t>(n));
        text[n] = 0;
      }
    });
  }

  int32_t tt_plan_prepared_size(const tt_plan *plan, int32_t operand, int64_t *elements)
  {
    return guarded([&] {
      const ttg::Program &p = *plan->program;
      if (operand < 0 || operand >= p.n_inputs) throw ttg::InvalidArgument("no operand " + std::to_string(operand));
      const int32_t b = p.prepared[static_cast<size_t>(operand)];
      *elements = b < 0 ? 0 : p.buffers[static_cast<size_t>(b)].size;
      // with the slices of its value that split-precision products read (float64 elements)
      if (b >= 0 && p.gemm_plans && !p.gemm_plans->prepared_bytes.empty())
        *elements = std::max<int64_t>(*elements, (p.gemm_plans->prepared_bytes[static_cast<size_t>(operand)] + 7) / 8);
    });
  }

  int32_t tt_plan_execute(const tt_plan *plan, int32_t dtype, int32_t precision, const void *const *inputs,
                          const void *const *prepared, void *output, void *workspace, void *stream)
  {
    if (!plan) return fail(TT_EINVAL, "no plan");
    if (dtype != TT_DTYPE_FLOAT64 && dtype != TT_DTYPE_COMPLEX128) return fail(TT_EINVAL, "unknown dtype");
    if (precision < TT_PRECISION_PER_BLOCK || precision > 8)
      return fail(TT_EINVAL, "precision is 0 (FP64), 1..8 slices, or -1 (per-block FP64)");
    if (precision > 0 && dtype != TT_DTYPE_FLOAT64)
      return fail(TT_EINVAL, "split precision is implemented for float64 arenas");
    ttg::ExecArgs args;
    args.complex = dtype == TT_DTYPE_COMPLEX128;
    args.precision = precision;
    args.inputs = inputs;
    args.prepared = prepared;
    args.output = output;
    args.workspace = workspace;
    args.stream = static_cast<cudaStream_t>(stream);
    if (plan->program->complex_coefficients && !args.complex)
    {
      // a float64 tensor keeps the real part of a complex coefficient, as the reference does
      // (tentorch/tensors/cache.cpp:84-92); nothing to do here, the kernel reads .re only
    }
    const cudaError_t e = ttg::execute(*plan->program, *plan->tables, args);
    if (e != cudaSuccess) return fail(TT_ECUDA, std::string("CUDA: ") + cudaGetErrorString(e));
    return TT_OK;
  }

  int32_t tt_plan_execute_batch(int32_t count, const tt_plan *const *plans, int32_t dtype, int32_t precision,
                                const void *const *const *inputs, const void *const *const *prepared,
                                void *const *outputs, void *const *workspaces, void *stream, int32_t *launched)
  {
    if (count < 0 || (count > 0 && (!plans || !inputs || !outputs || !workspaces)))
      return fail(TT_EINVAL, "a batch needs its plans, inputs, outputs and workspaces");
    if (precision < TT_PRECISION_PER_BLOCK || precision > 8)
      return fail(TT_EINVAL, "precision is 0 (FP64), 1..8 slices, or -1 (per-block FP64)");
    if (dtype != TT_DTYPE_FLOAT64 && dtype != TT_DTYPE_COMPLEX128) return fail(TT_EINVAL, "unknown dtype");
    if (precision > 0 && dtype != TT_DTYPE_FLOAT64) return fail(TT_EINVAL, "split precision is implemented for float64 arenas");
    for (int32_t i = 0; i < count; ++i)
      if (!plans[i]) return fail(TT_EINVAL, "no plan");
    if (launched) *launched = 0;
    const cudaStream_t s = static_cast<cudaStream_t>(stream);
    const auto args_of = [&](int32_t i)
    {
      ttg::ExecArgs args;
      args.complex = dtype == TT_DTYPE_COMPLEX128;
      args.precision = precision;
      args.inputs = inputs[i];
      args.prepared = prepared ? prepared[i] : nullptr;
      args.output = outputs[i];
      args.workspace = workspaces[i];
      args.stream = s;
      return args;
    };
    cudaError_t e = cudaSuccess;
    // one launch when every plan is an FP64 chain whose other ops are prepare phases
    bool one = count > 0 && count <= ttg::kChainBatch && dtype == TT_DTYPE_FLOAT64 && precision == 0;
    for (int32_t i = 0; i < count && one; ++i)
    {
      const ttg::Program &p = *plans[i]->program;
      if (p.chain_first < 0) one = false;
      for (size_t j = 0; j < p.ops.size() && one; ++j)
        if (p.ops[j].phase < 0 && static_cast<int32_t>(j) != p.chain_first && static_cast<int32_t>(j) != p.chain_move &&
            static_cast<int32_t>(j) != p.chain_second)
          one = false;
    }
    if (one)
    {
      std::vector<ttg::ChainBatchEntry> entries;
      for (int32_t i = 0; i < count && e == cudaSuccess; ++i)
      {
        const ttg::Program &p = *plans[i]->program;
        ttg::ExecArgs args = args_of(i);
        if ((e = plans[i]->tables->ensure(p)) != cudaSuccess) break;
        // the phases the caller has no prepared arena for run first, one plan after another
        args.phases_only = true;
        if ((e = ttg::execute(p, *plans[i]->tables, args)) != cudaSuccess) break;
        args.phases_only = false;
        const std::vector<char *> ptr = ttg::buffer_pointers(p, args);
        const ttg::Op &first = p.ops[static_cast<size_t>(p.chain_first)], &move = p.ops[static_cast<size_t>(p.chain_move)],
                      &second = p.ops[static_cast<size_t>(p.chain_second)];
        entries.push_back({&p, plans[i]->tables.get(), reinterpret_cast<const double *>(ptr[static_cast<size_t>(first.src)]),
                           reinterpret_cast<const double *>(ptr[static_cast<size_t>(first.src2)]),
                           reinterpret_cast<const double *>(ptr[static_cast<size_t>(second.src2)]),
                           reinterpret_cast<double *>(ptr[static_cast<size_t>(move.dst)]),
                           reinterpret_cast<double *>(ptr[static_cast<size_t>(second.dst)]), workspaces[i]});
      }
      bool used = false;
      if (e == cudaSuccess) e = ttg::launch_chain_batch(entries, s, &used);
      if (e != cudaSuccess) return fail(TT_ECUDA, std::string("CUDA: ") + cudaGetErrorString(e));
      if (used)
      {
        if (launched) *launched = 1;
        return TT_OK;
      }
    }
    // one plan after another (a plan whose phases already ran above runs them again, to the same values)
    for (int32_t i = 0; i < count && e == cudaSuccess; ++i)
    {
      ttg::ExecArgs args = args_of(i);
      e = ttg::execute(*plans[i]->program, *plans[i]->tables, args);
    }
    if (e != cudaSuccess) return fail(TT_ECUDA, std::string("CUDA: ") + cudaGetErrorString(e));
    if (launched) *launched = count;
    return TT_OK;
  }

  int32_t tt_plan_execute_timed(const tt_plan *plan, int32_t dtype, int32_t precision, const void *const *inputs,
                                const void *const *prepared, void *output, void *workspace, void *stream, int32_t cap,
                                float *op_ms, int32_t *op_kind)
  {
    if (!plan) return fail(TT_EINVAL, "no plan");
    if (precision < TT_PRECISION_PER_BLOCK || precision > 8)
      return fail(TT_EINVAL, "precision is 0 (FP64), 1..8 slices, or -1 (per-block FP64)");
    if (precision > 0 && dtype != TT_DTYPE_FLOAT64)
      return fail(TT_EINVAL, "split precision is implemented for float64 arenas");
    const ttg::Program &p = *plan->program;
    const size_t n = p.ops.size();
    std::vector<cudaEvent_t> events(2 * n, nullptr);
    cudaError_t e = cudaSuccess;
    for (size_t i = 0; i < events.size() && e == cudaSuccess; ++i) e = cudaEventCreate(&events[i]);
    if (e == cudaSuccess)
    {
      ttg::ExecArgs args;
      args.complex = dtype == TT_DTYPE_COMPLEX128;
      args.precision = precision;
      args.inputs = inputs;
      args.prepared = prepared;
      args.output = output;
      args.workspace = workspace;
      args.stream = static_cast<cudaStream_t>(stream);
      args.events = events.data();
      bool chained = false;
      args.chain_ran = &chained;
      e = ttg::execute(p, *plan->tables, args);
      if (e == cudaSuccess) e = cudaStreamSynchronize(args.stream);
      for (size_t i = 0; i < n && e == cudaSuccess; ++i)
      {
        float ms = -1.0f;
        // an op that did not run left its events unrecorded: cudaEventElapsedTime reports that
        if (cudaEventQuery(events[2 * i]) == cudaSuccess && cudaEventElapsedTime(&ms, events[2 * i], events[2 * i + 1]) != cudaSuccess)
          ms = -1.0f;
        cudaGetLastError();
        if (static_cast<int32_t>(i) < cap)
        {
          op_ms[i] = ms;
          // 7: the product chain as one launch (timed on its first op)
          op_kind[i] = chained && static_cast<int32_t>(i) == p.chain_first ? 7 : static_cast<int32_t>(p.ops[i].kind);
        }
      }
    }
    for (cudaEvent_t ev : events)
      if (ev) cudaEventDestroy(ev);
    if (e != cudaSuccess) return fail(TT_ECUDA, std::string("CUDA: ") + cudaGetErrorString(e));
    return TT_OK;
  }

  int32_t tt_plan_histogram(const tt_plan *plan, uint64_t *key)
  {
    if (!plan || !key) return fail(TT_EINVAL, "no plan");
    *key = plan->program->tune_key;
    return TT_OK;
  }

  int32_t tt_autotune(const tt_plan *plan, int32_t dtype, int32_t precision, const void *const *inputs,
                      const void *const *prepared, void *output, void *workspace, void *stream, int32_t *forms, float *ms)
  {
    if (!plan || !forms || !ms) return fail(TT_EINVAL, "no plan");
    if (dtype != TT_DTYPE_FLOAT64 && dtype != TT_DTYPE_COMPLEX128) return fail(TT_EINVAL, "unknown dtype");
    if (precision < TT_PRECISION_PER_BLOCK || precision > 8)
      return fail(TT_EINVAL, "precision is 0 (FP64), 1..8 slices, or -1 (per-block FP64)");
    if (precision > 0 && dtype != TT_DTYPE_FLOAT64)
      return fail(TT_EINVAL, "split precision is implemented for float64 arenas");
    const ttg::Program &p = *plan->program;
    if (cudaError_t e = plan->tables->ensure(p); e != cudaSuccess) return fail(TT_ECUDA, std::string("CUDA: ") + cudaGetErrorString(e));
    ttg::ExecArgs args;
    args.complex = dtype == TT_DTYPE_COMPLEX128;
    args.precision = precision;
    args.inputs = inputs;
    args.prepared = prepared;
    args.output = output;
    args.workspace = workspace;
    args.stream = static_cast<cudaStream_t>(stream);
    const cudaError_t e = ttg::autotune(p, *plan->tables, args, forms, ms);
    if (e != cudaSuccess) return fail(TT_ECUDA, std::string("CUDA: ") + cudaGetErrorString(e));
    return TT_OK;
  }

  int32_t tt_autotune_lookup(uint64_t key, int32_t dtype, int32_t precision, int32_t *forms, int32_t *found)
  {
    if (!forms || !found) return fail(TT_EINVAL, "no output");
    const int32_t f = ttg::tuned_forms(key, dtype == TT_DTYPE_COMPLEX128, precision);
    *found = f >= 0 ? 1 : 0;
    *forms = f >= 0 ? f : 0;
    return TT_OK;
  }

  int32_t tt_autotune_store(uint64_t key, int32_t dtype, int32_t precision, int32_t forms)
  {
    if (forms < 0 || forms > (TT_FORM_SEPARATE | TT_FORM_NO_TENSOR_CORES)) return fail(TT_EINVAL, "unknown forms");
    ttg::store_forms(key, dtype == TT_DTYPE_COMPLEX128, precision, forms);
    return TT_OK;
  }

  int32_t tt_autotune_clear(void)
  {
    ttg::clear_forms();
    return TT_OK;
  }

  int32_t tt_plan_prepare(const tt_plan *plan, int32_t dtype, int32_t operand, const void *input, void *prepared,
                          void *workspace, void *stream)
  {
    if (!plan) return fail(TT_EINVAL, "no plan");
    const ttg::Program &p = *plan->program;
    if (operand < 0 || operand >= p.n_inputs || p.prepared[static_cast<size_t>(operand)] < 0)
      return fail(TT_EINVAL, "operand " + std::to_string(operand) + " has no preparation");
    std::vector<const void *> inputs(static_cast<size_t>(p.n_inputs), nullptr);
    inputs[static_cast<size_t>(operand)] = input;
    ttg::ExecArgs args;
    args.complex = dtype == TT_DTYPE_COMPLEX128;
    args.inputs = inputs.data();
    args.workspace = workspace;
    args.stream = static_cast<cudaStream_t>(stream);
    args.only_phase = operand;
    args.prepared_out = prepared;
    cudaError_t e = ttg::execute(p, *plan->tables, args);
    if (e == cudaSuccess && !args.complex) e = ttg::fill_slice_caches(p, *plan->tables, operand, prepared, args.stream);
    if (e != cudaSuccess) return fail(TT_ECUDA, std::string("CUDA: ") + cudaGetErrorString(e));
    return TT_OK;
  }

  int32_t tt_step_plan(int32_t space, int32_t kind, int32_t arm, int64_t key_cod, int64_t key_dom, int32_t key_copy,
                       int64_t cap_shifts, int64_t *shifts, int64_t cap_pieces, double *pieces, int64_t *n_shifts,
                       int64_t *n_pieces)
  {
    return guarded([&] {
      ttg::Space s = ttg::space_by_id(space);
      if (kind < 0 || kind > 2) throw ttg::InvalidArgument("a step is 0 (exchange), 1 (bend down) or 2 (bend up)");
      std::vector<ttg::Leg> cod = s->codomain, dom = s->domain;
      if (kind == 0)
      {
        if (arm < 0 || arm + 1 >= static_cast<int32_t>(cod.size())) throw ttg::InvalidArgument("no such exchange");
        std::swap(cod[static_cast<size_t>(arm)], cod[static_cast<size_t>(arm + 1)]);
      }
      else if (kind == 1)
      {
        if (cod.empty()) throw ttg::InvalidArgument("no codomain leg to bend");
        dom.push_back(cod.back());
        cod.pop_back();
      }
      else
      {
        if (dom.empty()) throw ttg::InvalidArgument("no domain leg to bend");
        cod.push_back(dom.back());
        dom.pop_back();
      }
      ttg::Step step{kind, kind == 0 ? arm : 0, s, ttg::make_space(s->cat, cod, dom, s->qtotal)};
      const auto &plan = ttg::step_plan(step, ttg::BlockKey{S(key_cod), S(key_dom), key_copy});
      *n_shifts = static_cast<int64_t>(plan.size());
      int64_t np = 0;
      for (size_t i = 0; i < plan.size(); ++i)
      {
        const ttg::Shift &sh = plan[i];
        if (static_cast<int64_t>(i) < cap_shifts)
        {
          int64_t *o = shifts + 9 * i;
          o[0] = sh.from.codomain[0], o[1] = sh.from.domain[0], o[2] = sh.from.copy;
          o[3] = sh.to.codomain[0], o[4] = sh.to.domain[0], o[5] = sh.to.copy;
          o[6] = sh.rows, o[7] = sh.cols, o[8] = static_cast<int64_t>(sh.pieces.size());
        }
        for (const ttg::Piece &pc : sh.pieces)
        {
          if (np < cap_pieces)
          {
            double *o = pieces + 8 * np;
            o[0] = static_cast<double>(pc.first), o[1] = static_cast<double>(pc.last);
            o[2] = static_cast<double>(pc.from_step), o[3] = static_cast<double>(pc.to_step);
            o[4] = static_cast<double>(pc.run), o[5] = pc.coefficient.real(), o[6] = pc.coefficient.imag();
            o[7] = static_cast<double>(i);
          }
          ++np;
        }
      }
      *n_pieces = np;
    });
  }

  int32_t tt_chain(int32_t space, int32_t nabove, const int32_t *above, int32_t nbelow, const int32_t *below,
                   int32_t cap, int32_t *steps, int32_t *n)
  {
    return guarded([&] {
      const auto ch = ttg::chain(ttg::space_by_id(space), std::vector<int32_t>(above, above + nabove),
                                 std::vector<int32_t>(below, below + nbelow));
      *n = static_cast<int32_t>(ch.size());
      for (int32_t i = 0; i < std::min<int32_t>(cap, *n); ++i)
      {
        steps[3 * i] = ch[static_cast<size_t>(i)].kind;
        steps[3 * i + 1] = ch[static_cast<size_t>(i)].arm;
        steps[3 * i + 2] = ch[static_cast<size_t>(i)].after->id;
      }
    });
  }

  int32_t tt_lanczos_scratch(int64_t n, int32_t n_iter, int32_t dtype, int64_t *doubles)
  {
    return guarded([&] {
      if (n_iter < 1 || n_iter > 60) throw ttg::InvalidArgument("Lanczos takes 1 to 60 steps, not " + std::to_string(n_iter));
      *doubles = ttg::lanczos_scratch_doubles(n * (dtype == TT_DTYPE_COMPLEX128 ? 2 : 1), n_iter);
    });
  }

  namespace
  {
    // The checks and the Krylov loop of tt_lanczos / tt_lanczos_async.
    int32_t run_lanczos(const tt_plan *plan, int32_t dtype, int32_t precision, const void *const *inputs,
                        const void *const *prepared, int32_t vector_operand, const void *start, int32_t n_iter,
                        double tol, void *workspace, void *scratch, void *result, double *energy_dev, int32_t *size_dev,
                        void *stream)
    {
      if (!plan) return fail(TT_EINVAL, "no plan");
      if (dtype != TT_DTYPE_FLOAT64 && dtype != TT_DTYPE_COMPLEX128) return fail(TT_EINVAL, "unknown dtype");
      if (precision < TT_PRECISION_PER_BLOCK || precision > 8)
        return fail(TT_EINVAL, "precision is 0 (FP64), 1..8 slices, or -1 (per-block FP64)");
      if (precision > 0 && dtype != TT_DTYPE_FLOAT64)
        return fail(TT_EINVAL, "split precision is implemented for float64 arenas");
      if (n_iter < 1 || n_iter > 60) return fail(TT_EINVAL, "Lanczos takes 1 to 60 steps");
      const ttg::Program &p = *plan->program;
      if (vector_operand < 0 || vector_operand >= p.n_inputs) return fail(TT_ERANGE, "no such operand");
      if (p.input_spaces[static_cast<size_t>(vector_operand)] != p.output_space)
        return fail(TT_EINVAL, "the action has to map the vector's space to itself");
      if (start == nullptr || result == nullptr || scratch == nullptr) return fail(TT_EINVAL, "a missing arena");
      ttg::ExecArgs args;
      args.complex = dtype == TT_DTYPE_COMPLEX128;
      args.precision = precision;
      args.inputs = inputs;
      args.prepared = prepared;
      args.workspace = workspace;
      args.stream = static_cast<cudaStream_t>(stream);
      cudaError_t e = plan->tables->ensure(p);
      if (e == cudaSuccess)
      {
        const int64_t n = p.output_space->size * (args.complex ? 2 : 1);
        double *slot = ttg::lanczos_energy_slot(static_cast<double *>(scratch), n, n_iter);
        e = ttg::lanczos(p, *plan->tables, args, vector_operand, static_cast<const double *>(start), n, n_iter, tol,
                         static_cast<double *>(scratch), static_cast<double *>(result), energy_dev ? energy_dev : slot,
                         size_dev ? size_dev : reinterpret_cast<int32_t *>(slot + 1));
      }
      if (e != cudaSuccess) return fail(TT_ECUDA, std::string("CUDA: ") + cudaGetErrorString(e));
      return TT_OK;
    }
  } // namespace

  int32_t tt_lanczos(const tt_plan *plan, int32_t dtype, int32_t precision, const void *const *inputs,
                     const void *const *prepared, int32_t vector_operand, const void *start, int32_t n_iter,
                     double tol, void *workspace, void *scratch, void *result, double *energy, int32_t *size,
                     void *stream)
  {
    const int32_t status = run_lanczos(plan, dtype, precision, inputs, prepared, vector_operand, start, n_iter, tol,
                                       workspace, scratch, result, nullptr, nullptr, stream);
    if (status != TT_OK) return status;
    // the energy and the size from their place in the scratch, after the stream's work
    const ttg::Program &p = *plan->program;
    const int64_t n = p.output_space->size * (dtype == TT_DTYPE_COMPLEX128 ? 2 : 1);
    double found[2];
    const double *slot = ttg::lanczos_energy_slot(static_cast<double *>(scratch), n, n_iter);
    cudaError_t e = cudaMemcpyAsync(found, slot, sizeof(found), cudaMemcpyDeviceToHost, static_cast<cudaStream_t>(stream));
    if (e == cudaSuccess) e = cudaStreamSynchronize(static_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return fail(TT_ECUDA, std::string("CUDA: ") + cudaGetErrorString(e));
    *energy = found[0];
    std::memcpy(size, &found[1], sizeof(int32_t));
    return TT_OK;
  }

  int32_t tt_lanczos_async(const tt_plan *plan, int32_t dtype, int32_t precision, const void *const *inputs,
                           const void *const *prepared, int32_t vector_operand, const void *start, int32_t n_iter,
                           double tol, void *workspace, void *scratch, void *result, double *energy, int32_t *size,
                           void *stream)
  {
    if (energy == nullptr || size == nullptr)
      return fail(TT_EINVAL, "tt_lanczos_async writes its energy and size to device memory");
    return run_lanczos(plan, dtype, precision, inputs, prepared, vector_operand, start, n_iter, tol, workspace, scratch,
                       result, energy, size, stream);
  }

  int32_t tt_svd_workspace(int32_t count, const int64_t *shapes, int64_t *offsets, int64_t *total)
  {
    return guarded([&] {
      if (count < 0) throw ttg::InvalidArgument("a negative block count");
      int64_t at = 0;
      for (int32_t i = 0; i < count; ++i)
      {
        if (shapes[2 * i] > 1024 && shapes[2 * i + 1] > 1024)
          throw ttg::InvalidArgument("a block of the batched SVD has more than 1024 rows and columns");
        const int64_t need = ttg::svd_workspace_doubles(shapes[2 * i], shapes[2 * i + 1]);
        offsets[i] = need ? at : -1;
        at += (need + 31) / 32 * 32;
      }
      *total = at;
    });
  }

  int32_t tt_svd_blocks(int32_t count, int64_t largest, const int64_t *table, const double *a, double *u, double *s,
                        double *vh, double *workspace, int32_t *info, void *stream)
  {
    if (count < 0) return fail(TT_EINVAL, "a negative block count");
    if (largest < 0 || largest > 1024) return fail(TT_EINVAL, "the largest block of the batched SVD needs 0 to 1024 columns");
    const cudaError_t e =
      ttg::svd_blocks(count, largest, table, a, u, s, vh, workspace, info, static_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return fail(TT_ECUDA, std::string("CUDA: ") + cudaGetErrorString(e));
    return TT_OK;
  }

  int32_t tt_svd_keep(int32_t count, const int64_t *table, const double *u, const double *s, const double *vh,
                      double *first, double *second, double *values, void *stream)
  {
    if (count < 0) return fail(TT_EINVAL, "a negative block count");
    const cudaError_t e =
      ttg::svd_keep(count, table, u, s, vh, first, second, values, static_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return fail(TT_ECUDA, std::string("CUDA: ") + cudaGetErrorString(e));
    return TT_OK;
  }

  int32_t tt_svd_rank(const double *values, int32_t n_values, const int32_t *block_k, const int32_t *block_sector,
                      int32_t n_blocks, const int32_t *dual, int32_t n_sectors, double tol, int64_t max_bond, int32_t *kept,
                      void *stream)
  {
    if (n_values < 0 || n_blocks < 0 || n_sectors < 0) return fail(TT_EINVAL, "negative counts");
    if (n_blocks == 0) return TT_OK;
    if (ttg::rank_bytes(n_values, n_blocks, n_sectors) > ttg::kRankMaxBytes)
      return fail(TT_EINVAL, "too many singular values to rank in one CTA's shared memory (" + std::to_string(n_values) + ")");
    const cudaError_t e = ttg::svd_rank(values, n_values, block_k, block_sector, n_blocks, dual, n_sectors, tol, max_bond,
                                        kept, static_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return fail(TT_ECUDA, std::string("CUDA: ") + cudaGetErrorString(e));
    return TT_OK;
  }

  int32_t tt_dots(int32_t dtype, int32_t count, const void *const *as, const void *b, int64_t n, double *scratch,
                  double *out, void *stream)
  {
    if (count <= 0) return TT_OK;
    if (dtype != TT_DTYPE_FLOAT64 && dtype != TT_DTYPE_COMPLEX128)
      return fail(TT_EINVAL, "unknown dtype " + std::to_string(dtype));
    const bool complex = dtype == TT_DTYPE_COMPLEX128;
    const cudaError_t e = ttg::arena_dots(reinterpret_cast<const double *const *>(as), count,
                                          static_cast<const double *>(b), n * (complex ? 2 : 1), complex, scratch, out,
                                          static_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return fail(TT_ECUDA, std::string("CUDA: ") + cudaGetErrorString(e));
    return TT_OK;
  }
}
