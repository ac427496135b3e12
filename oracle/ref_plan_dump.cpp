// Test infrastructure, linked against the reference engine's own objects by oracle/build_ref.py:
// returns the reference's per-step regrouping plans and side layouts as plain Python data, so that
// the fixtures under tests/golden/ can pin the plan compiler bit for bit.  The reference binds
// neither `exchange_regrouping`/`bend_regrouping` (tentorch/tensors/regroup.h:69-96) nor
// `layout_of` (tentorch/tensors/layout.h:52-54) to Python.
#include <torch/extension.h>

#include <memory>
#include <string>
#include <vector>

#include "symmetry/cat/abelian/abelian.h"
#include "symmetry/cat/fibonacci/fibonacci.h"
#include "symmetry/cat/su2/su2.h"
#include "tensors/layout.h"
#include "tensors/regroup.h"

namespace
{
  using LegSpec = std::vector<std::pair<std::vector<int64_t>, int64_t>>;

  std::shared_ptr<const sym::FusionCategory> category(const std::string &name)
  {
    if (name == "u1") return sym::u1_symmetry();
    if (name == "su2") return sym::su2_symmetry();
    if (name == "fibonacci") return sym::fibonacci_category();
    if (name == "no_symmetry") return sym::no_symmetry();
    if (name == "fermion_parity") return sym::fermion_parity();
    throw std::invalid_argument("unknown category " + name);
  }

  std::vector<sym::Leg> legs_of(const std::shared_ptr<const sym::FusionCategory> &cat,
                                const std::vector<LegSpec> &specs)
  {
    std::vector<sym::Leg> out;
    for (const LegSpec &spec : specs)
    {
      std::vector<sym::Sector> sectors;
      std::vector<int64_t> mult;
      for (const auto &[sector, m] : spec)
      {
        sectors.emplace_back(sector);
        mult.push_back(m);
      }
      out.emplace_back(cat, sectors, mult);
    }
    return out;
  }

  py::tuple sector_tuple(const sym::Sector &s)
  {
    py::tuple out(static_cast<size_t>(s.size()));
    for (int64_t i = 0; i < s.size(); ++i) out[static_cast<size_t>(i)] = py::int_(s[i]);
    return out;
  }

  py::list plan_list(const sym::Regrouping &plan)
  {
    py::list shifts;
    for (const sym::Shift &shift : plan.shifts)
    {
      py::list pieces;
      for (const sym::Piece &p : shift.pieces)
        pieces.append(py::make_tuple(p.first, p.last, p.from_step, p.to_step, p.run, p.coefficient.real(),
                                     p.coefficient.imag()));
      shifts.append(py::make_tuple(
        py::make_tuple(sector_tuple(shift.from.codomain), sector_tuple(shift.from.domain), shift.from.copy),
        py::make_tuple(sector_tuple(shift.to.codomain), sector_tuple(shift.to.domain), shift.to.copy),
        shift.rows, shift.columns, pieces));
    }
    return shifts;
  }

  // One step of a chain on one block: kind 0 exchanges codomain legs `arm`, `arm + 1`; kind 1
  // bends the last codomain leg down (arm 1) or the last domain leg up (arm 0).
  py::list step_plan(const std::string &cat_name, const std::vector<LegSpec> &codomain,
                     const std::vector<LegSpec> &domain, const std::vector<int64_t> &key_codomain,
                     const std::vector<int64_t> &key_domain, int64_t key_copy,
                     const std::vector<int64_t> &qtotal, int64_t kind, int64_t arm)
  {
    const auto cat = category(cat_name);
    const auto cod = legs_of(cat, codomain);
    const auto dom = legs_of(cat, domain);
    const sym::BlockKey key{sym::Sector(key_codomain), sym::Sector(key_domain), key_copy};
    const sym::Sector q(qtotal);
    if (kind == 0)
      return plan_list(sym::exchange_regrouping(cat, cod, dom, key, q, arm, sym::layouts()));
    return plan_list(sym::bend_regrouping(cat, cod, dom, key, q, arm == 1, sym::layouts()));
  }

  py::tuple side_layout(const std::string &cat_name, const std::vector<LegSpec> &legs,
                        const std::vector<int64_t> &root)
  {
    const auto cat = category(cat_name);
    const sym::SideLayout layout = sym::layout_of(*cat, legs_of(cat, legs), sym::Sector(root));
    py::list trees;
    for (const sym::FusionTree &tree : layout.trees)
    {
      py::list sectors, inner, copies;
      for (const auto &s : tree.sectors) sectors.append(sector_tuple(s));
      for (const auto &s : tree.inner) inner.append(sector_tuple(s));
      for (const int64_t c : tree.copies) copies.append(py::int_(c));
      trees.append(py::make_tuple(sectors, inner, copies, sector_tuple(tree.coupled)));
    }
    return py::make_tuple(trees, layout.offsets);
  }

  py::list keys_of(const std::string &cat_name, const std::vector<LegSpec> &codomain,
                   const std::vector<LegSpec> &domain, const std::vector<int64_t> &qtotal)
  {
    const auto cat = category(cat_name);
    py::list out;
    for (const sym::BlockKey &key :
         sym::block_keys(*cat, legs_of(cat, codomain), legs_of(cat, domain), sym::Sector(qtotal)))
      out.append(py::make_tuple(sector_tuple(key.codomain), sector_tuple(key.domain), key.copy));
    return out;
  }
} // namespace

PYBIND11_MODULE(TORCH_EXTENSION_NAME, m)
{
  m.def("step_plan", &step_plan);
  m.def("side_layout", &side_layout);
  m.def("block_keys", &keys_of);
}
