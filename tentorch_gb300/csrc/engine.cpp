// Host side of the engine: categories, legs, trees, layouts, spaces and per-step plans.
// See engine.h for the conventions, each of which follows the reference (file:line cited there and
// at each function below), because the block layout is the contract of the drop-in.
#include "engine.h"

#include <algorithm>
#include <cmath>
#include <functional>
#include <mutex>
#include <numeric>
#include <set>
#include <tuple>

namespace ttg
{
  // ------------------------------------------------------------------------------------------
  // sectors
  // ------------------------------------------------------------------------------------------

  Sector::Sector(std::initializer_list<int64_t> values)
  {
    if (values.size() > 4) throw InvalidArgument("a sector holds at most 4 labels");
    size = static_cast<int32_t>(values.size());
    std::copy(values.begin(), values.end(), q.begin());
  }

  Sector Sector::of(const int64_t *values, int32_t n)
  {
    if (n < 0 || n > 4) throw InvalidArgument("a sector holds at most 4 labels");
    Sector s;
    s.size = n;
    for (int32_t i = 0; i < n; ++i) s.q[static_cast<size_t>(i)] = values[i];
    return s;
  }

  std::string Sector::str() const
  {
    std::string out = "(";
    for (int32_t i = 0; i < size; ++i)
    {
      if (i) out += ", ";
      out += std::to_string(q[static_cast<size_t>(i)]);
    }
    if (size == 1) out += ",";
    return out + ")";
  }

  std::string render(const std::vector<Sector> &sectors)
  {
    std::string out = "[";
    for (size_t i = 0; i < sectors.size(); ++i) out += (i ? ", " : "") + sectors[i].str();
    return out + "]";
  }

  // ------------------------------------------------------------------------------------------
  // categories
  // ------------------------------------------------------------------------------------------

  namespace
  {
    int64_t residue(int64_t x, int64_t m)
    {
      const int64_t r = x % m;
      return r < 0 ? r + m : r;
    }

    double golden_ratio() { return (1.0 + std::sqrt(5.0)) / 2.0; }

    // log(n!) table is not exact enough for the 6j sum; n! itself in double is exact to 22! and
    // correctly rounded beyond, which keeps the Racah sum accurate for the spins a tensor carries.
    double factorial(int64_t n)
    {
      static std::vector<double> table = []
      {
        std::vector<double> t(171, 1.0);
        for (size_t i = 1; i < t.size(); ++i) t[i] = t[i - 1] * static_cast<double>(i);
        return t;
      }();
      if (n < 0 || n > 170) throw InvalidArgument("a spin too large for the 6j table");
      return table[static_cast<size_t>(n)];
    }

    // Delta(a, b, c) of doubled spins: sqrt((a+b-c)!(a-b+c)!(-a+b+c)!/(a+b+c+1)!) with halves.
    double triangle(int64_t a, int64_t b, int64_t c)
    {
      return std::sqrt(factorial((a + b - c) / 2) * factorial((a - b + c) / 2) * factorial((-a + b + c) / 2) /
                       factorial((a + b + c) / 2 + 1));
    }

    bool admissible(int64_t a, int64_t b, int64_t c)
    {
      return a + b >= c && a + c >= b && b + c >= a && (a + b + c) % 2 == 0;
    }

    // The Wigner 6j symbol {j1 j2 j3; j4 j5 j6} of doubled spins, by Racah's single-sum formula
    // (G. Racah, Phys. Rev. 62, 438 (1942)).
    double six_j(int64_t j1, int64_t j2, int64_t j3, int64_t j4, int64_t j5, int64_t j6)
    {
      if (!admissible(j1, j2, j3) || !admissible(j1, j5, j6) || !admissible(j4, j2, j6) || !admissible(j4, j5, j3))
        return 0.0;
      const int64_t a1 = (j1 + j2 + j3) / 2, a2 = (j1 + j5 + j6) / 2, a3 = (j4 + j2 + j6) / 2,
                    a4 = (j4 + j5 + j3) / 2;
      const int64_t b1 = (j1 + j2 + j4 + j5) / 2, b2 = (j2 + j3 + j5 + j6) / 2, b3 = (j3 + j1 + j6 + j4) / 2;
      const int64_t lo = std::max({a1, a2, a3, a4}), hi = std::min({b1, b2, b3});
      double sum = 0.0;
      for (int64_t t = lo; t <= hi; ++t)
      {
        const double term = factorial(t + 1) /
                            (factorial(t - a1) * factorial(t - a2) * factorial(t - a3) * factorial(t - a4) *
                             factorial(b1 - t) * factorial(b2 - t) * factorial(b3 - t));
        sum += (t % 2 ? -term : term);
      }
      return triangle(j1, j2, j3) * triangle(j1, j5, j6) * triangle(j4, j2, j6) * triangle(j4, j5, j3) * sum;
    }
  } // namespace

  Category::Category(CategoryKind kind, int64_t param) : kind_(kind), param_(param)
  {
    switch (kind)
    {
    case CategoryKind::no_symmetry: name_ = "NoSymmetry"; break;
    case CategoryKind::u1: name_ = "U(1)"; break;
    case CategoryKind::su2: name_ = "SU(2)"; break;
    case CategoryKind::fibonacci: name_ = "FibonacciCategory"; break;
    case CategoryKind::z_n:
      if (param <= 0) throw InvalidArgument("The modulus of Z_N must be positive, not " + std::to_string(param) + ".");
      name_ = "Z_" + std::to_string(param);
      break;
    case CategoryKind::fermion_parity: name_ = "FermionParity"; break;
    }
  }

  bool Category::trivial_symbols() const
  {
    return kind_ == CategoryKind::no_symmetry || kind_ == CategoryKind::u1 || kind_ == CategoryKind::z_n;
  }

  bool Category::valid(const Sector &a) const
  {
    if (a.size != 1) return false;
    if (kind_ == CategoryKind::su2) return a[0] >= 0;
    return q_dim(a) > 0.0;
  }

  // tentorch/symmetry/cat/abelian/abelian.cpp:33-35,69-92,100-102; su2/su2.cpp:24-30;
  // fibonacci/fibonacci.cpp:24-28 — the order of the list is part of the contract.
  std::vector<Outcome> Category::compute_outcomes(const Sector &a, const Sector &b) const
  {
    switch (kind_)
    {
    case CategoryKind::no_symmetry: return {{Sector{0}, 1}};
    case CategoryKind::u1: return {{Sector{a[0] + b[0]}, 1}};
    case CategoryKind::z_n: return {{Sector{residue(a[0] + b[0], param_)}, 1}};
    case CategoryKind::fermion_parity: return {{Sector{residue(a[0] + b[0], 2)}, 1}};
    case CategoryKind::su2:
    {
      std::vector<Outcome> out;
      for (int64_t jj = std::llabs(a[0] - b[0]); jj <= a[0] + b[0]; jj += 2) out.push_back({Sector{jj}, 1});
      return out;
    }
    case CategoryKind::fibonacci:
      if (a[0] == 0) return {{b, 1}};
      if (b[0] == 0) return {{a, 1}};
      return {{Sector{0}, 1}, {Sector{1}, 1}};
    }
    return {};
  }

  const std::vector<Outcome> &Category::outcomes(const Sector &a, const Sector &b) const
  {
    if (a.size == 1 && b.size == 1 && a[0] == static_cast<int32_t>(a[0]) && b[0] == static_cast<int32_t>(b[0]))
    {
      const uint64_t packed = (static_cast<uint64_t>(static_cast<uint32_t>(a[0])) << 32) | static_cast<uint32_t>(b[0]);
      auto hit = outcomes_packed_.find(packed);
      if (hit == outcomes_packed_.end()) hit = outcomes_packed_.emplace(packed, compute_outcomes(a, b)).first;
      return hit->second;
    }
    const auto k = std::make_pair(a, b);
    auto found = outcomes_.find(k);
    if (found == outcomes_.end()) found = outcomes_.emplace(k, compute_outcomes(a, b)).first;
    return found->second;
  }

  int32_t Category::n_symbol(const Sector &a, const Sector &b, const Sector &c) const
  {
    for (const Outcome &o : outcomes(a, b))
      if (o.sector == c) return o.multiplicity;
    return 0;
  }

  Sector Category::dual(const Sector &a) const
  {
    switch (kind_)
    {
    case CategoryKind::no_symmetry: return Sector{0};
    case CategoryKind::u1: return Sector{-a[0]};
    case CategoryKind::z_n: return Sector{residue(-a[0], param_)};
    default: return a;
    }
  }

  double Category::q_dim(const Sector &a) const
  {
    if (kind_ == CategoryKind::su2) return static_cast<double>(a[0] + 1);
    if (kind_ == CategoryKind::fibonacci) return a[0] == 1 ? golden_ratio() : 1.0;
    return 1.0;
  }

  // tentorch/symmetry/cat/cat.cpp:61-77
  std::vector<FIndex> Category::f_rows(const Sector &a, const Sector &b, const Sector &c, const Sector &d) const
  {
    std::vector<FIndex> rows;
    for (const Outcome &e : outcomes(a, b))
    {
      const int32_t copies = n_symbol(e.sector, c, d);
      for (int32_t inner = 0; inner < e.multiplicity; ++inner)
        for (int32_t outer = 0; outer < copies; ++outer) rows.push_back({e.sector, inner, outer});
    }
    return rows;
  }

  // tentorch/symmetry/cat/cat.cpp:79-95
  std::vector<FIndex> Category::f_columns(const Sector &a, const Sector &b, const Sector &c, const Sector &d) const
  {
    std::vector<FIndex> cols;
    for (const Outcome &f : outcomes(b, c))
    {
      const int32_t copies = n_symbol(a, f.sector, d);
      for (int32_t inner = 0; inner < f.multiplicity; ++inner)
        for (int32_t outer = 0; outer < copies; ++outer) cols.push_back({f.sector, inner, outer});
    }
    return cols;
  }

  Matrix Category::compute_F(const Sector &a, const Sector &b, const Sector &c, const Sector &d) const
  {
    const std::vector<FIndex> rows = f_rows(a, b, c, d), cols = f_columns(a, b, c, d);
    Matrix m;
    m.rows = static_cast<int32_t>(rows.size());
    m.cols = static_cast<int32_t>(cols.size());
    m.v.assign(static_cast<size_t>(m.rows) * m.cols, cplx(0.0, 0.0));
    if (m.rows == 0 || m.cols == 0) return m;
    switch (kind_)
    {
    case CategoryKind::fermion_parity:
    {
      // tentorch/symmetry/cat/abelian/abelian.cpp:104-110: 1 when d is the fused parity
      const int32_t side = residue(a[0] + b[0] + c[0], 2) == d[0] ? 1 : 0;
      m.rows = m.cols = side;
      m.v.assign(static_cast<size_t>(side * side), cplx(1.0, 0.0));
      return m;
    }
    case CategoryKind::su2:
    {
      // The overlap of the two bracketings of Condon-Shortley vertices, divided by d_d
      // (tentorch/symmetry/cat/group.cpp:44-83), is the recoupling coefficient
      // (-1)^(a+b+c+d) sqrt((2e+1)(2f+1)) {a b e; c d f}.
      for (int32_t i = 0; i < m.rows; ++i)
        for (int32_t j = 0; j < m.cols; ++j)
        {
          const int64_t e = rows[static_cast<size_t>(i)].sector[0], f = cols[static_cast<size_t>(j)].sector[0];
          const int64_t phase = (a[0] + b[0] + c[0] + d[0]) / 2;
          const double value = (phase % 2 ? -1.0 : 1.0) * std::sqrt(static_cast<double>((e + 1) * (f + 1))) *
                               six_j(a[0], b[0], e, c[0], d[0], f);
          m.v[static_cast<size_t>(i) * m.cols + j] = cplx(value, 0.0);
        }
      return m;
    }
    case CategoryKind::fibonacci:
    {
      // tentorch/symmetry/cat/fibonacci/fibonacci.cpp:30-52: the golden matrix on tau tau tau -> tau
      if (a[0] == 1 && b[0] == 1 && c[0] == 1 && d[0] == 1)
      {
        const double phi = golden_ratio();
        const double golden[2][2] = {{1.0 / phi, 1.0 / std::sqrt(phi)}, {1.0 / std::sqrt(phi), -1.0 / phi}};
        for (int32_t i = 0; i < m.rows; ++i)
          for (int32_t j = 0; j < m.cols; ++j)
            m.v[static_cast<size_t>(i) * m.cols + j] =
              golden[rows[static_cast<size_t>(i)].sector[0]][cols[static_cast<size_t>(j)].sector[0]];
        return m;
      }
      std::fill(m.v.begin(), m.v.end(), cplx(1.0, 0.0));
      return m;
    }
    default:
      // an abelian group: every vertex is the entry 1, so the overlap is 1 (group.cpp:44-83)
      std::fill(m.v.begin(), m.v.end(), cplx(1.0, 0.0));
      return m;
    }
  }

  Matrix Category::compute_R(const Sector &b, const Sector &c) const
  {
    std::vector<Sector> rows;
    for (const Outcome &e : outcomes(b, c))
      for (int32_t k = 0; k < e.multiplicity; ++k) rows.push_back(e.sector);
    Matrix m;
    m.rows = m.cols = static_cast<int32_t>(rows.size());
    m.v.assign(static_cast<size_t>(m.rows) * m.cols, cplx(0.0, 0.0));
    for (int32_t i = 0; i < m.rows; ++i)
    {
      cplx phase(1.0, 0.0);
      const Sector &e = rows[static_cast<size_t>(i)];
      if (kind_ == CategoryKind::su2)
        phase = ((b[0] + c[0] - e[0]) / 2) % 2 ? cplx(-1.0, 0.0) : cplx(1.0, 0.0);  // group.cpp:93-130
      else if (kind_ == CategoryKind::fermion_parity)
        phase = b[0] == 1 && c[0] == 1 ? cplx(-1.0, 0.0) : cplx(1.0, 0.0);  // abelian.cpp:112-117
      else if (kind_ == CategoryKind::fibonacci && b[0] == 1 && c[0] == 1)
        phase = std::polar(1.0, e[0] == 0 ? -4.0 * M_PI / 5.0 : 3.0 * M_PI / 5.0);  // fibonacci.cpp:54-69
      m.v[static_cast<size_t>(i) * m.cols + i] = phase;
    }
    return m;
  }

  const Matrix &Category::F(const Sector &a, const Sector &b, const Sector &c, const Sector &d) const
  {
    const std::array<Sector, 4> k{a, b, c, d};
    auto found = f_.find(k);
    if (found == f_.end()) found = f_.emplace(k, compute_F(a, b, c, d)).first;
    return found->second;
  }

  const Matrix &Category::R(const Sector &b, const Sector &c) const
  {
    const auto k = std::make_pair(b, c);
    auto found = r_.find(k);
    if (found == r_.end()) found = r_.emplace(k, compute_R(b, c)).first;
    return found->second;
  }

  const Category *category(CategoryKind kind, int64_t param)
  {
    static std::map<std::pair<int32_t, int64_t>, std::unique_ptr<Category>> held;
    if (kind != CategoryKind::z_n) param = 0;
    auto &slot = held[{static_cast<int32_t>(kind), param}];
    if (!slot) slot = std::make_unique<Category>(kind, param);
    return slot.get();
  }

  // ------------------------------------------------------------------------------------------
  // legs
  // ------------------------------------------------------------------------------------------

  namespace
  {
    struct LegRegistry
    {
      std::map<std::tuple<const Category *, std::vector<Sector>, std::vector<int64_t>>, int32_t> index;
      std::vector<std::unique_ptr<LegData>> legs;
    };
    LegRegistry &leg_registry()
    {
      static LegRegistry r;
      return r;
    }
  } // namespace

  int64_t LegData::index_of(const Sector &s) const
  {
    const auto it = std::lower_bound(sectors.begin(), sectors.end(), s);
    if (it == sectors.end() || !(*it == s))
      throw InvalidArgument("a leg of " + std::to_string(sectors.size()) + " blocks carries none in sector " + s.str());
    return it - sectors.begin();
  }

  int64_t LegData::multiplicity_of(const Sector &s) const { return mult[static_cast<size_t>(index_of(s))]; }

  int64_t LegData::multiplets() const { return std::accumulate(mult.begin(), mult.end(), int64_t{0}); }

  // tentorch/symmetry/tree/tree.cpp:90-140: sorted, distinct, positive, every sector valid.
  Leg make_leg(const Category *cat, std::vector<Sector> sectors, std::vector<int64_t> mult)
  {
    if (!cat) throw InvalidArgument("A leg needs a category.");
    if (sectors.size() != mult.size())
      throw InvalidArgument("A leg needs one multiplicity per sector, got " + std::to_string(mult.size()) + " for " +
                            std::to_string(sectors.size()) + " sectors.");
    for (int64_t m : mult)
      if (m <= 0) throw InvalidArgument("A block multiplicity must be positive, got " + std::to_string(m) + ".");
    std::vector<size_t> order(sectors.size());
    std::iota(order.begin(), order.end(), 0);
    std::sort(order.begin(), order.end(), [&](size_t a, size_t b) { return sectors[a] < sectors[b]; });
    std::vector<Sector> s2;
    std::vector<int64_t> m2;
    for (size_t i : order)
    {
      s2.push_back(sectors[i]);
      m2.push_back(mult[i]);
    }
    for (size_t i = 1; i < s2.size(); ++i)
      if (s2[i] == s2[i - 1]) throw InvalidArgument("A leg cannot hold the sector " + s2[i].str() + " twice.");
    for (const Sector &s : s2)
      if (!cat->valid(s)) throw InvalidArgument("The sector " + s.str() + " has no components in " + cat->name() + ".");
    LegRegistry &reg = leg_registry();
    auto key = std::make_tuple(cat, s2, m2);
    const auto found = reg.index.find(key);
    if (found != reg.index.end()) return reg.legs[static_cast<size_t>(found->second)].get();
    auto leg = std::make_unique<LegData>();
    leg->cat = cat;
    leg->sectors = std::move(s2);
    leg->mult = std::move(m2);
    leg->id = static_cast<int32_t>(reg.legs.size());
    reg.index.emplace(std::move(key), leg->id);
    reg.legs.push_back(std::move(leg));
    return reg.legs.back().get();
  }

  Leg leg_by_id(int32_t id)
  {
    LegRegistry &reg = leg_registry();
    if (id < 0 || static_cast<size_t>(id) >= reg.legs.size()) throw InvalidArgument("no leg " + std::to_string(id));
    return reg.legs[static_cast<size_t>(id)].get();
  }

  // ------------------------------------------------------------------------------------------
  // trees and layouts
  // ------------------------------------------------------------------------------------------

  bool Tree::operator==(const Tree &o) const
  {
    return sectors == o.sectors && inner == o.inner && copies == o.copies && coupled == o.coupled;
  }

  bool Tree::operator<(const Tree &o) const
  {
    return std::tie(sectors, inner, copies, coupled) < std::tie(o.sectors, o.inner, o.copies, o.coupled);
  }

  // tentorch/symmetry/tree/tree.cpp:375-398
  std::vector<Sector> reachable_charges(const Category &cat, const std::vector<Leg> &legs)
  {
    std::vector<Sector> charges{cat.trivial()};
    for (Leg leg : legs)
    {
      std::vector<Sector> next;
      std::set<Sector> seen;
      for (const Sector &charge : charges)
        for (const Sector &s : leg->sectors)
          for (const Outcome &o : cat.outcomes(charge, s))
            if (seen.insert(o.sector).second) next.push_back(o.sector);
      charges = std::move(next);
    }
    return charges;
  }

  // tentorch/symmetry/tree/tree.cpp:400-471: depth first over the blocks of each leg, the
  // outcomes of each vertex in category order, and the copies of each outcome.
  std::vector<Tree> fusion_trees(const Category &cat, const std::vector<Leg> &legs, const Sector &coupled)
  {
    const size_t n = legs.size();
    std::vector<Tree> out;
    if (n == 0)
    {
      if (coupled == cat.trivial()) out.push_back(Tree{{}, {}, {}, coupled});
      return out;
    }
    // The walk below visits the trees in the reference's order; it only enters a partial fusion
    // that can still reach `coupled` through the legs left, found by one pass forward (the
    // partial fusions there are) and one backward (those that reach the root).
    std::vector<std::set<Sector>> alive(n + 1);
    {
      // the partial fusions after each leg depend on the legs only: kept per list of legs
      static std::map<std::pair<const Category *, std::vector<int32_t>>, std::vector<std::set<Sector>>> reaches;
      std::vector<int32_t> ids;
      for (Leg l : legs) ids.push_back(l->id);
      auto found = reaches.find({&cat, ids});
      if (found == reaches.end())
      {
        std::vector<std::set<Sector>> r(n + 1);
        r[1].insert(legs[0]->sectors.begin(), legs[0]->sectors.end());
        for (size_t k = 1; k < n; ++k)
          for (const Sector &x : r[k])
            for (const Sector &s : legs[k]->sectors)
              for (const Outcome &o : cat.outcomes(x, s)) r[k + 1].insert(o.sector);
        found = reaches.emplace(std::make_pair(&cat, std::move(ids)), std::move(r)).first;
      }
      const std::vector<std::set<Sector>> &reach = found->second;
      if (reach[n].count(coupled)) alive[n].insert(coupled);
      for (size_t k = n - 1; k >= 1; --k)
        for (const Sector &x : reach[k])
        {
          bool reaches = false;
          for (size_t j = 0; j < legs[k]->sectors.size() && !reaches; ++j)
            for (const Outcome &o : cat.outcomes(x, legs[k]->sectors[j]))
              if (alive[k + 1].count(o.sector))
              {
                reaches = true;
                break;
              }
          if (reaches) alive[k].insert(x);
        }
    }
    if (alive[n].empty()) return out;
    Tree tree;
    tree.sectors.resize(n);
    tree.inner.resize(n >= 2 ? n - 2 : 0);
    tree.copies.resize(n >= 2 ? n - 1 : 0);
    tree.coupled = coupled;
    std::function<void(size_t, const Sector &)> walk = [&](size_t leg, const Sector &previous)
    {
      for (const Sector &s : legs[leg]->sectors)
      {
        tree.sectors[leg] = s;
        if (leg == 0)
        {
          if (n == 1)
          {
            if (s == coupled) out.push_back(tree);
          }
          else if (alive[1].count(s))
            walk(1, s);
          continue;
        }
        for (const Outcome &o : cat.outcomes(previous, s))
        {
          if (leg + 1 == n && !(o.sector == coupled)) continue;
          if (leg + 1 < n && !alive[leg + 1].count(o.sector)) continue;
          if (leg + 1 < n) tree.inner[leg - 1] = o.sector;
          for (int32_t copy = 0; copy < o.multiplicity; ++copy)
          {
            tree.copies[leg - 1] = copy;
            if (leg + 1 == n)
              out.push_back(tree);
            else
              walk(leg + 1, o.sector);
          }
        }
      }
    };
    walk(0, cat.trivial());
    return out;
  }

  // tentorch/symmetry/tree/tree.cpp:473-484
  Tree trimmed(const Category &cat, const Tree &tree)
  {
    Tree out = tree;
    out.sectors.pop_back();
    if (!out.inner.empty()) out.inner.pop_back();
    if (!out.copies.empty()) out.copies.pop_back();
    const size_t n = tree.sectors.size();
    out.coupled = n <= 1 ? cat.trivial() : n == 2 ? tree.sectors[0] : tree.inner[n - 3];
    return out;
  }

  int32_t Layout::find(const Tree &t) const
  {
    if (position.empty())
      for (size_t i = 0; i < trees.size(); ++i) position.emplace(trees[i], static_cast<int32_t>(i));
    const auto it = position.find(t);
    return it == position.end() ? -1 : it->second;
  }

  // tentorch/tensors/layout.cpp:18-32, cached per (category, legs, root)
  const Layout &layout_of(const Category &cat, const std::vector<Leg> &legs, const Sector &root)
  {
    static std::map<std::tuple<const Category *, std::vector<int32_t>, Sector>, std::unique_ptr<Layout>> cache;
    std::vector<int32_t> ids;
    for (Leg l : legs) ids.push_back(l->id);
    auto key = std::make_tuple(&cat, std::move(ids), root);
    auto found = cache.find(key);
    if (found != cache.end()) return *found->second;
    auto layout = std::make_unique<Layout>();
    layout->trees = fusion_trees(cat, legs, root);
    layout->offsets.push_back(0);
    for (const Tree &t : layout->trees)
    {
      int64_t rows = 1;
      for (size_t axis = 0; axis < legs.size(); ++axis) rows *= legs[axis]->multiplicity_of(t.sectors[axis]);
      layout->offsets.push_back(layout->offsets.back() + rows);
    }
    return *cache.emplace(std::move(key), std::move(layout)).first->second;
  }

  // ------------------------------------------------------------------------------------------
  // spaces
  // ------------------------------------------------------------------------------------------

  bool BlockKey::operator<(const BlockKey &o) const
  {
    return std::tie(codomain, domain, copy) < std::tie(o.codomain, o.domain, o.copy);
  }

  bool BlockKey::operator==(const BlockKey &o) const
  {
    return codomain == o.codomain && domain == o.domain && copy == o.copy;
  }

  // tentorch/tensors/layout.cpp:34-47
  std::vector<BlockKey> block_keys(const Category &cat, const std::vector<Leg> &codomain,
                                   const std::vector<Leg> &domain, const Sector &qtotal)
  {
    std::vector<BlockKey> keys;
    const std::vector<Sector> out_roots = reachable_charges(cat, codomain);
    const std::vector<Sector> in_roots = reachable_charges(cat, domain);
    for (const Sector &r : out_roots)
      for (const Sector &s : in_roots)
        for (int32_t copy = 0; copy < cat.n_symbol(r, cat.dual(s), qtotal); ++copy) keys.push_back({r, s, copy});
    return keys;
  }

  namespace
  {
    struct SpaceRegistry
    {
      std::map<std::tuple<const Category *, std::vector<int32_t>, std::vector<int32_t>, Sector>, int32_t> index;
      std::vector<std::unique_ptr<SpaceData>> spaces;
    };
    SpaceRegistry &space_registry()
    {
      static SpaceRegistry r;
      return r;
    }
  } // namespace

  int32_t SpaceData::find(const BlockKey &key) const
  {
    const auto it = std::lower_bound(blocks.begin(), blocks.end(), key,
                                     [](const Block &b, const BlockKey &k) { return b.key < k; });
    if (it == blocks.end() || !(it->key == key)) return -1;
    return static_cast<int32_t>(it - blocks.begin());
  }

  std::vector<Leg> SpaceData::legs() const
  {
    std::vector<Leg> out = codomain;
    out.insert(out.end(), domain.begin(), domain.end());
    return out;
  }

  // The blocks of tentorch/tensors/tensor.cpp:23-61 in std::map order, each given a place in one
  // arena: packed in key order, every block starting on a 16-byte boundary.
  Space make_space(const Category *cat, std::vector<Leg> codomain, std::vector<Leg> domain, Sector qtotal)
  {
    for (Leg l : codomain)
      if (l->cat != cat) throw InvalidArgument("a codomain leg is over a different category");
    for (Leg l : domain)
      if (l->cat != cat) throw InvalidArgument("a domain leg is over a different category");
    std::vector<int32_t> cids, dids;
    for (Leg l : codomain) cids.push_back(l->id);
    for (Leg l : domain) dids.push_back(l->id);
    SpaceRegistry &reg = space_registry();
    auto key = std::make_tuple(cat, cids, dids, qtotal);
    const auto found = reg.index.find(key);
    if (found != reg.index.end()) return reg.spaces[static_cast<size_t>(found->second)].get();
    auto space = std::make_unique<SpaceData>();
    space->cat = cat;
    space->codomain = std::move(codomain);
    space->domain = std::move(domain);
    space->qtotal = qtotal;
    std::vector<BlockKey> keys = block_keys(*cat, space->codomain, space->domain, qtotal);
    std::sort(keys.begin(), keys.end());
    keys.erase(std::unique(keys.begin(), keys.end()), keys.end());
    int64_t offset = 0;
    for (const BlockKey &k : keys)
    {
      const int64_t rows = layout_of(*cat, space->codomain, k.codomain).rows();
      const int64_t cols = layout_of(*cat, space->domain, k.domain).rows();
      space->blocks.push_back({k, rows, cols, offset});
      offset += (rows * cols + 1) / 2 * 2;
    }
    space->size = offset;
    space->id = static_cast<int32_t>(reg.spaces.size());
    reg.index.emplace(std::move(key), space->id);
    reg.spaces.push_back(std::move(space));
    return reg.spaces.back().get();
  }

  Space space_by_id(int32_t id)
  {
    SpaceRegistry &reg = space_registry();
    if (id < 0 || static_cast<size_t>(id) >= reg.spaces.size()) throw InvalidArgument("no space " + std::to_string(id));
    return reg.spaces[static_cast<size_t>(id)].get();
  }

  // ------------------------------------------------------------------------------------------
  // per-step plans
  // ------------------------------------------------------------------------------------------

  namespace
  {
    // tentorch/tensors/regroup.cpp:16-22
    Sector chain_at(const Category &cat, const Tree &tree, int64_t last)
    {
      if (last < 0) return cat.trivial();
      if (last + 1 == static_cast<int64_t>(tree.sectors.size())) return tree.coupled;
      if (last == 0) return tree.sectors[0];
      return tree.inner[static_cast<size_t>(last - 1)];
    }

    void push_sector(std::vector<int64_t> &out, const Sector &s)
    {
      for (int32_t i = 0; i < s.size; ++i) out.push_back(s[i]);
    }
  } // namespace

  // tentorch/tensors/regroup.cpp:25-258: the trees that agree outside the pair recouple by
  // F^d_{ycb} R_{bc} (F^d_{ybc})^dagger; classes of equal multiplicity shape move as digit
  // permutations of the width index, coalesced into runs.
  std::vector<Shift> exchange_plan(const Category &cat, const std::vector<Leg> &codomain,
                                   const std::vector<Leg> &domain, const BlockKey &key, const Sector &qtotal,
                                   int32_t p)
  {
    (void)qtotal;
    const int32_t count = static_cast<int32_t>(codomain.size());
    std::vector<Leg> exchanged = codomain;
    std::swap(exchanged[static_cast<size_t>(p)], exchanged[static_cast<size_t>(p + 1)]);
    const Layout &source = layout_of(cat, codomain, key.codomain);
    const Layout &target = layout_of(cat, exchanged, key.codomain);
    const int64_t stride = layout_of(cat, domain, key.domain).rows();
    std::vector<Shift> plan;
    plan.push_back(Shift{key, key, 0, 0, {}});

    const auto signature = [&](const Tree &tree, bool exchanged_tree)
    {
      std::vector<int64_t> out;
      for (int32_t axis = 0; axis < count; ++axis)
      {
        const int32_t from = exchanged_tree && (axis == p || axis == p + 1) ? (axis == p ? p + 1 : p) : axis;
        push_sector(out, tree.sectors[static_cast<size_t>(from)]);
      }
      for (int32_t at = 0; at < static_cast<int32_t>(tree.inner.size()); ++at)
        if (at != p - 1) push_sector(out, tree.inner[static_cast<size_t>(at)]);
      for (int32_t at = 0; at < static_cast<int32_t>(tree.copies.size()); ++at)
        if (at != p - 1 && at != p) out.push_back(tree.copies[static_cast<size_t>(at)]);
      return out;
    };
    const auto moved = [p](int32_t axis) { return axis == p ? p + 1 : axis == p + 1 ? p : axis; };
    const auto shape_of = [&](const Tree &tree, const std::vector<Leg> &legs)
    {
      std::vector<int64_t> out;
      for (int32_t axis = 0; axis < count; ++axis)
        out.push_back(legs[static_cast<size_t>(axis)]->multiplicity_of(tree.sectors[static_cast<size_t>(axis)]));
      return out;
    };

    std::map<std::vector<int64_t>, std::vector<int32_t>> groups, partners;
    for (size_t at = 0; at < source.trees.size(); ++at)
      groups[signature(source.trees[at], false)].push_back(static_cast<int32_t>(at));
    for (size_t at = 0; at < target.trees.size(); ++at)
      partners[signature(target.trees[at], true)].push_back(static_cast<int32_t>(at));

    std::map<std::pair<int32_t, int32_t>, cplx> factors;
    for (const auto &[marks, olds] : groups)
    {
      const auto found = partners.find(marks);
      if (found == partners.end()) throw LogicError("the exchange has no image for a tree of the codomain");
      const std::vector<int32_t> &news = found->second;
      const Tree &sample = source.trees[static_cast<size_t>(olds.front())];
      const Sector y = chain_at(cat, sample, p - 1);
      const Sector d = chain_at(cat, sample, p + 1);
      const Sector &b = sample.sectors[static_cast<size_t>(p)];
      const Sector &c = sample.sectors[static_cast<size_t>(p + 1)];
      const Matrix &straight = cat.F(y, b, c, d);
      const Matrix &braided = cat.F(y, c, b, d);
      if (straight.rows != static_cast<int32_t>(olds.size()) || braided.rows != static_cast<int32_t>(news.size()))
        throw LogicError("the exchange does not match the trees of the block");
      std::vector<std::pair<Sector, int32_t>> offset;
      int32_t at = 0;
      for (const Outcome &o : cat.outcomes(b, c))
      {
        offset.emplace_back(o.sector, at);
        at += o.multiplicity;
      }
      const std::vector<FIndex> from = cat.f_columns(y, b, c, d);
      const std::vector<FIndex> to = cat.f_columns(y, c, b, d);
      const Matrix &braid = cat.R(b, c);
      const auto braid_at = [&](const FIndex &index) -> int32_t
      {
        for (const auto &[sector, start] : offset)
          if (sector == index.sector) return start + index.inner;
        return -1;
      };
      struct Term
      {
        int32_t i, braid_row, braid_col, j;
      };
      std::vector<Term> terms;
      for (size_t i = 0; i < to.size(); ++i)
      {
        const int32_t r = braid_at(to[i]);
        if (r < 0) continue;
        for (size_t j = 0; j < from.size(); ++j)
        {
          const int32_t cc = braid_at(from[j]);
          if (cc < 0) continue;
          if (!(to[i].sector == from[j].sector) || to[i].outer != from[j].outer) continue;
          terms.push_back({static_cast<int32_t>(i), r, cc, static_cast<int32_t>(j)});
        }
      }
      for (size_t one = 0; one < news.size(); ++one)
        for (size_t other = 0; other < olds.size(); ++other)
        {
          cplx value(0.0, 0.0);
          for (const Term &t : terms)
            value += braided.at(static_cast<int32_t>(one), t.i) * braid.at(t.braid_row, t.braid_col) *
                     std::conj(straight.at(static_cast<int32_t>(other), t.j));
          if (value.real() == 0.0 && value.imag() == 0.0) continue;
          factors.emplace(std::make_pair(news[one], olds[other]), value);
        }
    }

    std::map<std::vector<int64_t>, std::vector<int32_t>> before_classes, after_classes;
    std::vector<std::vector<int64_t>> after_shapes(target.trees.size());
    for (size_t at = 0; at < source.trees.size(); ++at)
      before_classes[shape_of(source.trees[at], codomain)].push_back(static_cast<int32_t>(at));
    for (size_t at = 0; at < target.trees.size(); ++at)
    {
      const std::vector<int64_t> shape = shape_of(target.trees[at], exchanged);
      std::vector<int64_t> back(shape.size(), 0);
      for (int32_t axis = 0; axis < count; ++axis) back[static_cast<size_t>(moved(axis))] = shape[static_cast<size_t>(axis)];
      after_shapes[at] = shape;
      after_classes[back].push_back(static_cast<int32_t>(at));
    }
    std::vector<Piece> &pieces = plan.back().pieces;
    std::vector<int64_t> width_of, digits(static_cast<size_t>(count)), placed(static_cast<size_t>(count));
    for (const auto &[shape, olds] : before_classes)
    {
      const auto partner = after_classes.find(shape);
      if (partner == after_classes.end()) throw LogicError("the exchange has no image for a block of trees");
      const std::vector<int32_t> &news = partner->second;
      int64_t width = 1;
      for (int64_t f : shape) width *= f;
      const std::vector<int64_t> &target_shape = after_shapes[static_cast<size_t>(news.front())];
      width_of.assign(static_cast<size_t>(width), 0);
      for (int64_t at = 0; at < width; ++at)
      {
        int64_t left = at;
        for (int32_t axis = count - 1; axis >= 0; --axis)
        {
          digits[static_cast<size_t>(axis)] = left % shape[static_cast<size_t>(axis)];
          left /= shape[static_cast<size_t>(axis)];
        }
        for (int32_t axis = 0; axis < count; ++axis) placed[static_cast<size_t>(moved(axis))] = digits[static_cast<size_t>(axis)];
        int64_t index = 0;
        for (int32_t axis = 0; axis < count; ++axis)
          index = index * target_shape[static_cast<size_t>(axis)] + placed[static_cast<size_t>(axis)];
        width_of[static_cast<size_t>(at)] = index;
      }
      for (const int32_t one : news)
        for (const int32_t other : olds)
        {
          const auto factor = factors.find(std::make_pair(one, other));
          if (factor == factors.end()) continue;
          for (int64_t at = 0; at < width;)
          {
            int64_t run = 1;
            while (at + run < width && width_of[static_cast<size_t>(at + run)] == width_of[static_cast<size_t>(at)] + run) ++run;
            pieces.push_back(Piece{(source.offsets[static_cast<size_t>(other)] + at) * stride,
                                   (target.offsets[static_cast<size_t>(one)] + width_of[static_cast<size_t>(at)]) * stride,
                                   1, 1, run * stride, factor->second});
            at += run;
          }
        }
    }
    return plan;
  }

  // tentorch/tensors/regroup.cpp:260-417: the giving side loses its last vertex, the taking side
  // gains one, and F^q(first, middle, last) carries the copies of the bent leg across; the bent
  // leg's sector reads as its dual on the other side.
  std::vector<Shift> bend_plan(const Category &cat, const std::vector<Leg> &codomain,
                               const std::vector<Leg> &domain, const BlockKey &key, const Sector &qtotal,
                               bool from_codomain)
  {
    const std::vector<Leg> &giving = from_codomain ? codomain : domain;
    const std::vector<Leg> &taking = from_codomain ? domain : codomain;
    const Leg moved_leg = giving.back();
    // The bent leg keeps its blocks and its sector reads as the dual one on the other side, so the
    // copies of a sector land in the rows of its dual: the two have to carry the same multiplets.
    // The reference assumes it (tentorch/linalg/graded/svd.cpp:97-100) and writes past its blocks
    // when it does not hold; here it is an error.
    for (size_t b = 0; b < moved_leg->sectors.size(); ++b)
    {
      const Sector d = cat.dual(moved_leg->sectors[b]);
      const auto it = std::lower_bound(moved_leg->sectors.begin(), moved_leg->sectors.end(), d);
      if (it != moved_leg->sectors.end() && *it == d &&
          moved_leg->mult[static_cast<size_t>(it - moved_leg->sectors.begin())] != moved_leg->mult[b])
        throw InvalidArgument("a leg bent across the tensor needs each sector and its dual to carry the same "
                              "multiplets, but " + moved_leg->sectors[b].str() + " has " +
                              std::to_string(moved_leg->mult[b]) + " and " + d.str() + " has " +
                              std::to_string(moved_leg->mult[static_cast<size_t>(it - moved_leg->sectors.begin())]));
    }
    const std::vector<Leg> kept_giving(giving.begin(), giving.end() - 1);
    std::vector<Leg> kept_taking = taking;
    kept_taking.push_back(moved_leg);
    const std::vector<Leg> &out_codomain = from_codomain ? kept_giving : kept_taking;
    const std::vector<Leg> &out_domain = from_codomain ? kept_taking : kept_giving;
    const Layout &moved_side = layout_of(cat, from_codomain ? codomain : domain, from_codomain ? key.codomain : key.domain);
    const Layout &gains_side = layout_of(cat, from_codomain ? domain : codomain, from_codomain ? key.domain : key.codomain);
    const Sector moved_root = from_codomain ? key.codomain : key.domain;
    const Sector gains_root = from_codomain ? key.domain : key.codomain;
    const int64_t source_stride = (from_codomain ? gains_side : moved_side).rows();

    std::vector<Shift> plan;
    std::map<BlockKey, size_t> at_of;
    std::map<std::pair<Sector, Sector>, std::pair<const Layout *, const Layout *>> out_layouts;
    const auto index_of = [&](const BlockKey &to, int64_t rows, int64_t cols) -> size_t
    {
      const auto found = at_of.find(to);
      if (found != at_of.end()) return found->second;
      const size_t index = plan.size();
      at_of.emplace(to, index);
      plan.push_back(Shift{key, to, rows, cols, {}});
      return index;
    };

    for (size_t gains_at = 0; gains_at < gains_side.trees.size(); ++gains_at)
    {
      const Tree &gains_tree = gains_side.trees[gains_at];
      const int64_t gains = gains_side.offsets[gains_at + 1] - gains_side.offsets[gains_at];
      for (size_t moved_at = 0; moved_at < moved_side.trees.size(); ++moved_at)
      {
        const Tree &moved_tree = moved_side.trees[moved_at];
        const Sector charge = moved_tree.sectors.back();
        const int64_t copies = moved_leg->multiplicity_of(charge);
        const int64_t span = moved_side.offsets[moved_at + 1] - moved_side.offsets[moved_at];
        const int64_t inside = span / copies;
        const Tree kept_tree = trimmed(cat, moved_tree);
        const Sector prefix = kept_tree.coupled;
        const int32_t copy = moved_tree.sectors.size() >= 2 ? moved_tree.copies.back() : 0;
        const Sector first = from_codomain ? prefix : gains_root;
        const Sector middle = from_codomain ? charge : cat.dual(charge);
        const Sector last = from_codomain ? cat.dual(gains_root) : cat.dual(prefix);
        const Matrix &coefficients = cat.F(first, middle, last, qtotal);
        const std::vector<FIndex> across = cat.f_rows(first, middle, last, qtotal);
        const std::vector<FIndex> along = cat.f_columns(first, middle, last, qtotal);
        const std::vector<FIndex> &named = from_codomain ? across : along;
        const std::vector<FIndex> &free = from_codomain ? along : across;
        const Sector named_root = from_codomain ? moved_root : cat.dual(moved_root);
        std::vector<int32_t> taken;
        for (size_t at = 0; at < named.size(); ++at)
          if (named[at].sector == named_root && named[at].inner == copy && named[at].outer == key.copy)
            taken.push_back(static_cast<int32_t>(at));
        if (taken.empty()) continue;
        const int64_t source_row = moved_side.offsets[moved_at];
        const int64_t source_column = gains_side.offsets[gains_at];
        for (const int32_t index : taken)
          for (size_t column = 0; column < free.size(); ++column)
          {
            const FIndex &taken_side = free[column];
            // entry [index * width + column] of the row-major matrix (regroup.cpp:350)
            const cplx value = coefficients.v[static_cast<size_t>(index) * coefficients.cols + column];
            if (value.real() == 0.0 && value.imag() == 0.0) continue;
            const Sector extended_root = from_codomain ? cat.dual(taken_side.sector) : taken_side.sector;
            Tree extended = gains_tree;
            extended.sectors.push_back(cat.dual(charge));
            if (gains_tree.sectors.size() >= 2) extended.inner.push_back(gains_root);
            if (gains_tree.sectors.size() >= 1) extended.copies.push_back(taken_side.inner);
            extended.coupled = extended_root;
            const Sector out_codomain_root = from_codomain ? prefix : extended_root;
            const Sector out_domain_root = from_codomain ? extended_root : prefix;
            const auto roots = std::make_pair(out_codomain_root, out_domain_root);
            auto found = out_layouts.find(roots);
            if (found == out_layouts.end())
              found = out_layouts
                        .emplace(roots, std::make_pair(&layout_of(cat, out_codomain, out_codomain_root),
                                                       &layout_of(cat, out_domain, out_domain_root)))
                        .first;
            const Layout &rows_layout = *found->second.first;
            const Layout &cols_layout = *found->second.second;
            const int32_t row_at = rows_layout.find(from_codomain ? kept_tree : extended);
            const int32_t column_at = cols_layout.find(from_codomain ? extended : kept_tree);
            if (row_at < 0 || column_at < 0) continue;
            const int64_t row = rows_layout.offsets[static_cast<size_t>(row_at)];
            const int64_t column_offset = cols_layout.offsets[static_cast<size_t>(column_at)];
            const int64_t target_stride = cols_layout.rows();
            std::vector<Piece> &pieces =
              plan[index_of(BlockKey{out_codomain_root, out_domain_root, taken_side.outer}, rows_layout.rows(),
                            cols_layout.rows())]
                .pieces;
            if (from_codomain)
            {
              for (int64_t shifted = 0; shifted < inside; ++shifted)
                for (int64_t gain = 0; gain < gains; ++gain)
                  pieces.push_back(Piece{(source_row + shifted * copies) * source_stride + source_column + gain,
                                         (row + shifted) * target_stride + column_offset + gain * copies,
                                         source_stride, 1, copies, value});
            }
            else
            {
              for (int64_t gain = 0; gain < gains; ++gain)
                for (int64_t copy_at = 0; copy_at < copies; ++copy_at)
                  pieces.push_back(Piece{(source_column + gain) * source_stride + source_row + copy_at,
                                         (row + gain * copies + copy_at) * target_stride + column_offset, copies, 1,
                                         inside, value});
            }
          }
      }
    }
    return plan;
  }

  // tentorch/tensors/place.cpp:199-214: the leading domain legs a place leaves where they are
  // (none when a codomain leg goes below)
  int32_t chain_kept(int32_t height, int32_t depth, const std::vector<int32_t> &below)
  {
    bool descends = false;
    for (size_t at = 0; !descends && at < below.size(); ++at) descends = below[at] < height;
    int32_t kept = 0;
    while (!descends && kept < depth && kept < static_cast<int32_t>(below.size()) &&
           below[static_cast<size_t>(kept)] == height + kept)
      ++kept;
    return kept;
  }

  // tentorch/tensors/place.cpp:41-107,199-247
  // tentorch/tensors/place.cpp:183-197: every leg named exactly once
  void check_place(Space space, const std::vector<int32_t> &above, const std::vector<int32_t> &below)
  {
    const int32_t total = space->nlegs();
    std::vector<bool> named(static_cast<size_t>(total), false);
    for (const std::vector<int32_t> *side : {&above, &below})
      for (const int32_t leg : *side)
      {
        if (leg < 0 || leg >= total)
          throw InvalidArgument("the leg " + std::to_string(leg) + " does not exist, the tensor has " +
                                std::to_string(total) + " legs");
        if (named[static_cast<size_t>(leg)]) throw InvalidArgument("the leg " + std::to_string(leg) + " is named twice");
        named[static_cast<size_t>(leg)] = true;
      }
    if (static_cast<int32_t>(above.size() + below.size()) != total)
    {
      int32_t left_out = 0;
      while (named[static_cast<size_t>(left_out)]) ++left_out;
      throw InvalidArgument("the leg " + std::to_string(left_out) + " is named on neither side");
    }
  }

  Space placed_space(Space space, const std::vector<int32_t> &above, const std::vector<int32_t> &below)
  {
    check_place(space, above, below);
    const std::vector<Leg> legs = space->legs();
    std::vector<Leg> cod, dom;
    for (const int32_t l : above) cod.push_back(legs[static_cast<size_t>(l)]);
    for (const int32_t l : below) dom.push_back(legs[static_cast<size_t>(l)]);
    return make_space(space->cat, std::move(cod), std::move(dom), space->qtotal);
  }

  bool place_is_identity(Space space, const std::vector<int32_t> &above, const std::vector<int32_t> &below)
  {
    const int32_t height = static_cast<int32_t>(space->codomain.size());
    if (static_cast<int32_t>(above.size()) != height) return false;
    for (int32_t i = 0; i < height; ++i)
      if (above[static_cast<size_t>(i)] != i) return false;
    for (size_t j = 0; j < below.size(); ++j)
      if (below[j] != height + static_cast<int32_t>(j)) return false;
    return true;
  }

  std::vector<Step> chain(Space space, const std::vector<int32_t> &above, const std::vector<int32_t> &below)
  {
    const int32_t height = static_cast<int32_t>(space->codomain.size());
    const int32_t depth = static_cast<int32_t>(space->domain.size());
    check_place(space, above, below);
    std::vector<Step> steps;
    std::vector<Leg> cod = space->codomain, dom = space->domain;
    Space current = space;
    const auto add = [&](int32_t kind, int32_t arm)
    {
      Space next = make_space(space->cat, cod, dom, space->qtotal);
      steps.push_back(Step{kind, arm, current, next});
      current = next;
    };
    const auto fold = [&](bool from_codomain)
    {
      if (from_codomain)
      {
        dom.push_back(cod.back());
        cod.pop_back();
      }
      else
      {
        cod.push_back(dom.back());
        dom.pop_back();
      }
      add(from_codomain ? 1 : 2, 0);
    };
    const int32_t kept = chain_kept(height, depth, below);
    for (int32_t at = kept; at < depth; ++at) fold(false);
    const auto position_of = [height, depth](int32_t leg)
    { return leg < height ? leg : height + (depth - 1 - (leg - height)); };
    std::vector<int32_t> order;
    for (const int32_t leg : above) order.push_back(position_of(leg));
    for (auto leg = below.rbegin(); leg != below.rend() - kept; ++leg) order.push_back(position_of(*leg));
    std::vector<int32_t> which(cod.size());
    std::iota(which.begin(), which.end(), 0);
    for (int32_t at = 0; at < static_cast<int32_t>(order.size()); ++at)
    {
      int32_t from = at;
      while (which[static_cast<size_t>(from)] != order[static_cast<size_t>(at)]) ++from;
      while (from > at)
      {
        std::swap(cod[static_cast<size_t>(from - 1)], cod[static_cast<size_t>(from)]);
        add(0, from - 1);
        std::swap(which[static_cast<size_t>(from - 1)], which[static_cast<size_t>(from)]);
        --from;
      }
    }
    for (int32_t at = kept; at < static_cast<int32_t>(below.size()); ++at) fold(true);
    return steps;
  }

  const std::vector<Shift> &step_plan(const Step &step, const BlockKey &key)
  {
    static std::map<std::tuple<int32_t, int32_t, int32_t, BlockKey>, std::vector<Shift>> cache;
    auto name = std::make_tuple(step.before->id, step.kind, step.arm, key);
    auto found = cache.find(name);
    if (found != cache.end()) return found->second;
    Space s = step.before;
    std::vector<Shift> plan = step.kind == 0 ? exchange_plan(*s->cat, s->codomain, s->domain, key, s->qtotal, step.arm)
                                             : bend_plan(*s->cat, s->codomain, s->domain, key, s->qtotal, step.kind == 1);
    return cache.emplace(std::move(name), std::move(plan)).first->second;
  }

} // namespace ttg
