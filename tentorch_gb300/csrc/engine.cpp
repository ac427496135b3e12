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
#include <unordered_map>

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

  namespace
  {
    // Hashes and key checks of the per-leg-list caches below, computed in place (no key is
    // allocated for a lookup): the category, the legs by their interned numbers.
    void mix(uint64_t &h, uint64_t v) { h ^= v + 0x9e3779b97f4a7c15ull + (h << 6) + (h >> 2); }

    uint64_t legs_hash(const Category &cat, const std::vector<Leg> &legs)
    {
      uint64_t h = 0x9e3779b97f4a7c15ull ^ static_cast<uint64_t>(reinterpret_cast<uintptr_t>(&cat));
      for (const Leg &l : legs) mix(h, static_cast<uint64_t>(l->id));
      mix(h, static_cast<uint64_t>(legs.size()));
      return h;
    }

    bool same_legs(const std::vector<int32_t> &ids, const std::vector<Leg> &legs)
    {
      if (ids.size() != legs.size()) return false;
      for (size_t i = 0; i < legs.size(); ++i)
        if (ids[i] != legs[i]->id) return false;
      return true;
    }

    std::vector<int32_t> ids_of(const std::vector<Leg> &legs)
    {
      std::vector<int32_t> ids;
      ids.reserve(legs.size());
      for (const Leg &l : legs) ids.push_back(l->id);
      return ids;
    }

    struct ChargesEntry
    {
      const Category *cat;
      std::vector<int32_t> ids;
      std::vector<Sector> charges;
    };
  } // namespace

  // tentorch/symmetry/tree/tree.cpp:375-398: the charges the legs fuse to, in the order a fusion
  // from the first leg meets them; kept per list of legs (every space and every einsum's output
  // check asks for them).
  std::vector<Sector> reachable_charges(const Category &cat, const std::vector<Leg> &legs)
  {
    static std::unordered_map<uint64_t, std::vector<ChargesEntry>> cache;
    std::vector<ChargesEntry> &bucket = cache[legs_hash(cat, legs)];
    for (const ChargesEntry &e : bucket)
      if (e.cat == &cat && same_legs(e.ids, legs)) return e.charges;
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
    bucket.push_back(ChargesEntry{&cat, ids_of(legs), charges});
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

  namespace
  {
    // A cached layout with the key it was built for: the category, the legs (interned, by number)
    // and the root.
    struct LayoutEntry
    {
      const Category *cat;
      std::vector<int32_t> ids;
      Sector root;
      std::unique_ptr<Layout> layout;
    };

    uint64_t layout_hash(const Category &cat, const std::vector<Leg> &legs, const Sector &root)
    {
      uint64_t h = legs_hash(cat, legs);
      mix(h, static_cast<uint64_t>(root.size));
      for (int32_t i = 0; i < root.size; ++i) mix(h, static_cast<uint64_t>(root[i]));
      return h;
    }
  } // namespace

  // tentorch/tensors/layout.cpp:18-32, cached per (category, legs, root).  A lookup hashes the key
  // in place and compares it against the entries of its hash, with no allocation: compiling a
  // plan looks layouts up for every block it touches.
  const Layout &layout_of(const Category &cat, const std::vector<Leg> &legs, const Sector &root)
  {
    static std::unordered_map<uint64_t, std::vector<LayoutEntry>> cache;
    std::vector<LayoutEntry> &bucket = cache[layout_hash(cat, legs, root)];
    for (const LayoutEntry &e : bucket)
      if (e.cat == &cat && e.root == root && same_legs(e.ids, legs)) return *e.layout;
    LayoutEntry entry{&cat, ids_of(legs), root, std::make_unique<Layout>()};
    Layout *layout = entry.layout.get();
    layout->trees = fusion_trees(cat, legs, root);
    layout->offsets.push_back(0);
    layout->index.reserve(layout->trees.size() * legs.size());
    for (const Tree &t : layout->trees)
    {
      int64_t rows = 1;
      for (size_t axis = 0; axis < legs.size(); ++axis)
      {
        const int64_t at = legs[axis]->index_of(t.sectors[axis]);
        layout->index.push_back(static_cast<int32_t>(at));
        rows *= legs[axis]->mult[static_cast<size_t>(at)];
      }
      layout->offsets.push_back(layout->offsets.back() + rows);
    }
    bucket.push_back(std::move(entry));
    return *layout;
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
  //
  // One step of a leg move regroups the entries of one block of its `before` space into blocks of
  // its `after` space.  Its plan is, per target block, a list of pieces {first, last, from_step,
  // to_step, run, c}: target[last + i * to_step] += c * source[first + i * from_step] for i < run
  // (the reference's Piece / Shift of tentorch/tensors/regroup.h:22-60; the set of pieces of every
  // shift is the same as the reference's, checked piece by piece).  Both kinds of step touch one or
  // two vertices of a tree: each source tree is mapped to the trees it recouples into by building
  // those trees directly and looking them up in the target layout.

  namespace
  {
    // The charge the first n legs of a tree fuse to: trivial for no leg, the first sector for one,
    // the root for all of them, else the inner charge after leg n - 1.
    Sector fused_through(const Category &cat, const Tree &tree, int32_t n)
    {
      const int32_t legs = static_cast<int32_t>(tree.sectors.size());
      if (n <= 0) return cat.trivial();
      if (n >= legs) return tree.coupled;
      if (n == 1) return tree.sectors[0];
      return tree.inner[static_cast<size_t>(n - 2)];
    }

    // The multiplicity index of the vertex at which leg v (v >= 1) joins the legs before it; leg 0
    // joins nothing and reads 0.
    int32_t joining_copy(const Tree &tree, int32_t v) { return v >= 1 ? tree.copies[static_cast<size_t>(v - 1)] : 0; }

    int32_t find_index(const std::vector<FIndex> &list, const Sector &sector, int32_t inner, int32_t outer)
    {
      for (size_t i = 0; i < list.size(); ++i)
        if (list[i].sector == sector && list[i].inner == inner && list[i].outer == outer) return static_cast<int32_t>(i);
      return -1;
    }

    // A recoupling coefficient this small is a cancellation that should have been zero: the
    // entries of F, R and their products are of order one.
    constexpr double kNegligible = 1e-13;

    // The exchange of two adjacent legs b, c between the charges y (of the legs before them) and d
    // (of the legs through them), as a matrix from the local bracketings before the exchange (the
    // rows of F^d_{y b c}: inner charge e, the copies of y x b -> e and e x c -> d) to those after
    // it (the rows of F^d_{y c b}):  Q = F_{ycb} . B . F_{ybc}^dagger, where B carries the braiding
    // R_{bc} between the right bracketings (f, copy of b x c -> f, copy of y x f -> d) that share f
    // and the outer copy.
    Matrix exchange_matrix(const Category &cat, const Sector &y, const Sector &b, const Sector &c, const Sector &d)
    {
      const Matrix &before = cat.F(y, b, c, d);
      const Matrix &after = cat.F(y, c, b, d);
      const std::vector<FIndex> right_before = cat.f_columns(y, b, c, d);
      const std::vector<FIndex> right_after = cat.f_columns(y, c, b, d);
      const Matrix &braid = cat.R(b, c);
      // the row (or column) of the braiding that a fusion channel (f, copy) of b and c takes
      std::vector<std::pair<Sector, int32_t>> channel_start;
      int32_t start = 0;
      for (const Outcome &o : cat.outcomes(b, c))
      {
        channel_start.emplace_back(o.sector, start);
        start += o.multiplicity;
      }
      const auto channel = [&](const FIndex &index)
      {
        for (const auto &entry : channel_start)
          if (entry.first == index.sector) return entry.second + index.inner;
        return -1;
      };
      // middle[i][j]: from right bracketing j before the exchange to i after it
      const int32_t ni = static_cast<int32_t>(right_after.size()), nj = static_cast<int32_t>(right_before.size());
      std::vector<cplx> middle(static_cast<size_t>(ni) * nj, cplx(0.0, 0.0));
      for (int32_t i = 0; i < ni; ++i)
        for (int32_t j = 0; j < nj; ++j)
        {
          if (right_after[static_cast<size_t>(i)].sector != right_before[static_cast<size_t>(j)].sector ||
              right_after[static_cast<size_t>(i)].outer != right_before[static_cast<size_t>(j)].outer)
            continue;
          const int32_t row = channel(right_after[static_cast<size_t>(i)]), col = channel(right_before[static_cast<size_t>(j)]);
          if (row >= 0 && col >= 0) middle[static_cast<size_t>(i) * nj + j] = braid.at(row, col);
        }
      // carried[i][s] = sum_j middle[i][j] conj(before[s][j]), then Q[t][s] = sum_i after[t][i] carried[i][s]
      std::vector<cplx> carried(static_cast<size_t>(ni) * before.rows, cplx(0.0, 0.0));
      for (int32_t i = 0; i < ni; ++i)
        for (int32_t s = 0; s < before.rows; ++s)
        {
          cplx sum(0.0, 0.0);
          for (int32_t j = 0; j < nj; ++j)
          {
            const cplx m = middle[static_cast<size_t>(i) * nj + j];
            if (m != cplx(0.0, 0.0)) sum += m * std::conj(before.at(s, j));
          }
          carried[static_cast<size_t>(i) * before.rows + s] = sum;
        }
      Matrix q;
      q.rows = after.rows;
      q.cols = before.rows;
      q.v.assign(static_cast<size_t>(q.rows) * q.cols, cplx(0.0, 0.0));
      for (int32_t t = 0; t < q.rows; ++t)
        for (int32_t s = 0; s < q.cols; ++s)
        {
          cplx sum(0.0, 0.0);
          for (int32_t i = 0; i < ni; ++i) sum += after.at(t, i) * carried[static_cast<size_t>(i) * before.rows + s];
          q.v[static_cast<size_t>(t) * q.cols + s] = sum;
        }
      return q;
    }

    // Shifts kept by their target block while a bend builds them, handed out in key order.
    struct ShiftsByTarget
    {
      BlockKey source;
      std::map<BlockKey, Shift> held;
      std::vector<Piece> &into(const BlockKey &to, int64_t rows, int64_t cols)
      {
        auto it = held.find(to);
        if (it == held.end()) it = held.emplace(to, Shift{source, to, rows, cols, {}}).first;
        return it->second.pieces;
      }
      std::vector<Shift> take()
      {
        std::vector<Shift> out;
        out.reserve(held.size());
        for (auto &entry : held) out.push_back(std::move(entry.second));
        return out;
      }
    };
  } // namespace

  // Exchange of the codomain legs p and p + 1 of one block (the step of
  // tentorch/tensors/regroup.cpp:25-258).  A tree (legs a_0 .. a_n-1) changes only at the two
  // vertices where a_p and a_p+1 join; its images are the trees of the exchanged legs that agree
  // with it everywhere else, one per local bracketing after the exchange, with the coefficient of
  // exchange_matrix.  Entries keep their place in the row but for the two legs' copy digits, which
  // trade places: when either leg carries a single copy the whole tree moves as one run, otherwise
  // in runs over the copies of the legs after the pair.
  std::vector<Shift> exchange_plan(const Category &cat, const std::vector<Leg> &codomain,
                                   const std::vector<Leg> &domain, const BlockKey &key, const Sector &qtotal,
                                   int32_t p)
  {
    (void)qtotal;
    const int32_t legs = static_cast<int32_t>(codomain.size());
    std::vector<Leg> swapped = codomain;
    std::swap(swapped[static_cast<size_t>(p)], swapped[static_cast<size_t>(p + 1)]);
    const Layout &before = layout_of(cat, codomain, key.codomain);
    const Layout &after = layout_of(cat, swapped, key.codomain);
    const int64_t row_length = layout_of(cat, domain, key.domain).rows();
    Shift shift{key, key, 0, 0, {}};
    std::map<std::array<Sector, 4>, Matrix> local;  // exchange_matrix per (y, b, c, d)

    for (size_t s = 0; s < before.trees.size(); ++s)
    {
      const Tree &tree = before.trees[s];
      const Sector &b = tree.sectors[static_cast<size_t>(p)], &c = tree.sectors[static_cast<size_t>(p + 1)];
      const Sector y = fused_through(cat, tree, p), d = fused_through(cat, tree, p + 2);
      auto found = local.find({y, b, c, d});
      if (found == local.end()) found = local.emplace(std::array<Sector, 4>{y, b, c, d}, exchange_matrix(cat, y, b, c, d)).first;
      const Matrix &q = found->second;
      const int32_t column = find_index(cat.f_rows(y, b, c, d), fused_through(cat, tree, p + 1), joining_copy(tree, p),
                                        joining_copy(tree, p + 1));
      if (column < 0) throw LogicError("a tree of the codomain is not a bracketing of its F symbol");
      // the copies of the two legs, of the legs after them, and of the whole tree
      const int64_t mb = codomain[static_cast<size_t>(p)]->multiplicity_of(b);
      const int64_t mc = codomain[static_cast<size_t>(p + 1)]->multiplicity_of(c);
      int64_t tail = 1, width = 1;
      for (int32_t l = 0; l < legs; ++l)
      {
        const int64_t m = codomain[static_cast<size_t>(l)]->multiplicity_of(tree.sectors[static_cast<size_t>(l)]);
        width *= m;
        if (l > p + 1) tail *= m;
      }
      const std::vector<FIndex> images = cat.f_rows(y, c, b, d);
      for (size_t r = 0; r < images.size(); ++r)
      {
        const cplx coefficient = q.at(static_cast<int32_t>(r), column);
        if (std::abs(coefficient) <= kNegligible) continue;
        // the image: legs p and p + 1 swapped, the local bracketing of row r
        Tree image = tree;
        std::swap(image.sectors[static_cast<size_t>(p)], image.sectors[static_cast<size_t>(p + 1)]);
        if (p >= 1)
        {
          // the charge after the first of the pair and the copy of its vertex (with no leg before
          // the pair that charge is the first sector itself and the vertex has one copy)
          image.inner[static_cast<size_t>(p - 1)] = images[r].sector;
          image.copies[static_cast<size_t>(p - 1)] = images[r].inner;
        }
        image.copies[static_cast<size_t>(p)] = images[r].outer;
        const int32_t t = after.find(image);
        if (t < 0) throw LogicError("the exchange has no image for a tree of the codomain");
        const int64_t from = before.offsets[s], to = after.offsets[static_cast<size_t>(t)];
        // source copy digits (high, beta, gamma, low) land at (high, gamma, beta, low): runs of
        // `tail` entries, merged where the next one continues the last on both sides (always when
        // either leg carries one copy, and across the step from one high digit to the next)
        const size_t first_piece = shift.pieces.size();
        const int64_t highs = width / (mb * mc * tail);
        for (int64_t h = 0; h < highs; ++h)
          for (int64_t beta = 0; beta < mb; ++beta)
            for (int64_t gamma = 0; gamma < mc; ++gamma)
            {
              const int64_t src = (from + ((h * mb + beta) * mc + gamma) * tail) * row_length;
              const int64_t dst = (to + ((h * mc + gamma) * mb + beta) * tail) * row_length;
              if (shift.pieces.size() > first_piece)
              {
                Piece &last = shift.pieces.back();
                if (last.first + last.run == src && last.last + last.run == dst)
                {
                  last.run += tail * row_length;
                  continue;
                }
              }
              shift.pieces.push_back(Piece{src, dst, 1, 1, tail * row_length, coefficient});
            }
      }
    }
    return {std::move(shift)};
  }

  // Bend of the last leg of one side onto the end of the other, for one block (the step of
  // tentorch/tensors/regroup.cpp:260-417).  The giving tree loses the vertex where the leg joins it
  // (charge x of its other legs, copy mu), the taking tree gains a vertex for the leg, which it
  // reads as the dual sector.  With Q the total charge, the recoupling is one row (codomain to
  // domain) or column (domain to codomain) of F^Q: for a leg q bent down from codomain root r onto
  // domain root s, F^Q_{x q s-bar} at row (r, mu, block copy) gives per column (f, kappa, lambda)
  // the new domain root f-bar, the new vertex's copy kappa and the block copy lambda; for a leg
  // bent up from domain root s onto codomain root r, F^Q_{r q-bar x-bar} at column (s-bar, mu,
  // block copy) gives per row (e, kappa, lambda) the new codomain root e.  The leg's copies are
  // the fastest digit of the tree that gains it, so one piece carries the copies of the leg for
  // one entry of the other legs (bent down), or one entry of the taking tree and one copy carry the
  // whole kept tree (bent up).
  std::vector<Shift> bend_plan(const Category &cat, const std::vector<Leg> &codomain,
                               const std::vector<Leg> &domain, const BlockKey &key, const Sector &qtotal,
                               bool from_codomain)
  {
    const std::vector<Leg> &giving = from_codomain ? codomain : domain;
    const std::vector<Leg> &taking = from_codomain ? domain : codomain;
    const Leg leg = giving.back();
    // The bent leg keeps its blocks and its sector reads as the dual one on the other side, so the
    // copies of a sector land in the rows of its dual: the two have to carry the same multiplets.
    // The reference assumes it (tentorch/linalg/graded/svd.cpp:97-100) and writes past its blocks
    // when it does not hold; here it is an error.
    for (size_t b = 0; b < leg->sectors.size(); ++b)
    {
      const Sector d = cat.dual(leg->sectors[b]);
      const auto it = std::lower_bound(leg->sectors.begin(), leg->sectors.end(), d);
      if (it != leg->sectors.end() && *it == d && leg->mult[static_cast<size_t>(it - leg->sectors.begin())] != leg->mult[b])
        throw InvalidArgument("a leg bent across the tensor needs each sector and its dual to carry the same "
                              "multiplets, but " + leg->sectors[b].str() + " has " + std::to_string(leg->mult[b]) +
                              " and " + d.str() + " has " +
                              std::to_string(leg->mult[static_cast<size_t>(it - leg->sectors.begin())]));
    }
    std::vector<Leg> shorter(giving.begin(), giving.end() - 1), longer = taking;
    longer.push_back(leg);
    const std::vector<Leg> &new_codomain = from_codomain ? shorter : longer;
    const std::vector<Leg> &new_domain = from_codomain ? longer : shorter;
    const Sector &giving_root = from_codomain ? key.codomain : key.domain;
    const Sector &taking_root = from_codomain ? key.domain : key.codomain;
    const Layout &givers = layout_of(cat, giving, giving_root);
    const Layout &takers = layout_of(cat, taking, taking_root);
    const int64_t source_cols = (from_codomain ? takers : givers).rows();
    ShiftsByTarget shifts{key, {}};

    for (size_t g = 0; g < givers.trees.size(); ++g)
    {
      const Tree &tree = givers.trees[g];
      const int32_t n = static_cast<int32_t>(tree.sectors.size());
      const Sector q = tree.sectors.back();
      const Sector x = fused_through(cat, tree, n - 1);
      const int32_t mu = joining_copy(tree, n - 1);
      const int64_t copies = leg->multiplicity_of(q);
      const int64_t kept_width = (givers.offsets[g + 1] - givers.offsets[g]) / copies;
      const Tree kept = trimmed(cat, tree);
      // the F symbol of the bend, the index this tree names and the indices it may land on
      const Sector a = from_codomain ? x : taking_root;
      const Sector b = from_codomain ? q : cat.dual(q);
      const Sector c = from_codomain ? cat.dual(taking_root) : cat.dual(x);
      const Matrix &f = cat.F(a, b, c, qtotal);
      const std::vector<FIndex> rows = cat.f_rows(a, b, c, qtotal), cols = cat.f_columns(a, b, c, qtotal);
      const int32_t named = from_codomain ? find_index(rows, giving_root, mu, key.copy)
                                          : find_index(cols, cat.dual(giving_root), mu, key.copy);
      if (named < 0) continue;
      const std::vector<FIndex> &landings = from_codomain ? cols : rows;
      for (size_t l = 0; l < landings.size(); ++l)
      {
        const FIndex &land = landings[l];
        // F is square; the reference reads it at (named index, landing index) in both directions
        const cplx coefficient = f.at(named, static_cast<int32_t>(l));
        if (coefficient == cplx(0.0, 0.0)) continue;
        const Sector grown_root = from_codomain ? cat.dual(land.sector) : land.sector;
        const Sector &row_root = from_codomain ? x : grown_root, &col_root = from_codomain ? grown_root : x;
        const Layout &out_rows = layout_of(cat, new_codomain, row_root);
        const Layout &out_cols = layout_of(cat, new_domain, col_root);
        const int64_t out_cols_n = out_cols.rows();
        for (size_t t = 0; t < takers.trees.size(); ++t)
        {
          const Tree &taker = takers.trees[t];
          Tree grown = taker;
          grown.sectors.push_back(cat.dual(q));
          if (taker.sectors.size() >= 2) grown.inner.push_back(taking_root);
          if (taker.sectors.size() >= 1) grown.copies.push_back(land.inner);
          grown.coupled = grown_root;
          const int32_t kept_at = (from_codomain ? out_rows : out_cols).find(kept);
          const int32_t grown_at = (from_codomain ? out_cols : out_rows).find(grown);
          if (kept_at < 0 || grown_at < 0) continue;
          const int64_t kept_offset = (from_codomain ? out_rows : out_cols).offsets[static_cast<size_t>(kept_at)];
          const int64_t grown_offset = (from_codomain ? out_cols : out_rows).offsets[static_cast<size_t>(grown_at)];
          const int64_t taker_offset = takers.offsets[t], taker_width = takers.offsets[t + 1] - takers.offsets[t];
          std::vector<Piece> &pieces = shifts.into(BlockKey{row_root, col_root, land.outer}, out_rows.rows(), out_cols_n);
          if (from_codomain)
            // source (row givers.offsets[g] + i * copies + k, column taker_offset + e) lands at
            // (row kept_offset + i, column grown_offset + e * copies + k); a piece runs over k
            for (int64_t i = 0; i < kept_width; ++i)
              for (int64_t e = 0; e < taker_width; ++e)
                pieces.push_back(Piece{(givers.offsets[g] + i * copies) * source_cols + taker_offset + e,
                                       (kept_offset + i) * out_cols_n + grown_offset + e * copies, source_cols, 1, copies,
                                       coefficient});
          else
            // source (row taker_offset + e, column givers.offsets[g] + j * copies + k) lands at
            // (row grown_offset + e * copies + k, column kept_offset + j); a piece runs over j
            for (int64_t e = 0; e < taker_width; ++e)
              for (int64_t k = 0; k < copies; ++k)
                pieces.push_back(Piece{(taker_offset + e) * source_cols + givers.offsets[g] + k,
                                       (grown_offset + e * copies + k) * out_cols_n + kept_offset, copies, 1, kept_width,
                                       coefficient});
        }
      }
    }
    return shifts.take();
  }

  // The leading domain legs a place leaves where they are: the longest prefix of `below` that
  // names the domain legs in their own order, or none when a codomain leg goes below (then every
  // domain leg is lifted before the sort).
  int32_t chain_kept(int32_t height, int32_t depth, const std::vector<int32_t> &below)
  {
    if (std::any_of(below.begin(), below.end(), [height](int32_t leg) { return leg < height; })) return 0;
    const int32_t limit = std::min<int32_t>(depth, static_cast<int32_t>(below.size()));
    int32_t kept = 0;
    while (kept < limit && below[static_cast<size_t>(kept)] == height + kept) ++kept;
    return kept;
  }

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

  // The steps of a place (the sequence tentorch/tensors/place.cpp:199-247 takes), tracking the legs
  // of each side by their number in `space`: (1) every domain leg behind the kept prefix is bent
  // up, the last first; (2) the codomain is brought to `above` followed by the legs that go below
  // (after the kept ones) last named first, each slot filled from left to right by exchanging its
  // leg leftwards one position at a time; (3) the tail of the codomain is bent down, the last leg
  // first, which lands the domain in the named order.
  std::vector<Step> chain(Space space, const std::vector<int32_t> &above, const std::vector<int32_t> &below)
  {
    const int32_t height = static_cast<int32_t>(space->codomain.size());
    const int32_t depth = static_cast<int32_t>(space->domain.size());
    check_place(space, above, below);
    const int32_t kept = chain_kept(height, depth, below);
    const std::vector<Leg> legs = space->legs();
    std::vector<int32_t> top(static_cast<size_t>(height)), bottom(static_cast<size_t>(depth));
    std::iota(top.begin(), top.end(), 0);
    std::iota(bottom.begin(), bottom.end(), height);
    std::vector<Step> steps;
    Space current = space;
    const auto record = [&](int32_t kind, int32_t arm)
    {
      std::vector<Leg> cod, dom;
      for (const int32_t l : top) cod.push_back(legs[static_cast<size_t>(l)]);
      for (const int32_t l : bottom) dom.push_back(legs[static_cast<size_t>(l)]);
      Space next = make_space(space->cat, std::move(cod), std::move(dom), space->qtotal);
      steps.push_back(Step{kind, arm, current, next});
      current = next;
    };
    while (static_cast<int32_t>(bottom.size()) > kept)
    {
      top.push_back(bottom.back());
      bottom.pop_back();
      record(2, 0);
    }
    std::vector<int32_t> wanted = above;
    wanted.insert(wanted.end(), below.rbegin(), below.rend() - kept);
    for (size_t slot = 0; slot < wanted.size(); ++slot)
    {
      size_t at = static_cast<size_t>(std::find(top.begin() + static_cast<std::ptrdiff_t>(slot), top.end(), wanted[slot]) - top.begin());
      for (; at > slot; --at)
      {
        std::swap(top[at - 1], top[at]);
        record(0, static_cast<int32_t>(at - 1));
      }
    }
    for (size_t n = static_cast<size_t>(kept); n < below.size(); ++n)
    {
      bottom.push_back(top.back());
      top.pop_back();
      record(1, 0);
    }
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
