// Host side of the GB300 block-sparse contraction engine: symmetry categories, legs, fusion trees,
// side layouts, tensor spaces (block keys and their places in one device arena) and the per-step
// regrouping plans of a leg move.  Everything here is host C++ with no CUDA dependency; the plan
// compiler (program.h) turns these into device descriptors that the kernels (kernels.cu) execute.
//
// The conventions that decide where an entry of a block lives follow the reference engine
// (Jumqyc/TenTorch) exactly, because the engine is a drop-in for it:
//   sector order        tentorch/symmetry/cat/cat.h:121-130 (lexicographic, shorter first)
//   tree enumeration     tentorch/symmetry/tree/tree.cpp:400-471 (DFS: leg blocks x outcomes x copies)
//   row offsets          tentorch/tensors/layout.cpp:18-32 (mixed radix, last leg fastest)
//   block keys           tentorch/tensors/layout.cpp:34-47 then std::map order
//   exchange / bend      tentorch/tensors/regroup.cpp:25-417
#pragma once

#include <array>
#include <complex>
#include <cstdint>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <vector>

namespace ttg
{
  using cplx = std::complex<double>;

  // Raised for a malformed request; the C ABI maps it to status TT_EINVAL (Python ValueError).
  struct InvalidArgument : std::invalid_argument
  {
    using std::invalid_argument::invalid_argument;
  };
  // Raised for a lookup outside a tensor (Python IndexError).
  struct OutOfRange : std::out_of_range
  {
    using std::out_of_range::out_of_range;
  };
  // Raised when an internal invariant fails (Python RuntimeError).
  struct LogicError : std::logic_error
  {
    using std::logic_error::logic_error;
  };

  // ------------------------------------------------------------------------------------------
  // sectors and categories
  // ------------------------------------------------------------------------------------------

  // A simple object of a category: up to four integer labels held inline.
  struct Sector
  {
    int32_t size = 0;
    std::array<int64_t, 4> q{};

    Sector() = default;
    Sector(std::initializer_list<int64_t> values);
    static Sector of(const int64_t *values, int32_t n);
    int64_t operator[](int32_t i) const { return q[static_cast<size_t>(i)]; }
    bool operator==(const Sector &o) const
    {
      if (size != o.size) return false;
      for (int32_t i = 0; i < size; ++i)
        if (q[static_cast<size_t>(i)] != o.q[static_cast<size_t>(i)]) return false;
      return true;
    }
    bool operator!=(const Sector &o) const { return !(*this == o); }
    // tentorch/symmetry/cat/cat.h:121-130: lexicographic, the shorter first when one is a prefix.
    bool operator<(const Sector &o) const
    {
      const int32_t common = size < o.size ? size : o.size;
      for (int32_t i = 0; i < common; ++i)
        if (q[static_cast<size_t>(i)] != o.q[static_cast<size_t>(i)]) return q[static_cast<size_t>(i)] < o.q[static_cast<size_t>(i)];
      return size < o.size;
    }
    std::string str() const;
  };

  struct Outcome
  {
    Sector sector;
    int32_t multiplicity;
  };

  // One row or column of an F symbol: the inner sector and the two vertex indices.
  struct FIndex
  {
    Sector sector;
    int32_t inner;
    int32_t outer;
  };

  // A small dense complex matrix, row major.
  struct Matrix
  {
    int32_t rows = 0, cols = 0;
    std::vector<cplx> v;
    cplx at(int32_t r, int32_t c) const { return v[static_cast<size_t>(r) * cols + c]; }
  };

  enum class CategoryKind : int32_t
  {
    no_symmetry = 0,
    u1 = 1,
    su2 = 2,
    fibonacci = 3,
    z_n = 4,
    fermion_parity = 5,
  };

  class Category
  {
  public:
    Category(CategoryKind kind, int64_t param);
    CategoryKind kind() const { return kind_; }
    int64_t param() const { return param_; }
    const std::string &name() const { return name_; }
    int32_t rank() const { return 1; }

    const std::vector<Outcome> &outcomes(const Sector &a, const Sector &b) const;
    int32_t n_symbol(const Sector &a, const Sector &b, const Sector &c) const;
    Sector dual(const Sector &a) const;
    Sector trivial() const { return Sector{0}; }
    double q_dim(const Sector &a) const;
    // Whether every F and R symbol is real (a float64 tensor is exact under it).
    bool real_symbols() const { return kind_ != CategoryKind::fibonacci; }
    // Whether F = R = 1 on every allowed vertex (abelian groups), so a move is a permutation.
    bool trivial_symbols() const;
    bool valid(const Sector &a) const;

    std::vector<FIndex> f_rows(const Sector &a, const Sector &b, const Sector &c, const Sector &d) const;
    std::vector<FIndex> f_columns(const Sector &a, const Sector &b, const Sector &c, const Sector &d) const;
    const Matrix &F(const Sector &a, const Sector &b, const Sector &c, const Sector &d) const;
    const Matrix &R(const Sector &b, const Sector &c) const;

  private:
    std::vector<Outcome> compute_outcomes(const Sector &a, const Sector &b) const;
    Matrix compute_F(const Sector &a, const Sector &b, const Sector &c, const Sector &d) const;
    Matrix compute_R(const Sector &b, const Sector &c) const;

    CategoryKind kind_;
    int64_t param_;
    std::string name_;
    mutable std::map<std::pair<Sector, Sector>, std::vector<Outcome>> outcomes_;
    // the same cache for single-label sectors with labels in 32 bits, keyed by the packed pair
    mutable std::unordered_map<uint64_t, std::vector<Outcome>> outcomes_packed_;
    mutable std::map<std::array<Sector, 4>, Matrix> f_;
    mutable std::map<std::pair<Sector, Sector>, Matrix> r_;
  };

  // The process-wide category of a kind (and modulus for Z_N), created on first use.
  const Category *category(CategoryKind kind, int64_t param = 0);

  // ------------------------------------------------------------------------------------------
  // legs, trees, layouts
  // ------------------------------------------------------------------------------------------

  // A graded space: sorted distinct sectors, each with a positive multiplicity.  Legs are interned,
  // so two legs over the same space are the same object and compare by pointer.
  struct LegData
  {
    const Category *cat;
    std::vector<Sector> sectors;
    std::vector<int64_t> mult;
    int32_t id;

    int64_t multiplicity_of(const Sector &s) const;
    int64_t index_of(const Sector &s) const;
    int64_t multiplets() const;
  };
  using Leg = const LegData *;

  // Intern a leg (sorting its blocks); raises InvalidArgument on repeats or non-positive counts.
  Leg make_leg(const Category *cat, std::vector<Sector> sectors, std::vector<int64_t> mult);
  Leg leg_by_id(int32_t id);
  std::string render(const std::vector<Sector> &sectors);

  struct Tree
  {
    std::vector<Sector> sectors;
    std::vector<Sector> inner;
    std::vector<int32_t> copies;
    Sector coupled;
    bool operator==(const Tree &o) const;
    bool operator<(const Tree &o) const;
  };

  std::vector<Sector> reachable_charges(const Category &cat, const std::vector<Leg> &legs);
  std::vector<Tree> fusion_trees(const Category &cat, const std::vector<Leg> &legs, const Sector &coupled);
  Tree trimmed(const Category &cat, const Tree &tree);

  // Trees of one side at one root and the first row of each (the last entry is the row count).
  struct Layout
  {
    std::vector<Tree> trees;
    std::vector<int64_t> offsets;
    std::vector<int32_t> index;  // per tree, the sector index of each leg on that leg (tree t at t * legs)
    int64_t rows() const { return offsets.back(); }
    // trees keyed for the lookups a bend makes, built on first use
    mutable std::map<Tree, int32_t> position;
    int32_t find(const Tree &t) const;
  };
  const Layout &layout_of(const Category &cat, const std::vector<Leg> &legs, const Sector &root);

  // ------------------------------------------------------------------------------------------
  // spaces: the shape of a tensor and where its blocks sit in one arena
  // ------------------------------------------------------------------------------------------

  struct BlockKey
  {
    Sector codomain;
    Sector domain;
    int32_t copy = 0;
    bool operator<(const BlockKey &o) const;
    bool operator==(const BlockKey &o) const;
  };

  struct Block
  {
    BlockKey key;
    int64_t rows;
    int64_t cols;
    int64_t offset;  // first element in the arena; every block starts on a 16-byte boundary
  };

  struct SpaceData
  {
    const Category *cat;
    std::vector<Leg> codomain;
    std::vector<Leg> domain;
    Sector qtotal;
    std::vector<Block> blocks;  // BlockKey order
    int64_t size;               // arena elements, padding included
    int32_t id;

    int32_t find(const BlockKey &key) const;  // -1 when absent
    std::vector<Leg> legs() const;
    int32_t nlegs() const { return static_cast<int32_t>(codomain.size() + domain.size()); }
  };
  using Space = const SpaceData *;

  std::vector<BlockKey> block_keys(const Category &cat, const std::vector<Leg> &codomain,
                                   const std::vector<Leg> &domain, const Sector &qtotal);
  Space make_space(const Category *cat, std::vector<Leg> codomain, std::vector<Leg> domain, Sector qtotal);
  Space space_by_id(int32_t id);

  // ------------------------------------------------------------------------------------------
  // per-step regrouping plans (the reference's Piece / Shift, tentorch/tensors/regroup.h:22-60)
  // ------------------------------------------------------------------------------------------

  struct Piece
  {
    int64_t first, last, from_step, to_step, run;
    cplx coefficient;
  };

  struct Shift
  {
    BlockKey from, to;
    int64_t rows, cols;
    std::vector<Piece> pieces;
  };

  std::vector<Shift> exchange_plan(const Category &cat, const std::vector<Leg> &codomain,
                                   const std::vector<Leg> &domain, const BlockKey &key, const Sector &qtotal,
                                   int32_t p);
  std::vector<Shift> bend_plan(const Category &cat, const std::vector<Leg> &codomain,
                               const std::vector<Leg> &domain, const BlockKey &key, const Sector &qtotal,
                               bool from_codomain);

  // One step of a leg move: kind 0 exchanges codomain legs arm, arm+1; kind 1 bends the last
  // codomain leg down; kind 2 bends the last domain leg up.  `after` is the space it lands in.
  struct Step
  {
    int32_t kind;
    int32_t arm;
    Space before;
    Space after;
  };
  // The chain of tentorch/tensors/place.cpp:199-247: fold the domain tail up, bubble sort, fold down.
  std::vector<Step> chain(Space space, const std::vector<int32_t> &above, const std::vector<int32_t> &below);
  // Raise the reference's errors for a place that does not name every leg exactly once.
  void check_place(Space space, const std::vector<int32_t> &above, const std::vector<int32_t> &below);
  // The space a place lands in (the chain's last space), without the spaces in between.
  Space placed_space(Space space, const std::vector<int32_t> &above, const std::vector<int32_t> &below);
  // Whether a place (already checked) leaves every leg where it is: the chain has no step.
  bool place_is_identity(Space space, const std::vector<int32_t> &above, const std::vector<int32_t> &below);
  // The leading domain legs the chain leaves in place: the others are bent up first, and every leg
  // of below[kept:] is bent down last.
  int32_t chain_kept(int32_t height, int32_t depth, const std::vector<int32_t> &below);

  // All shifts of one step for one block of its `before` space, cached.
  const std::vector<Shift> &step_plan(const Step &step, const BlockKey &key);

} // namespace ttg
