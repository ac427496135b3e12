// The plan compiler: place / contract / einsum -> device program (see program.h).
#include "program.h"

#include "gemm.h"

#include <algorithm>
#include <cmath>
#include <limits>
#include <map>
#include <numeric>
#include <optional>
#include <unordered_map>

namespace ttg
{
  namespace
  {
    // A value the program computes: an arena of `space`, read from `buffer` through an optional
    // pending gather (a composed chain of permutations not yet written out).
    // The tiles of a pending relabelling move and how many output entries they cover (the rest,
    // padding and dropped entries, is zero).
    struct TileMap
    {
      std::vector<Tile> tiles;
      int64_t covered = 0;
      bool conj = false;  // conjugate the values on the way
    };

    struct Value
    {
      int32_t buffer = -1;
      Space space = nullptr;
      std::shared_ptr<std::vector<int32_t>> pending;
      int32_t phase = -1;  // operand whose prepare phase computes it, -1 for the core
      std::shared_ptr<TileMap> tiled;  // a pending move as tiles (never together with `pending`)
    };

    class Builder
    {
    public:
      explicit Builder(Program &p) : p_(p) {}

      Value input(int32_t index, Space space)
      {
        Buffer b{BufferKind::input, index, 0, space->size};
        p_.buffers.push_back(b);
        return Value{static_cast<int32_t>(p_.buffers.size() - 1), space, nullptr, index};
      }

      int32_t output_buffer(Space space)
      {
        p_.buffers.push_back(Buffer{BufferKind::output, 0, 0, space->size});
        return static_cast<int32_t>(p_.buffers.size() - 1);
      }

      int32_t temp(Space space)
      {
        p_.buffers.push_back(Buffer{BufferKind::temp, -1, p_.workspace, space->size});
        p_.workspace += (space->size + 31) / 32 * 32;  // keep every temporary 256-byte aligned
        return static_cast<int32_t>(p_.buffers.size() - 1);
      }

      // Write a value out into a buffer of its own (or `into` when given).
      Value materialize(const Value &v, int32_t into = -1)
      {
        if (v.tiled)
        {
          const int32_t dst = into >= 0 ? into : temp(v.space);
          if (v.tiled->covered < v.space->size) emit(Op{OpKind::zero, -1, -1, dst, 0, 0, v.space->size, v.phase});
          Op op{OpKind::tiles, v.buffer, -1, dst, static_cast<int64_t>(p_.tile_chunks.size()), 0, v.space->size, v.phase};
          const int32_t first_tile = static_cast<int32_t>(p_.tiles.size());
          for (size_t i = 0; i < v.tiled->tiles.size(); ++i)
          {
            const Tile &t = v.tiled->tiles[i];
            const int32_t step = std::max<int32_t>(1, 2048 / std::max<int32_t>(1, t.cols));
            for (int32_t r = 0; r < t.rows; r += step)
              p_.tile_chunks.push_back(TileChunk{first_tile + static_cast<int32_t>(i), r, std::min(step, t.rows - r), 0});
          }
          p_.tiles.insert(p_.tiles.end(), v.tiled->tiles.begin(), v.tiled->tiles.end());
          op.count = static_cast<int64_t>(p_.tile_chunks.size()) - op.begin;
          op.flags = v.tiled->conj ? 1 : 0;
          p_.moved_elements += v.tiled->covered;
          if (op.count > 0) emit(op);
          return Value{dst, v.space, nullptr, v.phase};
        }
        if (!v.pending)
        {
          if (into < 0 || into == v.buffer) return v;
          emit(Op{OpKind::copy, v.buffer, -1, into, 0, 0, v.space->size, v.phase});
          return Value{into, v.space, nullptr, v.phase};
        }
        const std::vector<int32_t> &index = *v.pending;
        const Buffer &base = p_.buffers[static_cast<size_t>(v.buffer)];
        bool identity = into < 0 && base.size == static_cast<int64_t>(index.size());
        for (size_t i = 0; identity && i < index.size(); ++i) identity = index[i] == static_cast<int32_t>(i);
        if (identity) return Value{v.buffer, v.space, nullptr, v.phase};
        const int32_t dst = into >= 0 ? into : temp(v.space);
        Op op{OpKind::gather, v.buffer, -1, dst, static_cast<int64_t>(p_.gather_index.size()),
              static_cast<int64_t>(index.size()), static_cast<int64_t>(index.size()), v.phase};
        p_.gather_index.insert(p_.gather_index.end(), index.begin(), index.end());
        p_.moved_elements += static_cast<int64_t>(index.size());
        emit(op);
        return Value{dst, v.space, nullptr, v.phase};
      }

      // tentorch/tensors/place.cpp:199-247, compiled: the chain of steps becomes one composed
      // gather for categories whose symbols are all 1, and one RUNS pass per step otherwise.
      Value place(const Value &v, const std::vector<int32_t> &above, const std::vector<int32_t> &below)
      {
        const Category &cat = *v.space->cat;
        if (cat.trivial_symbols())
        {
          // a relabelling needs the space it lands in, not the chain's spaces in between
          const Space after = placed_space(v.space, above, below);
          if (place_is_identity(v.space, above, below)) return v;
          if (!v.pending && !v.tiled && v.space->nlegs() <= kTileLegs)
            return Value{v.buffer, after, nullptr, v.phase,
                         std::make_shared<TileMap>(relabel_tiles(v.space, above, below, after))};
          if (v.tiled) return place(materialize(v), above, below);
          std::vector<int32_t> back = relabel(v.space, above, below, after);
          if (v.pending)
            for (int32_t &b : back) b = b >= 0 ? (*v.pending)[static_cast<size_t>(b)] : -1;
          return Value{v.buffer, after, std::make_shared<std::vector<int32_t>>(std::move(back)), v.phase};
        }
        const std::vector<Step> steps = chain(v.space, above, below);
        if (steps.empty()) return v;
        Value at = materialize(v);
        for (const Step &step : steps)
        {
          const int32_t dst = temp(step.after);
          emit(Op{OpKind::zero, -1, -1, dst, 0, 0, step.after->size, v.phase});
          append_runs(step, at.buffer, dst, v.phase);
          at = Value{dst, step.after, nullptr, v.phase};
        }
        return at;
      }

      // tentorch/linalg/graded/contract.cpp:134-164 on operands already aligned: every output
      // block is the sum over the middle roots of the block products, one grouped GEMM.
      Value contract_aligned(const Value &a_in, const Value &b_in, const Sector &charge)
      {
        const Value a = materialize(a_in), b = materialize(b_in);
        const Category &cat = *a.space->cat;
        Space out = make_space(a.space->cat, a.space->codomain, b.space->domain, charge);
        for (const Block &blk : a.space->blocks) require_single_closing(cat, blk.key.codomain, blk.key.domain, a.space->qtotal, "the roots", "a contraction");
        for (const Block &blk : b.space->blocks) require_single_closing(cat, blk.key.codomain, blk.key.domain, b.space->qtotal, "the roots", "a contraction");
        for (const Block &blk : out->blocks) require_single_closing(cat, blk.key.codomain, blk.key.domain, charge, "the roots", "a contraction");
        const int32_t phase = a.phase == b.phase ? a.phase : -1;
        const int32_t dst = temp(out);
        // pairs per output block, in the order the reference sums them (A blocks in key order, B
        // blocks of the matching codomain root in key order)
        std::vector<std::vector<GemmPair>> pairs(out->blocks.size());
        std::map<Sector, std::vector<const Block *>> rows;
        for (const Block &blk : b.space->blocks) rows[blk.key.codomain].push_back(&blk);
        for (const Block &left : a.space->blocks)
        {
          const auto found = rows.find(left.key.domain);
          if (found == rows.end()) continue;
          for (const Block *right : found->second)
          {
            if (cat.n_symbol(left.key.codomain, cat.dual(right->key.domain), charge) == 0) continue;
            if (left.cols != right->rows)
              throw LogicError("the two blocks over the roots " + left.key.domain.str() + " do not line up: " +
                               std::to_string(left.cols) + " against " + std::to_string(right->rows));
            const int32_t at = out->find(BlockKey{left.key.codomain, right->key.domain, 0});
            if (at < 0) throw LogicError("a block product lands outside the output");
            pairs[static_cast<size_t>(at)].push_back(GemmPair{left.offset, right->offset, static_cast<int32_t>(left.cols), 0});
            p_.gemm_flops += 2.0 * static_cast<double>(left.rows) * static_cast<double>(left.cols) *
                             static_cast<double>(right->cols);
          }
        }
        Op op{OpKind::gemm, a.buffer, b.buffer, dst, static_cast<int64_t>(p_.gemm_blocks.size()), 0, out->size, phase};
        for (size_t i = 0; i < out->blocks.size(); ++i)
        {
          const Block &c = out->blocks[i];
          p_.gemm_blocks.push_back(GemmBlock{c.offset, static_cast<int32_t>(c.rows), static_cast<int32_t>(c.cols),
                                             static_cast<int32_t>(p_.gemm_pairs.size()),
                                             static_cast<int32_t>(pairs[i].size())});
          p_.gemm_pairs.insert(p_.gemm_pairs.end(), pairs[i].begin(), pairs[i].end());
        }
        op.count = static_cast<int64_t>(out->blocks.size());
        emit(op);
        return Value{dst, out, nullptr, phase};
      }

      // tentorch/linalg/graded/einsum.cpp:95-159: the trace of the last codomain leg against the
      // last domain leg, one result per charge the kept roots close to (in sector order).
      std::vector<Value> partial_trace(const Value &v_in)
      {
        const Value v = materialize(v_in);
        Space s = v.space;
        const Category &cat = *s->cat;
        const std::vector<Leg> out_cod(s->codomain.begin(), s->codomain.end() - 1);
        const std::vector<Leg> out_dom(s->domain.begin(), s->domain.end() - 1);
        struct Contribution
        {
          int64_t src, dst;
          int64_t inside_rows, inside_cols, copies, src_stride, dst_stride;
        };
        std::map<Sector, std::vector<Contribution>> by_charge;
        for (const Block &blk : s->blocks)
        {
          require_single_closing(cat, blk.key.codomain, blk.key.domain, s->qtotal, "the roots", "a trace");
          const Layout &rows = layout_of(cat, s->codomain, blk.key.codomain);
          const Layout &cols = layout_of(cat, s->domain, blk.key.domain);
          for (size_t ri = 0; ri < rows.trees.size(); ++ri)
          {
            const Tree &above_tree = rows.trees[ri];
            const int64_t row_span = rows.offsets[ri + 1] - rows.offsets[ri];
            const Tree kept_above = trimmed(cat, above_tree);
            for (size_t ci = 0; ci < cols.trees.size(); ++ci)
            {
              const Tree &under_tree = cols.trees[ci];
              if (!(above_tree.sectors.back() == under_tree.sectors.back())) continue;
              const Tree kept_under = trimmed(cat, under_tree);
              const Layout &out_rows = layout_of(cat, out_cod, kept_above.coupled);
              const Layout &out_cols = layout_of(cat, out_dom, kept_under.coupled);
              const int32_t new_row = out_rows.find(kept_above), new_col = out_cols.find(kept_under);
              if (new_row < 0 || new_col < 0) throw LogicError("a kept tree of a trace is not in the layout it was trimmed from");
              const int64_t inside_rows = out_rows.offsets[static_cast<size_t>(new_row) + 1] - out_rows.offsets[static_cast<size_t>(new_row)];
              const int64_t inside_cols = out_cols.offsets[static_cast<size_t>(new_col) + 1] - out_cols.offsets[static_cast<size_t>(new_col)];
              const int64_t copies = row_span / inside_rows;
              for (const Outcome &closing : cat.outcomes(kept_above.coupled, cat.dual(kept_under.coupled)))
              {
                require_single_closing(cat, kept_above.coupled, kept_under.coupled, closing.sector, "the kept roots", "a trace");
                Space out = make_space(s->cat, out_cod, out_dom, closing.sector);
                const int32_t at = out->find(BlockKey{kept_above.coupled, kept_under.coupled, 0});
                if (at < 0) throw LogicError("a trace lands outside its output");
                const Block &ob = out->blocks[static_cast<size_t>(at)];
                by_charge[closing.sector].push_back(Contribution{
                  blk.offset + rows.offsets[ri] * blk.cols + cols.offsets[ci],
                  ob.offset + out_rows.offsets[static_cast<size_t>(new_row)] * ob.cols + out_cols.offsets[static_cast<size_t>(new_col)],
                  inside_rows, inside_cols, copies, blk.cols, ob.cols});
              }
            }
          }
        }
        std::vector<Value> out;
        for (const auto &[charge, contributions] : by_charge)
        {
          Space space = make_space(s->cat, out_cod, out_dom, charge);
          const int32_t dst = temp(space);
          emit(Op{OpKind::zero, -1, -1, dst, 0, 0, space->size, v.phase});
          // element (i, j) of the kept block gathers sum_c src[(i*copies + c) * stride + j*copies + c]
          std::map<int64_t, std::vector<Term>> groups;
          for (const Contribution &c : contributions)
            for (int64_t i = 0; i < c.inside_rows; ++i)
              for (int64_t j = 0; j < c.inside_cols; ++j)
              {
                std::vector<Term> &terms = groups[c.dst + i * c.dst_stride + j];
                for (int64_t k = 0; k < c.copies; ++k)
                  terms.push_back(Term{c.src + (i * c.copies + k) * c.src_stride + j * c.copies + k, 0, 1.0, 0.0});
              }
          Op op{OpKind::runs, v.buffer, -1, dst, static_cast<int64_t>(p_.chunks.size()), 0, space->size, v.phase};
          for (const auto &[dst_at, terms] : groups)
          {
            p_.chunks.push_back(Chunk{dst_at, 1, 0, static_cast<int32_t>(p_.terms.size()), static_cast<int32_t>(terms.size())});
            p_.terms.insert(p_.terms.end(), terms.begin(), terms.end());
          }
          op.count = static_cast<int64_t>(p_.chunks.size()) - op.begin;
          emit(op);
          out.push_back(Value{dst, space, nullptr, v.phase});
        }
        return out;
      }

      void add_into(const Value &v, int32_t dst)
      {
        const Value m = materialize(v);
        emit(Op{OpKind::add, m.buffer, -1, dst, 0, 0, m.space->size, -1});
      }

      static void require_single_closing(const Category &cat, const Sector &above, const Sector &below,
                                         const Sector &charge, const std::string &subject, const std::string &what)
      {
        if (cat.n_symbol(above, cat.dual(below), charge) > 1)
          throw InvalidArgument(subject + " " + above.str() + " and " + below.str() + " close to " + charge.str() +
                                " in more than one way, which " + what + " does not recouple yet");
      }

      Program &p_;

    private:
      void emit(const Op &op) { p_.ops.push_back(op); }

      // One piece of a relabelling move: an (input row tree, input column tree) part of an input
      // block and the rectangle of an output block it lands in.  Strides and extents are per
      // input leg; out_stride is within the output block (rows times its columns, or columns).
      struct MovePiece
      {
        int64_t in_base, out_base, out_ld;
        const std::vector<int64_t> *extent, *in_stride, *out_stride;
      };

      // Tuples of sector indices over a list of legs, numbered mixed-radix: a dense table when the
      // legs have few sector combinations, a hash map when they have many, and tuples as vectors
      // when the numbering would not fit in 62 bits.
      class TupleIndex
      {
      public:
        explicit TupleIndex(const std::vector<Leg> &legs)
        {
          for (const Leg leg : legs)
          {
            const int64_t r = static_cast<int64_t>(leg->sectors.size());
            radix_.push_back(r);
            if (total_ > (int64_t{1} << 62) / std::max<int64_t>(r, 1)) wide_ = true;
            else total_ *= r;
          }
          dense_ = !wide_ && total_ <= (int64_t{1} << 20);
          if (dense_) table_.assign(static_cast<size_t>(total_), -1);
        }
        int32_t get(const int32_t *idx) const
        {
          if (wide_)
          {
            const auto it = wide_map_.find(std::vector<int32_t>(idx, idx + radix_.size()));
            return it == wide_map_.end() ? -1 : it->second;
          }
          const int64_t c = code(idx);
          if (dense_) return table_[static_cast<size_t>(c)];
          const auto it = hashed_.find(c);
          return it == hashed_.end() ? -1 : it->second;
        }
        // keeps the first value stored for a tuple
        void put_first(const int32_t *idx, int32_t value)
        {
          if (wide_) wide_map_.emplace(std::vector<int32_t>(idx, idx + radix_.size()), value);
          else if (dense_)
          {
            int32_t &slot = table_[static_cast<size_t>(code(idx))];
            if (slot < 0) slot = value;
          }
          else hashed_.emplace(code(idx), value);
        }

      private:
        int64_t code(const int32_t *idx) const
        {
          int64_t c = 0;
          for (size_t i = 0; i < radix_.size(); ++i) c = c * radix_[i] + idx[i];
          return c;
        }
        std::vector<int64_t> radix_;
        int64_t total_ = 1;
        bool wide_ = false, dense_ = false;
        std::vector<int32_t> table_;
        std::unordered_map<int64_t, int32_t> hashed_;
        std::map<std::vector<int32_t>, int32_t> wide_map_;
      };

      template <typename Fn>
      int64_t walk_pieces(Space in, const std::vector<int32_t> &above, const std::vector<int32_t> &below, Space out,
                          Fn &&fn)
      {
        const Category &cat = *in->cat;
        if (out->size > std::numeric_limits<int32_t>::max() || in->size > std::numeric_limits<int32_t>::max())
          throw InvalidArgument("an arena of more than 2^31 entries");
        const int32_t h = static_cast<int32_t>(in->codomain.size()), d = static_cast<int32_t>(in->domain.size());
        const int32_t n = h + d;
        const std::vector<Leg> legs = in->legs();
        const int32_t kept = chain_kept(h, d, below);
        std::vector<bool> bent(static_cast<size_t>(n), false), switched(static_cast<size_t>(n), false);
        for (int32_t l = h + kept; l < n; ++l) bent[static_cast<size_t>(l)] = true;
        for (size_t j = static_cast<size_t>(kept); j < below.size(); ++j) bent[static_cast<size_t>(below[j])] = true;
        for (const int32_t l : above) switched[static_cast<size_t>(l)] = l >= h;
        for (const int32_t l : below) switched[static_cast<size_t>(l)] = l < h;
        const std::vector<Leg> out_cod = out->codomain, out_dom = out->domain;
        // per leg and block of that leg: whether an entry survives the bends (the check bend_plan
        // makes on the paired multiplets), and the index of its sector on the output leg it
        // becomes (read as the dual when the leg changes side; -1 when that leg lacks it)
        std::vector<std::vector<bool>> survives(static_cast<size_t>(n));
        std::vector<std::vector<int32_t>> lands(static_cast<size_t>(n));
        std::vector<Leg> target(static_cast<size_t>(n));
        for (size_t i = 0; i < above.size(); ++i) target[static_cast<size_t>(above[i])] = out_cod[i];
        for (size_t j = 0; j < below.size(); ++j) target[static_cast<size_t>(below[j])] = out_dom[j];
        for (int32_t l = 0; l < n; ++l)
        {
          const Leg leg = legs[static_cast<size_t>(l)];
          survives[static_cast<size_t>(l)].assign(leg->sectors.size(), true);
          lands[static_cast<size_t>(l)].assign(leg->sectors.size(), -1);
          for (size_t b = 0; b < leg->sectors.size(); ++b)
          {
            const Sector label = switched[static_cast<size_t>(l)] ? cat.dual(leg->sectors[b]) : leg->sectors[b];
            const Leg to = target[static_cast<size_t>(l)];
            const auto it = std::lower_bound(to->sectors.begin(), to->sectors.end(), label);
            if (it != to->sectors.end() && *it == label)
              lands[static_cast<size_t>(l)][b] = static_cast<int32_t>(it - to->sectors.begin());
          }
          if (!bent[static_cast<size_t>(l)]) continue;
          for (size_t b = 0; b < leg->sectors.size(); ++b)
          {
            const Sector dual = cat.dual(leg->sectors[b]);
            const auto it = std::lower_bound(leg->sectors.begin(), leg->sectors.end(), dual);
            if (it == leg->sectors.end() || !(*it == dual))
            {
              survives[static_cast<size_t>(l)][b] = false;
              continue;
            }
            const int64_t other = leg->mult[static_cast<size_t>(it - leg->sectors.begin())];
            if (other != leg->mult[b] && !in->blocks.empty())
              throw InvalidArgument("a leg bent across the tensor needs each sector and its dual to carry the same "
                                    "multiplets, but " + leg->sectors[b].str() + " has " +
                                    std::to_string(leg->mult[b]) + " and " + dual.str() + " has " +
                                    std::to_string(other));
          }
        }
        // the output trees by the sector indices of their legs: (root, first row) on each side,
        // the first tree of a tuple kept; the output blocks (copy 0) by their pair of roots
        TupleIndex rows_of(out_cod), cols_of(out_dom);
        std::vector<std::pair<int32_t, int64_t>> row_at, col_at;  // (root number, first row)
        std::map<Sector, int32_t> cod_root, dom_root;
        for (const Block &ob : out->blocks)
        {
          cod_root.emplace(ob.key.codomain, static_cast<int32_t>(cod_root.size()));
          dom_root.emplace(ob.key.domain, static_cast<int32_t>(dom_root.size()));
        }
        std::vector<int32_t> block_of(cod_root.size() * dom_root.size(), -1);
        for (size_t bi = 0; bi < out->blocks.size(); ++bi)
        {
          const Block &ob = out->blocks[bi];
          const int32_t rr = cod_root.at(ob.key.codomain), cr = dom_root.at(ob.key.domain);
          if (ob.key.copy == 0) block_of[static_cast<size_t>(rr) * dom_root.size() + static_cast<size_t>(cr)] = static_cast<int32_t>(bi);
          if (ob.key.copy != 0) continue;  // the trees of a root are the same for every copy
          for (const auto &[side, root, number, table, at] :
               {std::make_tuple(&out_cod, ob.key.codomain, rr, &rows_of, &row_at),
                std::make_tuple(&out_dom, ob.key.domain, cr, &cols_of, &col_at)})
          {
            const Layout &lay = layout_of(cat, *side, root);
            const std::vector<int32_t> &idx = lay.index;
            for (size_t t = 0; t < lay.trees.size(); ++t)
            {
              table->put_first(idx.data() + t * side->size(), static_cast<int32_t>(at->size()));
              at->push_back({number, lay.offsets[t]});
            }
          }
        }
        std::vector<int32_t> idx_out(static_cast<size_t>(n));
        std::vector<int64_t> extent(static_cast<size_t>(n)), in_stride(static_cast<size_t>(n)),
          out_stride(static_cast<size_t>(n));
        std::vector<int32_t> at_of(static_cast<size_t>(n));
        int64_t covered = 0;
        for (const Block &blk : in->blocks)
        {
          const Layout &rl = layout_of(cat, in->codomain, blk.key.codomain);
          const Layout &cl = layout_of(cat, in->domain, blk.key.domain);
          const std::vector<int32_t> &r_idx = rl.index, &c_idx = cl.index;
          for (size_t rt = 0; rt < rl.trees.size(); ++rt)
            for (size_t ct = 0; ct < cl.trees.size(); ++ct)
            {
              bool keep = true;
              for (int32_t l = 0; l < n && keep; ++l)
              {
                const int32_t at = l < h ? r_idx[rt * static_cast<size_t>(h) + static_cast<size_t>(l)]
                                         : c_idx[ct * static_cast<size_t>(d) + static_cast<size_t>(l - h)];
                at_of[static_cast<size_t>(l)] = at;
                keep = survives[static_cast<size_t>(l)][static_cast<size_t>(at)] && lands[static_cast<size_t>(l)][static_cast<size_t>(at)] >= 0;
                extent[static_cast<size_t>(l)] = legs[static_cast<size_t>(l)]->mult[static_cast<size_t>(at)];
              }
              if (!keep) continue;
              for (size_t i = 0; i < above.size(); ++i)
                idx_out[i] = lands[static_cast<size_t>(above[i])][static_cast<size_t>(at_of[static_cast<size_t>(above[i])])];
              for (size_t j = 0; j < below.size(); ++j)
                idx_out[above.size() + j] = lands[static_cast<size_t>(below[j])][static_cast<size_t>(at_of[static_cast<size_t>(below[j])])];
              const int32_t r = rows_of.get(idx_out.data());
              const int32_t c = cols_of.get(idx_out.data() + above.size());
              if (r < 0 || c < 0) continue;
              const int32_t ob_at = block_of[static_cast<size_t>(row_at[static_cast<size_t>(r)].first) * dom_root.size() +
                                             static_cast<size_t>(col_at[static_cast<size_t>(c)].first)];
              if (ob_at < 0) continue;
              const Block &ob = out->blocks[static_cast<size_t>(ob_at)];
              // strides: input rows and columns with the last leg of each side fastest; the same
              // for the output sides
              int64_t run = blk.cols;
              for (int32_t l = h - 1; l >= 0; --l) in_stride[static_cast<size_t>(l)] = run, run *= extent[static_cast<size_t>(l)];
              run = 1;
              for (int32_t l = n - 1; l >= h; --l) in_stride[static_cast<size_t>(l)] = run, run *= extent[static_cast<size_t>(l)];
              run = ob.cols;
              int64_t entries = 1;
              for (size_t i = above.size(); i-- > 0;)
                out_stride[static_cast<size_t>(above[i])] = run, run *= extent[static_cast<size_t>(above[i])];
              run = 1;
              for (size_t j = below.size(); j-- > 0;)
                out_stride[static_cast<size_t>(below[j])] = run, run *= extent[static_cast<size_t>(below[j])];
              for (int32_t l = 0; l < n; ++l) entries *= extent[static_cast<size_t>(l)];
              covered += entries;
              fn(MovePiece{blk.offset + rl.offsets[rt] * blk.cols + cl.offsets[ct],
                           ob.offset + row_at[static_cast<size_t>(r)].second * ob.cols + col_at[static_cast<size_t>(c)].second,
                           ob.cols, &extent, &in_stride, &out_stride});
            }
        }
        return covered;
      }

      // The composed gather index of a whole chain of leg moves when every F and R symbol is 1:
      // after[i] = before[index[i]], -1 for entries nothing writes.  Such a chain only relabels:
      // the entry at sector s_l, copy c_l of every leg l lands at the same copies of the output
      // legs, a leg that ends on the other side reading its sector as the dual (each bend reads
      // the dual sector's rows, tentorch/tensors/regroup.cpp:260-417).  A bent leg that does not
      // hold the dual of an entry's sector drops the entry, as the chain's bends do; the chain
      // bends every leg of below[kept:] down and every domain leg past `kept` up.  The result is
      // the composition of the per-step permutations, built in one pass over the entries instead
      // of one pass per step.
      std::vector<int32_t> relabel(Space in, const std::vector<int32_t> &above, const std::vector<int32_t> &below,
                                   Space out)
      {
        std::vector<int32_t> back(static_cast<size_t>(out->size), -1);
        const int32_t n = in->nlegs();
        std::vector<int32_t> order(static_cast<size_t>(n));  // legs in output order, the last fastest
        for (size_t i = 0; i < above.size(); ++i) order[i] = above[i];
        for (size_t j = 0; j < below.size(); ++j) order[above.size() + j] = below[j];
        std::vector<int64_t> copy(static_cast<size_t>(n));
        walk_pieces(in, above, below, out, [&](const MovePiece &piece)
        {
          const std::vector<int64_t> &extent = *piece.extent, &in_stride = *piece.in_stride,
                                     &out_stride = *piece.out_stride;
          // walk every copy tuple in output order, the last output leg innermost
          std::fill(copy.begin(), copy.end(), 0);
          int64_t src = piece.in_base, dst = piece.out_base;
          const size_t inner = static_cast<size_t>(order[static_cast<size_t>(n - 1)]);
          while (true)
          {
            for (int64_t k = 0; k < extent[inner]; ++k)
              back[static_cast<size_t>(dst + k * out_stride[inner])] = static_cast<int32_t>(src + k * in_stride[inner]);
            int32_t at = n - 2;
            for (; at >= 0; --at)
            {
              const size_t l = static_cast<size_t>(order[static_cast<size_t>(at)]);
              if (++copy[l] < extent[l])
              {
                src += in_stride[l];
                dst += out_stride[l];
                break;
              }
              src -= (extent[l] - 1) * in_stride[l];
              dst -= (extent[l] - 1) * out_stride[l];
              copy[l] = 0;
            }
            if (at < 0) break;
          }
        });
        return back;
      }

      // The same move as tiles: one per piece, its rows the copies of the output codomain legs and
      // its columns those of the output domain legs.
      TileMap relabel_tiles(Space in, const std::vector<int32_t> &above, const std::vector<int32_t> &below, Space out)
      {
        TileMap map;
        // the pad entry of every odd block is a tile of its own that writes zero (in_base -1), so
        // that a move which drops nothing needs no zero pass
        for (const Block &ob : out->blocks)
          if ((ob.rows * ob.cols) & 1)
          {
            Tile t{};
            t.in_base = -1;
            t.out_base = ob.offset + ob.rows * ob.cols;
            t.out_ld = 1;
            t.rows = t.cols = 1;
            map.tiles.push_back(t);
            ++map.covered;
          }
        map.covered += walk_pieces(in, above, below, out, [&](const MovePiece &piece)
        {
          Tile t{};
          t.in_base = piece.in_base;
          t.out_base = piece.out_base;
          t.out_ld = static_cast<int32_t>(piece.out_ld);
          t.n_row = static_cast<int32_t>(above.size());
          t.n_col = static_cast<int32_t>(below.size());
          int64_t rows = 1, cols = 1;
          int32_t at = 0;
          for (const int32_t l : above)
          {
            t.extent[at] = static_cast<int32_t>((*piece.extent)[static_cast<size_t>(l)]);
            t.stride[at++] = (*piece.in_stride)[static_cast<size_t>(l)];
            rows *= (*piece.extent)[static_cast<size_t>(l)];
          }
          for (const int32_t l : below)
          {
            t.extent[at] = static_cast<int32_t>((*piece.extent)[static_cast<size_t>(l)]);
            t.stride[at++] = (*piece.in_stride)[static_cast<size_t>(l)];
            cols *= (*piece.extent)[static_cast<size_t>(l)];
          }
          t.rows = static_cast<int32_t>(rows);
          t.cols = static_cast<int32_t>(cols);
          map.tiles.push_back(t);
        });
        return map;
      }

      // One step with coefficients: the pieces of every block grouped by destination run.
      void append_runs(const Step &step, int32_t src, int32_t dst, int32_t phase)
      {
        Space before = step.before, after = step.after;
        struct RunKey
        {
          int64_t dst, step, len;
          bool operator<(const RunKey &o) const { return std::tie(dst, step, len) < std::tie(o.dst, o.step, o.len); }
        };
        std::map<RunKey, std::vector<Term>> groups;
        for (const Block &blk : before->blocks)
          for (const Shift &shift : step_plan(step, blk.key))
          {
            const int32_t t = after->find(shift.to);
            if (t < 0) throw LogicError("a move lands outside the tensor it builds");
            const int64_t ot = after->blocks[static_cast<size_t>(t)].offset;
            for (const Piece &piece : shift.pieces)
              groups[RunKey{ot + piece.last, piece.to_step, piece.run}].push_back(
                Term{blk.offset + piece.first, piece.from_step, piece.coefficient.real(), piece.coefficient.imag()});
          }
        // destination runs must not overlap; when they do the step is laid out entry by entry
        std::vector<uint8_t> seen(static_cast<size_t>(after->size), 0);
        bool overlap = false;
        for (const auto &[k, terms] : groups)
          for (int64_t i = 0; i < k.len && !overlap; ++i)
          {
            uint8_t &mark = seen[static_cast<size_t>(k.dst + i * k.step)];
            overlap = mark != 0;
            mark = 1;
          }
        if (overlap)
        {
          std::map<RunKey, std::vector<Term>> single;
          for (const auto &[k, terms] : groups)
            for (int64_t i = 0; i < k.len; ++i)
            {
              std::vector<Term> &into = single[RunKey{k.dst + i * k.step, 0, 1}];
              for (const Term &t : terms) into.push_back(Term{t.src + i * t.src_step, 0, t.re, t.im});
            }
          groups = std::move(single);
        }
        Op op{OpKind::runs, src, -1, dst, static_cast<int64_t>(p_.chunks.size()), 0, after->size, phase};
        for (const auto &[k, terms] : groups)
          for (int64_t c0 = 0; c0 < k.len; c0 += kChunk)
          {
            p_.chunks.push_back(Chunk{k.dst + c0 * k.step, static_cast<int32_t>(std::min<int64_t>(kChunk, k.len - c0)),
                                      static_cast<int32_t>(k.step), static_cast<int32_t>(p_.terms.size()),
                                      static_cast<int32_t>(terms.size())});
            for (const Term &t : terms)
            {
              p_.terms.push_back(Term{t.src + c0 * t.src_step, t.src_step, t.re, t.im});
              if (t.im != 0.0) p_.complex_coefficients = true;
            }
            p_.moved_elements += std::min<int64_t>(kChunk, k.len - c0);
          }
        op.count = static_cast<int64_t>(p_.chunks.size()) - op.begin;
        emit(op);
      }
    };

    std::vector<int32_t> without(int32_t total, const std::vector<int32_t> &taken)
    {
      std::vector<bool> named(static_cast<size_t>(total), false);
      for (int32_t leg : taken) named[static_cast<size_t>(leg)] = true;
      std::vector<int32_t> out;
      for (int32_t leg = 0; leg < total; ++leg)
        if (!named[static_cast<size_t>(leg)]) out.push_back(leg);
      return out;
    }

    void check_side(Space s, const std::vector<int32_t> &legs, const char *side)
    {
      std::vector<bool> named(static_cast<size_t>(s->nlegs()), false);
      for (int32_t leg : legs)
      {
        if (leg < 0 || leg >= s->nlegs())
          throw InvalidArgument("the leg " + std::to_string(leg) + " of the " + side + " tensor is out of range of its " +
                                std::to_string(s->nlegs()) + " legs");
        if (named[static_cast<size_t>(leg)])
          throw InvalidArgument("the leg " + std::to_string(leg) + " of the " + side + " tensor is summed twice");
        named[static_cast<size_t>(leg)] = true;
      }
    }

    // tentorch/linalg/graded/contract.cpp:47-77 (the scalar type is checked by the caller)
    void check_pairs(Space left, Space right, const std::vector<int32_t> &left_legs, const std::vector<int32_t> &right_legs)
    {
      if (left->cat != right->cat) throw InvalidArgument("a contraction needs both tensors over one category");
      if (left_legs.size() != right_legs.size())
        throw InvalidArgument("the two legs of a contraction must be given in pairs, got " + std::to_string(left_legs.size()) +
                              " and " + std::to_string(right_legs.size()));
      check_side(left, left_legs, "first");
      check_side(right, right_legs, "second");
      const std::vector<Leg> la = left->legs(), ra = right->legs();
      for (size_t at = 0; at < left_legs.size(); ++at)
      {
        Leg one = la[static_cast<size_t>(left_legs[at])], other = ra[static_cast<size_t>(right_legs[at])];
        if (one != other)
          throw InvalidArgument("the pair at position " + std::to_string(at) + " joins the leg " + std::to_string(left_legs[at]) +
                                " of the first tensor, over " + render(one->sectors) + ", to the leg " +
                                std::to_string(right_legs[at]) + " of the second, over " + render(other->sectors) +
                                ", and the two do not name one space");
      }
    }

    // Every descriptor stays inside the buffers its op reads and writes: checked once on the host
    // when the program is compiled, so no launch can be handed an offset outside an arena.
    void validate(const Program &p)
    {
      const auto size_of = [&](int32_t buffer) { return p.buffers[static_cast<size_t>(buffer)].size; };
      const auto require = [](bool ok, const char *what) {
        if (!ok) throw LogicError(std::string("a compiled program reaches outside its buffers: ") + what);
      };
      for (const Op &op : p.ops)
      {
        const int64_t dst = op.dst >= 0 ? size_of(op.dst) : 0;
        switch (op.kind)
        {
        case OpKind::zero:
        case OpKind::copy:
        case OpKind::add:
          require(op.elements <= dst && (op.src < 0 || op.elements <= size_of(op.src)), "arena op");
          break;
        case OpKind::gather:
          require(op.elements <= dst, "gather destination");
          for (int64_t i = op.begin; i < op.begin + op.count; ++i)
            require(p.gather_index[static_cast<size_t>(i)] < size_of(op.src), "gather source");
          break;
        case OpKind::tiles:
          for (int64_t c = op.begin; c < op.begin + op.count; ++c)
          {
            const TileChunk &ch = p.tile_chunks[static_cast<size_t>(c)];
            require(ch.tile >= 0 && static_cast<size_t>(ch.tile) < p.tiles.size(), "tile");
            const Tile &t = p.tiles[static_cast<size_t>(ch.tile)];
            require(ch.row0 >= 0 && ch.nrows >= 1 && ch.row0 + ch.nrows <= t.rows, "tile rows");
            require(t.n_row >= 0 && t.n_col >= 0 && t.n_row + t.n_col <= kTileLegs && t.cols >= 1, "tile legs");
            require(t.out_base >= 0 && t.out_base + static_cast<int64_t>(t.rows - 1) * t.out_ld + t.cols <= dst,
                    "tile destination");
            int64_t last = t.in_base, rows = 1, cols = 1;
            for (int32_t l = 0; l < t.n_row + t.n_col; ++l)
            {
              require(t.extent[l] >= 1 && t.stride[l] >= 0, "tile extent");
              last += static_cast<int64_t>(t.extent[l] - 1) * t.stride[l];
              (l < t.n_row ? rows : cols) *= t.extent[l];
            }
            require(rows == t.rows && cols == t.cols, "tile shape");
            require((t.in_base == -1 && t.n_row == 0 && t.n_col == 0) || (t.in_base >= 0 && last < size_of(op.src)),
                    "tile source");
          }
          break;
        case OpKind::runs:
          for (int64_t c = op.begin; c < op.begin + op.count; ++c)
          {
            const Chunk &ch = p.chunks[static_cast<size_t>(c)];
            require(ch.len >= 1 && ch.len <= kChunk && ch.dst >= 0 && ch.dst_step >= 0, "runs chunk");
            require(ch.dst + static_cast<int64_t>(ch.len - 1) * ch.dst_step < dst, "runs destination");
            for (int32_t t = 0; t < ch.term_count; ++t)
            {
              const Term &term = p.terms[static_cast<size_t>(ch.term_begin + t)];
              require(term.src >= 0 && term.src_step >= 0 &&
                        term.src + static_cast<int64_t>(ch.len - 1) * term.src_step < size_of(op.src),
                      "runs source");
            }
          }
          break;
        case OpKind::gemm:
          for (int64_t bi = op.begin; bi < op.begin + op.count; ++bi)
          {
            const GemmBlock &blk = p.gemm_blocks[static_cast<size_t>(bi)];
            const int64_t entries = static_cast<int64_t>(blk.m) * blk.n;
            require(blk.c >= 0 && blk.c + entries + (entries & 1) <= dst, "gemm output block");
            for (int32_t k = 0; k < blk.pair_count; ++k)
            {
              const GemmPair &pr = p.gemm_pairs[static_cast<size_t>(blk.pair_begin + k)];
              require(pr.a >= 0 && pr.a + static_cast<int64_t>(blk.m) * pr.k <= size_of(op.src), "gemm left block");
              require(pr.b >= 0 && pr.b + static_cast<int64_t>(pr.k) * blk.n <= size_of(op.src2), "gemm right block");
            }
          }
          break;
        }
      }
    }

    bool read_by_any(const Program &p, int32_t buffer)
    {
      for (const Op &op : p.ops)
        if (op.src == buffer || op.src2 == buffer) return true;
      return false;
    }

    void finish(Program &p, Builder &b, const std::vector<Value> &results)
    {
      if (results.empty()) throw LogicError("a program without a result");
      p.output_space = results.front().space;
      const int32_t out = b.output_buffer(p.output_space);
      // a result computed by the core (or a prepared value) writes straight into the output
      Value first = results.front();
      if (first.pending || first.tiled)
        b.materialize(first, out);
      else if (p.buffers[static_cast<size_t>(first.buffer)].kind == BufferKind::temp && first.phase < 0 &&
               !p.ops.empty() && p.ops.back().dst == first.buffer && !read_by_any(p, first.buffer))
      {
        // every op that writes the final temporary (a zero and its runs pass, or one gather or
        // GEMM) writes the output instead
        for (Op &op : p.ops)
          if (op.dst == first.buffer) op.dst = out;
      }
      else
        b.materialize(first, out);
      for (size_t i = 1; i < results.size(); ++i) b.add_into(results[i], out);
      // an operand's prepared value is the last buffer its phase writes that the core reads
      p.prepared.assign(static_cast<size_t>(p.n_inputs), -1);
      for (const Op &op : p.ops)
        if (op.phase < 0)
          for (int32_t src : {op.src, op.src2})
            if (src >= 0)
            {
              const Buffer &buf = p.buffers[static_cast<size_t>(src)];
              if (buf.kind == BufferKind::temp)
                for (const Op &producer : p.ops)
                  if (producer.dst == src && producer.phase >= 0)
                  {
                    // more than one prepared buffer per operand: leave the operand unprepared
                    int32_t &slot = p.prepared[static_cast<size_t>(producer.phase)];
                    slot = (slot == -1 || slot == src) ? src : -2;
                  }
            }
      for (int32_t i = 0; i < p.n_inputs; ++i)
        if (p.prepared[static_cast<size_t>(i)] >= 0)
          p.buffers[static_cast<size_t>(p.prepared[static_cast<size_t>(i)])].prepared_of = i;
        else
          p.prepared[static_cast<size_t>(i)] = -1;
      // ops of an unprepared operand's phase run as core ops
      for (Op &op : p.ops)
        if (op.phase >= 0 && p.prepared[static_cast<size_t>(op.phase)] < 0) op.phase = -1;
      // GEMM tickets ahead of the temporaries; every program that uses the workspace at all leaves
      // that region alone, since one workspace serves the programs of a stream in turn
      if (p.workspace > 0 ||
          std::any_of(p.ops.begin(), p.ops.end(), [](const Op &op) { return op.kind == OpKind::gemm; }))
      {
        for (Buffer &b : p.buffers)
          if (b.kind == BufferKind::temp) b.offset += kTicketElements;
        p.workspace += kTicketElements;
      }
      p.scratch_offset = p.workspace;
      detect_chain(p);
      p.workspace += plan_gemms(p);
      p.tune_key = tune_key(p);
      validate(p);
    }

    // --------------------------------------------------------------------------------------
    // einsum helpers (tentorch/linalg/graded/einsum.cpp:27-301)
    // --------------------------------------------------------------------------------------

    struct SideSpec
    {
      std::vector<char> labels;
      std::vector<bool> above;
    };

    SideSpec side_of(const std::string &text)
    {
      SideSpec out;
      for (const char letter : text)
      {
        if (letter == ' ') continue;
        out.labels.push_back(static_cast<char>(std::tolower(static_cast<unsigned char>(letter))));
        out.above.push_back(letter >= 'A' && letter <= 'Z');
      }
      return out;
    }

    bool holds(const std::vector<char> &labels, char label)
    {
      return std::find(labels.begin(), labels.end(), label) != labels.end();
    }

    int32_t position_of(const std::vector<char> &labels, char label)
    {
      const auto it = std::find(labels.begin(), labels.end(), label);
      if (it == labels.end()) throw LogicError(std::string("the label '") + label + "' left the equation");
      return static_cast<int32_t>(it - labels.begin());
    }

    std::vector<char> union_of(const std::vector<char> &a, const std::vector<char> &b)
    {
      std::vector<char> out = a;
      for (char l : b)
        if (!holds(out, l)) out.push_back(l);
      return out;
    }

    std::vector<char> shared_of(const std::vector<char> &a, const std::vector<char> &b)
    {
      std::vector<char> out;
      for (char l : a)
        if (holds(b, l)) out.push_back(l);
      return out;
    }

    std::vector<char> product_labels(const std::vector<char> &a, const std::vector<char> &b)
    {
      const std::vector<char> shared = shared_of(a, b);
      std::vector<char> out;
      for (char l : union_of(a, b))
        if (!holds(shared, l)) out.push_back(l);
      return out;
    }

    double leg_size(const Category &cat, Leg leg)
    {
      double out = 0;
      for (size_t i = 0; i < leg->sectors.size(); ++i) out += static_cast<double>(leg->mult[i]) * cat.q_dim(leg->sectors[i]);
      return out;
    }

    // A set of einsum labels as a bit mask over the equation's letters, with the size of a tensor
    // over them: the product of their dimensions, multiplied in the order the labels joined the set
    // (the order the reference multiplies them in, tentorch/linalg/graded/einsum.cpp:170-176, so
    // that equal costs compare equal there and here).
    struct LabelSet
    {
      uint64_t bits = 0;
      double size = 1;
    };

    // The order the operands of an einsum are folded in (the rule of
    // tentorch/linalg/graded/einsum.cpp:211-301): operand 0 first, then every other operand once,
    // so that the sum of the products' sizes is smallest, the size of a product being that of every
    // label the accumulator has met (summed labels included).
    //
    // Up to 12 operands the order is exact: over the subsets S of the other operands,
    //   best(S) = min over o in S of best(S - o) + size(labels of operand 0 and of S),
    // with o allowed only when it shares a label with operand 0 and S - o (outer products only when
    // no order without them exists).  Equal costs go to the step that sums more labels, then to the
    // operand written later.  Beyond 12 operands: greedily the operand whose product with the
    // accumulator is smallest, operands sharing a label first, the one written first on ties.
    std::vector<int32_t> fold_order(const std::vector<std::vector<char>> &inputs, const std::map<char, double> &dims)
    {
      const int32_t count = static_cast<int32_t>(inputs.size());
      std::map<char, int32_t> letter;
      for (const auto &labels : inputs)
        for (const char l : labels) letter.emplace(l, static_cast<int32_t>(letter.size()));
      std::vector<uint64_t> mask_of(inputs.size(), 0);
      for (size_t i = 0; i < inputs.size(); ++i)
        for (const char l : inputs[i]) mask_of[i] |= uint64_t(1) << letter[l];
      const auto joined = [&](LabelSet set, int32_t operand)
      {
        for (const char l : inputs[static_cast<size_t>(operand)])
        {
          const uint64_t bit = uint64_t(1) << letter[l];
          if (set.bits & bit) continue;
          set.bits |= bit;
          set.size *= dims.at(l);
        }
        return set;
      };
      const auto sums = [&](const LabelSet &set, int32_t operand)
      { return static_cast<int32_t>(__builtin_popcountll(set.bits & mask_of[static_cast<size_t>(operand)])); };
      std::vector<int32_t> order{0};
      if (count <= 12)
      {
        const int32_t others = count - 1;
        const size_t subsets = size_t(1) << others;
        // the labels of operand 0 and of subset S, joined highest operand first (as the reference
        // builds them: S's lowest operand joins the labels of the rest of S)
        std::vector<LabelSet> met(subsets);
        met[0] = joined(LabelSet{}, 0);
        for (size_t set = 1; set < subsets; ++set)
        {
          const int32_t low = __builtin_ctzll(static_cast<unsigned long long>(set));
          met[set] = joined(met[set & (set - 1)], low + 1);
        }
        for (const bool outer : {false, true})
        {
          std::vector<double> best(subsets, std::numeric_limits<double>::infinity());
          std::vector<int32_t> step(subsets, -1);
          best[0] = 0;
          for (size_t set = 1; set < subsets; ++set)
          {
            int32_t chosen_sums = -1;
            for (int32_t o = 0; o < others; ++o)
            {
              if (!(set >> o & 1)) continue;
              const size_t rest = set & ~(size_t(1) << o);
              if (best[rest] == std::numeric_limits<double>::infinity()) continue;
              const int32_t summed = sums(met[rest], o + 1);
              if (!outer && summed == 0) continue;
              const double cost = best[rest] + met[set].size;
              // (cost, -summed, -o) smallest wins; operands are visited in increasing o
              if (cost < best[set] || (cost == best[set] && summed >= chosen_sums))
              {
                best[set] = cost;
                chosen_sums = summed;
                step[set] = o;
              }
            }
          }
          if (step[subsets - 1] < 0 && subsets > 1) continue;
          std::vector<int32_t> tail;
          for (size_t set = subsets - 1; set; set &= ~(size_t(1) << step[set])) tail.push_back(step[set] + 1);
          order.insert(order.end(), tail.rbegin(), tail.rend());
          return order;
        }
        return order;
      }
      std::vector<bool> taken(inputs.size(), false);
      taken[0] = true;
      LabelSet live = joined(LabelSet{}, 0);
      while (static_cast<int32_t>(order.size()) < count)
      {
        int32_t pick = -1;
        double pick_size = 0;
        for (const bool outer : {false, true})
        {
          for (int32_t o = 1; o < count; ++o)
          {
            if (taken[static_cast<size_t>(o)] || (sums(live, o) == 0) != outer) continue;
            const double size = joined(live, o).size;
            if (pick < 0 || size < pick_size)
            {
              pick = o;
              pick_size = size;
            }
          }
          if (pick >= 0) break;
        }
        order.push_back(pick);
        taken[static_cast<size_t>(pick)] = true;
        live = joined(live, pick);
      }
      return order;
    }

    constexpr int64_t kMaxCharges = 4096;
  } // namespace

  std::vector<int32_t> expand_move(const Program &p, const Op &op)
  {
    if (op.kind == OpKind::gather)
      return std::vector<int32_t>(p.gather_index.begin() + op.begin, p.gather_index.begin() + op.begin + op.count);
    if (op.kind != OpKind::tiles) throw InvalidArgument("an operation that is neither a gather nor tiles");
    std::vector<int32_t> index(static_cast<size_t>(op.elements), -1);
    for (int64_t c = op.begin; c < op.begin + op.count; ++c)
    {
      const TileChunk &ch = p.tile_chunks[static_cast<size_t>(c)];
      const Tile &t = p.tiles[static_cast<size_t>(ch.tile)];
      if (t.in_base < 0) continue;  // a zero pad entry
      for (int32_t r = ch.row0; r < ch.row0 + ch.nrows; ++r)
        for (int32_t col = 0; col < t.cols; ++col)
        {
          // mixed radix over the copies of the row legs, then of the column legs, the last fastest
          int64_t in = t.in_base;
          int32_t rest = r;
          for (int32_t l = t.n_row - 1; l >= 0; --l) in += static_cast<int64_t>(rest % t.extent[l]) * t.stride[l], rest /= t.extent[l];
          rest = col;
          for (int32_t l = t.n_row + t.n_col - 1; l >= t.n_row; --l)
            in += static_cast<int64_t>(rest % t.extent[l]) * t.stride[l], rest /= t.extent[l];
          index[static_cast<size_t>(t.out_base + static_cast<int64_t>(r) * t.out_ld + col)] = static_cast<int32_t>(in);
        }
    }
    return index;
  }

  std::shared_ptr<Program> compile_conj(Space space)
  {
    const Category &cat = *space->cat;
    Space out = make_space(space->cat, space->domain, space->codomain, cat.dual(space->qtotal));
    auto p = std::make_shared<Program>();
    p->n_inputs = 1;
    p->input_spaces = {space};
    Builder b(*p);
    Value v = b.input(0, space);
    v.phase = -1;
    auto map = std::make_shared<TileMap>();
    map->conj = true;
    for (const Block &ob : out->blocks)
      if ((ob.rows * ob.cols) & 1)
      {
        Tile t{};
        t.in_base = -1;
        t.out_base = ob.offset + ob.rows * ob.cols;
        t.out_ld = 1;
        t.rows = t.cols = 1;
        map->tiles.push_back(t);
        ++map->covered;
      }
    for (const Block &blk : space->blocks)
    {
      if (blk.rows == 0 || blk.cols == 0) continue;
      const int32_t at = out->find(BlockKey{blk.key.domain, blk.key.codomain, blk.key.copy});
      if (at < 0) throw LogicError("a conjugate block lands outside the conjugate space");
      const Block &ob = out->blocks[static_cast<size_t>(at)];
      // out[c][r] = conj(in[r][c]): rows of the tile run over the input's columns, columns over its rows
      Tile t{};
      t.in_base = blk.offset;
      t.out_base = ob.offset;
      t.out_ld = static_cast<int32_t>(ob.cols);
      t.rows = static_cast<int32_t>(blk.cols);
      t.cols = static_cast<int32_t>(blk.rows);
      t.n_row = 1;
      t.n_col = 1;
      t.extent[0] = static_cast<int32_t>(blk.cols);
      t.stride[0] = 1;
      t.extent[1] = static_cast<int32_t>(blk.rows);
      t.stride[1] = blk.cols;
      map->tiles.push_back(t);
      map->covered += blk.rows * blk.cols;
    }
    finish(*p, b, {Value{v.buffer, out, nullptr, -1, map}});
    return p;
  }

  std::shared_ptr<Program> compile_place(Space space, const std::vector<int32_t> &above, const std::vector<int32_t> &below)
  {
    auto p = std::make_shared<Program>();
    p->n_inputs = 1;
    p->input_spaces = {space};
    Builder b(*p);
    Value v = b.input(0, space);
    v.phase = -1;
    finish(*p, b, {b.place(v, above, below)});
    return p;
  }

  std::shared_ptr<Program> compile_contract(Space left, Space right, const std::vector<int32_t> &left_legs,
                                            const std::vector<int32_t> &right_legs, bool has_charge, const Sector &charge_in)
  {
    const Category &cat = *left->cat;
    Sector charge = charge_in;
    if (!has_charge)
    {
      if (!(right->qtotal == cat.trivial()))
        throw InvalidArgument("the second tensor of a contraction must carry the trivial charge");
      charge = left->qtotal;
    }
    check_pairs(left, right, left_legs, right_legs);
    if (cat.n_symbol(left->qtotal, right->qtotal, charge) == 0)
      throw InvalidArgument("the charge " + charge.str() + " is not an outcome of " + left->qtotal.str() + " and " +
                            right->qtotal.str());
    Builder::require_single_closing(cat, left->qtotal, right->qtotal, charge, "the charges", "a contraction");
    auto p = std::make_shared<Program>();
    p->n_inputs = 2;
    p->input_spaces = {left, right};
    Builder b(*p);
    const Value l = b.input(0, left), r = b.input(1, right);
    const Value above = b.place(l, without(left->nlegs(), left_legs), left_legs);
    const Value under = b.place(r, right_legs, without(right->nlegs(), right_legs));
    finish(*p, b, {b.contract_aligned(above, under, charge)});
    return p;
  }

  std::shared_ptr<Program> compile_einsum(const std::string &spec, const std::vector<Space> &operands, bool has_charge,
                                          const Sector &charge_in)
  {
    if (operands.empty()) throw InvalidArgument("an einsum needs at least one operand");
    const size_t at_arrow = spec.find("->");
    if (at_arrow == std::string::npos) throw InvalidArgument("the equation '" + spec + "' does not say what it leaves");
    std::vector<SideSpec> groups;
    const std::string left = spec.substr(0, at_arrow);
    size_t start = 0;
    while (true)
    {
      const size_t comma = left.find(',', start);
      groups.push_back(side_of(left.substr(start, comma == std::string::npos ? std::string::npos : comma - start)));
      if (comma == std::string::npos) break;
      start = comma + 1;
    }
    const SideSpec output = side_of(spec.substr(at_arrow + 2));
    if (groups.size() != operands.size())
      throw InvalidArgument("the equation '" + spec + "' names " + std::to_string(groups.size()) + " operands but got " +
                            std::to_string(operands.size()));
    const Category &cat = *operands.front()->cat;
    const Sector charge = has_charge ? charge_in : cat.trivial();
    for (size_t at = 0; at < operands.size(); ++at)
    {
      if (operands[at]->cat != &cat) throw InvalidArgument("an einsum needs every operand over one category");
      if (groups[at].labels.size() != static_cast<size_t>(operands[at]->nlegs()))
        throw InvalidArgument("the group " + std::to_string(at) + " of '" + spec + "' names " +
                              std::to_string(groups[at].labels.size()) + " legs but the tensor has " +
                              std::to_string(operands[at]->nlegs()));
    }
    std::vector<char> seen;
    for (const SideSpec &g : groups)
      for (char label : g.labels)
      {
        if (std::count(seen.begin(), seen.end(), label) >= 2)
          throw InvalidArgument(std::string("the label '") + label + "' of '" + spec + "' names more than two legs");
        seen.push_back(label);
      }
    for (char label : seen)
    {
      const auto count = std::count(seen.begin(), seen.end(), label);
      if (count == 1 && !holds(output.labels, label))
        throw InvalidArgument(std::string("the label '") + label + "' of '" + spec +
                              "' names one leg but is not kept in the output, which would leave it open");
      if (count == 2 && holds(output.labels, label))
        throw InvalidArgument(std::string("the label '") + label + "' of '" + spec + "' is summed over and still kept");
    }
    for (char label : output.labels)
      if (std::count(seen.begin(), seen.end(), label) != 1)
        throw InvalidArgument(std::string("the output label '") + label + "' of '" + spec + "' does not name a leg of the operands");
    std::vector<char> summed;
    for (char label : seen)
      if (std::count(seen.begin(), seen.end(), label) == 2 && !holds(summed, label)) summed.push_back(label);

    auto p = std::make_shared<Program>();
    p->n_inputs = static_cast<int32_t>(operands.size());
    p->input_spaces = operands;
    Builder b(*p);
    // laid_out (einsum.cpp:65-81)
    std::vector<std::vector<Value>> prepared;
    std::vector<std::vector<char>> labels_of;
    for (size_t at = 0; at < operands.size(); ++at)
    {
      Space s = operands[at];
      const int32_t codomain = static_cast<int32_t>(s->codomain.size());
      std::vector<int32_t> above, below;
      for (int32_t leg = 0; leg < s->nlegs(); ++leg)
      {
        const bool stays = holds(summed, groups[at].labels[static_cast<size_t>(leg)]) ? leg < codomain
                                                                                       : static_cast<bool>(groups[at].above[static_cast<size_t>(leg)]);
        (stays ? above : below).push_back(leg);
      }
      std::vector<char> labels;
      for (int32_t leg : above) labels.push_back(groups[at].labels[static_cast<size_t>(leg)]);
      for (int32_t leg : below) labels.push_back(groups[at].labels[static_cast<size_t>(leg)]);
      std::vector<Value> alternatives{b.place(b.input(static_cast<int32_t>(at), s), above, below)};
      // self contractions (einsum.cpp:386-439)
      while (true)
      {
        int32_t first = -1, second = -1;
        for (size_t one = 0; one < labels.size() && first < 0; ++one)
          for (size_t other = one + 1; other < labels.size(); ++other)
            if (labels[one] == labels[other])
            {
              first = static_cast<int32_t>(one);
              second = static_cast<int32_t>(other);
              break;
            }
        if (first < 0) break;
        Space front = alternatives.front().space;
        const int32_t codomain_now = static_cast<int32_t>(front->codomain.size());
        const std::vector<Leg> legs = front->legs();
        if (legs[static_cast<size_t>(first)] != legs[static_cast<size_t>(second)])
          throw InvalidArgument(std::string("the label '") + labels[static_cast<size_t>(first)] + "' of '" + spec +
                                "' names two different spaces in the operand " + std::to_string(at) +
                                ", and a trace sums a space with itself");
        const int32_t above_leg = first < codomain_now ? first : second;
        const int32_t below_leg = first < codomain_now ? second : first;
        std::vector<int32_t> above2, below2;
        for (int32_t leg = 0; leg < front->nlegs(); ++leg)
          if (leg != above_leg && leg != below_leg) (leg < codomain_now ? above2 : below2).push_back(leg);
        above2.push_back(above_leg);
        below2.push_back(below_leg);
        std::vector<Value> traced;
        for (const Value &alt : alternatives)
          for (const Value &t : b.partial_trace(b.place(alt, above2, below2))) traced.push_back(t);
        alternatives = std::move(traced);
        labels.erase(labels.begin() + second);
        labels.erase(labels.begin() + first);
      }
      prepared.push_back(std::move(alternatives));
      labels_of.push_back(std::move(labels));
    }
    // the output legs must close to the charge (einsum.cpp:525-544)
    std::vector<Leg> above_legs, below_legs;
    for (size_t one = 0; one < output.labels.size(); ++one)
      for (size_t at = 0; at < labels_of.size(); ++at)
        if (holds(labels_of[at], output.labels[one]))
        {
          if (prepared[at].empty()) break;
          const Leg leg = prepared[at].front().space->legs()[static_cast<size_t>(position_of(labels_of[at], output.labels[one]))];
          (output.above[one] ? above_legs : below_legs).push_back(leg);
          break;
        }
    bool closes = output.labels.empty();
    if (!closes)
    {
      const std::vector<Sector> below_charges = reachable_charges(cat, below_legs);
      for (const Sector &a : reachable_charges(cat, above_legs))
      {
        for (const Sector &c : below_charges)
          if (cat.n_symbol(a, cat.dual(c), charge) > 0)
          {
            closes = true;
            break;
          }
        if (closes) break;
      }
    }
    if (!closes) throw InvalidArgument("the output legs of '" + spec + "' cannot close to " + charge.str());
    size_t combinations = 1;
    for (const std::vector<Value> &alts : prepared)
    {
      if (alts.empty()) throw InvalidArgument("the traces of '" + spec + "' leave nothing to sum");
      if (static_cast<int64_t>(alts.size()) > kMaxCharges / static_cast<int64_t>(combinations))
        throw InvalidArgument("the traces of '" + spec + "' leave more than " + std::to_string(kMaxCharges) +
                              " combinations of charges, which is more than this sums");
      combinations *= alts.size();
    }
    std::map<char, double> dims;
    for (size_t at = 0; at < labels_of.size(); ++at)
    {
      const std::vector<Leg> legs = prepared[at].front().space->legs();
      for (size_t leg = 0; leg < labels_of[at].size(); ++leg) dims[labels_of[at][leg]] = leg_size(cat, legs[leg]);
    }
    const std::vector<int32_t> order = fold_order(labels_of, dims);

    std::vector<Value> results;
    std::vector<size_t> choice(prepared.size(), 0);
    while (true)
    {
      // contract_path (einsum.cpp:351-376)
      std::vector<char> labels = labels_of.front();
      std::vector<Value> states{prepared[0][choice[0]]};
      for (size_t step = 1; step < order.size(); ++step)
      {
        const int32_t at = order[step];
        const Value right = prepared[static_cast<size_t>(at)][choice[static_cast<size_t>(at)]];
        const std::vector<char> &right_labels = labels_of[static_cast<size_t>(at)];
        // combine (einsum.cpp:306-345)
        const std::vector<char> shared = shared_of(labels, right_labels);
        std::vector<int32_t> left_legs, right_legs;
        for (char l : shared)
        {
          left_legs.push_back(position_of(labels, l));
          right_legs.push_back(position_of(right_labels, l));
        }
        std::vector<Value> folded;
        for (const Value &lv : states)
        {
          check_pairs(lv.space, right.space, left_legs, right_legs);
          const Value above = b.place(lv, without(lv.space->nlegs(), left_legs), left_legs);
          const Value under = b.place(right, right_legs, without(right.space->nlegs(), right_legs));
          std::vector<Sector> closings;
          for (const Outcome &o : cat.outcomes(lv.space->qtotal, right.space->qtotal))
            if (std::find(closings.begin(), closings.end(), o.sector) == closings.end()) closings.push_back(o.sector);
          for (const Sector &closed : closings)
          {
            Builder::require_single_closing(cat, lv.space->qtotal, right.space->qtotal, closed, "the charges", "a contraction");
            folded.push_back(b.contract_aligned(above, under, closed));
          }
        }
        if (static_cast<int64_t>(folded.size()) > kMaxCharges)
          throw InvalidArgument("the products of the equation leave more than " + std::to_string(kMaxCharges) +
                                " charges to sum, which is more than this takes");
        labels = product_labels(labels, right_labels);
        states = std::move(folded);
      }
      std::vector<int32_t> above, below;
      for (size_t at = 0; at < output.labels.size(); ++at)
        (output.above[at] ? above : below).push_back(position_of(labels, output.labels[at]));
      for (const Value &state : states)
      {
        if (!(state.space->qtotal == charge)) continue;
        const Value placed = b.place(state, above, below);
        if (placed.space->blocks.empty()) continue;
        results.push_back(placed);
      }
      size_t digit = 0;
      while (digit < choice.size() && ++choice[digit] == prepared[digit].size())
      {
        choice[digit] = 0;
        ++digit;
      }
      if (digit == choice.size()) break;
    }
    if (results.empty()) throw InvalidArgument("no way for the charges of '" + spec + "' to fuse to " + charge.str());
    finish(*p, b, results);
    p->fold = order;
    return p;
  }

} // namespace ttg
