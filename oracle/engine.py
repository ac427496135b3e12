'''
The oracle: a CPU restatement, in Python and numpy, of the reference's block-sparse contraction path
(Jumqyc/TenTorch: categories, fusion trees, layouts, the per-step regrouping plans, `place`,
`contract` and `einsum`).  Test infrastructure only.  It is imported by `tests/`, by
`__graft_entry__.smoke()` and by the CPU legs of `bench.py` (`cpu_baseline`, `--impl reference`),
always as the checker or the timed CPU baseline, never by the product.

Every function cites the reference file:line it restates.  The restatement keeps the reference's
orders (sector order, tree enumeration, block-key order, piece order) because the plan structures
are compared bit for bit; the arithmetic is plain numpy (`pieces` applied with vectorised
index arithmetic, block products with `@`).  Parity with the reference itself is pinned by the
fixtures in `tests/golden/`, produced by `tests/golden/make_golden.py` from the reference compiled
here by `oracle/build_ref.py`.

Tensors are float64 or complex128 numpy blocks keyed by `BlockKey` tuples
`(codomain_root, domain_root, copy)`.
'''
from __future__ import annotations

import math
from fractions import Fraction
from functools import lru_cache
from itertools import product as cartesian

import numpy as np

# --------------------------------------------------------------------------------------------
# categories (tentorch/symmetry/cat/*)
# --------------------------------------------------------------------------------------------


class Category:
    '''The category interface, tentorch/symmetry/cat/cat.h:190-429.'''
    name = 'category'
    real_symbols = True

    def outcomes(self, a, b):  # list of (sector, multiplicity)
        raise NotImplementedError

    def n_symbol(self, a, b, c):
        '''tentorch/symmetry/cat/cat.cpp:43-53'''
        for sector, mult in self.outcomes(a, b):
            if sector == c:
                return mult
        return 0

    def f_rows(self, a, b, c, d):
        '''tentorch/symmetry/cat/cat.cpp:61-77'''
        rows = []
        for e, mult in self.outcomes(a, b):
            copies = self.n_symbol(e, c, d)
            for inner in range(mult):
                for outer in range(copies):
                    rows.append((e, inner, outer))
        return rows

    def f_columns(self, a, b, c, d):
        '''tentorch/symmetry/cat/cat.cpp:79-95'''
        cols = []
        for f, mult in self.outcomes(b, c):
            copies = self.n_symbol(a, f, d)
            for inner in range(mult):
                for outer in range(copies):
                    cols.append((f, inner, outer))
        return cols

    def r_rows(self, b, c):
        '''tentorch/symmetry/cat/cat.cpp:97-108'''
        return [(e, copy) for e, mult in self.outcomes(b, c) for copy in range(mult)]


class Abelian(Category):
    '''tentorch/symmetry/cat/abelian/abelian.cpp:33-54: F = R = 1 from all-ones vertices.'''

    def outcomes(self, a, b):
        return [(self.combine(a, b), 1)]

    def trivial(self):
        return (0,)

    def dual(self, a):
        return self.inverse(a)

    def q_dim(self, a):
        return 1.0

    @lru_cache(maxsize = None)
    def F_symbol(self, a, b, c, d):
        return np.ones((len(self.f_rows(a, b, c, d)), len(self.f_columns(a, b, c, d))), complex)

    @lru_cache(maxsize = None)
    def R_symbol(self, b, c):
        n = len(self.r_rows(b, c))
        return np.ones((n, n), complex) if n else np.zeros((0, 0), complex)


class U1(Abelian):
    '''tentorch/symmetry/cat/abelian/abelian.cpp:75-83'''
    name = 'U(1)'

    def combine(self, a, b):
        return (a[0] + b[0],)

    def inverse(self, a):
        return (-a[0],)


class NoSymmetry(Abelian):
    '''tentorch/symmetry/cat/abelian/abelian.cpp:69-73'''
    name = 'NoSymmetry'

    def combine(self, a, b):
        return (0,)

    def inverse(self, a):
        return (0,)


class ZN(Abelian):
    '''tentorch/symmetry/cat/abelian/abelian.cpp:85-92'''

    def __init__(self, modulus):
        self.modulus = modulus
        self.name = f'Z_{modulus}'

    def combine(self, a, b):
        return ((a[0] + b[0]) % self.modulus,)

    def inverse(self, a):
        return ((-a[0]) % self.modulus,)


class FermionParity(Category):
    '''tentorch/symmetry/cat/abelian/abelian.cpp:94-124: trivial F, Koszul sign in R.'''
    name = 'FermionParity'

    def outcomes(self, a, b):
        return [(((a[0] + b[0]) % 2,), 1)]

    def trivial(self):
        return (0,)

    def dual(self, a):
        return a

    def q_dim(self, a):
        return 1.0

    def F_symbol(self, a, b, c, d):
        side = 1 if (a[0] + b[0] + c[0]) % 2 == d[0] else 0
        return np.ones((side, side), complex)

    def R_symbol(self, b, c):
        return np.full((1, 1), -1.0 if b[0] == 1 and c[0] == 1 else 1.0, complex)


def _cg_racah(j1, j2, j3, m1, m2):
    '''Clebsch-Gordan <j1 m1; j2 m2 | j3 m1+m2> in the Condon-Shortley phase, from Racah's closed
    formula (Racah 1942) with exact rational arithmetic; arguments are twice the spins.'''
    m3 = m1 + m2
    if abs(m1) > j1 or abs(m2) > j2 or abs(m3) > j3:
        return 0.0
    f = math.factorial
    a, b, c = j1, j2, j3
    # half-integer arguments are carried doubled, so every factorial argument is (sum)/2
    def h(x):
        assert x % 2 == 0, x
        return x // 2
    if a + b < c or abs(a - b) > c or (a + b + c) % 2:
        return 0.0
    pre = Fraction((c + 1) * f(h(a + b - c)) * f(h(a - b + c)) * f(h(-a + b + c)), f(h(a + b + c + 2)))
    pre *= f(h(c + m3)) * f(h(c - m3)) * f(h(a - m1)) * f(h(a + m1)) * f(h(b - m2)) * f(h(b + m2))
    total = Fraction(0)
    for k in range(0, h(a + b - c) + 1):
        args = [k, h(a + b - c) - k, h(a - m1) - k, h(b + m2) - k, h(c - b + m1) + k, h(c - a - m2) + k]
        if min(args) < 0:
            continue
        term = Fraction(1, math.prod(f(x) for x in args))
        total += -term if k % 2 else term
    if not total:
        return 0.0
    # one correctly rounded square root of the exact square
    return math.copysign(math.sqrt(pre * total * total), float(total))


class SU2(Category):
    '''tentorch/symmetry/cat/su2/su2.cpp:20-58 with the group layer tentorch/symmetry/cat/group.cpp:
    F and R are overlaps of Clebsch-Gordan tensors divided by the quantum dimension.'''
    name = 'SU(2)'

    def outcomes(self, a, b):
        return [((jj,), 1) for jj in range(abs(a[0] - b[0]), a[0] + b[0] + 1, 2)]

    def trivial(self):
        return (0,)

    def dual(self, a):
        return a

    def q_dim(self, a):
        return float(a[0] + 1)

    @lru_cache(maxsize = None)
    def cg(self, a, b, c):
        '''The vertex tensor of shape (dim a, dim b, dim c), components ordered m = -j..j
        (tentorch/symmetry/cat/su2/su2.cpp:62-125 indexes k = (m + j)/2).'''
        j1, j2, j3 = a[0], b[0], c[0]
        out = np.zeros((j1 + 1, j2 + 1, j3 + 1))
        for k1 in range(j1 + 1):
            for k2 in range(j2 + 1):
                m1, m2 = 2 * k1 - j1, 2 * k2 - j2
                m3 = m1 + m2
                if abs(m3) <= j3:
                    out[k1, k2, (m3 + j3) // 2] = _cg_racah(j1, j2, j3, m1, m2)
        return out

    @lru_cache(maxsize = None)
    def F_symbol(self, a, b, c, d):
        '''tentorch/symmetry/cat/group.cpp:44-83'''
        rows, cols = self.f_rows(a, b, c, d), self.f_columns(a, b, c, d)
        if not rows or not cols:
            return np.zeros((len(rows), len(cols)), complex)
        left = [np.einsum('abe,ecd->abcd', self.cg(a, b, e), self.cg(e, c, d)).ravel() for e, _, _ in rows]
        right = [np.einsum('bce,aed->abcd', self.cg(b, c, f), self.cg(a, f, d)).ravel() for f, _, _ in cols]
        return (np.stack(left) @ np.stack(right).T / self.q_dim(d)).astype(complex)

    @lru_cache(maxsize = None)
    def R_symbol(self, b, c):
        '''tentorch/symmetry/cat/group.cpp:93-130 (multiplicity free: one entry per outcome)'''
        rows = self.r_rows(b, c)
        out = np.zeros((len(rows), len(rows)), complex)
        for i, (e, _) in enumerate(rows):
            straight = self.cg(b, c, e).ravel()
            swapped = self.cg(c, b, e).transpose(1, 0, 2).ravel()
            out[i, i] = straight @ swapped / self.q_dim(e)
        return out


class Fibonacci(Category):
    '''tentorch/symmetry/cat/fibonacci/fibonacci.cpp:24-86'''
    name = 'FibonacciCategory'
    real_symbols = False

    def outcomes(self, a, b):
        if a[0] == 0:
            return [(b, 1)]
        if b[0] == 0:
            return [(a, 1)]
        return [((0,), 1), ((1,), 1)]

    def trivial(self):
        return (0,)

    def dual(self, a):
        return a

    def q_dim(self, a):
        return (1 + math.sqrt(5)) / 2 if a[0] == 1 else 1.0

    @lru_cache(maxsize = None)
    def F_symbol(self, a, b, c, d):
        rows, cols = self.f_rows(a, b, c, d), self.f_columns(a, b, c, d)
        out = np.zeros((len(rows), len(cols)), complex)
        if not rows or not cols:
            return out
        if a == b == c == d == (1,):
            phi = (1 + math.sqrt(5)) / 2
            golden = [[1 / phi, 1 / math.sqrt(phi)], [1 / math.sqrt(phi), -1 / phi]]
            for i, r in enumerate(rows):
                for j, col in enumerate(cols):
                    out[i, j] = golden[r[0][0]][col[0][0]]
            return out
        out[:] = 1.0
        return out

    @lru_cache(maxsize = None)
    def R_symbol(self, b, c):
        rows = self.r_rows(b, c)
        out = np.zeros((len(rows), len(rows)), complex)
        for i, (e, _) in enumerate(rows):
            phase = 1.0 + 0j
            if b[0] == 1 and c[0] == 1:
                angle = -4 * math.pi / 5 if e[0] == 0 else 3 * math.pi / 5
                phase = complex(math.cos(angle), math.sin(angle))
            out[i, i] = phase
        return out


u1, su2, fibonacci, no_symmetry, fermion_parity = U1(), SU2(), Fibonacci(), NoSymmetry(), FermionParity()
CATEGORIES = {'u1': u1, 'su2': su2, 'fibonacci': fibonacci, 'no_symmetry': no_symmetry,
              'fermion_parity': fermion_parity}

# --------------------------------------------------------------------------------------------
# legs, trees, layouts (tentorch/symmetry/tree/tree.cpp, tentorch/tensors/layout.cpp)
# --------------------------------------------------------------------------------------------


class Leg:
    '''tentorch/symmetry/tree/tree.cpp:90-140: blocks sorted by sector, distinct, positive.'''

    def __init__(self, cat, sectors, multiplicities):
        pairs = sorted(zip((tuple(s) for s in sectors), (int(m) for m in multiplicities)))
        for (s, m) in pairs:
            if m <= 0:
                raise ValueError(f'A block multiplicity must be positive, got {m}.')
        for i in range(1, len(pairs)):
            if pairs[i][0] == pairs[i - 1][0]:
                raise ValueError(f'A leg cannot hold the sector {pairs[i][0]} twice.')
        self.cat = cat
        self.sectors = tuple(p[0] for p in pairs)
        self.multiplicities = tuple(p[1] for p in pairs)

    def nblocks(self):
        return len(self.sectors)

    def multiplicity_of(self, sector):
        '''tentorch/tensors/layout.cpp:8-16 (block_of) then the multiplicity'''
        i = self.sectors.index(sector)
        return self.multiplicities[i]

    def multiplets(self):
        return sum(self.multiplicities)

    def __eq__(self, other):
        return (isinstance(other, Leg) and self.cat is other.cat and self.sectors == other.sectors and
                self.multiplicities == other.multiplicities)

    def __hash__(self):
        return hash((id(self.cat), self.sectors, self.multiplicities))

    def __repr__(self):
        return f'Leg({self.cat.name}: ' + ', '.join(f'{s}:{m}' for s, m in zip(self.sectors, self.multiplicities)) + ')'


def reachable_charges(cat, legs):
    '''tentorch/symmetry/tree/tree.cpp:375-398'''
    charges = [cat.trivial()]
    for leg in legs:
        nxt, seen = [], set()
        for charge in charges:
            for s in leg.sectors:
                for out, _ in cat.outcomes(charge, s):
                    if out not in seen:
                        seen.add(out)
                        nxt.append(out)
        charges = nxt
    return charges


def fusion_trees(cat, legs, coupled):
    '''tentorch/symmetry/tree/tree.cpp:400-471: DFS over leg blocks x outcomes x copies.
    A tree is (sectors, inner, copies, coupled), all tuples.'''
    n = len(legs)
    if n == 0:
        return [((), (), (), coupled)] if coupled == cat.trivial() else []
    out = []
    sectors = [None] * n
    inner = [None] * max(n - 2, 0)
    copies = [None] * max(n - 1, 0)

    def walk(leg, previous):
        for s in legs[leg].sectors:
            sectors[leg] = s
            if leg == 0:
                if n == 1:
                    if s == coupled:
                        out.append(((s,), (), (), coupled))
                else:
                    walk(1, s)
                continue
            for o, mult in cat.outcomes(previous, s):
                if leg + 1 == n and o != coupled:
                    continue
                if leg + 1 < n:
                    inner[leg - 1] = o
                for copy in range(mult):
                    copies[leg - 1] = copy
                    if leg + 1 == n:
                        out.append((tuple(sectors), tuple(inner), tuple(copies), coupled))
                    else:
                        walk(leg + 1, o)
    walk(0, cat.trivial())
    return out


def trimmed(cat, tree):
    '''tentorch/symmetry/tree/tree.cpp:473-484'''
    sectors, inner, copies, coupled = tree
    n = len(sectors)
    root = cat.trivial() if n <= 1 else (sectors[0] if n == 2 else inner[n - 3])
    return (sectors[:-1], inner[:-1] if inner else (), copies[:-1] if copies else (), root)


_layouts = {}


def layout_of(cat, legs, root):
    '''tentorch/tensors/layout.cpp:18-32: trees and the first row of each (cached).'''
    key = (id(cat), tuple(legs), root)
    got = _layouts.get(key)
    if got is None:
        trees = fusion_trees(cat, legs, root)
        offsets = [0]
        for tree in trees:
            rows = 1
            for leg, s in zip(legs, tree[0]):
                rows *= leg.multiplicity_of(s)
            offsets.append(offsets[-1] + rows)
        got = (trees, offsets)
        _layouts[key] = got
    return got


def block_keys(cat, codomain, domain, qtotal):
    '''tentorch/tensors/layout.cpp:34-47 (the tensor then holds them in std::map order)'''
    keys = []
    for r in reachable_charges(cat, codomain):
        for s in reachable_charges(cat, domain):
            for copy in range(cat.n_symbol(r, cat.dual(s), qtotal)):
                keys.append((r, s, copy))
    return keys


# --------------------------------------------------------------------------------------------
# tensors (tentorch/tensors/tensor.cpp)
# --------------------------------------------------------------------------------------------


class Tensor:
    '''tentorch/tensors/tensor.h:43-216: one dense row-major matrix per block key, all allocated.'''

    def __init__(self, cat, codomain, domain, qtotal, dtype = np.float64):
        self.cat, self.codomain, self.domain = cat, list(codomain), list(domain)
        self.qtotal, self.dtype = tuple(qtotal), np.dtype(dtype)
        self.blocks = {}
        for key in sorted(block_keys(cat, self.codomain, self.domain, self.qtotal)):
            rows = layout_of(cat, self.codomain, key[0])[1][-1]
            cols = layout_of(cat, self.domain, key[1])[1][-1]
            self.blocks[key] = np.zeros((rows, cols), self.dtype)

    def legs(self):
        return self.codomain + self.domain

    def nlegs(self):
        return len(self.codomain) + len(self.domain)

    def copy(self):
        out = Tensor.__new__(Tensor)
        out.cat, out.codomain, out.domain, out.qtotal, out.dtype = (self.cat, list(self.codomain),
                                                                     list(self.domain), self.qtotal, self.dtype)
        out.blocks = {k: v.copy() for k, v in self.blocks.items()}
        return out

    def conj(self):
        '''tentorch/tensors/tensor.cpp:99-107'''
        out = Tensor(self.cat, self.domain, self.codomain, self.cat.dual(self.qtotal), self.dtype)
        for (r, s, c), block in self.blocks.items():
            out.blocks[(s, r, c)][...] = block.conj().T
        return out

    def fill_random(self, generator):
        '''Fill every block in key order with standard normal float64 draws from a torch generator.'''
        import torch
        for key in self.blocks:
            shape = self.blocks[key].shape
            self.blocks[key][...] = torch.randn(shape, dtype = torch.float64, generator = generator).numpy()
        return self

    def place(self, above, below = None):
        return place(self, above, below)


def inner(a, b):
    '''tentorch/linalg/graded/compare.cpp:31-43'''
    if a.qtotal != b.qtotal:
        return 0.0
    return sum(np.vdot(block, b.blocks[key]) for key, block in a.blocks.items())


def norm(t):
    '''tentorch/linalg/graded/compare.cpp:45'''
    return math.sqrt(abs(inner(t, t)))


# --------------------------------------------------------------------------------------------
# regrouping plans (tentorch/tensors/regroup.cpp)
# --------------------------------------------------------------------------------------------


def _chain_at(cat, tree, last):
    '''tentorch/tensors/regroup.cpp:16-22'''
    sectors, inner, _, coupled = tree
    if last < 0:
        return cat.trivial()
    if last + 1 == len(sectors):
        return coupled
    if last == 0:
        return sectors[0]
    return inner[last - 1]


def exchange_regrouping(cat, codomain, domain, key, qtotal, p):
    '''tentorch/tensors/regroup.cpp:25-258.  Returns shifts [(from, to, rows, cols, pieces)] with
    pieces (first, last, from_step, to_step, run, coefficient).'''
    count = len(codomain)
    exchanged = list(codomain)
    exchanged[p], exchanged[p + 1] = exchanged[p + 1], exchanged[p]
    src_trees, src_off = layout_of(cat, codomain, key[0])
    dst_trees, dst_off = layout_of(cat, exchanged, key[0])
    stride = layout_of(cat, domain, key[1])[1][-1]

    def signature(tree, exchanged_tree):
        sectors, inner, copies, _ = tree
        out = []
        for axis in range(count):
            frm = (p + 1 if axis == p else p) if exchanged_tree and axis in (p, p + 1) else axis
            out.extend(sectors[frm])
        for at, charge in enumerate(inner):
            if at != p - 1:
                out.extend(charge)
        for at, c in enumerate(copies):
            if at not in (p - 1, p):
                out.append(c)
        return tuple(out)

    def moved(axis):
        return p + 1 if axis == p else (p if axis == p + 1 else axis)

    def shape_of(tree, legs):
        return tuple(legs[axis].multiplicity_of(tree[0][axis]) for axis in range(count))

    groups, partners = {}, {}
    for at, tree in enumerate(src_trees):
        groups.setdefault(signature(tree, False), []).append(at)
    for at, tree in enumerate(dst_trees):
        partners.setdefault(signature(tree, True), []).append(at)

    factors = {}
    for marks in sorted(groups):
        olds = groups[marks]
        if marks not in partners:
            raise RuntimeError('the exchange has no image for a tree of the codomain')
        news = partners[marks]
        sample = src_trees[olds[0]]
        y, d = _chain_at(cat, sample, p - 1), _chain_at(cat, sample, p + 1)
        b, c = sample[0][p], sample[0][p + 1]
        straight = cat.F_symbol(y, b, c, d)
        braided = cat.F_symbol(y, c, b, d)
        offset, at = [], 0
        for sector, mult in cat.outcomes(b, c):
            offset.append((sector, at))
            at += mult
        frm = cat.f_columns(y, b, c, d)
        to = cat.f_columns(y, c, b, d)
        braid = cat.R_symbol(b, c)

        def braid_at(index):
            for sector, start in offset:
                if sector == index[0]:
                    return start + index[1]
            return -1
        rows = [braid_at(i) for i in to]
        cols = [braid_at(j) for j in frm]
        terms = []
        for i in range(len(to)):
            if rows[i] < 0:
                continue
            for j in range(len(frm)):
                if cols[j] < 0 or to[i][0] != frm[j][0] or to[i][2] != frm[j][2]:
                    continue
                terms.append((i, rows[i], cols[j], j))
        for one_i, one in enumerate(news):
            for other_i, other in enumerate(olds):
                value = 0j
                for (i, br, bc, j) in terms:
                    value += braided[one_i, i] * braid[br, bc] * np.conj(straight[other_i, j])
                if value == 0:
                    continue
                factors[(one, other)] = value

    before, after = {}, {}
    after_shapes = [None] * len(dst_trees)
    for at, tree in enumerate(src_trees):
        before.setdefault(shape_of(tree, codomain), []).append(at)
    for at, tree in enumerate(dst_trees):
        shape = shape_of(tree, exchanged)
        back = [0] * count
        for axis in range(count):
            back[moved(axis)] = shape[axis]
        after_shapes[at] = shape
        after.setdefault(tuple(back), []).append(at)
    pieces = []
    for shape in sorted(before):
        olds = before[shape]
        if shape not in after:
            raise RuntimeError('the exchange has no image for a block of trees')
        news = after[shape]
        width = math.prod(shape)
        target_shape = after_shapes[news[0]]
        width_of = []
        for at in range(width):
            digits, left = [0] * count, at
            for axis in range(count - 1, -1, -1):
                digits[axis] = left % shape[axis]
                left //= shape[axis]
            placed = [0] * count
            for axis in range(count):
                placed[moved(axis)] = digits[axis]
            index = 0
            for axis in range(count):
                index = index * target_shape[axis] + placed[axis]
            width_of.append(index)
        for one in news:
            for other in olds:
                factor = factors.get((one, other))
                if factor is None:
                    continue
                at = 0
                while at < width:
                    run = 1
                    while at + run < width and width_of[at + run] == width_of[at] + run:
                        run += 1
                    pieces.append(((src_off[other] + at) * stride, (dst_off[one] + width_of[at]) * stride,
                                   1, 1, run * stride, factor))
                    at += run
    return [(key, key, 0, 0, pieces)]


def bend_regrouping(cat, codomain, domain, key, qtotal, from_codomain):
    '''tentorch/tensors/regroup.cpp:260-417'''
    giving = codomain if from_codomain else domain
    taking = domain if from_codomain else codomain
    moved_leg = giving[-1]
    kept_giving = list(giving[:-1])
    kept_taking = list(taking) + [moved_leg]
    out_codomain = kept_giving if from_codomain else kept_taking
    out_domain = kept_taking if from_codomain else kept_giving
    moved_trees, moved_off = layout_of(cat, codomain if from_codomain else domain, key[0] if from_codomain else key[1])
    gains_trees, gains_off = layout_of(cat, domain if from_codomain else codomain, key[1] if from_codomain else key[0])
    moved_root = key[0] if from_codomain else key[1]
    gains_root = key[1] if from_codomain else key[0]
    source_stride = (gains_off if from_codomain else moved_off)[-1]
    shifts, at_of, out_layouts = [], {}, {}

    def index_of(to, rows, cols):
        if to not in at_of:
            at_of[to] = len(shifts)
            shifts.append((key, to, rows, cols, []))
        return at_of[to]

    for gains_at, gains_tree in enumerate(gains_trees):
        gains = gains_off[gains_at + 1] - gains_off[gains_at]
        for moved_at, moved_tree in enumerate(moved_trees):
            charge = moved_tree[0][-1]
            copies = moved_leg.multiplicity_of(charge)
            span = moved_off[moved_at + 1] - moved_off[moved_at]
            inside = span // copies
            kept_tree = trimmed(cat, moved_tree)
            prefix = kept_tree[3]
            copy = moved_tree[2][-1] if len(moved_tree[0]) >= 2 else 0
            first = prefix if from_codomain else gains_root
            middle = charge if from_codomain else cat.dual(charge)
            last = cat.dual(gains_root) if from_codomain else cat.dual(prefix)
            coefficients = cat.F_symbol(first, middle, last, qtotal)
            across = cat.f_rows(first, middle, last, qtotal)
            along = cat.f_columns(first, middle, last, qtotal)
            named = across if from_codomain else along
            free = along if from_codomain else across
            named_root = moved_root if from_codomain else cat.dual(moved_root)
            taken = [i for i, n in enumerate(named) if n[0] == named_root and n[1] == copy and n[2] == key[2]]
            if not taken:
                continue
            source_row = moved_off[moved_at]
            source_column = gains_off[gains_at]
            for index in taken:
                for column, taken_side in enumerate(free):
                    # entry [index * width + column] of the row-major matrix in both directions
                    # (tentorch/tensors/regroup.cpp:350), `index` counting the named side
                    value = coefficients.reshape(-1)[index * coefficients.shape[1] + column]
                    if value == 0:
                        continue
                    extended_root = cat.dual(taken_side[0]) if from_codomain else taken_side[0]
                    g_sectors, g_inner, g_copies, _ = gains_tree
                    ext = (g_sectors + (cat.dual(charge),),
                           g_inner + ((gains_root,) if len(g_sectors) >= 2 else ()),
                           g_copies + ((taken_side[1],) if len(g_sectors) >= 1 else ()),
                           extended_root)
                    out_cod_root = prefix if from_codomain else extended_root
                    out_dom_root = extended_root if from_codomain else prefix
                    roots = (out_cod_root, out_dom_root)
                    if roots not in out_layouts:
                        r_trees, r_off = layout_of(cat, out_codomain, out_cod_root)
                        c_trees, c_off = layout_of(cat, out_domain, out_dom_root)
                        out_layouts[roots] = (r_off, c_off, {t: i for i, t in enumerate(r_trees)},
                                              {t: i for i, t in enumerate(c_trees)})
                    r_off, c_off, row_of, col_of = out_layouts[roots]
                    ra = row_of.get(kept_tree if from_codomain else ext)
                    ca = col_of.get(ext if from_codomain else kept_tree)
                    if ra is None or ca is None:
                        continue
                    row, column_offset = r_off[ra], c_off[ca]
                    target_stride = c_off[-1]
                    pieces = shifts[index_of((out_cod_root, out_dom_root, taken_side[2]), r_off[-1], c_off[-1])][4]
                    if from_codomain:
                        for shifted in range(inside):
                            for gain in range(gains):
                                pieces.append(((source_row + shifted * copies) * source_stride + source_column + gain,
                                               (row + shifted) * target_stride + column_offset + gain * copies,
                                               source_stride, 1, copies, value))
                    else:
                        for gain in range(gains):
                            for copy_at in range(copies):
                                pieces.append(((source_column + gain) * source_stride + source_row + copy_at,
                                               (row + gain * copies + copy_at) * target_stride + column_offset,
                                               copies, 1, inside, value))
    return shifts


# --------------------------------------------------------------------------------------------
# chains and place (tentorch/tensors/place.cpp)
# --------------------------------------------------------------------------------------------


def chain_steps(codomain, domain, above, below):
    '''The step sequence of tentorch/tensors/place.cpp:199-247 (Chain: folds up, bubble sort, folds
    down).  Each step is (kind, arm, codomain_after, domain_after); kind 'x' exchange at `arm`,
    'up' bends the last domain leg up, 'down' the last codomain leg down.'''
    height, depth = len(codomain), len(domain)
    total = height + depth
    named = [False] * total
    for side in (above, below):
        for leg in side:
            if leg < 0 or leg >= total:
                raise ValueError(f'the leg {leg} does not exist, the tensor has {total} legs')
            if named[leg]:
                raise ValueError(f'the leg {leg} is named twice')
            named[leg] = True
    if len(above) + len(below) != total:
        raise ValueError(f'the leg {named.index(False)} is named on neither side')
    cod, dom = list(codomain), list(domain)
    steps = []

    def fold(from_codomain):
        if from_codomain:
            dom.append(cod.pop())
        else:
            cod.append(dom.pop())
        steps.append(('down' if from_codomain else 'up', 0, list(cod), list(dom)))

    def exchange(position):
        cod[position], cod[position + 1] = cod[position + 1], cod[position]
        steps.append(('x', position, list(cod), list(dom)))

    descends = any(leg < height for leg in below)
    kept = 0
    while not descends and kept < depth and kept < len(below) and below[kept] == height + kept:
        kept += 1
    for _ in range(kept, depth):
        fold(False)

    def position_of(leg):
        return leg if leg < height else height + (depth - 1 - (leg - height))
    order = [position_of(leg) for leg in above] + [position_of(leg) for leg in reversed(below[kept:])]
    which = list(range(len(cod)))
    for at in range(len(order)):
        frm = at
        while which[frm] != order[at]:
            frm += 1
        while frm > at:
            exchange(frm - 1)
            which[frm - 1], which[frm] = which[frm], which[frm - 1]
            frm -= 1
    for _ in range(kept, len(below)):
        fold(True)
    return steps


_plans = {}


def plan_of(cat, codomain, domain, key, qtotal, step):
    '''tentorch/tensors/place.cpp:110-123 with the cache of tentorch/tensors/cache.cpp:197-218'''
    kind, arm = step[0], step[1]
    name = (id(cat), tuple(codomain), tuple(domain), key, qtotal, kind, arm)
    got = _plans.get(name)
    if got is None:
        if kind == 'x':
            got = exchange_regrouping(cat, codomain, domain, key, qtotal, arm)
        else:
            got = bend_regrouping(cat, codomain, domain, key, qtotal, kind == 'down')
        got = [(frm, to, rows, cols, pieces, _piece_arrays(pieces)) for frm, to, rows, cols, pieces in got]
        _plans[name] = got
    return got


def _piece_arrays(pieces):
    '''The runs of a shift expanded to flat index arrays, so a plan applies in one numpy pass.'''
    if not pieces:
        return np.zeros(0, np.int64), np.zeros(0, np.int64), np.zeros(0, complex), True
    arr = np.array([(p[0], p[1], p[2], p[3], p[4]) for p in pieces], np.int64)
    runs = arr[:, 4]
    rep = np.repeat(np.arange(len(pieces)), runs)
    starts = np.cumsum(runs) - runs
    step = np.arange(rep.size) - starts[rep]
    src = arr[rep, 0] + step * arr[rep, 2]
    dst = arr[rep, 1] + step * arr[rep, 3]
    coef = np.array([p[5] for p in pieces], complex)[rep]
    unique = np.unique(dst).size == dst.size
    return src, dst, coef, unique


def _apply(arrays, source, target):
    '''tentorch/tensors/cache.cpp:66-92: to[last + i*ts] += c * from[first + i*fs]; a float64
    block takes the real part of the coefficient (tentorch/tensors/cache.cpp:84-92).'''
    src, dst, coef, unique = arrays
    if src.size == 0:
        return
    flat = target.reshape(-1)
    c = coef if np.iscomplexobj(target) else coef.real
    if unique:
        flat[dst] += c * source.reshape(-1)[src]
    else:
        np.add.at(flat, dst, c * source.reshape(-1)[src])


def carried(tensor, steps):
    '''tentorch/tensors/place.cpp:127-180: every block through every step, buffers per step.'''
    if not steps:
        return tensor
    out = Tensor(tensor.cat, steps[-1][2], steps[-1][3], tensor.qtotal, tensor.dtype)
    for start, block in tensor.blocks.items():
        live = {start: block}
        codomain, domain = tensor.codomain, tensor.domain
        for at, step in enumerate(steps):
            last = at + 1 == len(steps)
            nxt = {}
            for key, buffer in live.items():
                plan = plan_of(tensor.cat, codomain, domain, key, tensor.qtotal, step)
                for frm, to, rows, cols, pieces, arrays in plan:
                    if last:
                        target = out.blocks[to]
                    else:
                        if to not in nxt:
                            shape = (rows if rows else buffer.shape[0], cols if cols else buffer.shape[1])
                            nxt[to] = np.zeros(shape, tensor.dtype)
                        target = nxt[to]
                    _apply(arrays, buffer, target)
            codomain, domain = step[2], step[3]
            live = nxt
    return out


def place(tensor, above, below = None):
    '''tentorch/tensors/place.cpp:183-247'''
    total = tensor.nlegs()
    if below is None:
        below = [leg for leg in range(total) if leg not in set(above)]
    steps = chain_steps(tensor.codomain, tensor.domain, list(above), list(below))
    return carried(tensor, steps)


# --------------------------------------------------------------------------------------------
# contraction (tentorch/linalg/graded/contract.cpp)
# --------------------------------------------------------------------------------------------


def _without(total, taken):
    return [leg for leg in range(total) if leg not in set(taken)]


def _check_pairs(left, right, left_legs, right_legs):
    '''tentorch/linalg/graded/contract.cpp:47-77'''
    if left.cat is not right.cat:
        raise ValueError('a contraction needs both tensors over one category')
    if left.dtype != right.dtype:
        raise ValueError('a contraction needs both tensors of one scalar type')
    if len(left_legs) != len(right_legs):
        raise ValueError('the two legs of a contraction must be given in pairs')
    for t, legs in ((left, left_legs), (right, right_legs)):
        if len(set(legs)) != len(legs) or any(l < 0 or l >= t.nlegs() for l in legs):
            raise ValueError('a summed leg is out of range or named twice')
    la, ra = left.legs(), right.legs()
    for a, b in zip(left_legs, right_legs):
        if la[a] != ra[b]:
            raise ValueError(f'the pair joins the leg {a} to the leg {b}, and the two do not name one space')


def align(left, right, left_legs, right_legs):
    '''tentorch/linalg/graded/contract.cpp:80-91,108-115'''
    _check_pairs(left, right, left_legs, right_legs)
    return (place(left, _without(left.nlegs(), left_legs), list(left_legs)),
            place(right, list(right_legs), _without(right.nlegs(), right_legs)))


def _single_closing(cat, above, below, charge):
    '''tentorch/linalg/graded/contract.cpp:95-106'''
    if cat.n_symbol(above, cat.dual(below), charge) > 1:
        raise ValueError('the roots close in more than one way, which a contraction does not recouple yet')


def contract_aligned(above, under, charge):
    '''tentorch/linalg/graded/contract.cpp:123-165, on operands that are already aligned.'''
    cat = above.cat
    out = Tensor(cat, above.codomain, under.domain, charge, above.dtype)
    for key in above.blocks:
        _single_closing(cat, key[0], key[1], above.qtotal)
    for key in under.blocks:
        _single_closing(cat, key[0], key[1], under.qtotal)
    for key in out.blocks:
        _single_closing(cat, key[0], key[1], charge)
    rows = {}
    for key, block in under.blocks.items():
        rows.setdefault(key[0], []).append((key[1], block))
    for key, left_block in above.blocks.items():
        for domain_root, right_block in rows.get(key[1], []):
            if cat.n_symbol(key[0], cat.dual(domain_root), charge) == 0:
                continue
            out.blocks[(key[0], domain_root, 0)] += left_block @ right_block
    return out


def contract(left, right, left_legs, right_legs, charge = None):
    '''tentorch/linalg/graded/contract.cpp:117-175'''
    if charge is None:
        if right.qtotal != left.cat.trivial():
            raise ValueError('the second tensor of a contraction must carry the trivial charge')
        charge = left.qtotal
    _check_pairs(left, right, left_legs, right_legs)
    cat = left.cat
    if cat.n_symbol(left.qtotal, right.qtotal, charge) == 0:
        raise ValueError(f'the charge {charge} is not an outcome of {left.qtotal} and {right.qtotal}')
    _single_closing(cat, left.qtotal, right.qtotal, charge)
    above, under = align(left, right, left_legs, right_legs)
    return contract_aligned(above, under, charge)


# --------------------------------------------------------------------------------------------
# einsum (tentorch/linalg/graded/einsum.cpp)
# --------------------------------------------------------------------------------------------


def _side_of(text):
    '''tentorch/linalg/graded/einsum.cpp:35-45'''
    labels, above = [], []
    for ch in text:
        if ch == ' ':
            continue
        labels.append(ch.lower())
        above.append('A' <= ch <= 'Z')
    return labels, above


def _laid_out(tensor, side, summed):
    '''tentorch/linalg/graded/einsum.cpp:65-81'''
    labels, wants = side
    codomain = len(tensor.codomain)
    above, below = [], []
    for leg in range(tensor.nlegs()):
        stays = (leg < codomain) if labels[leg] in summed else wants[leg]
        (above if stays else below).append(leg)
    return place(tensor, above, below), [labels[l] for l in above] + [labels[l] for l in below]


def _partial_trace(tensor):
    '''tentorch/linalg/graded/einsum.cpp:95-159'''
    cat, q = tensor.cat, tensor.qtotal
    out_cod, out_dom = tensor.codomain[:-1], tensor.domain[:-1]
    out = {}
    for key, matrix in tensor.blocks.items():
        _single_closing(cat, key[0], key[1], q)
        r_trees, r_off = layout_of(cat, tensor.codomain, key[0])
        c_trees, c_off = layout_of(cat, tensor.domain, key[1])
        for ri, above_tree in enumerate(r_trees):
            row_span = r_off[ri + 1] - r_off[ri]
            kept_above = trimmed(cat, above_tree)
            for ci, under_tree in enumerate(c_trees):
                col_span = c_off[ci + 1] - c_off[ci]
                if above_tree[0][-1] != under_tree[0][-1]:
                    continue
                kept_under = trimmed(cat, under_tree)
                o_r_trees, o_r_off = layout_of(cat, out_cod, kept_above[3])
                o_c_trees, o_c_off = layout_of(cat, out_dom, kept_under[3])
                new_row = o_r_trees.index(kept_above)
                new_col = o_c_trees.index(kept_under)
                inside_rows = o_r_off[new_row + 1] - o_r_off[new_row]
                inside_cols = o_c_off[new_col + 1] - o_c_off[new_col]
                copies = row_span // inside_rows
                piece = matrix[r_off[ri]:r_off[ri] + row_span, c_off[ci]:c_off[ci] + col_span]
                piece = piece.reshape(inside_rows, copies, inside_cols, copies)
                piece = np.einsum('iaja->ij', piece)
                seen = []
                for closing, _ in cat.outcomes(kept_above[3], cat.dual(kept_under[3])):
                    _single_closing(cat, kept_above[3], kept_under[3], closing)
                    if closing not in out:
                        out[closing] = Tensor(cat, out_cod, out_dom, closing, tensor.dtype)
                    t = out[closing]
                    t.blocks[(kept_above[3], kept_under[3], 0)][
                        o_r_off[new_row]:o_r_off[new_row] + inside_rows,
                        o_c_off[new_col]:o_c_off[new_col] + inside_cols] += piece
    return [out[k] for k in sorted(out)]


def _leg_size(cat, leg):
    '''tentorch/linalg/graded/einsum.cpp:162-168'''
    return sum(m * cat.q_dim(s) for s, m in zip(leg.sectors, leg.multiplicities))


def _union(a, b):
    out = list(a)
    for label in b:
        if label not in out:
            out.append(label)
    return out


def _shared(a, b):
    return [label for label in a if label in b]


def _product_labels(a, b):
    shared = _shared(a, b)
    return [label for label in _union(a, b) if label not in shared]


def fold_order(inputs, dims):
    '''tentorch/linalg/graded/einsum.cpp:216-301'''
    count = len(inputs)
    if count <= 12:
        masks = 1 << (count - 1)
        labels = [list(inputs[0])] * masks
        for mask in range(1, masks):
            bit = (mask & -mask).bit_length() - 1
            labels[mask] = _union(labels[mask ^ (1 << bit)], inputs[bit + 1])
        for pss in range(2):
            cost = [math.inf] * masks
            summed = [0] * masks
            last = [0] * masks
            cost[0] = 0
            for mask in range(1, masks):
                for bit in range(count - 1):
                    if not mask & (1 << bit):
                        continue
                    shared = _shared(labels[mask ^ (1 << bit)], inputs[bit + 1])
                    if pss == 0 and not shared:
                        continue
                    size = 1.0
                    for label in labels[mask]:
                        size *= dims[label]
                    candidate = cost[mask ^ (1 << bit)] + size
                    better = (candidate < cost[mask] or
                              (candidate == cost[mask] and len(shared) > summed[mask]) or
                              (candidate == cost[mask] and len(shared) == summed[mask] and bit > last[mask]))
                    if better:
                        cost[mask], summed[mask], last[mask] = candidate, len(shared), bit
            if cost[masks - 1] == math.inf:
                continue
            order, mask = [], masks - 1
            while mask:
                order.append(last[mask] + 1)
                mask ^= 1 << last[mask]
            order.append(0)
            return order[::-1]
    taken = [False] * count
    live = list(inputs[0])
    order = [0]
    taken[0] = True
    for _ in range(1, count):
        best, best_size, found = -1, 0.0, False
        for pss in range(2):
            if found:
                break
            for at in range(count):
                if taken[at] or ((not _shared(live, inputs[at])) != (pss == 1)):
                    continue
                size = 1.0
                for label in _union(live, inputs[at]):
                    size *= dims[label]
                if not found or size < best_size:
                    found, best, best_size = True, at, size
        order.append(best)
        taken[best] = True
        live = _union(live, inputs[best])
    return order


def _combine(left_states, left_labels, right_states, right_labels):
    '''tentorch/linalg/graded/einsum.cpp:306-345'''
    shared = _shared(left_labels, right_labels)
    left_legs = [left_labels.index(l) for l in shared]
    right_legs = [right_labels.index(l) for l in shared]
    folded = []
    for left in left_states:
        for right in right_states:
            above, under = align(left, right, left_legs, right_legs)
            closings = []
            for o, _ in left.cat.outcomes(left.qtotal, right.qtotal):
                if o not in closings:
                    closings.append(o)
            for closed in closings:
                _single_closing(left.cat, left.qtotal, right.qtotal, closed)
                if left.cat.n_symbol(left.qtotal, right.qtotal, closed) == 0:
                    raise ValueError('the charge is not an outcome')
                folded.append(contract_aligned(above, under, closed))
    return folded


def einsum(spec, *operands, outcharge = None):
    '''tentorch/linalg/graded/einsum.cpp:444-605'''
    if not operands:
        raise ValueError('an einsum needs at least one operand')
    if '->' not in spec:
        raise ValueError(f"the equation '{spec}' does not say what it leaves")
    lhs, rhs = spec.split('->', 1)
    groups = [_side_of(g) for g in lhs.split(',')]
    output = _side_of(rhs)
    if len(groups) != len(operands):
        raise ValueError(f"the equation '{spec}' names {len(groups)} operands but got {len(operands)}")
    cat = operands[0].cat
    charge = cat.trivial() if outcharge is None else tuple(outcharge)
    for g, t in zip(groups, operands):
        if t.cat is not cat:
            raise ValueError('an einsum needs every operand over one category')
        if len(g[0]) != t.nlegs():
            raise ValueError('a group names a different number of legs than its tensor has')
    seen = []
    for labels, _ in groups:
        for label in labels:
            if seen.count(label) >= 2:
                raise ValueError(f"the label '{label}' of '{spec}' names more than two legs")
            seen.append(label)
    for label in seen:
        n = seen.count(label)
        if n == 1 and label not in output[0]:
            raise ValueError(f"the label '{label}' of '{spec}' names one leg but is not kept in the output")
        if n == 2 and label in output[0]:
            raise ValueError(f"the label '{label}' of '{spec}' is summed over and still kept")
    for label in output[0]:
        if seen.count(label) != 1:
            raise ValueError(f"the output label '{label}' of '{spec}' does not name a leg of the operands")
    summed = []
    for label in seen:
        if seen.count(label) == 2 and label not in summed:
            summed.append(label)
    laid, inputs = [], []
    for t, g in zip(operands, groups):
        tensor, labels = _laid_out(t, g, summed)
        laid.append(tensor)
        inputs.append(labels)
    # self contractions (tentorch/linalg/graded/einsum.cpp:386-439)
    prepared, prep_labels = [], []
    for at, tensor in enumerate(laid):
        alternatives, labels = [tensor], list(inputs[at])
        while True:
            first = second = -1
            for one in range(len(labels)):
                for other in range(one + 1, len(labels)):
                    if labels[one] == labels[other]:
                        first, second = one, other
                        break
                if first >= 0:
                    break
            if first < 0:
                break
            front = alternatives[0]
            codomain = len(front.codomain)
            if front.legs()[first] != front.legs()[second]:
                raise ValueError(f"the label '{labels[first]}' names two different spaces")
            above_leg = first if first < codomain else second
            below_leg = second if first < codomain else first
            above = [l for l in range(front.nlegs()) if l not in (above_leg, below_leg) and l < codomain]
            below = [l for l in range(front.nlegs()) if l not in (above_leg, below_leg) and l >= codomain]
            above.append(above_leg)
            below.append(below_leg)
            traced = []
            for alt in alternatives:
                traced.extend(_partial_trace(place(alt, above, below)))
            alternatives = traced
            del labels[second]
            del labels[first]
        prepared.append(alternatives)
        prep_labels.append(labels)
    above_legs, below_legs = [], []
    for one, label in enumerate(output[0]):
        for at, labels in enumerate(prep_labels):
            if label in labels:
                leg = prepared[at][0].legs()[labels.index(label)]
                (above_legs if output[1][one] else below_legs).append(leg)
                break
    closes = not output[0]
    for a in reachable_charges(cat, above_legs):
        for b in reachable_charges(cat, below_legs):
            if cat.n_symbol(a, cat.dual(b), charge) > 0:
                closes = True
    if not closes:
        raise ValueError(f"the output legs of '{spec}' cannot close to {charge}")
    for alts in prepared:
        if not alts:
            raise ValueError(f"the traces of '{spec}' leave nothing to sum")
    dims = {}
    for at, labels in enumerate(prep_labels):
        legs = prepared[at][0].legs()
        for i, label in enumerate(labels):
            dims[label] = _leg_size(cat, legs[i])
    order = fold_order(prep_labels, dims)
    total = None
    for choice in cartesian(*[range(len(a)) for a in prepared]):
        ops = [prepared[i][c] for i, c in enumerate(choice)]
        labels = list(prep_labels[0])
        states = [ops[0]]
        for step in range(1, len(order)):
            at = order[step]
            states = _combine(states, labels, [ops[at]], prep_labels[at])
            labels = _product_labels(labels, prep_labels[at])
        above = [labels.index(l) for l, up in zip(*output) if up]
        below = [labels.index(l) for l, up in zip(*output) if not up]
        for state in states:
            result = place(state, above, below)
            if result.qtotal != charge or not result.blocks:
                continue
            if total is None:
                total = result
            else:
                for key, block in result.blocks.items():
                    total.blocks[key] += block
    if total is None:
        raise ValueError(f"no way for the charges of '{spec}' to fuse to {charge}")
    return total


# --------------------------------------------------------------------------------------------
# the configurations' inputs
# --------------------------------------------------------------------------------------------


def degeneracies(chi, qmax = 8):
    '''Multiplets per U(1) charge q = -qmax..qmax for a bond of `chi` multiplets: one each, then the
    rest apportioned proportional to exp(-q^2/8), floors first, leftover pairs (+1 to q and -q) by
    descending fractional part (ties to smaller |q|), an odd leftover to q = 0.  Symmetric in q, so a
    bond bends without reading a missing dual block.'''
    qs = list(range(-qmax, qmax + 1))
    w = {q: math.exp(-q * q / 8) for q in qs}
    total_w = sum(w.values())
    rest = chi - len(qs)
    raw = {q: rest * w[q] / total_w for q in qs}
    m = {q: 1 + int(raw[q]) for q in qs}
    left = chi - sum(m.values())
    for q in sorted(range(1, qmax + 1), key = lambda q: (-(raw[q] - int(raw[q])), q)):
        if left >= 2:
            m[q] += 1
            m[-q] += 1
            left -= 2
    m[0] += left
    return qs, [m[q] for q in qs]


def heisenberg_site(cat, first = False, last = False, coupling = 1.0, dtype = np.float64):
    '''One site of the Heisenberg MPO over the codomain (w_left, phys) and the domain (phys, w_right),
    restating tentorch/models/heisenberg.py:104-201 for a U(1) category (charge = 2 Sz).'''
    START, CLOSED = 0, 4
    state_of_charged = {(0,): {0: START, 1: 1, 2: CLOSED}, (2,): {0: 2}, (-2,): {0: 3}}
    op = {
        (START, START): lambda o, i: 1.0 if o == i else 0.0,
        (CLOSED, CLOSED): lambda o, i: 1.0 if o == i else 0.0,
        (START, 1): lambda o, i: 0.5 if o == i == 1 else (-0.5 if o == i else 0.0),
        (1, CLOSED): lambda o, i: 0.5 if o == i == 1 else (-0.5 if o == i else 0.0),
        (START, 2): lambda o, i: 1.0 if o == i + 2 else 0.0,
        (2, CLOSED): lambda o, i: 0.5 if o == i - 2 else 0.0,
        (START, 3): lambda o, i: 1.0 if o == i - 2 else 0.0,
        (3, CLOSED): lambda o, i: 0.5 if o == i + 2 else 0.0,
    }
    phys = Leg(cat, [(1,), (-1,)], [1, 1])
    bond = Leg(cat, [(0,), (2,), (-2,)], [3, 1, 1])
    edge = Leg(cat, [cat.trivial()], [1])
    w_left = edge if first else bond
    w_right = edge if last else bond
    t = Tensor(cat, [w_left, phys], [phys, w_right], cat.trivial(), dtype)
    for key in t.blocks:
        rows = _rows(cat, t.codomain, key[0])
        cols = _rows(cat, t.domain, key[1])
        for r, (tree_out, copy_out) in enumerate(rows):
            for c, (tree_in, copy_in) in enumerate(cols):
                before = START if first else state_of_charged[tree_out[0][0]][copy_out[0]]
                after = CLOSED if last else state_of_charged[tree_in[0][1]][copy_in[1]]
                write = op.get((before, after))
                if write is None:
                    continue
                weight = coupling if before not in (START, CLOSED) and after == CLOSED else 1.0
                t.blocks[key][r, c] = weight * write(tree_out[0][1][0], tree_in[0][0][0])
    return t, phys, bond


def _rows(cat, legs, root):
    '''tentorch/tensors/tree.py:236-248: every row of a root as (tree, copy of each leg).'''
    out = []
    for tree in fusion_trees(cat, legs, root):
        mults = [leg.multiplicity_of(s) for leg, s in zip(legs, tree[0])]
        for copy in cartesian(*[range(m) for m in mults]):
            out.append((tree, copy))
    return out


def matvec_inputs(chi, seed = 0, dtype = np.float64):
    '''The single two-site effective-Hamiltonian matvec: environments L, R = (bond, w | bond),
    the Heisenberg bulk site W, and theta = (bond, phys | phys, bond) at the trivial charge, all
    entries N(0, 1) float64 drawn in block-key order from one torch generator seeded `seed`
    (L, then R, then theta).  Returns (head, tail, theta) with head = einsum('EIa,IPqj->EPaqj', L, W)
    and tail = einsum('JRsk,Fkb->JRSFb', W, R) as tentorch/algorithms/dmrg.py:113-114 builds them.'''
    import torch
    cat = u1
    qs, deg = degeneracies(chi)
    bond = Leg(cat, [(2 * q,) for q in qs], deg)
    site, phys, w = heisenberg_site(cat, dtype = dtype)
    gen = torch.Generator().manual_seed(seed)
    left = Tensor(cat, [bond, w], [bond], cat.trivial(), dtype).fill_random(gen)
    right = Tensor(cat, [bond, w], [bond], cat.trivial(), dtype).fill_random(gen)
    theta = Tensor(cat, [bond, phys], [phys, bond], cat.trivial(), dtype).fill_random(gen)
    head = einsum('EIa,IPqj->EPaqj', left, site)
    tail = einsum('JRsk,Fkb->JRSFb', site, right)
    return head, tail, theta


MATVEC = 'EPaqj,JRSFb,AQsb->EPrf'
