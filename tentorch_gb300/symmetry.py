'''
The categories, legs and fusion trees, with the Python surface of the reference's
`tentorch.symmetry` (tentorch/_ext/bindings.cpp:170-231, :464-470): the module singletons `u1`,
`su2`, `fibonacci`, `no_symmetry`, `fermion_parity`, `z_n(modulus)`, the `Leg` class and the tree
functions.  Everything is answered by the engine library; a sector is a tuple `(label,)`.
'''
from __future__ import annotations

import ctypes
from typing import NamedTuple

import torch

from tentorch_gb300._lib import check, f64, i32, i64, ints32, lib

Sector = tuple[int, ...]


def _label(sector) -> int:
    sector = tuple(sector)
    if len(sector) != 1:
        raise ValueError(f'a sector of this engine holds one label, got {sector}')
    return int(sector[0])


class Outcome(NamedTuple):
    '''One term of a fusion (tentorch/symmetry/cat/cat.h:150-160).'''
    sector: Sector
    multiplicity: int


class FusionCategory:
    '''A fusion category (tentorch/symmetry/cat/cat.h:190-429), answered by the engine.'''
    _kind = -1

    def __init__(self, param: int = 0):
        out = i32()
        check(lib.tt_category(self._kind, param, ctypes.byref(out)))
        self._id = out.value
        self._param = param

    @property
    def name(self) -> str:
        return self._name

    def outcomes(self, a, b) -> list[Outcome]:
        sectors, mult, n = (i64 * 64)(), (i32 * 64)(), i32()
        check(lib.tt_outcomes(self._id, _label(a), _label(b), 64, sectors, mult, ctypes.byref(n)))
        return [Outcome((sectors[i],), mult[i]) for i in range(n.value)]

    def n_symbol(self, a, b, c) -> int:
        for o in self.outcomes(a, b):
            if o.sector == tuple(c):
                return o.multiplicity
        return 0

    def can_fuse_to(self, a, b, c) -> bool:
        return self.n_symbol(a, b, c) > 0

    def _matrix(self, fn, *labels) -> torch.Tensor:
        cap = 4096
        values, rows, cols = (f64 * (2 * cap))(), i32(), i32()
        check(fn(self._id, *labels, cap, values, ctypes.byref(rows), ctypes.byref(cols)))
        n = rows.value * cols.value
        flat = torch.tensor(values[:2 * n], dtype = torch.float64).view(n, 2) if n else torch.zeros(0, 2, dtype = torch.float64)
        return torch.complex(flat[:, 0], flat[:, 1]).reshape(rows.value, cols.value)

    def F_symbol(self, a, b, c, d) -> torch.Tensor:
        '''F^d_{abc} on the host (tentorch/symmetry/cat/cat.h:250-288).'''
        return self._matrix(lib.tt_F_symbol, _label(a), _label(b), _label(c), _label(d))

    def R_symbol(self, b, c) -> torch.Tensor:
        '''R_{bc} on the host (tentorch/symmetry/cat/cat.h:290-301).'''
        return self._matrix(lib.tt_R_symbol, _label(b), _label(c))

    def q_dim(self, a) -> float:
        out = f64()
        check(lib.tt_q_dim(self._id, _label(a), ctypes.byref(out)))
        return out.value

    def dual(self, a) -> Sector:
        out = i64()
        check(lib.tt_dual(self._id, _label(a), ctypes.byref(out)))
        return (out.value,)

    def frobenius_schur_sign(self, a) -> float:
        return 1.0

    def trivial(self) -> Sector:
        return (0,)

    @property
    def dtype(self) -> torch.dtype:
        '''Every category of the reference defaults its tensors to complex128
        (tentorch/symmetry/cat/abelian/abelian.cpp:47, su2/su2.cpp:37, fibonacci/fibonacci.cpp:82).'''
        return torch.complex128

    @property
    def device(self) -> torch.device:
        return default_device()

    def clear_cache(self) -> None:
        '''The symbol tables are small and held for the life of the process.'''

    def __repr__(self) -> str:
        return f'<{type(self).__name__} {self.name}>'


class Group(FusionCategory):
    pass


class AbelianGroup(Group):
    pass


class NoSymmetry(AbelianGroup):
    _kind, _name = 0, 'NoSymmetry'


class U1Symmetry(AbelianGroup):
    _kind, _name = 1, 'U(1)'


class SU2Symmetry(Group):
    _kind, _name = 2, 'SU(2)'

    def frobenius_schur_sign(self, a) -> float:
        return 1.0 if _label(a) % 2 == 0 else -1.0


class FibonacciCategory(FusionCategory):
    _kind, _name = 3, 'FibonacciCategory'


class ZNSymmetry(AbelianGroup):
    _kind = 4

    def __init__(self, modulus: int):
        super().__init__(modulus)
        self._name = f'Z_{modulus}'

    @property
    def modulus(self) -> int:
        return self._param


class FermionParity(FusionCategory):
    _kind, _name = 5, 'FermionParity'

    def frobenius_schur_sign(self, a) -> float:
        return -1.0 if _label(a) == 1 else 1.0


no_symmetry = NoSymmetry()
u1 = U1Symmetry()
su2 = SU2Symmetry()
fibonacci = FibonacciCategory()
fermion_parity = FermionParity()
_z_n = {}


def z_n(modulus: int) -> ZNSymmetry:
    '''The Z_N singleton of one modulus.'''
    if modulus not in _z_n:
        _z_n[modulus] = ZNSymmetry(modulus)
    return _z_n[modulus]


def default_device() -> torch.device:
    '''The CUDA device when one is visible (the engine computes there), else the host, where a
    tensor is only a container.'''
    return torch.device('cuda') if torch.cuda.is_available() else torch.device('cpu')


_legs = {}


class Leg:
    '''A graded space: blocks sorted by sector, one multiplicity each
    (tentorch/symmetry/tree/tree.h:33-118).  Interned by the engine, so equal legs share a handle.'''
    __slots__ = ('cat', '_id', 'sectors', 'multiplicities')

    def __init__(self, cat: FusionCategory, sectors, multiplicities):
        sectors = [tuple(s) for s in sectors]
        multiplicities = [int(m) for m in multiplicities]
        labels, n = (i64 * max(len(sectors), 1))(*[_label(s) for s in sectors]), len(sectors)
        mult = (i64 * max(len(multiplicities), 1))(*multiplicities)
        if len(multiplicities) != n:
            raise ValueError(f'A leg needs one multiplicity per sector, got {len(multiplicities)} for {n} sectors.')
        out = i32()
        check(lib.tt_leg(cat._id, n, labels, mult, ctypes.byref(out)))
        self.cat = cat
        self._id = out.value
        cached = _legs.get(self._id)
        if cached is None:
            got_s, got_m, count = (i64 * max(n, 1))(), (i64 * max(n, 1))(), i32()
            check(lib.tt_leg_blocks(self._id, n, got_s, got_m, ctypes.byref(count)))
            cached = (tuple((got_s[i],) for i in range(count.value)), tuple(got_m[i] for i in range(count.value)))
            _legs[self._id] = cached
        self.sectors, self.multiplicities = cached

    @classmethod
    def _of(cls, cat, leg_id):
        leg = cls.__new__(cls)
        leg.cat, leg._id = cat, leg_id
        leg.sectors, leg.multiplicities = _legs[leg_id]
        return leg

    @staticmethod
    def trivial(multiplets: int, cat: FusionCategory) -> 'Leg':
        if multiplets <= 0:
            raise ValueError(f'A trivial leg needs at least one component, got {multiplets}.')
        return Leg(cat, [cat.trivial()], [multiplets])

    @staticmethod
    def from_blocks(cat: FusionCategory, entries) -> tuple['Leg', list[int]]:
        entries = [(tuple(s), int(m)) for s, m in entries]
        leg = Leg(cat, [s for s, _ in entries], [m for _, m in entries])
        return leg, [leg.sectors.index(s) for s, _ in entries]

    def nblocks(self) -> int:
        return len(self.sectors)

    def sector(self, block: int) -> Sector:
        return self.sectors[block]

    def multiplicity(self, block: int) -> int:
        return self.multiplicities[block]

    def multiplets(self) -> int:
        return sum(self.multiplicities)

    def fuse(self, other: 'Leg') -> 'Leg':
        '''tentorch/symmetry/tree/tree.cpp:172-200'''
        if self.cat is not other.cat:
            raise ValueError(f'Cannot fuse a leg of {self.cat.name} with one of {other.cat.name}.')
        fused = {}
        for s1, m1 in zip(self.sectors, self.multiplicities):
            for s2, m2 in zip(other.sectors, other.multiplicities):
                for o in self.cat.outcomes(s1, s2):
                    fused[o.sector] = fused.get(o.sector, 0) + m1 * m2 * o.multiplicity
        keys = sorted(fused)
        return Leg(self.cat, keys, [fused[k] for k in keys])

    def conj(self) -> 'Leg':
        return Leg(self.cat, [self.cat.dual(s) for s in self.sectors], self.multiplicities)

    def capped(self, max_multiplets: int) -> 'Leg':
        if max_multiplets <= 0:
            raise ValueError(f'A cap must keep at least one multiplet, got {max_multiplets}.')
        sectors, mult, kept = [], [], 0
        for s, m in zip(self.sectors, self.multiplicities):
            if kept >= max_multiplets:
                break
            take = min(m, max_multiplets - kept)
            sectors.append(s)
            mult.append(take)
            kept += take
        return Leg(self.cat, sectors, mult)

    def __eq__(self, other) -> bool:
        return isinstance(other, Leg) and self._id == other._id

    def __ne__(self, other) -> bool:
        return not self == other

    def __hash__(self) -> int:
        return hash(('Leg', self._id))

    def __repr__(self) -> str:
        return f'Leg({self.cat.name}: ' + ', '.join(
            f'{_render(s)}:{m}' for s, m in zip(self.sectors, self.multiplicities)) + ')'


def _render(sector) -> str:
    return '(' + ', '.join(str(x) for x in sector) + (',)' if len(sector) == 1 else ')')


class FusionTree(NamedTuple):
    '''A left-nested fusion tree (tentorch/symmetry/tree/tree.h:120-155).'''
    sectors: tuple
    inner: tuple
    copies: tuple
    coupled: Sector

    def size(self) -> int:
        return len(self.sectors)

    def chain(self) -> list:
        if len(self.sectors) <= 1:
            return list(self.sectors)
        return [self.sectors[0], *self.inner, self.coupled]


def reachable_charges(cat: FusionCategory, legs) -> list[Sector]:
    '''tentorch/symmetry/tree/tree.cpp:375-398'''
    ids, n = ints32(leg._id for leg in legs)
    out, count = (i64 * 4096)(), i32()
    check(lib.tt_reachable_charges(cat._id, n, ids, 4096, out, ctypes.byref(count)))
    return [(out[i],) for i in range(count.value)]


def fusion_trees(cat: FusionCategory, legs, coupled) -> list[FusionTree]:
    '''tentorch/symmetry/tree/tree.cpp:400-471'''
    legs = list(legs)
    ids, n = ints32(leg._id for leg in legs)
    total, stride = i64(), i32()
    check(lib.tt_fusion_trees(cat._id, n, ids, _label(coupled), 0, (i64 * 1)(), ctypes.byref(total), ctypes.byref(stride)))
    buf = (i64 * max(1, total.value * stride.value))()
    check(lib.tt_fusion_trees(cat._id, n, ids, _label(coupled), total.value * stride.value, buf, ctypes.byref(total),
                              ctypes.byref(stride)))
    trees, per = [], stride.value
    ni, nc = max(n - 2, 0), max(n - 1, 0)
    for t in range(total.value):
        row = buf[t * per:(t + 1) * per]
        trees.append(FusionTree(tuple((x,) for x in row[:n]), tuple((x,) for x in row[n:n + ni]),
                                tuple(row[n + ni:n + ni + nc]), (row[-1],)))
    return trees


def validate(category: FusionCategory, tree: FusionTree) -> None:
    '''tentorch/symmetry/tree/tree.cpp:318-373'''
    legs = tree.size()
    if legs <= 1:
        if tree.inner or tree.copies:
            raise ValueError(f'A tree of {legs} legs has no inner coupling or vertex.')
        if legs == 1 and tuple(tree.coupled) != tuple(tree.sectors[0]):
            raise ValueError(f'A tree of one leg couples to {tree.sectors[0]}, not to {tree.coupled}.')
        return
    if len(tree.inner) != legs - 2 or len(tree.copies) != legs - 1:
        raise ValueError(f'A tree of {legs} legs has {legs - 2} inner couplings and {legs - 1} vertices.')
    for vertex in range(legs - 1):
        left = tree.sectors[0] if vertex == 0 else tree.inner[vertex - 1]
        right = tree.sectors[vertex + 1]
        out = tree.coupled if vertex + 2 == legs else tree.inner[vertex]
        copies = category.n_symbol(left, right, out)
        if copies == 0:
            raise ValueError(f'The vertex {left} x {right} -> {out} is not allowed by {category.name}.')
        if not 0 <= tree.copies[vertex] < copies:
            raise ValueError(f'Vertex {vertex} has {copies} copies, got copy {tree.copies[vertex]}.')
