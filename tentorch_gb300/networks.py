'''
The callers of the contraction path, with the reference's surface: the entry-by-entry tensor
builder (tentorch/tensors/tree.py), the MPS (tentorch/networks/mps.py), the MPO
(tentorch/networks/mpo.py), the Heisenberg model (tentorch/models/heisenberg.py, model.py) and the
two-site DMRG driver (tentorch/algorithms/dmrg.py).  They run their einsums, SVDs and Lanczos on the
GPU through this package.
'''
from __future__ import annotations

import itertools
import math
from dataclasses import dataclass
from typing import Callable, Literal, Optional, Sequence

import numpy as np
import torch

from tentorch_gb300.lanczos import lanczos, lanczos_einsum
from tentorch_gb300.linalg import (_split_over, conj_plan, contract, contract_plan, einsum, einsum_plan, inner,
                                   inner_device, place_plan, precision, qr, rq)
from tentorch_gb300.symmetry import (AbelianGroup, FusionCategory, FusionTree, Leg, NoSymmetry, fusion_trees,
                                     reachable_charges, u1)
from tentorch_gb300.tensor import BlockKey, Space, Tensor, block_keys, domain_legs

# ---------------------------------------------------------------------------------------------
# entry-by-entry tensors (tentorch/tensors/tree.py)
# ---------------------------------------------------------------------------------------------


def block_of(leg: Leg, sector) -> int:
    '''tentorch/tensors/tree.py:18-32'''
    for block in range(leg.nblocks()):
        if leg.sector(block) == tuple(sector):
            return block
    raise ValueError(f'the leg carries none of the sector {sector}')


def rows(cat: FusionCategory, legs: Sequence[Leg], root):
    '''Every row of a root's block in storage order: (tree, copy of each leg)
    (tentorch/tensors/tree.py:35-47).'''
    for tree in fusion_trees(cat, legs, root):
        mults = [leg.multiplicity(block_of(leg, s)) for leg, s in zip(legs, tree.sectors)]
        yield from ((tree, copy) for copy in itertools.product(*[range(m) for m in mults]))


def entered(cat: FusionCategory, codomain, domain, entry: Callable, root = None, dtype = None, device = None) -> Tensor:
    '''A tensor written entry by entry (tentorch/tensors/tree.py:50-75).'''
    charge = cat.trivial() if root is None else tuple(root)
    out = Tensor(cat, list(codomain), list(domain), charge, dtype = dtype, device = device)
    host = {}
    for key in out.keys():
        out_rows = list(rows(cat, codomain, key.codomain))
        in_rows = list(rows(cat, domain, key.domain))
        data = np.zeros((len(out_rows), len(in_rows)), dtype = np.complex128)
        for r, (tree_out, copy_out) in enumerate(out_rows):
            for c, (tree_in, copy_in) in enumerate(in_rows):
                data[r, c] = entry(tree_out, copy_out, tree_in, copy_in)
        host[key] = data
    for key, data in host.items():
        block = out.block(key.codomain, key.domain, key.copy)
        block.copy_(torch.from_numpy(data if block.is_complex() else data.real).to(block.dtype))
    return out


# ---------------------------------------------------------------------------------------------
# MPS and MPO (tentorch/networks/mps.py, mpo.py)
# ---------------------------------------------------------------------------------------------


def _identity(cat: FusionCategory, bond: Leg, middle: Optional[Leg] = None, dtype = None, device = None) -> Tensor:
    '''tentorch/networks/mps.py:12-28'''
    def entry(tree_out, copy_out, tree_in, copy_in):
        same = tree_out.sectors[0] == tree_in.sectors[0] and copy_out[0] == copy_in[0]
        return 1.0 if same and (middle is None or tree_out.sectors[1] == cat.trivial()) else 0.0
    codomain = [bond] if middle is None else [bond, middle]
    return entered(cat, codomain, [bond], entry, dtype = dtype, device = device)


class MPS:
    '''A matrix product state in mixed canonical form (tentorch/networks/mps.py:31-204).'''

    def __init__(self, tensors: Sequence[Tensor], physical: Leg, center: int = 0) -> None:
        if not tensors:
            raise ValueError('A state needs at least one site.')
        for at, tensor in enumerate(tensors):
            if tensor.nlegs() != 3:
                raise ValueError(f'site {at} needs three legs, not {tensor.nlegs()}')
        if not 0 <= center < len(tensors):
            raise IndexError(f'the centre {center} is outside the chain of {len(tensors)} sites')
        self.tensors = list(tensors)
        self.physical = physical
        self.center = center
        self.canonicalize()

    @property
    def L(self) -> int:
        return len(self.tensors)

    @property
    def cat(self) -> FusionCategory:
        return self.tensors[0].cat

    @property
    def dtype(self) -> torch.dtype:
        return self.tensors[0].dtype

    @property
    def device(self) -> torch.device:
        return self.tensors[0].device

    @property
    def bond_dims(self) -> list[int]:
        return [self.tensors[at].domain[0].multiplets() for at in range(self.L - 1)]

    @classmethod
    def random(cls, cat: FusionCategory, physical: Leg, length: int, sector = None, seed: int = 0,
               multiplets: int = 1, dtype = None, device = None, generator: Optional[torch.Generator] = None) -> 'MPS':
        '''tentorch/networks/mps.py:85-118.  With `generator` (a CPU torch.Generator) the blocks are
        float64 N(0, 1) draws in block-key order from it, the reproducible form the reference's
        float64 harness uses; without it every block is `normal_()` after `torch.manual_seed(seed)`.'''
        charge = cat.trivial() if sector is None else tuple(sector)
        left = [reachable_charges(cat, [physical] * at) for at in range(length + 1)]
        tail = [reachable_charges(cat, [physical] * (length - at)) for at in range(length + 1)]
        bonds = []
        for at in range(length + 1):
            sectors = [b for b in left[at] if any(cat.can_fuse_to(b, r, charge) for r in tail[at])]
            bonds.append(Leg(cat, sectors, [multiplets] * len(sectors)))
        bonds[0] = bonds[-1] = Leg(cat, [charge], (1,))
        if not bonds[0].nblocks() or not bonds[-1].nblocks():
            raise ValueError(f'the charge {charge} admits no state of {length} sites')
        tensors = []
        if generator is None:
            torch.manual_seed(seed)
        for at in range(length):
            t = Tensor(cat, [bonds[at], physical], [bonds[at + 1]], charge, dtype = dtype, device = device)
            for key in t.keys():
                block = t.block(key.codomain, key.domain, key.copy)
                if generator is None:
                    block.normal_()
                else:
                    block.copy_(torch.randn(block.shape, dtype = torch.float64, generator = generator).to(block.dtype))
            tensors.append(t)
        return cls(tensors, physical)

    def _left_canonicalize(self, at: int) -> None:
        if at < 0 or at >= self.L - 1:
            raise IndexError(f'index {at} has no site to its right in a chain of {self.L} sites')
        factor, rest = qr(self.tensors[at], [0, 1])
        self.tensors[at] = factor
        joined = contract(rest, self.tensors[at + 1], domain_legs(rest), [0])
        self.tensors[at + 1] = joined.place([0, 1])
        self.center = at + 1

    def _right_canonicalize(self, at: int) -> None:
        if at <= 0 or at >= self.L:
            raise IndexError(f'index {at} has no site to its left in a chain of {self.L} sites')
        factor, rest = rq(self.tensors[at], [0])
        self.tensors[at] = rest.place([0, 1])
        self.tensors[at - 1] = contract(self.tensors[at - 1], factor, domain_legs(self.tensors[at - 1]), [0])
        self.center = at - 1

    def move_center(self, at: int) -> None:
        if not 0 <= at < self.L:
            raise IndexError(f'the centre {at} is outside the chain of {self.L} sites')
        while self.center < at:
            self._left_canonicalize(self.center)
        while self.center > at:
            self._right_canonicalize(self.center)

    def canonicalize(self) -> None:
        for at in range(self.center):
            self._left_canonicalize(at)
        for at in range(self.L - 1, self.center, -1):
            self._right_canonicalize(at)

    def norm(self) -> float:
        '''tentorch/networks/mps.py:165-170 (the arena padding is zero)'''
        return float(torch.linalg.vector_norm(self.tensors[self.center].data))

    def normalize(self) -> None:
        self.tensors[self.center] /= self.norm()

    def expectation(self, operator: 'MPO') -> complex:
        '''tentorch/networks/mps.py:176-195'''
        dtype, device = self.dtype, self.device
        left = _identity(self.cat, self.tensors[0].codomain[0], operator.tensors[0].codomain[0], dtype, device)
        for at, tensor in enumerate(self.tensors):
            left = einsum('AIe,aPb,Feq,IPqj->BJf', left, tensor, tensor.conj(), operator.tensors[at])
        return inner(_identity(self.cat, self.tensors[-1].domain[0], operator.tensors[-1].domain[1], dtype, device), left)

    def __len__(self) -> int:
        return self.L

    def __repr__(self) -> str:
        return (f'MPS(L={self.L}, blocks={self.physical.nblocks()}, bond_dim={self.bond_dims}, '
                f'center={self.center})')


class MPO:
    '''A matrix product operator (tentorch/networks/mpo.py:7-86).'''

    def __init__(self, sites: Sequence[Tensor], physical: Leg, cat: FusionCategory, sector = None, dtype = None,
                 device = None) -> None:
        self.tensors = list(sites)
        if not self.tensors:
            raise ValueError('an operator needs at least one site')
        for at, site in enumerate(self.tensors):
            if site.nlegs() != 4:
                raise ValueError(f'site {at} has {site.nlegs()} legs, not the four of an operator')
        self.L = len(self.tensors)
        self.cat = cat
        self.physical = physical
        self.sector = cat.trivial() if sector is None else sector
        self.dtype = self.tensors[0].dtype if dtype is None else dtype
        self.device = self.tensors[0].device if device is None else device
        self.bond_dim = [site.codomain[0].multiplets() for site in self.tensors]
        self.bond_dim.append(self.tensors[-1].domain[1].multiplets())

    @property
    def physical_dim(self) -> int:
        return sum(self.physical.multiplicity(b) for b in range(self.physical.nblocks()))

    def __len__(self) -> int:
        return self.L

    def __iter__(self):
        return iter(self.tensors)

    def __getitem__(self, at: int) -> Tensor:
        return self.tensors[at]

    def __repr__(self) -> str:
        return f'MPO(L={self.L}, physical_dim={self.physical_dim}, bond_dim={self.bond_dim[1:self.L]})'


# ---------------------------------------------------------------------------------------------
# the Heisenberg chain (tentorch/models/heisenberg.py, model.py)
# ---------------------------------------------------------------------------------------------

START, CLOSED = 0, 4
_STATE_OF_CHARGED = {(0,): {0: START, 1: 1, 2: CLOSED}, (2,): {0: 2}, (-2,): {0: 3}}
_OPERATOR = {
    (START, START): lambda out, into: 1.0 if out == into else 0.0,
    (CLOSED, CLOSED): lambda out, into: 1.0 if out == into else 0.0,
    (START, 1): lambda out, into: 0.5 if out == into == 1 else (-0.5 if out == into else 0.0),
    (1, CLOSED): lambda out, into: 0.5 if out == into == 1 else (-0.5 if out == into else 0.0),
    (START, 2): lambda out, into: 1.0 if out == into + 2 else 0.0,
    (2, CLOSED): lambda out, into: 0.5 if out == into - 2 else 0.0,
    (START, 3): lambda out, into: 1.0 if out == into - 2 else 0.0,
    (3, CLOSED): lambda out, into: 0.5 if out == into + 2 else 0.0,
}


def _table(cat):
    '''tentorch/models/heisenberg.py:40-55'''
    if isinstance(cat, NoSymmetry):
        return (Leg(cat, [(0,)], (2,)), Leg(cat, [(0,)], (5,)), lambda sector, copy: copy,
                lambda sector, copy: 1 - 2 * copy)
    return (Leg(cat, [(1,), (-1,)], (1, 1)), Leg(cat, [(0,), (2,), (-2,)], (3, 1, 1)),
            lambda sector, copy: _STATE_OF_CHARGED[tuple(sector)][copy], lambda sector, copy: sector[0])


def heisenberg(cat: FusionCategory, length: int, coupling: float = 1.0, dtype = None, device = None) -> MPO:
    '''The nearest-neighbour Heisenberg chain as an MPO automaton (tentorch/models/heisenberg.py:58-115).'''
    if not isinstance(cat, AbelianGroup):
        raise ValueError(f'the rows of {cat.name} would need the recoupling to dress them')
    phys, bond, state_of, spin_of = _table(cat)
    edge = Leg(cat, [cat.trivial()], (1,))

    def site(w_left, w_right, first, last):
        def entry(tree_out, copy_out, tree_in, copy_in):
            before = START if first else state_of(tree_out.sectors[0], copy_out[0])
            after = CLOSED if last else state_of(tree_in.sectors[1], copy_in[1])
            write = _OPERATOR.get((before, after))
            if write is None:
                return 0.0
            weight = coupling if before not in (START, CLOSED) and after == CLOSED else 1.0
            return weight * write(spin_of(tree_out.sectors[1], copy_out[1]), spin_of(tree_in.sectors[0], copy_in[0]))
        return entered(cat, [w_left, phys], [phys, w_right], entry, dtype = dtype, device = device)

    sites = [site(edge if at == 0 else bond, edge if at == length - 1 else bond, at == 0, at == length - 1)
             for at in range(length)]
    return MPO(sites, phys, cat)


@dataclass
class Model:
    '''A chain and its couplings (tentorch/models/model.py:5-34).'''
    length: int
    coupling: complex = 1.0
    cat: FusionCategory = u1
    physical: Optional[Leg] = None
    sector: Optional[tuple] = None
    state: Optional[object] = None
    energy: Optional[float] = None

    def __post_init__(self) -> None:
        if self.length < 1:
            raise ValueError(f'a chain needs at least one site, not {self.length}')
        if self.sector is None:
            self.sector = self.cat.trivial()


# ---------------------------------------------------------------------------------------------
# two-site DMRG (tentorch/algorithms/dmrg.py)
# ---------------------------------------------------------------------------------------------


class DMRG:
    '''The two-site DMRG of a chain (tentorch/algorithms/dmrg.py:13-217) on the GPU engine.

    `dtype` selects the scalar type of the state and the operator (the reference builds complex128;
    float64 is exact for U(1) and no symmetry).  `generator` draws the starting state reproducibly
    (see `MPS.random`).  `precision` chooses the block products of the Lanczos matvec (0: FP64;
    k: k bf16 slices, see `tentorch_gb300.precision`); with `all_products` also those of the
    environments, head and tail and the two-site contraction.  The SVDs, the Lanczos vector algebra
    and the tridiagonal eigensolve stay FP64 either way.  With `refine_energy` a window's energy is
    the FP64 Rayleigh quotient <v|H v> / <v|v> of the Ritz vector v the split-precision Lanczos found
    (one FP64 matvec per window): its error is second order in the vector's, so a coarse split
    (three slices, ~2^-21 per matvec) still reports energies near FP64.'''

    def __init__(self, model: Model, max_bond_dim: int = 50, svd_tol: float = 1e-14, n_iter: int = 5, seed: int = 0,
                 dtype = None, device = None, generator: Optional[torch.Generator] = None, precision: int = 0,
                 all_products: bool = False, refine_energy: bool = False) -> None:
        self.model = model
        self.max_bond_dim = max_bond_dim
        self.svd_tol = svd_tol
        self.n_iter = n_iter
        self.precision = precision
        self.all_products = all_products
        self.refine_energy = refine_energy
        self.operator = heisenberg(model.cat, model.length, model.coupling, dtype = dtype, device = device)
        physical = model.physical if model.physical is not None else self.operator.physical
        self.state = MPS.random(model.cat, physical, model.length, model.sector, seed = seed, dtype = dtype,
                                device = device, generator = generator)
        self.left: dict[int, Tensor] = {}
        self.right: dict[int, Tensor] = {}
        self.matvecs = 0

    @property
    def L(self) -> int:
        return self.model.length

    @property
    def center(self) -> int:
        return self.state.center

    @center.setter
    def center(self, at: int) -> None:
        self.state.center = at

    def _advance_left(self, left: Tensor, at: int) -> Tensor:
        tensor = self.state.tensors[at]
        return einsum('EIa,Feq,aPb,IqPj->FJb', left, tensor.conj(), tensor, self.operator.tensors[at])

    def _advance_right(self, right: Tensor, at: int) -> Tensor:
        tensor = self.state.tensors[at]
        return einsum('Gfq,aPb,IqPk,Gkb->FIa', tensor.conj(), tensor, self.operator.tensors[at], right)

    def cache_environments(self) -> None:
        dtype, device = self.state.dtype, self.state.device
        self.left = {0: _identity(self.model.cat, self.state.tensors[0].codomain[0],
                                  self.operator.tensors[0].codomain[0], dtype, device)}
        self.right = {self.L: _identity(self.model.cat, self.state.tensors[-1].domain[0],
                                        self.operator.tensors[-1].domain[1], dtype, device)}
        for at in range(self.L - 1, 1, -1):
            self.right[at] = self._advance_right(self.right[at + 1], at)

    def update(self, direction: Literal['left', 'right']) -> tuple[float, float]:
        '''tentorch/algorithms/dmrg.py:96-129'''
        energy, lost = self._update(direction)
        return float(energy), float(lost)

    def _update(self, direction: Literal['left', 'right']) -> tuple[torch.Tensor, torch.Tensor]:
        '''One window, with its energy and discarded weight left on the device and the centre
        normalised there: the window's only host wait is the split's read of its singular values.'''
        at = self.center
        first, second = self.state.tensors[at], self.state.tensors[at + 1]
        bond = second.codomain[0]  # the bond the split replaces
        two = contract(first, second, domain_legs(first), [0])
        site, following = self.operator.tensors[at], self.operator.tensors[at + 1]
        head = einsum('EIa,IPqj->EPaqj', self.left[at], site)
        tail = einsum('JRsk,Fkb->JRSFb', following, self.right[at + 2])

        # the reference's action, einsum('EPaqj,JRSFb,AQsb->EPrf', head, tail, vector), with the
        # Krylov loop on the device
        with precision(self.precision):
            energy, vector = lanczos_einsum('EPaqj,JRSFb,AQsb->EPrf', [head, tail, two], 2, two, self.n_iter,
                                            wait = False)
        self.matvecs += self.n_iter
        if self.refine_energy and self.precision != 0:
            # the Ritz vector's Rayleigh quotient in FP64, on the device
            with precision(0):
                image = einsum('EPaqj,JRSFb,AQsb->EPrf', head, tail, vector)
            energy = (inner_device(vector, image) / inner_device(vector, vector)).real
            self.matvecs += 1
        factor = 2 if direction == 'right' else 1
        # svd(vector, max_bond, tol, factor), compiling what follows while the split runs
        left, values, right = _split_over(vector, None, self.max_bond_dim, self.svd_tol, factor,
                                          lambda: self._compile_ahead(at, direction, vector._space, bond))
        self.state.tensors[at], self.state.tensors[at + 1] = left, right.place([0, 1])
        self.center = at + 1 if direction == 'right' else at
        centre = self.state.tensors[self.center]._data
        centre.div_(torch.linalg.vector_norm(centre))
        return energy, 1.0 - torch.sum(values * values).real

    def _compile_ahead(self, at: int, direction: str, theta: Space, bond: Leg) -> None:
        '''Compile, while the split of window `at` runs on the device, the plans of what follows it
        (the right factor's leg move, the environment update, the next window's contraction, head,
        tail and matvec) for the shapes they get when the split keeps the bond it replaces: near
        convergence a DMRG bond keeps its multiplets from sweep to sweep, and the calls then find
        their plans compiled.  A bond that changed compiles its own plans when the calls run; a
        predicted shape the engine refuses is left to them.'''
        cat, ops = theta.cat, self.operator.tensors
        domain = lambda space: list(range(len(space.codomain), len(space.codomain) + len(space.domain)))
        try:
            first = Space.of(cat, theta.codomain, [bond], theta.qtotal)
            second = Space.of(cat, [bond], theta.domain, cat.trivial())
            moved = place_plan(second, [0, 1], [2])
            placed = moved.out_space if moved.n_ops else second
            if direction == 'right':
                if at >= self.L - 2 or at + 3 not in self.right:
                    return
                env = einsum_plan('EIa,Feq,aPb,IqPj->FJb', [self.left[at]._space, conj_plan(first).out_space, first,
                                                            ops[at]._space]).out_space
                two = contract_plan(placed, self.state.tensors[at + 2]._space, domain(placed), [0]).out_space
                head = einsum_plan('EIa,IPqj->EPaqj', [env, ops[at + 1]._space]).out_space
                tail = einsum_plan('JRsk,Fkb->JRSFb', [ops[at + 2]._space, self.right[at + 3]._space]).out_space
            else:
                if at <= 0 or at - 1 not in self.left or at + 2 not in self.right:
                    return
                env = einsum_plan('Gfq,aPb,IqPk,Gkb->FIa', [conj_plan(placed).out_space, placed, ops[at + 1]._space,
                                                            self.right[at + 2]._space]).out_space
                before = self.state.tensors[at - 1]._space
                two = contract_plan(before, first, domain(before), [0]).out_space
                head = einsum_plan('EIa,IPqj->EPaqj', [self.left[at - 1]._space, ops[at - 1]._space]).out_space
                tail = einsum_plan('JRsk,Fkb->JRSFb', [ops[at]._space, env]).out_space
            einsum_plan('EPaqj,JRSFb,AQsb->EPrf', [head, tail, two])
        except ValueError:
            pass

    def sweep(self) -> tuple[float, float]:
        '''tentorch/algorithms/dmrg.py:131-161'''
        if self.all_products and self.precision > 0:
            with precision(self.precision):
                return self._sweep()
        return self._sweep()

    def _sweep(self) -> tuple[float, float]:
        self.state.move_center(0)
        self.cache_environments()
        energy, lost = 0.0, []
        for at in range(self.L - 1):
            energy, weight = self._update('right')
            lost.append(weight)
            if at < self.L - 2:
                self.left[at + 1] = self._advance_left(self.left[at], at)
        self.state._right_canonicalize(self.L - 1)
        self.right[self.L - 1] = self._advance_right(self.right[self.L], self.L - 1)
        for at in range(self.L - 3, -1, -1):
            self.center = at
            energy, weight = self._update('left')
            lost.append(weight)
            if at > 0:
                self.right[at + 1] = self._advance_right(self.right[at + 2], at + 1)
        # the energy of the last window and the largest weight any window discarded, read once per sweep
        discarded = float(torch.stack(lost).max()) if lost else 0.0
        return float(energy), max(discarded, 0.0)

    def energy(self) -> complex:
        '''tentorch/algorithms/dmrg.py:163-179'''
        if not self.left:
            raise RuntimeError('the energy needs the environments of a sweep, and none has run')
        at = min(self.center, self.L - 2)
        two = contract(self.state.tensors[at], self.state.tensors[at + 1], domain_legs(self.state.tensors[at]), [0])
        image = einsum('AIe,IPqj,JRsk,Dkf,EQSf->APrd', self.left[at], self.operator.tensors[at],
                       self.operator.tensors[at + 1], self.right[at + 2], two)
        return complex(inner(two, image) / inner(two, two))

    def run(self, num_sweeps: int = 5, energy_tol: float = 1e-10, patience: int = 2, verbose: bool = True) -> Model:
        '''tentorch/algorithms/dmrg.py:181-212'''
        if num_sweeps < 1:
            raise ValueError(f'a run needs at least one sweep, not {num_sweeps}')
        energy, best, stale = float('inf'), float('inf'), 0
        for sweep in range(1, num_sweeps + 1):
            energy, discarded = self.sweep()
            if verbose:
                print(f'sweep {sweep}: energy = {energy:.12f}, truncated = {discarded:.2e}, '
                      f'bond = {self.state.bond_dims}')
            if abs(energy - best) <= energy_tol:
                stale += 1
                if stale >= patience:
                    break
            else:
                stale, best = 0, energy
        self.model.state = self.state
        self.model.energy = energy
        return self.model

    def __repr__(self) -> str:
        return f'DMRG(L={self.L}, max_bond_dim={self.max_bond_dim}, bond_dim={self.state.bond_dims})'


def dmrg(model: Model, max_bond_dim: int = 50, svd_tol: float = 1e-14, num_sweeps: int = 5, energy_tol: float = 1e-10,
         patience: int = 2, n_iter: int = 5, seed: int = 0, verbose: bool = True, **kw) -> Model:
    '''tentorch/algorithms/dmrg.py:220-240'''
    return DMRG(model, max_bond_dim, svd_tol, n_iter, seed, **kw).run(num_sweeps, energy_tol, patience, verbose)
