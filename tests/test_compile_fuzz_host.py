'''Random two-site windows compiled without a GPU: the output space of every DMRG einsum (head, tail,
matvec, both environment updates) and of the two-site contraction, block keys and shapes, against
the oracle's own einsum of tensors with the same legs, for U(1) bonds of random charges and
multiplets (each charge's multiplets equal to its dual's, as truncated bonds have them).  Every draw
brings new legs and leg lists through the engine's per-leg-list caches (layouts, reachable charges),
so a lookup that handed back another list's entry would show as a wrong key set or shape.'''
import random

import numpy as np
import torch

import tentorch_gb300 as tg
from tentorch_gb300 import linalg as la
from tentorch_gb300.tensor import Space
from oracle import engine as orc

SPECS = [('EIa,IPqj->EPaqj', ('left', 'site')), ('JRsk,Fkb->JRSFb', ('site', 'right')),
         ('EIa,Feq,aPb,IqPj->FJb', ('left', 'bra', 'mps', 'site')),
         ('Gfq,aPb,IqPk,Gkb->FIa', ('bra', 'mps', 'site', 'right'))]


def _bond(rng):
    top = rng.randint(1, 5)
    charges = list(range(-top, top + 1))
    mult = {}
    for q in charges:
        if q <= 0:
            mult[q] = mult[-q] = rng.randint(1, 4)
    return [(2 * q,) for q in charges], [mult[q] for q in charges]


def _shapes_of_space(space):
    return {(tuple(k.codomain), tuple(k.domain), k.copy): tuple(s) for k, s in zip(space.keys, space.shapes)}


def _shapes_of_oracle(t):
    return {(tuple(k[0]), tuple(k[1]), k[2]): b.shape for k, b in t.blocks.items()}


def test_random_windows_compile_to_the_oracles_output_spaces():
    rng = random.Random(5)
    site_o, phys_o, w_o = orc.heisenberg_site(orc.u1)
    legs = lambda ls: [tg.Leg(tg.u1, list(l.sectors), list(l.multiplicities)) for l in ls]
    site = Space.of(tg.u1, legs(site_o.codomain), legs(site_o.domain), site_o.qtotal)
    gen = torch.Generator().manual_seed(3)
    la.clear_plans()
    for draw in range(12):
        sectors, mults = _bond(rng)
        bond_o = orc.Leg(orc.u1, sectors, mults)
        left_o = orc.Tensor(orc.u1, [bond_o, w_o], [bond_o], orc.u1.trivial(), np.float64).fill_random(gen)
        right_o = orc.Tensor(orc.u1, [bond_o, w_o], [bond_o], orc.u1.trivial(), np.float64).fill_random(gen)
        mps_o = orc.Tensor(orc.u1, [bond_o, phys_o], [bond_o], orc.u1.trivial(), np.float64).fill_random(gen)
        bra_o = mps_o.conj()
        oracle = {'left': left_o, 'right': right_o, 'mps': mps_o, 'bra': bra_o, 'site': site_o}
        product = {name: Space.of(tg.u1, legs(t.codomain), legs(t.domain), t.qtotal) for name, t in oracle.items()
                   if name != 'site'}
        product['site'] = site
        outs = {}
        for spec, names in SPECS:
            plan = la.einsum_plan(spec, [product[n] for n in names])
            want = orc.einsum(spec, *[oracle[n] for n in names])
            assert _shapes_of_space(plan.out_space) == _shapes_of_oracle(want), (draw, spec)
            outs[spec] = (plan.out_space, want)
        # the two-site contraction and the matvec over the head and tail just compiled
        two = la.contract_plan(product['mps'], product['mps'], [2], [0]).out_space
        two_o = orc.contract(mps_o, mps_o, [2], [0])
        assert _shapes_of_space(two) == _shapes_of_oracle(two_o), draw
        head, head_o = outs['EIa,IPqj->EPaqj']
        tail, tail_o = outs['JRsk,Fkb->JRSFb']
        plan = la.einsum_plan(orc.MATVEC, [head, tail, two])
        assert _shapes_of_space(plan.out_space) == _shapes_of_oracle(orc.einsum(orc.MATVEC, head_o, tail_o, two_o)), draw


def test_random_su2_recouplings_compile_to_the_oracles_output_spaces():
    '''SU(2) legs of random spins and multiplets through the recoupling einsum of the named config
    ('ABcd,DCef->ABef': the second operand's codomain read in the other order, an exchange with F
    and R symbols), an exchange of the domain's legs ('ABcd->ABdc') and bends of a leg across the
    sides ('ABcd->ABCd', 'ABcd->Abcd'; a label's case names its side): the compiled output spaces
    against the oracle's.'''
    rng = random.Random(11)
    gen = torch.Generator().manual_seed(4)
    legs = lambda ls: [tg.Leg(tg.su2, list(l.sectors), list(l.multiplicities)) for l in ls]
    la.clear_plans()
    for draw in range(8):
        spins = sorted(rng.sample(range(0, 5), rng.randint(1, 3)))
        leg_o = orc.Leg(orc.su2, [(j,) for j in spins], [rng.randint(1, 2) for _ in spins])
        a_o = orc.Tensor(orc.su2, [leg_o, leg_o], [leg_o, leg_o], orc.su2.trivial(), np.float64).fill_random(gen)
        a = Space.of(tg.su2, legs(a_o.codomain), legs(a_o.domain), a_o.qtotal)
        for spec in ('ABcd,DCef->ABef', 'ABcd->ABdc', 'ABcd->ABCd', 'ABcd->Abcd'):
            operands_o = [a_o, a_o] if ',' in spec else [a_o]
            plan = la.einsum_plan(spec, [a] * len(operands_o))
            want = orc.einsum(spec, *operands_o)
            assert _shapes_of_space(plan.out_space) == _shapes_of_oracle(want), (draw, spec, spins)
