'''The split's host hook and the plan getters on spaces, without a GPU.  `_split_over` runs the
caller's `while_waiting` once, after the split's device work is queued and before its read (here
the per-block path on host tensors), and gives the factors `svd` gives; the getters over spaces
(`einsum_plan`, `contract_plan`, `place_plan`, `conj_plan`) are the cache entries the tensor calls
read, so a plan compiled ahead from predicted spaces is the one the call finds.'''
import torch

import tentorch_gb300 as tg
from tentorch_gb300 import linalg as la
from tentorch_gb300.tensor import Tensor


def _tensor(cat, codomain, domain, seed):
    t = Tensor(cat, codomain, domain, (0,), dtype = torch.float64, device = 'cpu')
    gen = torch.Generator().manual_seed(seed)
    t.data.copy_(torch.randn(t.data.shape, dtype = torch.float64, generator = gen))
    return t


def test_the_split_runs_its_hook_once_before_reading():
    cat = tg.u1
    leg = tg.Leg(cat, [(-1,), (0,), (1,)], [2, 3, 2])
    t = _tensor(cat, [leg, leg], [leg], 3)
    calls = []
    first, values, second = la._split_over(t, None, 5, 1e-14, 0, lambda: calls.append(1))
    assert calls == [1]
    want = la.svd(t, 5, 1e-14, 0)
    assert first._space is want[0]._space and second._space is want[2]._space
    assert torch.equal(values, want[1])
    assert torch.allclose(first.data, want[0].data, atol = 1e-13) and torch.allclose(second.data, want[2].data, atol = 1e-13)


def test_plans_over_spaces_are_the_entries_the_calls_read():
    cat = tg.u1
    bond = tg.Leg(cat, [(-1,), (0,), (1,)], [2, 3, 2])
    phys = tg.Leg(cat, [(-1,), (1,)], [1, 1])
    a = _tensor(cat, [bond, phys], [bond], 1)
    b = _tensor(cat, [bond, phys], [bond], 2)
    la.clear_plans()
    by_tensors = la.plan_of('aPb,bQc->aPQc', a, b)
    assert la.einsum_plan('aPb,bQc->aPQc', [a._space, b._space]) is by_tensors
    contracted = la.contract_plan(a._space, b._space, [2], [0])
    assert la.contract_plan(a._space, b._space, (2,), (0,)) is contracted
    moved = la.place_plan(a._space, [0], [1, 2])
    assert la._plans[('place', a._space.id, (0,), (1, 2))] is moved
    bra = la.conj_plan(a._space)
    assert la._plans[('conj', a._space.id)] is bra
    assert la.cached_plans() == 4


def _stand_in(space):
    return Tensor._wrap(space, None)


def test_compile_ahead_fills_the_next_windows_plans():
    '''A DMRG window compiles, during its split, the plans its successor's calls read when the
    split keeps the bond: with the bond kept the state's spaces stay as they are, and the next
    window's environment update, contraction, head, tail and matvec (keys built here from the
    state's own spaces, as the sweep's calls build them) are all in the cache already.'''
    from types import SimpleNamespace
    from tentorch_gb300 import networks as nw
    cat, length = tg.u1, 8
    operator = nw.heisenberg(cat, length, dtype = torch.float64, device = 'cpu')
    phys = operator.physical
    # the MPS's spaces (bond legs of the reachable charges, three multiplets each), not canonicalised
    bonds = [tg.Leg(cat, [(0,)], [1])]
    for at in range(1, length):
        bonds.append(tg.Leg(cat, [(q,) for q in range(-min(at, length - at), min(at, length - at) + 1, 2)],
                            [3] * (min(at, length - at) + 1)))
    bonds.append(tg.Leg(cat, [(0,)], [1]))
    state = [_stand_in(tg.tensor.Space.of(cat, [bonds[at], phys], [bonds[at + 1]], (0,))) for at in range(length)]
    driver = SimpleNamespace(L = length, operator = operator, state = SimpleNamespace(tensors = state))
    T = [t._space for t in state]
    ops = [o._space for o in operator.tensors]
    domain = lambda s: list(range(len(s.codomain), len(s.codomain) + len(s.domain)))
    bra = lambda s: la.conj_plan(s).out_space
    advance_left = lambda env, at: la.einsum_plan('EIa,Feq,aPb,IqPj->FJb', [env, bra(T[at]), T[at], ops[at]]).out_space
    advance_right = lambda env, at: la.einsum_plan('Gfq,aPb,IqPk,Gkb->FIa', [bra(T[at]), T[at], ops[at], env]).out_space
    left = {0: nw._identity(cat, bonds[0], operator.tensors[0].codomain[0], torch.float64, 'cpu')._space}
    right = {length: nw._identity(cat, bonds[-1], operator.tensors[-1].domain[1], torch.float64, 'cpu')._space}
    for at in range(1, length - 1):
        left[at] = advance_left(left[at - 1], at - 1)
    for at in range(length - 1, 1, -1):
        right[at] = advance_right(right[at + 1], at)
    driver.left = {k: _stand_in(v) for k, v in left.items()}
    driver.right = {k: _stand_in(v) for k, v in right.items()}

    def window_plans(at):
        two = la.contract_plan(T[at], T[at + 1], domain(T[at]), [0]).out_space
        head = la.einsum_plan('EIa,IPqj->EPaqj', [left[at], ops[at]]).out_space
        tail = la.einsum_plan('JRsk,Fkb->JRSFb', [ops[at + 1], right[at + 2]]).out_space
        la.einsum_plan('EPaqj,JRSFb,AQsb->EPrf', [head, tail, two])
        return two

    for at, direction in ((2, 'right'), (4, 'left')):
        la.clear_plans()
        theta = window_plans(at)
        bond = T[at + 1].codomain[0]
        nw.DMRG._compile_ahead(driver, at, direction, theta, bond)
        ahead = la.cached_plans()
        # with the bond kept, the split leaves the state's spaces as they were
        first = tg.tensor.Space.of(cat, theta.codomain, [bond], theta.qtotal)
        second = tg.tensor.Space.of(cat, [bond], theta.domain, cat.trivial())
        assert first is T[at]
        assert la.place_plan(second, [0, 1], [2]).out_space is T[at + 1]
        if direction == 'right':
            assert advance_left(left[at], at) is left[at + 1]
            window_plans(at + 1)
        else:
            assert advance_right(right[at + 2], at + 1) is right[at + 1]
            window_plans(at - 1)
        assert la.cached_plans() == ahead, direction


def test_compile_ahead_stops_at_the_turns():
    '''At the last window of each half-sweep there is no next window to compile for: the right
    half-sweep's last window and the left half-sweep's window at the chain's start compile nothing
    beyond the right factor's leg move.'''
    from types import SimpleNamespace
    from tentorch_gb300 import networks as nw
    cat, length = tg.u1, 4
    operator = nw.heisenberg(cat, length, dtype = torch.float64, device = 'cpu')
    phys = operator.physical
    bonds = [tg.Leg(cat, [(0,)], [1]), tg.Leg(cat, [(-1,), (1,)], [1, 1]), tg.Leg(cat, [(-2,), (0,), (2,)], [1, 2, 1]),
             tg.Leg(cat, [(-1,), (1,)], [1, 1]), tg.Leg(cat, [(0,)], [1])]
    state = [_stand_in(tg.tensor.Space.of(cat, [bonds[at], phys], [bonds[at + 1]], (0,))) for at in range(length)]
    driver = SimpleNamespace(L = length, operator = operator, state = SimpleNamespace(tensors = state), left = {}, right = {})
    T = [t._space for t in state]
    for at, direction in ((length - 2, 'right'), (0, 'left')):
        la.clear_plans()
        theta = la.contract_plan(T[at], T[at + 1], [2], [0]).out_space
        la.clear_plans()
        nw.DMRG._compile_ahead(driver, at, direction, theta, T[at + 1].codomain[0])
        assert la.cached_plans() == 1, direction  # the place of the right factor
