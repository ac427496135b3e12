'''The product's host engine (no GPU needed): the C ABI loads and exports what include/ declares,
and the categories, trees, layouts, block keys and per-step regrouping plans match the reference's
own outputs (tests/golden/, produced from the reference) — the plans bit for bit.'''
import ctypes
import os
import re

import numpy as np
import pytest

from golden_io import load_json

import tentorch_gb300 as tg
from tentorch_gb300 import _lib
from tentorch_gb300.tensor import Space

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CATS = {'u1': tg.u1, 'su2': tg.su2, 'fibonacci': tg.fibonacci, 'no_symmetry': tg.no_symmetry}


def declared():
    text = open(os.path.join(ROOT, 'include', 'tentorch_gb300.h')).read()
    return sorted(set(re.findall(r'\b(tt_[a-z_A-Z0-9]+)\s*\(', text)))


def test_library_exports_every_declared_symbol():
    names = declared()
    assert len(names) >= 25
    for name in names:
        assert hasattr(_lib.lib, name), name
    assert _lib.lib.tt_version() >= 1
    assert set(names) == set(_lib.EXPORTED)


def legs(cat, specs):
    return [tg.Leg(cat, [tuple(s) for s, _ in spec], [m for _, m in spec]) for spec in specs]


@pytest.mark.parametrize('name', ['su2', 'fibonacci'])
def test_symbols_match_the_reference(name):
    cat = CATS[name]
    table = load_json('symbols.json')[name]
    for a, b, c, d, re_, im_ in table['F']:
        got = cat.F_symbol(tuple(a), tuple(b), tuple(c), tuple(d)).numpy()
        want = np.array(re_) + 1j * np.array(im_)
        assert got.shape == want.shape
        assert np.abs(got - want).max(initial = 0) < 1e-13, (a, b, c, d)
    for b, c, re_, im_ in table['R']:
        got = cat.R_symbol(tuple(b), tuple(c)).numpy()
        want = np.array(re_) + 1j * np.array(im_)
        assert got.shape == want.shape and np.abs(got - want).max(initial = 0) < 1e-13


def test_trees_layouts_and_keys_match_the_reference():
    data = load_json('structure.json')
    for case in data['layouts']:
        cat = CATS[case['cat']]
        ls = legs(cat, case['legs'])
        trees = tg.fusion_trees(cat, ls, tuple(case['root']))
        want = [(tuple(map(tuple, t[0])), tuple(map(tuple, t[1])), tuple(t[2]), tuple(t[3])) for t in case['trees']]
        assert [tuple(t) for t in trees] == want
        offsets = [0]
        for t in trees:
            rows = 1
            for leg, s in zip(ls, t.sectors):
                rows *= leg.multiplicities[leg.sectors.index(s)]
            offsets.append(offsets[-1] + rows)
        assert offsets == case['offsets']
    for case in data['keys']:
        cat = CATS[case['cat']]
        space = Space.of(cat, legs(cat, case['codomain']), legs(cat, case['domain']), tuple(case['qtotal']))
        want = sorted((tuple(k[0]), tuple(k[1]), k[2]) for k in case['keys'])
        assert [tuple(k) for k in space.keys] == want


def step_plan(space_id, kind, arm, key):
    ns, npc = ctypes.c_int64(), ctypes.c_int64()
    args = (space_id, kind, arm, key[0][0], key[1][0], key[2])
    _lib.check(_lib.lib.tt_step_plan(*args, 0, (ctypes.c_int64 * 1)(), 0, (ctypes.c_double * 1)(),
                                     ctypes.byref(ns), ctypes.byref(npc)))
    shifts = (ctypes.c_int64 * max(9 * ns.value, 1))()
    pieces = (ctypes.c_double * max(8 * npc.value, 1))()
    _lib.check(_lib.lib.tt_step_plan(*args, ns.value, shifts, npc.value, pieces, ctypes.byref(ns), ctypes.byref(npc)))
    out, at = [], 0
    for i in range(ns.value):
        s = shifts[9 * i:9 * i + 9]
        count = s[8]
        ps = [pieces[8 * j:8 * j + 7] for j in range(at, at + count)]
        at += count
        out.append(((s[0], s[1], s[2]), (s[3], s[4], s[5]), s[6], s[7], ps))
    return out


def test_step_plans_match_the_reference_bit_for_bit():
    '''Every shift of every block of every step, matched by the block it writes: the same pieces
    (first, last, steps and run exactly, the coefficient to 1e-12), in whatever order each side
    lists them.'''
    kinds = {'x': 0, 'down': 1, 'up': 2}
    checked = 0
    for record in load_json('plans.json'):
        cat = CATS[record['cat']]
        for step in record['steps']:
            space = Space.of(cat, legs(cat, step['codomain']), legs(cat, step['domain']), tuple(record['qtotal']))
            for block in step['blocks']:
                key = (tuple(block['key'][0]), tuple(block['key'][1]), block['key'][2])
                got = {tuple(shift[1]): shift for shift in step_plan(space.id, kinds[step['kind']], step['arm'], key)}
                want = {tuple(s[1][0] + s[1][1] + [s[1][2]]): s for s in block['shifts']}
                assert set(got) == set(want)
                for to, theirs in want.items():
                    mine = got[to]
                    assert list(mine[0]) == theirs[0][0] + theirs[0][1] + [theirs[0][2]]
                    assert (mine[2], mine[3]) == (theirs[2], theirs[3])
                    ours = sorted((tuple(int(x) for x in p[:5]), p[5] + 1j * p[6]) for p in mine[4])
                    ref = sorted((tuple(p[:5]), p[5] + 1j * p[6]) for p in theirs[4])
                    assert [k for k, _ in ours] == [k for k, _ in ref]
                    assert max((abs(a - b) for (_, a), (_, b) in zip(ours, ref)), default = 0.0) < 1e-12
                    checked += len(mine[4])
    assert checked > 1000


def test_chain_matches_the_oracle_step_sequence():
    from oracle import engine as orc
    for record in load_json('plans.json'):
        cat = CATS[record['cat']]
        space = Space.of(cat, legs(cat, record['codomain']), legs(cat, record['domain']), tuple(record['qtotal']))
        above, n_above = _lib.ints32(record['above'])
        below, n_below = _lib.ints32(record['below'])
        steps, n = (ctypes.c_int32 * 192)(), ctypes.c_int32()
        _lib.check(_lib.lib.tt_chain(space.id, n_above, above, n_below, below, 64, steps, ctypes.byref(n)))
        kinds = {0: 'x', 1: 'down', 2: 'up'}
        got = [(kinds[steps[3 * i]], steps[3 * i + 1]) for i in range(n.value)]
        assert got == [(s['kind'], s['arm']) for s in record['steps']]


def test_errors_map_to_the_reference_exceptions():
    leg = tg.Leg(tg.u1, [(1,), (-1,)], [1, 1])
    with pytest.raises(ValueError, match = 'twice'):
        tg.Leg(tg.u1, [(1,), (1,)], [1, 1])
    with pytest.raises(ValueError, match = 'positive'):
        tg.Leg(tg.u1, [(1,)], [0])
    with pytest.raises(ValueError, match = 'no components'):
        tg.Leg(tg.su2, [(-1,)], [1])
    t = tg.Tensor(tg.u1, [leg, leg], [leg], (1,), device = 'cpu')
    with pytest.raises(ValueError, match = 'named twice'):
        _lib.check(_lib.lib.tt_plan_place(t._space.id, 2, _lib.ints32([0, 0])[0], 1, _lib.ints32([2])[0],
                                          ctypes.byref(ctypes.c_void_p())))
    with pytest.raises(IndexError):
        t.block((5,), (5,))
    with pytest.raises(ValueError, match = 'does not say what it leaves'):
        tg.linalg.plan_of('ab', t)
    with pytest.raises(ValueError, match = 'names more than two legs'):
        tg.linalg.plan_of('abc,aab->c', t, t)
    with pytest.raises(ValueError, match = "does not take the keyword 'charge'"):
        tg.einsum('ABc->ABc', t, charge = (1,))
    with pytest.raises(RuntimeError, match = 'CUDA device'):
        tg.einsum('ABc->ABc', t, outcharge = (1,))


def test_dot_entry_points_refuse_an_unknown_dtype_before_any_device_work():
    # both dot products check their arguments on the host, so the refusal needs no GPU
    for call in (lambda: _lib.lib.tt_dots(7, 1, None, None, 16, None, None, None),
                 lambda: _lib.lib.tt_dots_noalloc(7, 1, None, None, 16, None, None)):
        with pytest.raises(ValueError, match = 'unknown dtype'):
            _lib.check(call())


def test_einsum_plan_compiles_on_the_host():
    '''The matvec plan compiles without a GPU and reports its work.'''
    from oracle import engine as orc
    qs, deg = orc.degeneracies(64)
    bond = tg.Leg(tg.u1, [(2 * q,) for q in qs], deg)
    phys = tg.Leg(tg.u1, [(1,), (-1,)], [1, 1])
    w = tg.Leg(tg.u1, [(0,), (2,), (-2,)], [3, 1, 1])
    head = tg.Tensor(tg.u1, [bond, phys], [bond, phys, w], (0,), device = 'cpu')
    tail = tg.Tensor(tg.u1, [w, phys, phys, bond], [bond], (0,), device = 'cpu')
    theta = tg.Tensor(tg.u1, [bond, phys], [phys, bond], (0,), device = 'cpu')
    plan = tg.linalg.plan_of('EPaqj,JRSFb,AQsb->EPrf', head, tail, theta)
    assert plan.flops > 0 and plan.n_ops >= 3
    assert plan.prepared_size(0) > 0 and plan.prepared_size(1) > 0 and plan.prepared_size(2) == 0
    assert plan.out_space.codomain == [bond, phys] and plan.out_space.domain == [phys, bond]


def test_every_golden_case_compiles_on_the_host():
    '''place / contract / einsum plans of every golden case compile and pass the descriptor bounds
    validation the engine runs on every program.'''
    from convert import PRODUCT_CATS, case_category
    import torch
    for case in load_json('cases.json'):
        cat = PRODUCT_CATS[case_category(case['inputs'][0]['name'])]
        ts = [tg.Tensor(cat, legs(cat, e['codomain']), legs(cat, e['domain']), tuple(e['qtotal']),
                        dtype = torch.float64, device = 'cpu') for e in case['inputs']]
        if case['op'] == 'place':
            a, na = _lib.ints32(case['above'])
            b, nb = _lib.ints32(case['below'])
            _lib.check(_lib.lib.tt_plan_place(ts[0]._space.id, na, a, nb, b, ctypes.byref(ctypes.c_void_p())))
        elif case['op'] == 'contract':
            l, n = _lib.ints32(case['left_legs'])
            r, _ = _lib.ints32(case['right_legs'])
            _lib.check(_lib.lib.tt_plan_contract(ts[0]._space.id, ts[1]._space.id, n, l, r, 1, case['charge'][0],
                                                 ctypes.byref(ctypes.c_void_p())))
        else:
            oc = case.get('outcharge')
            plan = tg.linalg.plan_of(case['spec'], *ts, outcharge = tuple(oc) if oc else None)
            assert plan.out_space.keys == [tg.BlockKey(*k) for k in
                                           sorted((tuple(k[0]), tuple(k[1]), k[2]) for k in case['output']['keys'])]


def test_bending_a_leg_with_unpaired_dual_multiplets_is_an_error():
    '''A bent leg's sector reads as its dual on the other side, so a sector and its dual must carry
    the same multiplets (the reference's assumption, tentorch/linalg/graded/svd.cpp:97-100; it
    writes past its blocks when the assumption fails).  The engine refuses the plan.'''
    import torch
    cat = tg.u1
    bond = tg.Leg(cat, [(0,)], [3])
    unpaired = tg.Leg(cat, [(-1,), (1,)], [2, 3])
    w = tg.Leg(cat, [(0,), (2,), (-2,)], [3, 1, 1])
    phys = tg.Leg(cat, [(1,), (-1,)], [1, 1])
    T = lambda cod, dom: tg.Tensor(cat, cod, dom, (0,), dtype = torch.float64, device = 'cpu')
    left, mps, site = T([bond, w], [bond]), T([bond, phys], [unpaired]), T([w, phys], [phys, w])
    with pytest.raises(ValueError, match = 'same multiplets'):
        tg.linalg.plan_of('EIa,Feq,aPb,IqPj->FJb', left, mps.conj(), mps, site)
    paired = tg.Leg(cat, [(-1,), (1,)], [3, 3])
    mps = T([bond, phys], [paired])
    tg.linalg.plan_of('EIa,Feq,aPb,IqPj->FJb', left, mps.conj(), mps, site)


def _composed_chain_index(space, above, below):
    '''The gather index of a place composed from the per-step plans of its chain (tt_chain and
    tt_step_plan, which match the reference's plans bit for bit): after[i] = before[index[i]].'''
    a, na = _lib.ints32(above)
    b, nb = _lib.ints32(below)
    steps, n = (ctypes.c_int32 * 3 * 256)(), ctypes.c_int32()
    _lib.check(_lib.lib.tt_chain(space.id, na, a, nb, b, 256, ctypes.cast(steps, ctypes.POINTER(ctypes.c_int32)),
                                 ctypes.byref(n)))
    flat = ctypes.cast(steps, ctypes.POINTER(ctypes.c_int32))
    current = np.arange(space.size, dtype = np.int64)
    before = space
    for i in range(n.value):
        kind, arm, after_id = flat[3 * i], flat[3 * i + 1], flat[3 * i + 2]
        after = Space._load(space.cat, after_id)
        back = np.full(after.size, -1, dtype = np.int64)
        for key, offset in zip(before.keys, before.offsets):
            for _, to, _, _, pieces in step_plan(before.id, kind, arm, (key[0], key[1], key[2])):
                ot = after.offsets[after.index[tg.BlockKey(to[0:1], to[1:2], to[2])]]
                for first, last, from_step, to_step, run, re_, im_ in pieces:
                    assert (re_, im_) == (1.0, 0.0)
                    for k in range(int(run)):
                        slot = ot + int(last) + k * int(to_step)
                        assert back[slot] < 0
                        back[slot] = offset + int(first) + k * int(from_step)
        current = np.where(back >= 0, current[np.maximum(back, 0)], -1)
        before = after
    return current


def _compiled_gather(space, above, below):
    from tentorch_gb300 import linalg as la
    a, na = _lib.ints32(above)
    b, nb = _lib.ints32(below)
    plan = la._plan(('place', space.id, tuple(above), tuple(below)),
                    lambda out: _lib.lib.tt_plan_place(space.id, na, a, nb, b, out), space.cat)
    text = ctypes.create_string_buffer(1 << 16)
    length = ctypes.c_int64()
    _lib.check(_lib.lib.tt_plan_describe(plan.handle, len(text), text, ctypes.byref(length)))
    gathers = [int(m.group(1)) for m in re.finditer(r"op (\d+) (?:gather|tiles)", text.value.decode())]
    if not gathers:
        return 'zero' if re.search(r'op \d+ zero', text.value.decode()) else None
    assert len(gathers) == 1
    count = ctypes.c_int64()
    _lib.check(_lib.lib.tt_plan_gather(plan.handle, gathers[0], 0, None, ctypes.byref(count)))
    index = (ctypes.c_int32 * max(count.value, 1))()
    _lib.check(_lib.lib.tt_plan_gather(plan.handle, gathers[0], count.value, index, ctypes.byref(count)))
    return np.array(index[:count.value], dtype = np.int64)


def test_compiled_leg_moves_are_the_composed_step_plans():
    '''For categories whose symbols are all 1 a place compiles to one gather, built in one pass over
    the entries; it equals the composition of the chain's per-step plans, including legs that do
    not hold the dual of a sector (their entries are dropped by the bends) and qtotal != 0.'''
    rng = np.random.default_rng(5)
    checked = 0
    for cat, pool in ((tg.u1, [-3, -2, -1, 0, 1, 2, 3]), (tg.z_n(3), [0, 1, 2]), (tg.no_symmetry, [0])):
        for trial in range(12):
            nlegs = int(rng.integers(2, 5))
            legs = []
            for _ in range(nlegs):
                sectors = sorted(rng.choice(pool, size = int(rng.integers(1, len(pool) + 1)), replace = False).tolist())
                mult = {}
                for s in sectors:
                    d = (-s) % 3 if cat is not tg.u1 and cat is not tg.no_symmetry else -s
                    mult[s] = mult.get(d, int(rng.integers(1, 4)))
                legs.append(tg.Leg(cat, [(s,) for s in sectors], [mult[s] for s in sectors]))
            height = int(rng.integers(0, nlegs + 1))
            charges = sorted({s[0] for l in legs for s in l.sectors})
            qtotal = (int(rng.choice(charges)) if cat is tg.u1 else 0,)
            space = Space.of(cat, legs[:height], legs[height:], qtotal)
            if space.size == 0:
                continue
            order = rng.permutation(nlegs).tolist()
            cut = int(rng.integers(0, nlegs + 1))
            above, below = order[:cut], order[cut:]
            want = _composed_chain_index(space, above, below)
            got = _compiled_gather(space, above, below)
            if got is None:
                assert np.array_equal(want, np.arange(space.size))
                continue
            if isinstance(got, str):
                assert (want < 0).all()
                continue
            assert np.array_equal(got, want), (cat.name, legs, height, above, below)
            checked += 1
    assert checked >= 20


def test_plan_cache_clears_wholesale_at_its_budget_and_held_plans_recompile(monkeypatch):
    '''Past the budget the whole plan cache goes (tentorch/tensors/cache.cpp:203-217); a Plan held
    across the clear compiles its program again on its next use and describes the same program.'''
    import torch
    import tentorch_gb300 as tg
    from tentorch_gb300 import linalg as la
    monkeypatch.setattr(la, '_PLAN_BUDGET', 3)
    la.clear_plans()
    cat = tg.u1
    plans = []
    for m in range(1, 6):
        leg = tg.Leg(cat, [(0,), (2,)], [m, m + 1])
        t = tg.Tensor(cat, [leg], [leg], (0,), dtype = torch.float64, device = 'cpu')
        plans.append(la.plan_of('ab,bc->ac', t, t))
        assert len(la._plans) <= 3
    first = plans[0]
    text = first.describe()
    assert first.generation == la._generation
    assert first.describe() == text
    la.clear_plans()


def _random_network(rng, count, sizes):
    '''A random einsum over `count` operands: every label joins two different operands or stays
    open (one to three open labels), legs of no symmetry whose multiplets are drawn from `sizes`.'''
    while True:
        slots = [list(range(int(rng.integers(2, 4)))) for _ in range(count)]
        ends = [(o, s) for o, legs_of in enumerate(slots) for s in legs_of]
        rng.shuffle(ends)
        labels = [[None] * len(legs_of) for legs_of in slots]
        letters = iter('abcdefghijklmnopqrstuvwxyz')
        open_left = int(rng.integers(1, 4))
        pending = list(ends)
        while pending:
            o, s = pending.pop()
            partner = next((i for i, (o2, _) in enumerate(pending) if o2 != o), None)
            letter = next(letters, None)
            if letter is None:
                break
            labels[o][s] = letter
            if partner is not None and (open_left == 0 or rng.random() < 0.8):
                o2, s2 = pending.pop(partner)
                labels[o2][s2] = letter
            else:
                open_left -= 1
        if any(l is None for ls in labels for l in ls):
            continue
        opened = [l for ls in labels for l in ls if sum(l in other for other in labels) == 1]
        if opened:
            break
    dims = {l: int(rng.choice(sizes)) for ls in labels for l in ls}
    leg_of = {l: tg.Leg(tg.no_symmetry, [(0,)], [dims[l]]) for l in dims}
    tensors = [tg.Tensor(tg.no_symmetry, [leg_of[l] for l in ls], [], (0,), device = 'cpu') for ls in labels]
    spec = ','.join(''.join(ls) for ls in labels) + '->' + ''.join(opened)
    return spec, labels, {l: float(d) for l, d in dims.items()}, tensors


def test_einsum_fold_order_is_the_reference_rule():
    '''The order an einsum folds its operands in (tentorch/linalg/graded/einsum.cpp:216-301), on
    random networks of 2 to 14 operands whose leg sizes tie often, against the oracle's restatement:
    the exact search up to 12 operands (ties broken by the labels a step sums, then the operand
    written later) and the greedy rule beyond.'''
    from oracle import engine as orc
    rng = np.random.default_rng(11)
    checked = 0
    for trial in range(60):
        count = int(rng.integers(2, 8)) if trial < 50 else int(rng.integers(13, 15))
        spec, labels, dims, tensors = _random_network(rng, count, [2, 3] if trial % 2 else [2, 3, 5, 7])
        text = tg.linalg.plan_of(spec, *tensors).describe()
        line = next(l for l in text.splitlines() if l.startswith('fold order'))
        got = [int(x) for x in line.split()[2:]]
        assert got == orc.fold_order(labels, dims), spec
        checked += 1
    assert checked == 60
