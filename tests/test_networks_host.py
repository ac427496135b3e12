'''Host-side checks of the callers around the contraction path: the Heisenberg MPO written entry by
entry against the reference's own site tensor (a golden fixture), the row order of a block, the
chain ends, and the argument errors of the reference's MPS, MPO, Model and DMRG.  The tensors live
in host containers; nothing here contracts.'''
import numpy as np
import pytest
import torch

import tentorch_gb300 as tg
from tentorch_gb300 import networks as nw
from golden_io import case_blocks, load_json


def _case_input(name):
    for case in load_json('cases.json'):
        for entry in case['inputs']:
            if entry['name'] == name:
                return entry
    raise KeyError(name)


def test_heisenberg_site_is_the_references():
    '''tentorch/models/heisenberg.py:58-115 at site 1 of four, read back as float64.'''
    mpo = nw.heisenberg(tg.u1, 4, dtype = torch.float64, device = 'cpu')
    site = mpo.tensors[1]
    entry = _case_input('mv/W')
    want = case_blocks(entry, entry['name'])
    got = {(k.codomain, k.domain, k.copy): b.numpy() for k, b in site.to_tuple()[3].items()}
    assert set(got) == set(want)
    for key, block in want.items():
        assert np.array_equal(got[key], block), key


def test_heisenberg_chain_ends_and_bonds():
    mpo = nw.heisenberg(tg.u1, 5, dtype = torch.float64, device = 'cpu')
    assert len(mpo) == 5 and mpo.physical_dim == 2
    assert mpo.bond_dim == [1, 5, 5, 5, 5, 1]
    assert repr(mpo) == 'MPO(L=5, physical_dim=2, bond_dim=[5, 5, 5, 5])'
    assert mpo[0].codomain[0].multiplets() == 1 and mpo[4].domain[1].multiplets() == 1
    plain = nw.heisenberg(tg.no_symmetry, 3, dtype = torch.float64, device = 'cpu')
    assert plain.bond_dim == [1, 5, 5, 1]


def test_heisenberg_needs_an_abelian_category():
    with pytest.raises(ValueError, match = 'recoupling'):
        nw.heisenberg(tg.su2, 4, device = 'cpu')


def test_rows_run_trees_then_copies_last_leg_fastest():
    '''tentorch/tensors/tree.py:35-47'''
    a = tg.Leg(tg.u1, [(-1,), (1,)], [2, 3])
    rows = list(nw.rows(tg.u1, [a, a], (0,)))
    assert [tree.sectors for tree, _ in rows] == [((-1,), (1,))] * 6 + [((1,), (-1,))] * 6
    assert [copy for _, copy in rows[:6]] == [(0, 0), (0, 1), (0, 2), (1, 0), (1, 1), (1, 2)]
    with pytest.raises(ValueError):
        nw.block_of(a, (3,))


def test_identity_closes_the_chain():
    bond = tg.Leg(tg.u1, [(0,)], [1])
    w = tg.Leg(tg.u1, [(0,), (2,), (-2,)], [3, 1, 1])
    t = nw._identity(tg.u1, bond, w, dtype = torch.float64, device = 'cpu')
    blocks = {(k.codomain, k.domain): b.numpy() for k, b in t.to_tuple()[3].items()}
    assert list(blocks) == [((0,), (0,))]
    # rows: (bond copy, w copy) over the trees of (0,) then (2,)/(−2,) cannot couple to 0 with bond 0
    assert blocks[((0,), (0,))][:, 0].tolist() == [1.0, 1.0, 1.0]


def test_argument_errors():
    with pytest.raises(ValueError):
        nw.Model(0)
    assert nw.Model(4).sector == tg.u1.trivial()
    with pytest.raises(ValueError):
        nw.MPS([], tg.Leg(tg.u1, [(1,)], [1]))
    with pytest.raises(ValueError):
        nw.MPO([], tg.Leg(tg.u1, [(1,)], [1]), tg.u1)


def test_bench_bond_layout_is_the_matvec_workload_layout():
    '''The benchmark builds its bond with the layout the oracle's matvec inputs use (17 charges,
    multiplicities from exp(-q^2/8) summing to chi, symmetric in q).'''
    import importlib.util
    import pathlib
    from oracle import engine as orc
    path = pathlib.Path(__file__).resolve().parents[1] / 'bench.py'
    spec = importlib.util.spec_from_file_location('bench_under_test', path)
    bench = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bench)
    for chi in (32, 64, 100, 256, 512, 1024):
        sectors, mult = bench.bond_multiplicities(chi)
        qs, deg = orc.degeneracies(chi)
        assert sectors == [(2 * q,) for q in qs] and mult == deg and sum(mult) == chi
        assert mult == mult[::-1]
