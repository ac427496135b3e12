'''The behaviour the reference's own MPS and DMRG tests check (tests/test_mps.py,
tests/test_dmrg.py), on the GPU engine, in the reference's default dtype (complex128) and for both
of its test categories (no symmetry and U(1)): the mixed canonical form keeps the norm and the
expectation wherever the centre sits, a product state has the energy of its spins, DMRG reaches
exact diagonalisation on short chains, keeps its bond within the cap, drops weight only when
capped, and approaches the bulk energy density 1/4 - ln 2 on a long chain.'''
import math

import pytest
import torch

import tentorch_gb300 as tg
from tentorch_gb300 import networks as nw
from golden_io import load_json

pytestmark = pytest.mark.gpu
CATEGORIES = [tg.no_symmetry, tg.u1]
DEVICE = 'cuda'


def _exact(length):
    return load_json('dmrg.json')['exact'][str(length)]


def _driver(cat, length, bond, n_iter = 5):
    return nw.DMRG(nw.Model(length, cat = cat), max_bond_dim = bond, n_iter = n_iter, device = DEVICE)


@pytest.mark.parametrize('cat', CATEGORIES, ids = ['no_symmetry', 'u1'])
def test_the_norm_does_not_depend_on_the_center(cat):
    operator = nw.heisenberg(cat, 4, device = DEVICE)
    state = nw.MPS.random(cat, operator.physical, 4, seed = 1, multiplets = 2, device = DEVICE)
    state.normalize()
    for center in list(range(state.L)) + list(range(state.L - 1, -1, -1)):
        state.move_center(center)
        assert state.center == center
        assert abs(state.norm() - 1.0) < 1e-12


@pytest.mark.parametrize('cat', CATEGORIES, ids = ['no_symmetry', 'u1'])
def test_the_expectation_does_not_depend_on_the_center(cat):
    operator = nw.heisenberg(cat, 4, device = DEVICE)
    state = nw.MPS.random(cat, operator.physical, 4, seed = 2, multiplets = 2, device = DEVICE)
    state.normalize()
    values = []
    for center in range(state.L):
        state.move_center(center)
        values.append(complex(state.expectation(operator)))
    assert max(abs(value - values[0]) for value in values) < 1e-12


def test_a_product_state_has_the_energy_of_its_spins():
    '''Only the Sz Sz terms act on a product state: +1/4 per aligned neighbour pair, -1/4 per
    anti-aligned one.'''
    cat = tg.no_symmetry
    spins = [1, -1, 1, -1]
    operator = nw.heisenberg(cat, len(spins), device = DEVICE)
    bonds = [tg.Leg(cat, [(0,)], (1,)) for _ in range(len(spins) + 1)]

    def site(at):
        def fill(tree_out, copy_out, tree_in, copy_in):
            return 1.0 if 1 - 2 * copy_out[1] == spins[at] else 0.0
        return nw.entered(cat, [bonds[at], operator.physical], [bonds[at + 1]], fill, device = DEVICE)
    state = nw.MPS([site(at) for at in range(len(spins))], operator.physical)
    assert abs(state.norm() - 1.0) < 1e-12
    want = sum(0.25 if a == b else -0.25 for a, b in zip(spins, spins[1:]))
    assert abs(complex(state.expectation(operator)) - want) < 1e-12


@pytest.mark.parametrize('length', [4, 6, 8])
@pytest.mark.parametrize('cat', CATEGORIES, ids = ['no_symmetry', 'u1'])
def test_the_energy_matches_exact_diagonalisation(cat, length):
    driver = _driver(cat, length, 64)
    driver.run(num_sweeps = 6, verbose = False)
    assert abs(driver.energy().real - _exact(length)) < 1e-10


@pytest.mark.parametrize('cat', CATEGORIES, ids = ['no_symmetry', 'u1'])
def test_the_driver_writes_the_state_and_the_energy_onto_the_model(cat):
    model = nw.Model(6, cat = cat)
    result = nw.dmrg(model, max_bond_dim = 64, num_sweeps = 4, verbose = False, device = DEVICE)
    assert result is model
    assert result.state is not None
    assert abs(result.energy - _exact(6)) < 1e-10


@pytest.mark.parametrize('cat', CATEGORIES, ids = ['no_symmetry', 'u1'])
def test_a_sweep_leaves_a_normalised_state_and_its_energy_is_the_expectation(cat):
    driver = _driver(cat, 6, 64)
    driver.sweep()
    assert abs(driver.state.norm() - 1.0) < 1e-12
    assert driver.center == driver.state.center
    driver.run(num_sweeps = 5, verbose = False)
    assert abs(driver.energy() - driver.state.expectation(driver.operator)) < 1e-10


@pytest.mark.parametrize('cat', CATEGORIES, ids = ['no_symmetry', 'u1'])
def test_the_bond_cap_holds_and_truncation_is_variational(cat):
    capped = _driver(cat, 12, 4)
    capped.run(num_sweeps = 4, verbose = False)
    assert max(capped.state.bond_dims) <= 4
    small = _driver(cat, 8, 2)
    small.run(num_sweeps = 6, verbose = False)
    large = _driver(cat, 8, 64)
    large.run(num_sweeps = 6, verbose = False)
    assert small.energy().real > large.energy().real - 1e-10


@pytest.mark.parametrize('cat', CATEGORIES, ids = ['no_symmetry', 'u1'])
def test_a_capped_bond_throws_weight_away(cat):
    capped = _driver(cat, 10, 2)
    _, capped_lost = capped.sweep()
    full = _driver(cat, 10, 64)
    full.sweep()
    _, full_lost = full.sweep()
    assert capped_lost > 1e-3
    assert full_lost < 1e-12


def test_the_energy_and_a_run_need_a_sweep():
    driver = _driver(tg.u1, 4, 16)
    with pytest.raises(RuntimeError):
        driver.energy()
    with pytest.raises(ValueError):
        driver.run(num_sweeps = 0)


def test_the_energy_density_of_a_long_chain_approaches_the_known_limit():
    '''The bulk energy per site of the spin-1/2 chain is 1/4 - ln 2 (L = 64, bond 64, 5 sweeps).'''
    length = 64
    model = nw.Model(length, cat = tg.u1)
    energy = nw.dmrg(model, max_bond_dim = 64, num_sweeps = 5, verbose = False, device = DEVICE,
                     dtype = torch.float64).energy
    assert abs(energy / length - (0.25 - math.log(2))) < 5e-3
