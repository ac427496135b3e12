'''The callers of the contraction path on the GPU against the reference: the Lanczos solver and the
two-site DMRG of the Heisenberg chain, in the reference's float64 harness (float64 MPS blocks drawn
N(0, 1) in block-key order from `torch.Generator().manual_seed(seed)`, float64 MPO and identities).
Every sweep energy of the reference (L = 4, 6, 8 with bond 64; L = 16 with bond 32) is met within
1e-10, the bond dimensions exactly, and the final energies within 1e-10 of exact diagonalisation
where the bond is not truncating; the split-precision matvec and every block product of a sweep
in 8 bf16 slices give the same energies within 1e-10.'''
import numpy as np
import pytest
import torch

import tentorch_gb300 as tg
from tentorch_gb300 import networks as nw
from tentorch_gb300.lanczos import lanczos
from golden_io import load_json

pytestmark = pytest.mark.gpu
ENERGY_TOL = 1e-10


def _driver(length, bond, seed = 0, precision = 0, n_iter = 5, all_products = False):
    return nw.DMRG(nw.Model(length, cat = tg.u1), max_bond_dim = bond, n_iter = n_iter, seed = seed,
                   dtype = torch.float64, device = 'cuda', generator = torch.Generator().manual_seed(seed),
                   precision = precision, all_products = all_products)


@pytest.mark.parametrize('length', [4, 6, 8])
def test_small_chains_match_the_reference_and_exact_diagonalisation(length):
    golden = load_json('dmrg.json')
    want = golden['small'][str(length)]
    driver = _driver(length, 64)
    energies = [driver.sweep()[0] for _ in range(4)]
    assert np.max(np.abs(np.array(energies) - np.array(want['sweeps']))) < ENERGY_TOL, energies
    final = driver.energy()
    assert abs(final.real - want['energy']) < ENERGY_TOL
    assert abs(final.imag) < 1e-12
    assert abs(final.real - golden['exact'][str(length)]) < ENERGY_TOL


def _config1(precision, all_products = False):
    golden = load_json('dmrg.json')['config1']
    driver = _driver(golden['length'], golden['max_bond_dim'], golden['seed'], precision, golden['n_iter'], all_products)
    out = []
    for want in golden['sweeps']:
        energy, lost = driver.sweep()
        out.append((energy, lost, driver.state.bond_dims, want))
    return out, golden


def test_sixteen_sites_bond_32_matches_the_reference_sweep_by_sweep():
    sweeps, golden = _config1(0)
    for energy, lost, bonds, want in sweeps:
        assert abs(energy - want['energy']) < ENERGY_TOL, (energy, want['energy'])
        assert bonds == want['bond']
        assert abs(lost - want['discarded']) < 1e-12
    assert sweeps[-1][0] - golden['exact'] < 1e-8


@pytest.mark.parametrize('slices, all_products', [(8, False), (8, True)])
def test_split_precision_sweeps_keep_the_fp64_energies(slices, all_products):
    '''The Lanczos matvec in split precision, or every block product of the sweep (environments,
    head and tail too): the reference's FP64 sweep energies within 1e-10, the bonds exactly.'''
    sweeps, _ = _config1(slices, all_products)
    for energy, lost, bonds, want in sweeps:
        assert abs(energy - want['energy']) < ENERGY_TOL, (energy, want['energy'])
        assert bonds == want['bond']


def test_lanczos_finds_the_lowest_eigenvalue_of_a_dense_operator():
    '''tentorch/linalg/lanczos.py:8-64 on a Hermitian action with a known spectrum: with as many
    steps as the dimension the Krylov space is the whole space.'''
    cat = tg.u1
    leg = tg.Leg(cat, [(0,)], [6])
    start = tg.Tensor(cat, [leg], [], (0,), dtype = torch.complex128, device = 'cuda')
    gen = torch.Generator().manual_seed(3)
    start.data.copy_(torch.randn(start.data.shape, dtype = torch.complex128, generator = gen))
    a = torch.randn(6, 6, dtype = torch.complex128, generator = gen)
    h = (a + a.conj().T).cuda()

    def action(v):
        return tg.Tensor._wrap(v._space, h @ v.data)
    energy, vector = lanczos(action, start, 6)
    exact = torch.linalg.eigvalsh(h)[0].item()
    assert abs(energy - exact) < 1e-10
    residual = h @ vector.data - energy * vector.data
    assert torch.linalg.vector_norm(residual).item() < 1e-8
    assert abs(tg.norm(vector) - 1.0) < 1e-12


def test_lanczos_stops_when_the_krylov_space_closes():
    '''A start inside a two-dimensional invariant subspace: the third beta is zero, the reference
    stops there, and the eigenpair is that subspace's.'''
    cat = tg.u1
    leg = tg.Leg(cat, [(0,)], [4])
    start = tg.Tensor(cat, [leg], [], (0,), dtype = torch.float64, device = 'cuda')
    start.data.copy_(torch.tensor([1.0, 1.0, 0.0, 0.0], dtype = torch.float64))
    h = torch.diag(torch.tensor([-2.0, 1.0, 5.0, 7.0], dtype = torch.float64)).cuda()

    def action(v):
        return tg.Tensor._wrap(v._space, h @ v.data)
    energy, vector = lanczos(action, start, 4)
    assert abs(energy + 2.0) < 1e-12
    assert torch.allclose(vector.data.abs().cpu(), torch.tensor([1.0, 0.0, 0.0, 0.0], dtype = torch.float64),
                          atol = 1e-12)


def test_lanczos_argument_errors():
    cat = tg.u1
    leg = tg.Leg(cat, [(0,)], [2])
    start = tg.Tensor(cat, [leg], [], (0,), dtype = torch.float64, device = 'cuda')
    with pytest.raises(ValueError, match = 'at least one step'):
        lanczos(lambda v: v, start, 0)
    with pytest.raises(ValueError, match = 'non-zero norm'):
        lanczos(lambda v: v, start, 3)


def test_mps_expectation_of_the_heisenberg_chain_is_the_dmrg_energy():
    driver = _driver(6, 64)
    for _ in range(3):
        driver.sweep()
    value = driver.state.expectation(driver.operator)
    assert abs(value.real - load_json('dmrg.json')['exact']['6']) < ENERGY_TOL


@pytest.mark.parametrize('dtype', [torch.float64, torch.complex128])
def test_device_lanczos_matches_the_python_loop(dtype):
    '''tt_lanczos (the Krylov loop on the device) against the loop driven from Python on the same
    window (site 3 of an L = 8 chain after one sweep): energies within 1e-10 and Ritz vectors equal
    up to a phase; the split-precision block products give the same energy.'''
    from tentorch_gb300.lanczos import lanczos_einsum
    driver = _driver(8, 64)
    driver.sweep()
    at = 3
    driver.state.move_center(at)
    driver.cache_environments()
    for site in range(at):
        driver.left[site + 1] = driver._advance_left(driver.left[site], site)
    first, second = driver.state.tensors[at], driver.state.tensors[at + 1]
    two = tg.contract(first, second, tg.domain_legs(first), [0])
    head = tg.einsum('EIa,IPqj->EPaqj', driver.left[at], driver.operator.tensors[at])
    tail = tg.einsum('JRsk,Fkb->JRSFb', driver.operator.tensors[at + 1], driver.right[at + 2])
    if dtype == torch.complex128:
        head, tail, two = head.to(dtype = dtype), tail.to(dtype = dtype), two.to(dtype = dtype)
    spec = 'EPaqj,JRSFb,AQsb->EPrf'
    e_py, v_py = lanczos(lambda v: tg.einsum(spec, head, tail, v), two, 5)
    e_dev, v_dev = lanczos_einsum(spec, [head, tail, two], 2, two, 5)
    assert abs(e_py - e_dev) < 1e-10
    overlap = abs(tg.inner(v_py, v_dev))
    assert abs(overlap - 1.0) < 1e-8
    if dtype == torch.float64:
        with tg.precision(8):
            e_split, _ = lanczos_einsum(spec, [head, tail, two], 2, two, 5)
        assert abs(e_split - e_dev) < 1e-10


def test_sixty_four_sites_bond_256_meet_the_reference_sweeps():
    '''The headline chain (U(1) Heisenberg, L = 64, bond 256, n_iter = 10, seed 0) against the
    reference's own float64 run of the same seed (tests/golden/dmrg_chi256.json): from the fourth
    sweep on, when every bond is at 256, the grouped FP64 sweeps meet the reference's energies
    within 1e-10, and one sweep from the same fourth-sweep state in each other form does too: the
    six-slice split matvec and the per-block form (one cuBLAS product per block pair, one cuSOLVER
    SVD per block).  The first sweeps start from a random state whose truncations (the +-q pairing
    of the bond) pick among nearly equal values, so they follow their own path until the bond fills
    (their energies are not compared); the bond dimensions also differ at a few bonds, where
    singular values sit at the 1e-14 cut and round to either side in two SVD implementations.'''
    from tentorch_gb300.linalg import PER_BLOCK
    golden = load_json('dmrg_chi256.json')
    driver = _driver(64, 256, golden['seed'], 0, golden['n_iter'])
    energies = []
    for _ in range(4):
        energies.append(driver.sweep()[0])
    start = ([t.clone() for t in driver.state.tensors], driver.state.center)
    for _ in range(2):
        energies.append(driver.sweep()[0])
    want = [s['energy'] for s in golden['sweeps']]
    for at in (3, 4, 5):
        assert abs(energies[at] - want[at]) < ENERGY_TOL, (at + 1, energies[at], want[at])
    assert max(driver.state.bond_dims) == 256
    assert abs(driver.energy().real - golden['energy']) < ENERGY_TOL
    for form in (6, PER_BLOCK):
        driver.state.tensors = [t.clone() for t in start[0]]
        driver.state.center = start[1]
        driver.precision = form
        with tg.precision(PER_BLOCK if form == PER_BLOCK else 0):
            energy, _ = driver.sweep()
        assert abs(energy - want[4]) < ENERGY_TOL, (form, energy, want[4])


def test_three_slice_sweeps_report_fp64_rayleigh_quotients():
    '''The three-slice form (bf16 x 3 matvecs in Lanczos) with the window energy refined by the
    FP64 Rayleigh quotient of its Ritz vector: on the L = 16, bond 32 chain every sweep energy is
    within 1e-5 of the reference's (the state carries the three-slice Ritz vectors' error, so the
    energy error is that error squared, not FP64 round-off), and each refined energy is the FP64
    Rayleigh quotient of the window's vector (it does not sit below the FP64 sweep's energy by more
    than round-off: the quotient is variational).'''
    golden = load_json('dmrg.json')['config1']
    driver = _driver(golden['length'], golden['max_bond_dim'], golden['seed'], 3, golden['n_iter'])
    driver.refine_energy = True
    for want in golden['sweeps']:
        energy, _ = driver.sweep()
        assert abs(energy - want['energy']) < 1e-5, (energy, want['energy'])
    assert energy > golden['exact'] - 1e-10


def test_windows_find_their_matvec_plans_compiled_during_the_previous_split(monkeypatch):
    '''Near convergence a window's bond keeps its multiplets, so the matvec plan of each window but
    the first of a half-sweep is compiled while the previous window's split runs (DMRG._compile_ahead),
    and the sweep's energy matches a sweep from the same state that compiles every plan in its call.'''
    from tentorch_gb300 import linalg as la
    driver = _driver(16, 32, n_iter = 5)
    for _ in range(6):
        driver.sweep()
    state = ([t.clone() for t in driver.state.tensors], driver.state.center)
    matvec = 'EPaqj,JRSFb,AQsb->EPrf'
    misses = {'ahead': 0, 'call': 0}
    inside = [False]
    real_plan, real_ahead = la._plan, nw.DMRG._compile_ahead

    def counting(key, build, cat):
        if key not in la._plans and key[0] == 'einsum' and key[1] == matvec:
            misses['ahead' if inside[0] else 'call'] += 1
        return real_plan(key, build, cat)

    def ahead(self, *args):
        inside[0] = True
        try:
            real_ahead(self, *args)
        finally:
            inside[0] = False

    monkeypatch.setattr(la, '_plan', counting)
    monkeypatch.setattr(nw.DMRG, '_compile_ahead', ahead)
    la.clear_plans()
    energy, _ = driver.sweep()
    # the right half-sweep meets every window's shapes first; a window whose bond changed, and the
    # first window, compile in the call
    assert misses['ahead'] >= driver.L // 2 and misses['ahead'] >= misses['call'], misses

    monkeypatch.setattr(nw.DMRG, '_compile_ahead', lambda self, *args: None)
    driver.state.tensors = [t.clone() for t in state[0]]
    driver.state.center = state[1]
    la.clear_plans()
    plain, _ = driver.sweep()
    assert abs(energy - plain) < ENERGY_TOL, (energy, plain)
