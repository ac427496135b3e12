'''The recoupling and batched-window workloads at the sizes the benchmark runs them, checked against
the oracle rather than against another form of this engine:

- the exchange-forcing contraction 'ABcd,DCef->ABef' of two rank-4 tensors over SU(2) legs of spins
  j = 0 .. 4 (2j = 0 .. 8) with 8 multiplets each, float64 (17 blocks per tensor, 85.9 GFLOP of block
  products), and over Fibonacci legs (vacuum 16, tau 16) in complex128 (the Fibonacci R symbol is
  complex); F and R recouplings on every block (tentorch/linalg/graded/einsum.cpp:444-598,
  tentorch/tensors/regroup.cpp:25-258); its split products run on the tensor cores (tcgen05);
- windows of the batched U(1) two-site matvec at the bonds the benchmark draws (chi from
  {32, 64, 128, 256, 512}), one by one and as one launch.

FP64 block products within 1e-12 of the oracle relative to the largest entry; split products with
S slices within their truncation bound (100 * 2^-7S relative, plus FP64 rounding).'''
import numpy as np
import pytest
import torch

import tentorch_gb300 as tg
from convert import max_relative, to_product
from oracle import engine as orc

pytestmark = pytest.mark.gpu
TOL = 1e-12
SPEC = 'ABcd,DCef->ABef'


def split_bound(slices):
    return 100 * 2.0 ** (-7 * slices) + 1e-14


def _operands(catname, top, mult, dtype):
    ocat = orc.CATEGORIES[catname]
    leg = orc.Leg(ocat, [(j,) for j in range(top + 1)], [mult] * (top + 1))
    gen = torch.Generator().manual_seed(0)
    return [orc.Tensor(ocat, [leg, leg], [leg, leg], (0,), dtype).fill_random(gen) for _ in range(2)]


@pytest.fixture(scope = 'module')
def su2_case():
    a, b = _operands('su2', 8, 8, np.float64)
    return a, b, orc.einsum(SPEC, a, b).blocks


def _tickets_clear():
    from tentorch_gb300 import linalg as la
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream().cuda_stream
    pool = la._pools[(torch.cuda.current_device(), stream, torch.float64)]
    return int(torch.count_nonzero(pool[:8192]).item()) == 0


def test_su2_recoupling_at_the_benchmark_size_matches_the_oracle(su2_case):
    a, b, want = su2_case
    pa, pb = to_product(a, tg.su2), to_product(b, tg.su2)
    assert pa.nblocks() == 17
    with tg.precision(0):
        got = tg.einsum(SPEC, pa, pb)
    assert max_relative(got, want) < TOL


@pytest.mark.parametrize('slices', [2, 4, 6])
def test_tensor_core_split_products_match_the_oracle(su2_case, slices):
    '''The SU(2) recoupling at the benchmark size runs its split products on the tensor cores
    (tcgen05: 128 x 64 tiles, one level sum per slice pair in tensor memory): against the FP64
    oracle within the truncation bound of `slices` slices, twice in a row (the kernel leaves its
    tensor memory and barriers as it found them), with the workspace's error flag still clear.'''
    a, b, want = su2_case
    pa, pb = to_product(a, tg.su2), to_product(b, tg.su2)
    with tg.precision(slices):
        for _ in range(2):
            assert max_relative(tg.einsum(SPEC, pa, pb), want) < split_bound(slices)
    assert _tickets_clear()


def test_fibonacci_recoupling_at_the_benchmark_size_matches_the_oracle():
    a, b = _operands('fibonacci', 1, 16, np.complex128)
    for t in (a, b):
        for key in t.blocks:
            t.blocks[key] = t.blocks[key] * (1 + 0.5j)
    want = orc.einsum(SPEC, a, b)
    with tg.precision(0):
        got = tg.einsum(SPEC, to_product(a, tg.fibonacci), to_product(b, tg.fibonacci))
    assert max_relative(got, want.blocks) < TOL


def _window_chis():
    return [int(c) for c in np.random.default_rng(0).choice([32, 64, 128, 256, 512], size = 64)]


@pytest.mark.parametrize('window', [0, 3, 5, 12])  # chi 512, 64, 32, 128
def test_batched_window_matches_the_oracle(window):
    '''Window i of the batched workload: chi drawn from the workload's seeded generator, inputs
    seeded with the workload's seed + i (the benchmark draws them the same way), in FP64 (one launch
    with the leg move between the products) and in six-slice split precision (the first product
    storing through the move).'''
    head, tail, theta = orc.matvec_inputs(_window_chis()[window], seed = window)
    want = orc.einsum(orc.MATVEC, head, tail, theta)
    h, t, v = (to_product(x, tg.u1) for x in (head, tail, theta))
    for _ in range(2):  # the second call with the operator prepared
        with tg.precision(0):
            assert max_relative(tg.einsum(orc.MATVEC, h, t, v), want.blocks) < TOL
        with tg.precision(6):
            assert max_relative(tg.einsum(orc.MATVEC, h, t, v), want.blocks) < split_bound(6)
    assert _tickets_clear()


def test_batched_windows_run_as_one_launch():
    '''Windows of different bond dimension (the first eight of the batched workload's draw) through
    einsum_batch: in FP64 their matvec chains run as ONE persistent launch whose results meet the
    oracle within 1e-12, twice in a row (the second call with prepared operators); in split
    precision the same call runs the windows one after another.'''
    from tentorch_gb300 import linalg as la
    chis = _window_chis()[:8]
    cases = [orc.matvec_inputs(chi, seed = 100 + i) for i, chi in enumerate(chis)]
    wants = [orc.einsum(orc.MATVEC, *c).blocks for c in cases]
    windows = [[to_product(x, tg.u1) for x in c] for c in cases]
    with tg.precision(0):
        for _ in range(2):
            outs = la.einsum_batch(orc.MATVEC, windows)
            assert la.last_batch_launches == 1
            for got, want in zip(outs, wants):
                assert max_relative(got, want) < TOL
    with tg.precision(6):
        outs = la.einsum_batch(orc.MATVEC, windows)
        assert la.last_batch_launches == len(windows)
        for got, want in zip(outs, wants):
            assert max_relative(got, want) < split_bound(6)


def test_tensor_core_form_is_an_autotuned_choice(su2_case):
    '''At the benchmark size the split products can run on tcgen05 or on mma.sync: the autotuner
    times both (tt_autotune) and caches the faster under the plan's histogram; either form meets
    the oracle within the six-slice bound.'''
    from tentorch_gb300 import linalg as la
    a, b, want = su2_case
    pa, pb = to_product(a, tg.su2), to_product(b, tg.su2)
    la.clear_tuning()
    with tg.precision(6):
        plan = la.plan_of(SPEC, pa, pb)
        chosen, ms = la.autotune(SPEC, pa, pb)
        assert chosen in (0, la.FORM_NO_TENSOR_CORES) and ms > 0
        assert la.tuned_forms(plan) == chosen
        for forms in (0, la.FORM_NO_TENSOR_CORES):
            la.store_forms(plan, forms)
            assert max_relative(tg.einsum(SPEC, pa, pb), want) < split_bound(6)
    la.clear_tuning()
