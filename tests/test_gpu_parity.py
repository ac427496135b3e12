'''Parity of the CUDA path with the reference: every golden case (place, contract, einsum over U(1),
SU(2), Fibonacci and no symmetry) run on the GPU through the C ABI against the reference's own
outputs, and the seeded two-site matvec (chi = 64 and 256) against the oracle.  FP64 block products:
values within 1e-12 relative of the reference.'''
import numpy as np
import pytest
import torch

import tentorch_gb300 as tg
from convert import PRODUCT_CATS, case_category, fixture_tensor, max_relative, to_oracle, to_product
from golden_io import case_blocks, load_json
from oracle import engine as orc

pytestmark = pytest.mark.gpu
TOL = 1e-12


@pytest.fixture(autouse = True)
def fp64():
    with tg.precision(0):
        yield


@pytest.mark.parametrize('index', range(len(load_json('cases.json'))))
def test_golden_case_on_the_gpu(index):
    case = load_json('cases.json')[index]
    catname = case_category(case['inputs'][0]['name'])
    cat = PRODUCT_CATS[catname]
    dtype = torch.complex128 if catname == 'fibonacci' else torch.float64
    inputs = [fixture_tensor(e, cat, dtype) for e in case['inputs']]
    if case['op'] == 'place':
        out = inputs[0].place(case['above'], case['below'])
    elif case['op'] == 'contract':
        out = tg.contract(inputs[0], inputs[1], case['left_legs'], case['right_legs'], tuple(case['charge']))
    else:
        kw = {'outcharge': tuple(case['outcharge'])} if case.get('outcharge') else {}
        out = tg.einsum(case['spec'], *inputs, **kw)
    torch.cuda.synchronize()
    assert out.device.type == 'cuda'
    want = case_blocks(case['output'], case['output']['name'])
    assert max_relative(out, want) < TOL


@pytest.mark.parametrize('chi', [32, 64, 256])
def test_matvec_matches_the_oracle(chi):
    head, tail, theta = orc.matvec_inputs(chi, seed = 7)
    want = orc.einsum(orc.MATVEC, head, tail, theta)
    h, t, v = (to_product(x, tg.u1) for x in (head, tail, theta))
    got = tg.einsum(orc.MATVEC, h, t, v)
    assert max_relative(got, want.blocks) < TOL
    # a second call reuses the prepared head and tail; a changed vector changes the image
    v2 = v * 2.0
    got2 = tg.einsum(orc.MATVEC, h, t, v2)
    assert max_relative(got2, {k: 2 * b for k, b in want.blocks.items()}) < TOL


def test_head_and_tail_builds_match_the_oracle():
    qs, deg = orc.degeneracies(64)
    cat = orc.u1
    bond = orc.Leg(cat, [(2 * q,) for q in qs], deg)
    site, phys, w = orc.heisenberg_site(cat)
    gen = torch.Generator().manual_seed(3)
    left = orc.Tensor(cat, [bond, w], [bond], (0,)).fill_random(gen)
    right = orc.Tensor(cat, [bond, w], [bond], (0,)).fill_random(gen)
    for spec, ops in (('EIa,IPqj->EPaqj', (left, site)), ('JRsk,Fkb->JRSFb', (site, right))):
        want = orc.einsum(spec, *ops)
        got = tg.einsum(spec, *(to_product(x, tg.u1) for x in ops))
        assert max_relative(got, want.blocks) < TOL


def test_a_changed_operator_is_prepared_again():
    head, tail, theta = orc.matvec_inputs(32, seed = 9)
    h, t, v = (to_product(x, tg.u1) for x in (head, tail, theta))
    tg.einsum(orc.MATVEC, h, t, v)
    h.data.mul_(-1.0)  # in place: the cached preparation of h must not be reused
    got = tg.einsum(orc.MATVEC, h, t, v)
    want = orc.einsum(orc.MATVEC, head, tail, theta)
    assert max_relative(got, {k: -b for k, b in want.blocks.items()}) < TOL


@pytest.mark.parametrize('catname,mult,top', [('su2', 2, 6), ('fibonacci', 4, 1)])
def test_recoupling_einsum_matches_the_oracle(catname, mult, top):
    '''The exchange-forcing contraction of two rank-4 tensors, F and R on every block.'''
    ocat, cat = orc.CATEGORIES[catname], PRODUCT_CATS[catname]
    dtype = np.complex128 if catname == 'fibonacci' else np.float64
    leg = orc.Leg(ocat, [(j,) for j in range(top + 1)], [mult] * (top + 1))
    gen = torch.Generator().manual_seed(5)
    a = orc.Tensor(ocat, [leg, leg], [leg, leg], (0,), dtype).fill_random(gen)
    b = orc.Tensor(ocat, [leg, leg], [leg, leg], (0,), dtype).fill_random(gen)
    if dtype == np.complex128:
        for t in (a, b):
            for key in t.blocks:
                t.blocks[key] = t.blocks[key] * (1 + 0.5j)
    want = orc.einsum('ABcd,DCef->ABef', a, b)
    got = tg.einsum('ABcd,DCef->ABef', to_product(a, cat), to_product(b, cat))
    assert max_relative(got, want.blocks) < TOL


def test_place_round_trip_is_the_identity():
    '''A leg move and its inverse give back the same arena (a size-independent property).'''
    head, tail, theta = orc.matvec_inputs(256, seed = 11)
    t = to_product(tail, tg.u1)
    moved = t.place([0, 2, 4], [1, 3])
    back = moved.place([0, 3, 1, 4], [2])
    assert torch.equal(back.data, t.data)


def test_inner_and_norm_on_the_device():
    head, tail, theta = orc.matvec_inputs(64, seed = 13)
    v = to_product(theta, tg.u1)
    assert abs(tg.norm(v) - orc.norm(theta)) < 1e-12 * orc.norm(theta)
    w = v * 0.5
    assert abs(tg.inner(v, w) - 0.5 * orc.norm(theta) ** 2) < 1e-10 * orc.norm(theta) ** 2


@pytest.mark.parametrize('slices', [2, 3, 4, 6, 8])
def test_split_precision_matvec_accuracy(slices):
    '''Split bf16 products: the error of the chi = 256 matvec against the FP64 oracle stays within
    the truncation bound of `slices` 7-bit slices (100 * 2^-7s relative to the largest entry, plus
    FP64 rounding).'''
    head, tail, theta = orc.matvec_inputs(256, seed = 21)
    want = orc.einsum(orc.MATVEC, head, tail, theta)
    h, t, v = (to_product(x, tg.u1) for x in (head, tail, theta))
    with tg.precision(slices):
        got = tg.einsum(orc.MATVEC, h, t, v)
    err = max_relative(got, want.blocks)
    assert err < 100 * 2.0 ** (-7 * slices) + 1e-14, err
    if slices == 8:
        assert err < 1e-14


def test_split_precision_is_deterministic():
    '''Repeated split products are bit-identical, including once head and tail are prepared (from
    the second call on) and their slices are read from the prepared arenas instead of being cut at
    each launch: the first S of the eight cached digits are the digits an S-slice cut makes.'''
    head, tail, theta = orc.matvec_inputs(128, seed = 23)
    h, t, v = (to_product(x, tg.u1) for x in (head, tail, theta))
    plan = tg.linalg.plan_of(orc.MATVEC, h, t, v)
    for slices in (4, 6, 8):
        with tg.precision(slices):
            runs = [tg.einsum(orc.MATVEC, h, t, v).data.clone() for _ in range(3)]
            cut_now = tg.linalg.run(plan, [h, t, v], reuse_prepared = False).data
        assert torch.equal(runs[0], runs[1]) and torch.equal(runs[0], runs[2])
        assert torch.equal(runs[0], cut_now)


def test_large_blocks_split_over_k():
    '''Blocks whose K is long enough to be cut into several work items (partial tiles reduced in a
    fixed order): an SU(2) contraction with multiplicity 8, in FP64 and split precision.'''
    ocat = orc.su2
    leg = orc.Leg(ocat, [(j,) for j in range(5)], [8] * 5)
    gen = torch.Generator().manual_seed(29)
    a = orc.Tensor(ocat, [leg, leg], [leg, leg], (0,)).fill_random(gen)
    b = orc.Tensor(ocat, [leg, leg], [leg, leg], (0,)).fill_random(gen)
    want = orc.einsum('ABcd,DCef->ABef', a, b)
    pa, pb = to_product(a, tg.su2), to_product(b, tg.su2)
    assert max_relative(tg.einsum('ABcd,DCef->ABef', pa, pb), want.blocks) < TOL
    with tg.precision(8):
        assert max_relative(tg.einsum('ABcd,DCef->ABef', pa, pb), want.blocks) < 1e-14


@pytest.mark.parametrize('dtype', [torch.float64, torch.complex128])
def test_device_dot_products(dtype):
    '''tt_dots: <a_j, b> for several arenas in one pass, no host synchronisation, against torch.'''
    import ctypes
    from tentorch_gb300 import _lib
    n, count = 100_003, 5
    gen = torch.Generator(device = 'cuda').manual_seed(31)
    make = lambda: torch.randn(n, dtype = dtype, device = 'cuda', generator = gen)
    arenas, b = [make() for _ in range(count)], make()
    table = torch.tensor([a.data_ptr() for a in arenas], dtype = torch.int64, device = 'cuda')
    scratch = torch.empty(2 * 120 * count, dtype = torch.float64, device = 'cuda')
    out = torch.empty(2 * count, dtype = torch.float64, device = 'cuda')
    _lib.check(_lib.lib.tt_dots(0 if dtype == torch.float64 else 1, count, table.data_ptr(), b.data_ptr(), n,
                                scratch.data_ptr(), out.data_ptr(), torch.cuda.current_stream().cuda_stream))
    got = torch.complex(out[0::2], out[1::2]).cpu()
    want = torch.stack([torch.vdot(a, b) for a in arenas]).to(torch.complex128).cpu()
    assert torch.allclose(got, want, rtol = 1e-12, atol = 1e-10)


@pytest.mark.parametrize('catname', ['u1', 'su2', 'fibonacci'])
def test_conjugate_transpose_is_the_blockwise_one(catname):
    '''tentorch/tensors/tensor.cpp:99-107: the compiled bra (one tiles pass) against the block-by-block
    conjugate transpose on the host container.'''
    cases = load_json('cases.json')
    entry = next(e for c in cases for e in c['inputs'] if case_category(e['name']) == catname)
    cat = PRODUCT_CATS[catname]
    dtype = torch.complex128 if catname == 'fibonacci' else torch.float64
    t = fixture_tensor(entry, cat, dtype)
    if dtype == torch.complex128:
        t.data.mul_(torch.exp(1j * torch.arange(t.data.numel(), dtype = torch.float64, device = 'cuda')))
    got = t.conj()
    want = t.to(device = 'cpu').conj()
    assert got._space is want._space
    assert torch.equal(got.data.cpu(), want.data)


def test_gemm_tickets_are_left_zero_in_the_workspace():
    '''The head of a stream's workspace holds the counters of split output tiles: every launch of
    the grouped kernels leaves them zero (the last finisher of a tile resets its counter), so runs
    after runs of plans with and without block products on one workspace stay correct.'''
    from tentorch_gb300 import linalg as la
    head, tail, theta = orc.matvec_inputs(256, seed = 11)
    want = orc.einsum(orc.MATVEC, head, tail, theta)
    h, t, v = (to_product(x, tg.u1) for x in (head, tail, theta))
    for precision in (0, 6, 0, 8):
        with tg.precision(precision):
            for _ in range(3):
                got = tg.einsum(orc.MATVEC, h, t, v)
                moved = v.place([0, 3], [1, 2])  # a program with temporaries and no block products
        assert max_relative(got, want.blocks) < (TOL if precision in (0, 8) else 1e-10)
        assert moved is not None
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream().cuda_stream
    pool = la._pools[(torch.cuda.current_device(), stream, torch.float64)]
    assert int(torch.count_nonzero(pool[:8192]).item()) == 0


@pytest.mark.parametrize('slices, tol', [(0, TOL), (6, 1000 * 2.0 ** -42)])
def test_full_size_matvec_is_linear(slices, tol):
    '''The matvec at the largest bond of the DMRG workloads (chi = 1024, 562,412 entries a vector;
    beyond what the oracle builds within a test's time) through a size-independent property: the
    image of 2x + 3y is 2 Hx + 3 Hy, in FP64 to round-off and in six slices within ten times the
    split's bound on each of the three images (relative to the largest entry).'''
    import bench
    head, tail, x = bench.matvec_operands(tg, torch, 'cuda', 1024, 31)
    y = x.clone()
    gen = torch.Generator().manual_seed(32)
    for block in y.to_tuple()[3].values():
        block.copy_(torch.randn(block.shape, dtype = torch.float64, generator = gen))
    z = x * 2.0
    z += y * 3.0
    with tg.precision(slices):
        hx, hy, hz = (tg.einsum(orc.MATVEC, head, tail, v) for v in (x, y, z))
    blocks = lambda t: torch.cat([b.flatten() for b in t.to_tuple()[3].values()])
    want = blocks(hx) * 2.0 + blocks(hy) * 3.0
    scale = float(want.abs().max())
    err = float((blocks(hz) - want).abs().max()) / scale
    assert scale > 0 and err < tol, err
