'''The truncating splittings on the GPU (tentorch/linalg/graded/svd.cpp): the engine's batched Jacobi
SVD against the per-block LAPACK-style SVD (at::linalg_svd, the reference's call) on the same
blocks, the truncation, the +-q pairing and the absorbed values, and QR / RQ.  Singular values
within 1e-13 relative, factors orthonormal within 1e-13, products within 1e-12.'''
import numpy as np
import pytest
import torch

import tentorch_gb300 as tg
from tentorch_gb300 import linalg as la

pytestmark = pytest.mark.gpu


def _tensor(rows_by_charge, cols_by_charge, seed):
    '''A U(1) matrix-like tensor with one block per charge: codomain [a], domain [b].'''
    cat = tg.u1
    charges = sorted(rows_by_charge)
    a = tg.Leg(cat, [(q,) for q in charges], [rows_by_charge[q] for q in charges])
    b = tg.Leg(cat, [(q,) for q in charges], [cols_by_charge[q] for q in charges])
    t = tg.Tensor(cat, [a], [b], (0,), dtype = torch.float64, device = 'cuda')
    _fill(t, seed)
    return t


def _fill(t, seed):
    """N(0, 1) blocks in key order; the arena's padding stays zero."""
    gen = torch.Generator().manual_seed(seed)
    for block in t.to_tuple()[3].values():
        block.copy_(torch.randn(block.shape, dtype = torch.float64, generator = gen))


# charge-symmetric (the split pairs q with -q, svd.cpp:97-120, so a bond sector without its dual
# partner would be dropped): tall and wide blocks, small ones, ones whose working set fits in
# shared memory and ones that need the global workspace
SHAPES = {-5: (300, 200), -4: (130, 140), -3: (1, 1), -2: (1, 5), -1: (60, 90), 0: (117, 117), 1: (90, 60),
          2: (5, 1), 3: (1, 1), 4: (140, 130), 5: (200, 300)}


def _blocks(t):
    return {k: v for k, v in t.to_tuple()[3].items()}


def test_batched_svd_matches_per_block_svd():
    t = _tensor({q: r for q, (r, c) in SHAPES.items()}, {q: c for q, (r, c) in SHAPES.items()}, seed = 1)
    first, values, second = tg.svd(t)
    with tg.precision(la.PER_BLOCK):
        first_ref, values_ref, second_ref = tg.svd(t)
    torch.cuda.synchronize()
    assert torch.allclose(values, values_ref, rtol = 1e-13, atol = 0)
    # with the values absorbed the factors multiply back to the tensor; without, they are orthonormal
    scaled, _, rest = tg.svd(t, None, 0.0, 1)
    product = tg.contract(scaled, rest, [1], [0])
    assert torch.max(torch.abs(product.data - t.data)).item() < 1e-12 * torch.max(torch.abs(t.data)).item()
    for key, u in _blocks(first).items():
        eye = torch.eye(u.shape[1], dtype = torch.float64, device = 'cuda')
        assert torch.max(torch.abs(u.T @ u - eye)).item() < 1e-13
    for key, vh in _blocks(second).items():
        eye = torch.eye(vh.shape[0], dtype = torch.float64, device = 'cuda')
        assert torch.max(torch.abs(vh @ vh.T - eye)).item() < 1e-13


def test_a_spectrum_over_twelve_decades_agrees_with_lapack():
    """Singular values from 1 down to 1e-12: the Jacobi values agree with LAPACK's on the same
    block to 1e-14 absolute (both are accurate to a few ulps of the largest value)."""
    cat = tg.u1
    leg = tg.Leg(cat, [(0,)], [40])
    t = tg.Tensor(cat, [leg], [leg], (0,), dtype = torch.float64, device = 'cuda')
    gen = torch.Generator().manual_seed(3)
    q1, _ = torch.linalg.qr(torch.randn(40, 40, dtype = torch.float64, generator = gen))
    q2, _ = torch.linalg.qr(torch.randn(40, 40, dtype = torch.float64, generator = gen))
    sigma = torch.logspace(0, -12, 40, dtype = torch.float64)
    t.data[:1600].copy_((q1 @ torch.diag(sigma) @ q2.T).reshape(-1))
    _, values, _ = tg.svd(t)
    want = torch.linalg.svdvals(t.data[:1600].reshape(40, 40).cpu())
    assert torch.max(torch.abs(values.cpu() - want)).item() < 1e-14
    assert torch.max(torch.abs(values.cpu() - sigma)).item() < 1e-14


def test_rank_deficient_and_zero_blocks_through_the_preconditioned_path():
    """Blocks of 32 columns or more are sorted and QR-factored before the sweeps: a tall and a wide
    block of rank 12 (the split pairs the bond sectors of q and -q, so the two keep as many values)
    and an all-zero block (40 columns each) give LAPACK's values, factors that multiply back to the
    tensor, and singular vectors orthonormal wherever their value is not zero."""
    t = _tensor({-1: 48, 0: 40, 1: 40}, {-1: 40, 0: 40, 1: 48}, seed = 4)
    gen = torch.Generator().manual_seed(5)
    for block in _blocks(t).values():
        if block.shape == (40, 40):
            block.zero_()
        else:
            m, n = block.shape
            block.copy_(torch.randn(m, 12, dtype = torch.float64, generator = gen) @
                        torch.randn(12, n, dtype = torch.float64, generator = gen))
    # values below 1e-10 of the largest (the zero block's and the rank-12 block's round-off) are cut
    first, values, second = tg.svd(t, None, 1e-10)
    with tg.precision(la.PER_BLOCK):
        _, values_ref, _ = tg.svd(t, None, 1e-10)
    torch.cuda.synchronize()
    big = torch.max(torch.abs(values_ref)).item()
    assert values.shape == values_ref.shape
    assert torch.max(torch.abs(values - values_ref)).item() < 1e-13 * big
    scaled, _, rest = tg.svd(t, None, 1e-10, 1)
    product = tg.contract(scaled, rest, [1], [0])
    assert torch.max(torch.abs(product.data - t.data)).item() < 1e-12 * torch.max(torch.abs(t.data)).item()
    for factor, columns in ((first, True), (second, False)):
        for key, f in _blocks(factor).items():
            g = f.T @ f if columns else f @ f.T
            d = torch.diagonal(g)
            assert torch.all((torch.abs(d - 1) < 1e-13) | (torch.abs(d) < 1e-13))
            assert torch.max(torch.abs(g - torch.diag(d))).item() < 1e-13


@pytest.mark.parametrize('absorb', [0, 1, 2, 3])
def test_truncating_split_matches_the_per_block_form(absorb):
    rows = {-2: 20, 0: 40, 2: 20}
    t = _tensor(rows, rows, seed = 2)
    first, values, second = tg.svd(t, 30, 1e-14, absorb)
    with tg.precision(la.PER_BLOCK):
        first_ref, values_ref, second_ref = tg.svd(t, 30, 1e-14, absorb)
    assert first.domain == first_ref.domain and second.codomain == second_ref.codomain
    assert torch.allclose(values, values_ref, rtol = 1e-13, atol = 0)
    # the kept factors agree up to the sign of each singular vector pair
    product = tg.contract(first, second, [1], [0])
    product_ref = tg.contract(first_ref, second_ref, [1], [0])
    assert torch.max(torch.abs(product.data - product_ref.data)).item() < 1e-12


def test_split_of_the_two_site_tensor_pairs_the_bond():
    '''A two-site tensor [bond, phys] -> [phys, bond] with charge-symmetric bonds: the kept bond
    carries as many multiplets in q as in -q (svd.cpp:97-117).'''
    cat = tg.u1
    bond = tg.Leg(cat, [(-2,), (0,), (2,)], [6, 9, 6])
    phys = tg.Leg(cat, [(-1,), (1,)], [1, 1])
    t = tg.Tensor(cat, [bond, phys], [phys, bond], (0,), dtype = torch.float64, device = 'cuda')
    _fill(t, 4)
    first, values, second = tg.svd(t, 11, 1e-14, 2)
    leg = first.domain[0]
    mult = {leg.sector(b): leg.multiplicity(b) for b in range(leg.nblocks())}
    for sector, count in mult.items():
        assert mult.get((-sector[0],), count) == count
    with tg.precision(la.PER_BLOCK):
        first_ref, values_ref, second_ref = tg.svd(t, 11, 1e-14, 2)
    assert first.domain == first_ref.domain
    assert torch.allclose(values, values_ref, rtol = 1e-13, atol = 0)


def test_qr_and_rq_factor_the_tensor():
    rows = {-1: 7, 0: 12, 1: 5}
    cols = {-1: 4, 0: 12, 1: 9}
    t = _tensor(rows, cols, seed = 5)
    q, r = tg.qr(t)
    assert torch.max(torch.abs(tg.contract(q, r, [1], [0]).data - t.data)).item() < 1e-13
    for u in _blocks(q).values():
        assert torch.max(torch.abs(u.T @ u - torch.eye(u.shape[1], dtype = torch.float64, device = 'cuda'))).item() < 1e-13
    l, qq = tg.rq(t)
    assert torch.max(torch.abs(tg.contract(l, qq, [1], [0]).data - t.data)).item() < 1e-13
    for v in _blocks(qq).values():
        assert torch.max(torch.abs(v @ v.T - torch.eye(v.shape[0], dtype = torch.float64, device = 'cuda'))).item() < 1e-13


def test_a_block_too_large_for_shared_memory_splits_through_the_workspace():
    '''A 700 x 600 block: its rows dealt over a cluster still do not fit in shared memory, so the
    FP32 and FP64 sweeps keep W and V in the global workspace.  Values against LAPACK to 1e-12
    relative, factors orthonormal to 1e-13, the product back to the block to 1e-12.'''
    t = _tensor({0: 700}, {0: 600}, seed = 7)
    first, values, second = tg.svd(t)
    block = t.data[:700 * 600].reshape(700, 600)
    want = torch.linalg.svdvals(block.cpu())
    assert torch.allclose(values.cpu(), want, rtol = 1e-12, atol = 0)
    u = first.data[:700 * 600].reshape(700, 600)
    vh = second.data[:600 * 600].reshape(600, 600)
    eye = torch.eye(600, dtype = torch.float64, device = 'cuda')
    assert torch.max(torch.abs(u.T @ u - eye)).item() < 1e-13
    assert torch.max(torch.abs(vh @ vh.T - eye)).item() < 1e-13
    product = (u * values) @ vh
    assert torch.max(torch.abs(product - block)).item() < 1e-12 * torch.max(torch.abs(block)).item()
