'''The engine's launches captured in a CUDA graph: several two-site windows (two of them on one
plan) issued as one graph once warm-up calls have compiled the plans and uploaded their tables.
A graph reads every operand from its own buffer (no prepared copies).  Replays equal the eager
calls on the same operands in both forms of the block products, and after new vectors and a new
environment are written into the captured buffers a replay equals the eager calls on them: the
graph reads its inputs and caches no result.'''
import pytest
import torch

import tentorch_gb300 as tg

pytestmark = pytest.mark.gpu
MATVEC = 'EPaqj,JRSFb,AQsb->EPrf'


def _window(chi, seed):
    cat = tg.u1
    site = tg.heisenberg(cat, 4, dtype = torch.float64, device = 'cuda').tensors[1]
    w, phys = site.codomain[0], site.codomain[1]
    share = [1, 2, 3, 4, 3, 2, 1]
    mult = [max(1, chi * s // sum(share)) for s in share]
    bond = tg.Leg(cat, [(2 * q,) for q in range(-3, 4)], mult)
    gen = torch.Generator().manual_seed(seed)

    def filled(cod, dom):
        t = tg.Tensor(cat, cod, dom, (0,), dtype = torch.float64, device = 'cuda')
        for block in t.to_tuple()[3].values():
            block.copy_(torch.randn(block.shape, dtype = torch.float64, generator = gen))
        return t
    left, right = filled([bond, w], [bond]), filled([bond, w], [bond])
    theta = filled([bond, phys], [phys, bond])
    head = tg.einsum('EIa,IPqj->EPaqj', left, site)
    tail = tg.einsum('JRsk,Fkb->JRSFb', site, right)
    return head, tail, theta


@pytest.mark.parametrize('precision', [0, 8])
def test_graph_replay_of_batched_windows_equals_eager_calls(precision):
    windows = [_window(chi, seed) for seed, chi in enumerate([24, 40, 24])]
    with tg.precision(precision):
        for _ in range(3):
            eager = [tg.einsum(MATVEC, *win).data.clone() for win in windows]
        torch.cuda.synchronize()
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph):
            images = [tg.einsum(MATVEC, *win) for win in windows]
        graph.replay()
        torch.cuda.synchronize()
        for got, want in zip(images, eager):
            assert torch.max(torch.abs(got.data - want)).item() <= 1e-13 * torch.max(torch.abs(want)).item()
        gen = torch.Generator().manual_seed(99)
        for win in windows:
            win[2].data.copy_(torch.randn(win[2].data.shape, dtype = torch.float64, generator = gen))
        windows[1][0].data.mul_(-0.5)
        graph.replay()
        torch.cuda.synchronize()
        for got, win in zip(images, windows):
            want = tg.einsum(MATVEC, *win).data
            assert torch.max(torch.abs(got.data - want)).item() <= 1e-13 * torch.max(torch.abs(want)).item()


@pytest.mark.parametrize('precision', [0, 6])
def test_lanczos_window_captured_in_a_graph(precision):
    '''A whole Lanczos window (ten matvecs, the orthogonalisation passes, the tridiagonal's lowest
    Ritz pair on the device and the normalised Ritz vector) captured as one CUDA graph: the call with
    `wait=False` has no host synchronisation inside.  A replay gives the eager call's energy and
    vector; after a new start vector and a scaled head are written into the captured buffers, a
    replay gives the eager call's result on them (the graph prepares the head and tail itself).'''
    from tentorch_gb300.lanczos import lanczos_einsum
    head, tail, theta = _window(40, 7)

    def eager():
        energy, vector = lanczos_einsum(MATVEC, [head, tail, theta], 2, theta, 10, wait = False)
        return energy.item(), vector.data.clone()
    with tg.precision(precision):
        for _ in range(2):
            want_e, want_v = eager()
        torch.cuda.synchronize()
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph):
            energy, vector = lanczos_einsum(MATVEC, [head, tail, theta], 2, theta, 10, wait = False)
        graph.replay()
        torch.cuda.synchronize()
        assert abs(energy.item() - want_e) <= 1e-12 * abs(want_e)
        assert torch.max(torch.abs(vector.data - want_v)).item() <= 1e-9
        gen = torch.Generator().manual_seed(5)
        theta.data.copy_(torch.randn(theta.data.shape, dtype = torch.float64, generator = gen))
        head.data.mul_(-0.5)
        graph.replay()
        torch.cuda.synchronize()
        want_e, want_v = eager()
        assert abs(energy.item() - want_e) <= 1e-12 * abs(want_e)
        assert torch.max(torch.abs(vector.data - want_v)).item() <= 1e-9


def test_batched_windows_as_one_launch_in_a_graph():
    '''Windows of different bond dimension through einsum_batch captured in a CUDA graph: in FP64
    their matvec chains are one persistent launch inside the graph; replays equal the eager batch,
    also after new vectors are written into the captured buffers.'''
    from tentorch_gb300 import linalg as la
    windows = [_window(chi, 20 + seed) for seed, chi in enumerate([16, 40, 24, 56])]
    with tg.precision(0):
        for _ in range(2):
            eager = [o.data.clone() for o in la.einsum_batch(MATVEC, windows)]
        assert la.last_batch_launches == 1
        torch.cuda.synchronize()
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph):
            images = la.einsum_batch(MATVEC, windows)
        assert la.last_batch_launches == 1
        graph.replay()
        torch.cuda.synchronize()
        for got, want in zip(images, eager):
            assert torch.max(torch.abs(got.data - want)).item() <= 1e-13 * torch.max(torch.abs(want)).item()
        gen = torch.Generator().manual_seed(98)
        for win in windows:
            win[2].data.copy_(torch.randn(win[2].data.shape, dtype = torch.float64, generator = gen))
        graph.replay()
        torch.cuda.synchronize()
        for got, win in zip(images, windows):
            want = tg.einsum(MATVEC, *win).data
            assert torch.max(torch.abs(got.data - want)).item() <= 1e-13 * torch.max(torch.abs(want)).item()
