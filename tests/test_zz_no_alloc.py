'''tt_dots_noalloc: the Krylov dot products for callers that cannot allocate device memory where
they need them (a host framework that forbids allocation inside its solver loop, or one whose memory
pool belongs to another runtime).  It keeps its partial sums in a static device array of the library
instead of caller scratch.  Checked through the C ABI against tt_dots, which takes caller scratch,
on two calls in a row (the array keeps the previous call's partial sums, which must not leak into the
next result).  This file is collected last so that a run stopping at the first failure has already
run every other test; it also passes alone in a fresh process, where its first call does the
per-device set-up.'''
import pytest
import torch

from tentorch_gb300 import _lib

pytestmark = pytest.mark.gpu
TOL = 1e-12


def _dots(dtype, arenas, b, no_alloc):
    count, n = len(arenas), b.numel()
    table = torch.tensor([a.data_ptr() for a in arenas], dtype = torch.int64, device = b.device)
    out = torch.full((2 * count,), float('nan'), dtype = torch.float64, device = b.device)
    stream = torch.cuda.current_stream().cuda_stream
    code = 0 if dtype == torch.float64 else 1
    if no_alloc:
        _lib.check(_lib.lib.tt_dots_noalloc(code, count, table.data_ptr(), b.data_ptr(), n, out.data_ptr(), stream))
    else:
        scratch = torch.empty(2 * 120 * count, dtype = torch.float64, device = b.device)
        _lib.check(_lib.lib.tt_dots(code, count, table.data_ptr(), b.data_ptr(), n, scratch.data_ptr(),
                                    out.data_ptr(), stream))
    torch.cuda.synchronize()
    return torch.complex(out[0::2], out[1::2]).cpu()


@pytest.mark.parametrize('dtype', [torch.float64, torch.complex128])
def test_no_alloc_dots_match_the_scratch_entry_point(dtype):
    gen = torch.Generator(device = 'cuda').manual_seed(41)
    make = lambda n: torch.randn(n, dtype = dtype, device = 'cuda', generator = gen)
    for call, (n, count) in enumerate([(250_001, 64), (33_068, 7)]):  # two calls in a row
        arenas, b = [make(n) for _ in range(count)], make(n)
        want = _dots(dtype, arenas, b, no_alloc = False)
        got = _dots(dtype, arenas, b, no_alloc = True)
        scale = want.abs().max().item()
        assert (got - want).abs().max().item() <= TOL * scale, f'call {call}'


def test_no_alloc_rejects_more_vectors_than_its_array_holds():
    b = torch.zeros(16, dtype = torch.float64, device = 'cuda')
    with pytest.raises(ValueError, match = 'at most 64 vectors'):
        _dots(torch.float64, [b] * 65, b, no_alloc = True)
