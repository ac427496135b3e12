'''Host <-> device transfers by a kernel over the coherent CPU-GPU link (tt_link_copy).'''
import pytest
import torch

from tentorch_gb300 import linalg as la

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize('n', [1, 7, 33080, 33081])
def test_link_copy_both_ways_equals_the_data(n):
    gen = torch.Generator().manual_seed(n)
    host = torch.randn(n, dtype = torch.float64, generator = gen).pin_memory()
    device = torch.empty(n, dtype = torch.float64, device = 'cuda')
    la.link_copy(device, host)
    torch.cuda.synchronize()
    assert torch.equal(device.cpu(), host)
    back = torch.empty(n, dtype = torch.float64).pin_memory()
    la.link_copy(back, device * 2)
    torch.cuda.synchronize()
    assert torch.equal(back, host * 2)


def test_link_copy_refuses_unpinned_host_memory():
    host = torch.zeros(16, dtype = torch.float64)
    device = torch.empty(16, dtype = torch.float64, device = 'cuda')
    with pytest.raises(ValueError):
        la.link_copy(device, host)
    with pytest.raises(ValueError):
        la.link_copy(device, torch.zeros(8, dtype = torch.float64).pin_memory())
