'''The autotuner's host side (no GPU): histogram keys of compiled plans and the form cache.'''
import torch

import tentorch_gb300 as tg
from tentorch_gb300 import linalg as la
from tentorch_gb300.tensor import Tensor

MATVEC = 'EPaqj,JRSFb,AQsb->EPrf'


def _matvec_plan(chi):
    '''The two-site matvec plan at bond chi, compiled from host tensors (nothing executes).'''
    import bench
    cat = tg.u1
    site = tg.heisenberg(cat, 4, dtype = torch.float64, device = 'cpu').tensors[1]
    w, phys = site.codomain[0], site.codomain[1]
    bond = tg.Leg(cat, *bench.bond_multiplicities(chi))
    mk = lambda cod, dom: tg.Tensor(cat, cod, dom, (0,), dtype = torch.float64, device = 'cpu')
    left, right, theta = mk([bond, w], [bond]), mk([bond, w], [bond]), mk([bond, phys], [phys, bond])

    def blank(spec, *ts):
        plan = la.plan_of(spec, *ts)
        return Tensor._wrap(plan.out_space, torch.zeros(plan.out_space.size, dtype = torch.float64))
    head = blank('EIa,IPqj->EPaqj', left, site)
    tail = blank('JRsk,Fkb->JRSFb', site, right)
    return la.plan_of(MATVEC, head, tail, theta)


def test_histogram_keys_tell_bond_dimensions_apart():
    a, b, c = _matvec_plan(64), _matvec_plan(128), _matvec_plan(64)
    assert a is c
    assert la.histogram_key(a) == la.histogram_key(c)
    assert la.histogram_key(a) != la.histogram_key(b)


def test_form_cache_stores_looks_up_and_clears():
    plan = _matvec_plan(32)
    la.clear_tuning()
    assert la.tuned_forms(plan, precision = 0) is None
    la.store_forms(plan, la.FORM_SEPARATE, precision = 0)
    assert la.tuned_forms(plan, precision = 0) == la.FORM_SEPARATE
    assert la.tuned_forms(plan, precision = 6) is None  # per precision
    la.store_forms(plan, la.FORM_NO_TENSOR_CORES, precision = 6)
    assert la.tuned_forms(plan, precision = 6) == la.FORM_NO_TENSOR_CORES
    la.clear_tuning()
    assert la.tuned_forms(plan, precision = 0) is None


def test_unknown_forms_are_refused():
    import pytest
    plan = _matvec_plan(32)
    with pytest.raises(ValueError):
        la.store_forms(plan, 7, precision = 0)


def test_the_matvec_plan_is_a_product_chain_and_a_plain_contraction_is_not():
    '''The compiler finds the two-site matvec's chain (a product, the leg move of its result, the
    product that reads the moved result: one FP64 launch on the GPU), and a single contraction has
    none; the histogram key records the difference.'''
    plan = _matvec_plan(64)
    text = plan.describe()
    assert text.splitlines()[0].startswith('chain ops ')
    ops = [int(x) for x in text.splitlines()[0].split()[2:]]
    kinds = {int(line.split()[1]): line.split()[2] for line in text.splitlines() if line.startswith('op ')}
    assert [kinds[o] for o in ops] == ['gemm', 'tiles', 'gemm']
    cat = tg.u1
    leg = tg.Leg(cat, [(q,) for q in (-1, 0, 1)], [2, 3, 2])
    a = tg.Tensor(cat, [leg], [leg], (0,), dtype = torch.float64, device = 'cpu')
    single = la.plan_of('ab,bc->ac', a, a)
    assert not single.describe().startswith('chain ops')
    assert la.histogram_key(single) != la.histogram_key(plan)
