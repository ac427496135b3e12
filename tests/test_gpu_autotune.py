'''The autotuner on the GPU: tt_autotune times the forms a plan's products can run in, caches the
fastest by the plan's block-size histogram, and every form gives the oracle's result.'''
import pytest
import torch

import tentorch_gb300 as tg
from tentorch_gb300 import linalg as la
from convert import max_relative, to_product
from oracle import engine as orc

pytestmark = pytest.mark.gpu
TOL = 1e-12


def _split_bound(slices):
    return 100 * 2.0 ** (-7 * slices) + 1e-14


def test_matvec_forms_are_timed_cached_and_exact():
    '''The chi = 128 two-site matvec: FP64 (one chain launch or separate launches) and six-slice
    split precision; the choice is cached under the plan's histogram and every form meets the
    oracle.'''
    head, tail, theta = orc.matvec_inputs(128, seed = 3)
    want = orc.einsum(orc.MATVEC, head, tail, theta).blocks
    h, t, v = (to_product(x, tg.u1) for x in (head, tail, theta))
    la.clear_tuning()
    for precision, forms in ((0, (0, la.FORM_SEPARATE)), (6, (0, la.FORM_SEPARATE))):
        with tg.precision(precision):
            plan = la.plan_of(orc.MATVEC, h, t, v)
            chosen, ms = la.autotune(orc.MATVEC, h, t, v)
            assert chosen in forms and ms > 0
            assert la.tuned_forms(plan) == chosen
            bound = TOL if precision == 0 else _split_bound(6)
            for f in forms:
                la.store_forms(plan, f)
                assert max_relative(tg.einsum(orc.MATVEC, h, t, v), want) < bound
    la.clear_tuning()
