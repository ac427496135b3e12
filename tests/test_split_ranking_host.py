'''The split's ranking (tentorch/linalg/graded/svd.cpp:68-118) as the host restates it
(`linalg._rank_candidates`: a stable sort of (value, block, index), the cut, the kept prefix of each
block, the +-q pairing) against the order of work the device ranking kernel (`tt_svd_rank`) does:
sort by (value descending, position), cut at `tol` and `max_bond`, count each block's values below
the cut, then pair by counting each domain sector's values in sorted order.  Random cases with ties,
zeros and unpaired sectors; the two agree on every block's kept count.'''
import random
from collections import namedtuple

from tentorch_gb300 import linalg as la

Key = namedtuple('Key', 'codomain domain copy')


class _Dual:
    def __init__(self, dual):
        self.d = dual

    def dual(self, sector):
        return self.d[sector]


def _kernel_order(values, domains, dual, tol, max_bond):
    flat, block = [], []
    for fi, vs in enumerate(values):
        for v in vs:
            flat.append(v)
            block.append(fi)
    order = sorted(range(len(flat)), key = lambda p: (-flat[p], p))
    cut = sum(1 for v in flat if v > tol)
    if max_bond is not None:
        cut = min(cut, max_bond)
    kept = [0] * len(values)
    for r in range(cut):
        kept[block[order[r]]] += 1
    sectors = sorted(set(domains) | {dual[s] for s in domains})
    mult = {s: 0 for s in sectors}
    for fi, k in enumerate(kept):
        mult[domains[fi]] += k
    paired, differs, anything = {}, False, False
    for s in sectors:
        if mult[s] == 0:
            continue
        if mult[dual[s]] > 0:
            paired[s] = min(mult[s], mult[dual[s]])
            anything = True
            differs |= paired[s] != mult[s]
        else:
            differs = True
    if anything and differs:
        kept = [0] * len(values)
        used = {s: 0 for s in sectors}
        for r in range(cut):
            fi = block[order[r]]
            s = domains[fi]
            if s not in paired or used[s] >= paired[s]:
                continue
            used[s] += 1
            kept[fi] += 1
    return kept


def test_device_ranking_order_equals_the_host_ranking():
    rng = random.Random(7)
    for _ in range(3000):
        n_sectors = rng.randint(1, 6)
        dual = list(range(n_sectors))
        order = list(range(n_sectors))
        rng.shuffle(order)
        for i in range(0, n_sectors - 1, 2):
            if rng.random() < 0.7:
                a, b = order[i], order[i + 1]
                dual[a], dual[b] = b, a
        nb = rng.randint(1, 8)
        domains = [rng.randrange(n_sectors) for _ in range(nb)]
        values = [sorted((rng.choice([1.0, 0.5, 0.25, 1e-3, 1e-15, 0.0, rng.random()]) for _ in range(rng.randint(0, 6))),
                         reverse = True) for _ in range(nb)]
        tol = rng.choice([0.0, 1e-14, 0.3])
        max_bond = rng.choice([None, 1, 3, 5, 100])
        factors = [[Key(None, domains[fi], 0), None, None, None, 0, 0] for fi in range(nb)]
        candidates = [(v, fi, i) for fi, vs in enumerate(values) for i, v in enumerate(vs)]
        la._rank_candidates(factors, candidates, max_bond, tol, _Dual(dual))
        assert [f[4] for f in factors] == _kernel_order(values, domains, dual, tol, max_bond)
