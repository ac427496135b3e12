'''Readers of the golden fixtures in tests/golden/ (produced by the reference, see make_golden.py).'''
import json
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'golden')


def load_json(name):
    with open(os.path.join(GOLDEN, name)) as handle:
        return json.load(handle)


_arrays = None


def arrays():
    global _arrays
    if _arrays is None:
        _arrays = dict(np.load(os.path.join(GOLDEN, 'cases.npz')))
    return _arrays


def case_blocks(entry, name):
    '''The blocks of a stored tensor as {(codomain_root, domain_root, copy): ndarray}.'''
    store = arrays()
    out = {}
    for i, key in enumerate(entry['keys']):
        out[(tuple(key[0]), tuple(key[1]), key[2])] = store[f'{name}/{i}']
    return out


def case_names():
    '''The npz prefix of every stored tensor, in the order make_golden.py stored them.'''
    names = sorted({k.rsplit('/', 1)[0] for k in arrays()})
    return names


def leg_args(spec):
    '''(sectors, multiplicities) of a leg spec [[sector, mult], ...].'''
    return [tuple(s) for s, _ in spec], [m for _, m in spec]


def relative_error(a, b):
    a, b = np.asarray(a), np.asarray(b)
    scale = max(np.abs(b).max(initial = 0.0), 1e-300)
    return float(np.abs(a - b).max(initial = 0.0) / scale)
