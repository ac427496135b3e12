'''The oracle (CPU restatement of the reference) pinned against the reference's own outputs: symbols,
layouts, block keys, per-step plans bit for bit, and place/contract/einsum block values.'''
import numpy as np
import pytest

from golden_io import case_blocks, leg_args, load_json, relative_error
from oracle import engine as orc

SYMBOL_TOL = 1e-13
VALUE_TOL = 1e-12


def legs(cat, specs):
    return [orc.Leg(cat, *leg_args(s)) for s in specs]


def tensor_of(entry, cat, dtype):
    t = orc.Tensor(cat, legs(cat, entry['codomain']), legs(cat, entry['domain']), tuple(entry['qtotal']), dtype)
    for key, block in case_blocks(entry, entry['name']).items():
        t.blocks[key][...] = block
    return t


@pytest.mark.parametrize('name', ['su2', 'fibonacci'])
def test_symbols_match_the_reference(name):
    cat = orc.CATEGORIES[name]
    table = load_json('symbols.json')[name]
    for a, b, c, d, re, im in table['F']:
        got = cat.F_symbol(tuple(a), tuple(b), tuple(c), tuple(d))
        assert np.abs(got - (np.array(re) + 1j * np.array(im))).max(initial = 0) < SYMBOL_TOL, (a, b, c, d)
    for b, c, re, im in table['R']:
        got = cat.R_symbol(tuple(b), tuple(c))
        want = np.array(re) + 1j * np.array(im)
        assert got.shape == want.shape and np.abs(got - want).max(initial = 0) < SYMBOL_TOL


def test_layouts_and_keys_match_the_reference():
    data = load_json('structure.json')
    for case in data['layouts']:
        cat = orc.CATEGORIES[case['cat']]
        trees, offsets = orc.layout_of(cat, legs(cat, case['legs']), tuple(case['root']))
        assert offsets == case['offsets']
        want = [(tuple(map(tuple, t[0])), tuple(map(tuple, t[1])), tuple(t[2]), tuple(t[3])) for t in case['trees']]
        assert trees == want
    for case in data['keys']:
        cat = orc.CATEGORIES[case['cat']]
        keys = orc.block_keys(cat, legs(cat, case['codomain']), legs(cat, case['domain']), tuple(case['qtotal']))
        assert [[list(k[0]), list(k[1]), k[2]] for k in keys] == case['keys']


def test_step_plans_match_the_reference_bit_for_bit():
    '''Every piece of every shift: the five integers exactly, the coefficient to 1e-12.'''
    for record in load_json('plans.json'):
        cat = orc.CATEGORIES[record['cat']]
        q = tuple(record['qtotal'])
        for step in record['steps']:
            cod, dom = legs(cat, step['codomain']), legs(cat, step['domain'])
            for block in step['blocks']:
                key = (tuple(block['key'][0]), tuple(block['key'][1]), block['key'][2])
                if step['kind'] == 'x':
                    got = orc.exchange_regrouping(cat, cod, dom, key, q, step['arm'])
                else:
                    got = orc.bend_regrouping(cat, cod, dom, key, q, step['kind'] == 'down')
                assert len(got) == len(block['shifts'])
                for mine, theirs in zip(got, block['shifts']):
                    assert [list(mine[0][0]), list(mine[0][1]), mine[0][2]] == theirs[0]
                    assert [list(mine[1][0]), list(mine[1][1]), mine[1][2]] == theirs[1]
                    assert (mine[2], mine[3]) == (theirs[2], theirs[3])
                    assert [p[:5] for p in mine[4]] == [tuple(p[:5]) for p in theirs[4]]
                    coef = np.array([p[5] for p in mine[4]], complex)
                    ref = np.array([p[5] + 1j * p[6] for p in theirs[4]], complex)
                    assert np.abs(coef - ref).max(initial = 0) < VALUE_TOL






@pytest.mark.parametrize('index', range(len(load_json('cases.json'))))
def test_values_match_the_reference(index):
    case = load_json('cases.json')[index]
    name = case['inputs'][0]['name']
    catname = ('fibonacci' if name.startswith(('place6', 'place7', 'fibonacci')) else
               'su2' if name.startswith(('place0', 'place1', 'place2', 'place3', 'su2', 'outer', 'trace/')) else
               'no_symmetry' if name.startswith('place8') else 'u1')
    cat = orc.CATEGORIES[catname]
    dtype = np.complex128 if catname == 'fibonacci' else np.float64
    inputs = [tensor_of(e, cat, dtype) for e in case['inputs']]
    if case['op'] == 'place':
        out = orc.place(inputs[0], case['above'], case['below'])
    elif case['op'] == 'contract':
        out = orc.contract(inputs[0], inputs[1], case['left_legs'], case['right_legs'], tuple(case['charge']))
    else:
        out = orc.einsum(case['spec'], *inputs, outcharge = case.get('outcharge'))
    want = case_blocks(case['output'], case['output']['name'])
    assert [list(map(list, k[:2])) + [k[2]] for k in out.blocks] == case['output']['keys']
    for key, block in want.items():
        assert out.blocks[key].shape == block.shape
        assert relative_error(out.blocks[key], block) < VALUE_TOL, key
