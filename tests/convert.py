'''Moving tensors between the oracle (numpy blocks) and the product (one device arena).'''
import numpy as np
import torch

import tentorch_gb300 as tg
from golden_io import case_blocks
from oracle import engine as orc

PRODUCT_CATS = {'u1': tg.u1, 'su2': tg.su2, 'fibonacci': tg.fibonacci, 'no_symmetry': tg.no_symmetry}
ORACLE_OF = {id(tg.u1): orc.u1, id(tg.su2): orc.su2, id(tg.fibonacci): orc.fibonacci,
             id(tg.no_symmetry): orc.no_symmetry}


def product_leg(cat, leg):
    return tg.Leg(cat, list(leg.sectors), list(leg.multiplicities))


def to_product(t, cat, device = 'cuda'):
    '''An oracle tensor as a product tensor on `device`.'''
    dtype = torch.complex128 if t.dtype == np.complex128 else torch.float64
    out = tg.Tensor(cat, [product_leg(cat, l) for l in t.codomain], [product_leg(cat, l) for l in t.domain],
                    t.qtotal, dtype = dtype, device = device)
    for key, block in t.blocks.items():
        out.block(key[0], key[1], key[2]).copy_(torch.from_numpy(np.ascontiguousarray(block)))
    return out


def to_oracle(t):
    '''A product tensor as an oracle tensor (host numpy blocks).'''
    ocat = ORACLE_OF[id(t.cat)]
    dtype = np.complex128 if t.dtype == torch.complex128 else np.float64
    out = orc.Tensor(ocat, [orc.Leg(ocat, l.sectors, l.multiplicities) for l in t.codomain],
                     [orc.Leg(ocat, l.sectors, l.multiplicities) for l in t.domain], t.qtotal, dtype)
    for key, block in t.to_tuple()[3].items():
        out.blocks[(key.codomain, key.domain, key.copy)][...] = block.cpu().numpy()
    return out


def fixture_tensor(entry, cat, dtype, device = 'cuda'):
    '''A stored golden tensor as a product tensor.'''
    legs = lambda specs: [tg.Leg(cat, [tuple(s) for s, _ in spec], [m for _, m in spec]) for spec in specs]
    t = tg.Tensor(cat, legs(entry['codomain']), legs(entry['domain']), tuple(entry['qtotal']), dtype = dtype,
                  device = device)
    for key, block in case_blocks(entry, entry['name']).items():
        t.block(*key).copy_(torch.from_numpy(block))
    return t


def max_relative(product, reference_blocks):
    '''max |a - b| / max |b| over all blocks, and whether the key sets and shapes agree.'''
    mine = {(k.codomain, k.domain, k.copy): v.cpu().numpy() for k, v in product.to_tuple()[3].items()}
    if set(mine) != set(reference_blocks):
        return float('inf')
    scale = max((np.abs(b).max(initial = 0.0) for b in reference_blocks.values()), default = 0.0) or 1.0
    worst = 0.0
    for key, block in reference_blocks.items():
        if mine[key].shape != block.shape:
            return float('inf')
        worst = max(worst, float(np.abs(mine[key] - block).max(initial = 0.0)))
    return worst / scale


def case_category(name):
    if name.startswith(('place6', 'place7', 'fibonacci')):
        return 'fibonacci'
    if name.startswith(('place0', 'place1', 'place2', 'place3', 'su2', 'outer', 'trace/')):
        return 'su2'
    if name.startswith('place8'):
        return 'no_symmetry'
    return 'u1'
