'''
Generate the golden fixtures in this directory from the reference itself (Jumqyc/TenTorch compiled
from its own sources by `oracle/build_ref.py`, imported by `oracle/ref_import.py`).

Run from the repository root, where the reference checkout exists:

    TENTORCH_REFERENCE=<reference checkout> TENTORCH_DEVICE=cpu python tests/golden/make_golden.py

Every fixture is produced by the reference's own code path, on the CPU, in float64 (and complex128
for the Fibonacci category, whose R symbol is complex):

- `symbols.json`: SU(2) and Fibonacci F and R symbols (`FusionCategory.F_symbol/R_symbol`).
- `structure.json`: side layouts (trees and row offsets, `layout_of`), block keys (`block_keys`).
- `plans.json`: the reference's per-step regrouping plans (`exchange_regrouping`,
  `bend_regrouping`) for every block of every step of a set of `place` calls.
- `cases.npz` + `cases.json`: inputs and outputs of `place`, `contract` and `einsum` calls.
- `dmrg.json`: DMRG energies of the reference's float64 harness and exact diagonalisation.

Inputs are N(0, 1) float64 entries drawn in block-key order from `torch.Generator().manual_seed`;
complex inputs draw the real part and then the imaginary part of each block.
'''
import json
import math
import os
import sys

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
os.environ.setdefault('TENTORCH_DEVICE', 'cpu')

from oracle import engine as orc  # noqa: E402  (only for the chain step sequence and the sector rule)
from oracle.ref_import import reference  # noqa: E402

tt, dump = reference()
CATS = {'u1': tt.u1, 'su2': tt.su2, 'fibonacci': tt.fibonacci, 'no_symmetry': tt.no_symmetry}
CPU = torch.device('cpu')


def leg_spec(leg):
    return [[list(s), int(m)] for s, m in zip(leg.sectors, leg.multiplicities)]


def make_leg(cat, spec):
    return tt.Leg(CATS[cat], [tuple(s) for s, _ in spec], [m for _, m in spec])


def key_tuple(key):
    return [list(key.codomain), list(key.domain), int(key.copy)]


def filled(cat, cod, dom, q, dtype, gen):
    t = tt.Tensor(CATS[cat], [make_leg(cat, s) for s in cod], [make_leg(cat, s) for s in dom], tuple(q),
                  dtype = dtype, device = CPU)
    for key, block in t.to_tuple()[3].items():
        re = torch.randn(block.shape, dtype = torch.float64, generator = gen)
        if dtype == torch.complex128:
            im = torch.randn(block.shape, dtype = torch.float64, generator = gen)
            block.copy_(torch.complex(re, im))
        else:
            block.copy_(re)
    return t


ARRAYS = {}


def store(name, tensor):
    '''Record a tensor's structure in the case list and its blocks in the npz.'''
    cod, dom, q, blocks = tensor.to_tuple()
    entry = {'name': name, 'codomain': [leg_spec(l) for l in cod], 'domain': [leg_spec(l) for l in dom],
             'qtotal': list(q), 'keys': []}
    for i, (key, block) in enumerate(blocks.items()):
        entry['keys'].append(key_tuple(key))
        ARRAYS[f'{name}/{i}'] = block.numpy().copy()
    return entry


def symbols():
    out = {'su2': {'F': [], 'R': []}, 'fibonacci': {'F': [], 'R': []}}
    for name, cat, top in (('su2', tt.su2, 4), ('fibonacci', tt.fibonacci, 1)):
        labels = [(j,) for j in range(top + 1)]
        for a in labels:
            for b in labels:
                r = cat.R_symbol(a, b)
                out[name]['R'].append([a, b, r.real.tolist(), r.imag.tolist()])
                for c in labels:
                    for d in range(0, 3 * top + 1):
                        f = cat.F_symbol(a, b, c, (d,))
                        if f.numel():
                            out[name]['F'].append([a, b, c, [d], f.real.tolist(), f.imag.tolist()])
    return out


SU2_LEG = [[[j], 1 + (j % 2)] for j in range(0, 4)]
U1_LEG = [[[q], m] for q, m in ((-2, 1), (0, 2), (2, 1))]
U1_PHYS = [[[-1], 1], [[1], 1]]
FIB_LEG = [[[0], 2], [[1], 2]]

STRUCTURE_CASES = [
    ('su2', [SU2_LEG, SU2_LEG], [0]), ('su2', [SU2_LEG, SU2_LEG, SU2_LEG], [2]),
    ('su2', [SU2_LEG, SU2_LEG, SU2_LEG], [1]), ('u1', [U1_LEG, U1_PHYS, U1_LEG], [1]),
    ('fibonacci', [FIB_LEG, FIB_LEG, FIB_LEG], [1]), ('fibonacci', [FIB_LEG, FIB_LEG], [0]), ('su2', [], [0]),
]

# (category, codomain, domain, qtotal, above, below)
PLACE_CASES = [
    ('su2', [SU2_LEG, SU2_LEG], [SU2_LEG, SU2_LEG], [0], [1, 0], [2, 3]),
    ('su2', [SU2_LEG, SU2_LEG], [SU2_LEG, SU2_LEG], [0], [0, 1, 3], [2]),
    ('su2', [SU2_LEG, SU2_LEG], [SU2_LEG, SU2_LEG], [0], [0], [3, 1, 2]),
    ('su2', [SU2_LEG, SU2_LEG, SU2_LEG], [SU2_LEG], [1], [2, 3], [1, 0]),
    ('u1', [U1_LEG, U1_PHYS], [U1_PHYS, U1_LEG], [0], [3, 0], [2, 1]),
    ('u1', [U1_LEG, U1_PHYS, U1_PHYS], [U1_LEG], [0], [1], [3, 2, 0]),
    ('fibonacci', [FIB_LEG, FIB_LEG], [FIB_LEG, FIB_LEG], [0], [1, 0], [3, 2]),
    ('fibonacci', [FIB_LEG, FIB_LEG], [FIB_LEG], [1], [2, 0], [1]),
    ('no_symmetry', [[[[0], 2]], [[[0], 3]]], [[[[0], 2]]], [0], [2, 1], [0]),
]


def structure():
    out = {'layouts': [], 'keys': []}
    for cat, legs, root in STRUCTURE_CASES:
        trees, offsets = dump.side_layout(cat, legs, root)
        out['layouts'].append({'cat': cat, 'legs': legs, 'root': root, 'offsets': list(offsets),
                               'trees': [[[list(s) for s in t[0]], [list(s) for s in t[1]], list(t[2]), list(t[3])]
                                         for t in trees]})
    for cat, cod, dom, q, _, _ in PLACE_CASES:
        keys = dump.block_keys(cat, cod, dom, q)
        out['keys'].append({'cat': cat, 'codomain': cod, 'domain': dom, 'qtotal': q,
                            'keys': [[list(k[0]), list(k[1]), k[2]] for k in keys]})
    return out


def plans():
    out = []
    for cat, cod, dom, q, above, below in PLACE_CASES:
        ocat = orc.CATEGORIES[cat]
        ocod = [orc.Leg(ocat, [tuple(s) for s, _ in l], [m for _, m in l]) for l in cod]
        odom = [orc.Leg(ocat, [tuple(s) for s, _ in l], [m for _, m in l]) for l in dom]
        steps = orc.chain_steps(ocod, odom, above, below)
        cur_c, cur_d = cod, dom
        record = {'cat': cat, 'codomain': cod, 'domain': dom, 'qtotal': q, 'above': above, 'below': below,
                  'steps': []}
        for kind, arm, new_c, new_d in steps:
            keys = dump.block_keys(cat, cur_c, cur_d, q)
            step = {'kind': kind, 'arm': arm, 'codomain': cur_c, 'domain': cur_d, 'blocks': []}
            for k in keys:
                shifts = dump.step_plan(cat, cur_c, cur_d, list(k[0]), list(k[1]), k[2], q,
                                        0 if kind == 'x' else 1, arm if kind == 'x' else (1 if kind == 'down' else 0))
                step['blocks'].append({'key': [list(k[0]), list(k[1]), k[2]], 'shifts': [
                    [[list(s[0][0]), list(s[0][1]), s[0][2]], [list(s[1][0]), list(s[1][1]), s[1][2]], s[2], s[3],
                     [list(p) for p in s[4]]] for s in shifts]})
            record['steps'].append(step)
            cur_c = [[[list(s), m] for s, m in zip(l.sectors, l.multiplicities)] for l in new_c]
            cur_d = [[[list(s), m] for s, m in zip(l.sectors, l.multiplicities)] for l in new_d]
        out.append(record)
    return out


def cases():
    gen = torch.Generator().manual_seed(1234)
    out = []
    f64, c128 = torch.float64, torch.complex128
    # place
    for i, (cat, cod, dom, q, above, below) in enumerate(PLACE_CASES):
        dtype = c128 if cat == 'fibonacci' else f64
        t = filled(cat, cod, dom, q, dtype, gen)
        out.append({'op': 'place', 'above': above, 'below': below, 'inputs': [store(f'place{i}/in', t)],
                    'output': store(f'place{i}/out', t.place(above, below))})
    # einsum: the two-site matvec at chi = 32 (float64), head and tail builds included
    qs, deg = orc.degeneracies(32)
    bond = [[[2 * q], m] for q, m in zip(qs, deg)]
    w = [[[0], 3], [[2], 1], [[-2], 1]]
    mpo = tt.heisenberg(tt.u1, 4)
    site = mpo.tensors[1]
    site64 = tt.Tensor(tt.u1, list(site.codomain), list(site.domain), site.qtotal, dtype = f64, device = CPU)
    for key, block in site64.to_tuple()[3].items():
        block.copy_(site.to_tuple()[3][key].real)
    left = filled('u1', [bond, w], [bond], [0], f64, gen)
    right = filled('u1', [bond, w], [bond], [0], f64, gen)
    theta = filled('u1', [bond, U1_PHYS], [U1_PHYS, bond], [0], f64, gen)
    head = tt.einsum('EIa,IPqj->EPaqj', left, site64)
    tail = tt.einsum('JRsk,Fkb->JRSFb', site64, right)
    image = tt.einsum('EPaqj,JRSFb,AQsb->EPrf', head, tail, theta)
    out.append({'op': 'einsum', 'spec': 'EIa,IPqj->EPaqj', 'inputs': [store('mv/L', left), store('mv/W', site64)],
                'output': store('mv/head', head)})
    out.append({'op': 'einsum', 'spec': 'JRsk,Fkb->JRSFb', 'inputs': [store('mv/W2', site64), store('mv/R', right)],
                'output': store('mv/tail', tail)})
    out.append({'op': 'einsum', 'spec': 'EPaqj,JRSFb,AQsb->EPrf',
                'inputs': [store('mv/head2', head), store('mv/tail2', tail), store('mv/theta', theta)],
                'output': store('mv/image', image)})
    # einsum with F and R: SU(2) and Fibonacci, the exchange-forcing contraction
    for cat, leg, dtype in (('su2', SU2_LEG, f64), ('fibonacci', FIB_LEG, c128)):
        a = filled(cat, [leg, leg], [leg, leg], [0], dtype, gen)
        b = filled(cat, [leg, leg], [leg, leg], [0], dtype, gen)
        r = tt.einsum('ABcd,DCef->ABef', a, b)
        out.append({'op': 'einsum', 'spec': 'ABcd,DCef->ABef', 'inputs': [store(f'{cat}x/a', a), store(f'{cat}x/b', b)],
                    'output': store(f'{cat}x/out', r)})
    # a charged contraction, an outer product and traces
    a = filled('u1', [U1_LEG, U1_PHYS], [U1_LEG], [1], f64, gen)
    b = filled('u1', [U1_LEG], [U1_PHYS, U1_LEG], [-1], f64, gen)
    r = tt.contract(a, b, [2], [0], (0,))
    out.append({'op': 'contract', 'left_legs': [2], 'right_legs': [0], 'charge': [0],
                'inputs': [store('ch/a', a), store('ch/b', b)], 'output': store('ch/out', r)})
    a = filled('su2', [SU2_LEG], [SU2_LEG], [0], f64, gen)
    b = filled('su2', [SU2_LEG, SU2_LEG], [SU2_LEG], [1], f64, gen)
    r = tt.einsum('Ab,CDe->ACDbe', a, b, outcharge = (1,))
    out.append({'op': 'einsum', 'spec': 'Ab,CDe->ACDbe', 'outcharge': [1],
                'inputs': [store('outer/a', a), store('outer/b', b)], 'output': store('outer/out', r)})
    t = filled('su2', [SU2_LEG, SU2_LEG], [SU2_LEG, SU2_LEG], [0], f64, gen)
    r = tt.einsum('ABcb->Ac', t)
    out.append({'op': 'einsum', 'spec': 'ABcb->Ac', 'inputs': [store('trace/t', t)], 'output': store('trace/out', r)})
    t = filled('u1', [U1_LEG, U1_PHYS], [U1_PHYS, U1_LEG], [0], f64, gen)
    r = tt.einsum('ABba->', t)
    out.append({'op': 'einsum', 'spec': 'ABba->', 'inputs': [store('trace2/t', t)], 'output': store('trace2/out', r)})
    # a four-operand environment update (tentorch/algorithms/dmrg.py:65)
    env = filled('u1', [bond, w], [bond], [0], f64, gen)
    mps = filled('u1', [bond, U1_PHYS], [bond], [0], f64, gen)
    r = tt.einsum('EIa,Feq,aPb,IqPj->FJb', env, mps.conj(), mps, site64)
    out.append({'op': 'einsum', 'spec': 'EIa,Feq,aPb,IqPj->FJb',
                'inputs': [store('env/L', env), store('env/bra', mps.conj()), store('env/ket', mps), store('env/W', site64)],
                'output': store('env/out', r)})
    return out


def float64_harness():
    '''Patch the reference's DMRG to run in float64: its random MPS draws float64 blocks in key order
    from a seeded generator, its identities and MPO blocks are cast to float64 (the reference builds
    complex128 by default).  Returns the patched DMRG module and the exact-diagonalisation helper.'''
    import tentorch.networks.mps as mps_module
    dmrg_module = sys.modules['tentorch.algorithms.dmrg']
    import importlib.util
    from oracle.build_ref import REFERENCE
    spec = importlib.util.spec_from_file_location('reference_exact', os.path.join(REFERENCE, 'tests', 'exact.py'))
    exact = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(exact)

    def exact_energy_of(length):
        return exact.exact_energy(tt.Model(length, cat = tt.u1))
    original_random = mps_module.MPS.random.__func__
    original_identity = mps_module._identity

    def random64(cls, cat, physical, length, sector = None, seed = 0, multiplets = 1):
        charge = cat.trivial() if sector is None else sector
        left = [sys.modules['tentorch._ext'].reachable_charges(cat, [physical] * at) for at in range(length + 1)]
        tail = [sys.modules['tentorch._ext'].reachable_charges(cat, [physical] * (length - at)) for at in range(length + 1)]
        bonds = []
        for at in range(length + 1):
            sectors = [b for b in left[at] if any(cat.can_fuse_to(b, r, charge) for r in tail[at])]
            bonds.append(tt.Leg(cat, sectors, [multiplets] * len(sectors)))
        bonds[0] = bonds[-1] = tt.Leg(cat, [charge], (1,))
        gen = torch.Generator().manual_seed(seed)
        tensors = []
        for at in range(length):
            t = tt.Tensor(cat, [bonds[at], physical], [bonds[at + 1]], charge, dtype = torch.float64, device = CPU)
            for _, block in t.to_tuple()[3].items():
                block.copy_(torch.randn(block.shape, dtype = torch.float64, generator = gen))
            tensors.append(t)
        return cls(tensors, physical)

    def identity64(cat, bond, middle = None):
        src = original_identity(cat, bond, middle)
        out = tt.Tensor(cat, list(src.codomain), list(src.domain), src.qtotal, dtype = torch.float64, device = CPU)
        for key, block in out.to_tuple()[3].items():
            block.copy_(src.to_tuple()[3][key].real)
        return out

    mps_module.MPS.random = classmethod(random64)
    mps_module._identity = identity64
    dmrg_module._identity = identity64
    heis = sys.modules['tentorch.models.heisenberg']
    original_heisenberg = heis.heisenberg

    def heisenberg64(cat, length, coupling = 1.0):
        mpo = original_heisenberg(cat, length, coupling)
        sites = []
        for s in mpo.tensors:
            o = tt.Tensor(cat, list(s.codomain), list(s.domain), s.qtotal, dtype = torch.float64, device = CPU)
            for key, block in o.to_tuple()[3].items():
                block.copy_(s.to_tuple()[3][key].real)
            sites.append(o)
        mpo.tensors = sites
        return mpo
    dmrg_module.heisenberg = heisenberg64
    return dmrg_module, exact_energy_of


def dmrg_energies():
    '''The reference's float64 DMRG at small lengths, against exact diagonalisation, and config 1.'''
    dmrg_module, exact_energy_of = float64_harness()
    out = {'exact': {}, 'small': {}, 'config1': {}}
    for length in (4, 6, 8):
        model = tt.Model(length, cat = tt.u1)
        out['exact'][str(length)] = exact_energy_of(length)
        driver = dmrg_module.DMRG(model, max_bond_dim = 64, n_iter = 5)
        energies = [driver.sweep()[0] for _ in range(4)]
        out['small'][str(length)] = {'sweeps': energies, 'energy': driver.energy().real}
    driver = dmrg_module.DMRG(tt.Model(16, cat = tt.u1), max_bond_dim = 32, n_iter = 5, seed = 0)
    sweeps = []
    for _ in range(3):
        energy, lost = driver.sweep()
        sweeps.append({'energy': energy, 'discarded': lost, 'bond': driver.state.bond_dims})
    out['config1'] = {'length': 16, 'max_bond_dim': 32, 'n_iter': 5, 'seed': 0, 'sweeps': sweeps,
                      'exact': exact_energy_of(16)}
    return out


def dmrg_chi256(sweeps = 6):
    '''The reference's float64 DMRG of the U(1) Heisenberg chain at L = 64, max bond 256, n_iter = 10,
    seed 0: per sweep its energy (the last window's Ritz value), the largest discarded weight and the
    bond dimensions, and after the last sweep the expectation `DMRG.energy()`.  The first four sweeps
    bring every bond to 256; the later ones are the steady state.'''
    dmrg_module, _ = float64_harness()
    driver = dmrg_module.DMRG(tt.Model(64, cat = tt.u1), max_bond_dim = 256, n_iter = 10, seed = 0)
    out = []
    for _ in range(sweeps):
        energy, lost = driver.sweep()
        out.append({'energy': energy, 'discarded': lost, 'bond': driver.state.bond_dims})
        print('sweep', len(out), energy, lost, max(driver.state.bond_dims), flush = True)
    return {'length': 64, 'max_bond_dim': 256, 'n_iter': 10, 'seed': 0, 'svd_tol': driver.svd_tol,
            'sweeps': out, 'energy': driver.energy().real}


if __name__ == '__main__':
    sys.path.insert(0, HERE)
    if sys.argv[1:] == ['dmrg_chi256']:
        # about a minute and a half per sweep on eight cores: run on its own, not by default
        json.dump(dmrg_chi256(), open(os.path.join(HERE, 'dmrg_chi256.json'), 'w'), indent = 1)
        raise SystemExit(0)
    if sys.argv[1:] == ['dmrg']:
        # the reference's buffer pool is keyed by shape and not by dtype (tentorch/tensors/cache.cpp:
        # 120-130), so the float64 DMRG runs in a process that never held a complex128 tensor
        json.dump(dmrg_energies(), open(os.path.join(HERE, 'dmrg.json'), 'w'), indent = 1)
        raise SystemExit(0)
    import subprocess
    subprocess.run([sys.executable, os.path.abspath(__file__), 'dmrg'], check = True)
    json.dump(symbols(), open(os.path.join(HERE, 'symbols.json'), 'w'))
    json.dump(structure(), open(os.path.join(HERE, 'structure.json'), 'w'))
    json.dump(plans(), open(os.path.join(HERE, 'plans.json'), 'w'))
    case_list = cases()
    json.dump(case_list, open(os.path.join(HERE, 'cases.json'), 'w'))
    np.savez_compressed(os.path.join(HERE, 'cases.npz'), **ARRAYS)
    for name in ('symbols.json', 'structure.json', 'plans.json', 'cases.json', 'cases.npz', 'dmrg.json'):
        print(name, os.path.getsize(os.path.join(HERE, name)))
