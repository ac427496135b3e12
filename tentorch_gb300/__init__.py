'''
tentorch_gb300: a GB300-native (sm_103a) engine for TenTorch's block-sparse contraction path.

The public names mirror the reference package `tentorch` for that path: the categories, `Leg`,
`Tensor` (with `place`, `to_tuple`, `from_tuple`, `random`), `einsum`, `contract`, `inner`,
`norm`, `is_close`, the splittings, the Lanczos solver and the callers that drive the path (`MPS`,
`MPO`, `heisenberg`, `Model`, `DMRG`), so a caller of the reference switches
by changing the import.  The contraction runs on the GPU through the C ABI of
`libtentorch_gb300.so` (include/tentorch_gb300.h); there is no CPU path for it.
'''
from tentorch_gb300.symmetry import (AbelianGroup, FermionParity, FibonacciCategory, FusionCategory, FusionTree,
                                     Group, Leg, NoSymmetry, Outcome, Sector, SU2Symmetry, U1Symmetry, ZNSymmetry,
                                     default_device, fermion_parity, fibonacci, fusion_trees, no_symmetry,
                                     reachable_charges, su2, u1, validate, z_n)
from tentorch_gb300.tensor import BlockKey, Tensor, block_keys, codomain_legs, domain_legs
from tentorch_gb300.linalg import (contract, einsum, get_precision, inner, is_close, norm, place, precision, qr, rq,
                                   set_precision, svd, svdvals)
from tentorch_gb300.lanczos import lanczos
from tentorch_gb300.networks import DMRG, MPO, MPS, Model, dmrg, entered, heisenberg

__all__ = [
    'DMRG', 'MPO', 'MPS', 'Model', 'dmrg', 'entered', 'heisenberg', 'lanczos',
    'AbelianGroup', 'BlockKey', 'FermionParity', 'FibonacciCategory', 'FusionCategory', 'FusionTree', 'Group', 'Leg',
    'NoSymmetry', 'Outcome', 'SU2Symmetry', 'Sector', 'Tensor', 'U1Symmetry', 'ZNSymmetry', 'block_keys',
    'codomain_legs', 'contract', 'default_device', 'domain_legs', 'einsum', 'fermion_parity', 'fibonacci',
    'fusion_trees', 'get_precision', 'inner', 'is_close', 'no_symmetry', 'norm', 'place', 'precision', 'qr',
    'reachable_charges', 'rq', 'set_precision', 'su2', 'svd', 'svdvals', 'u1', 'validate', 'z_n',
]
