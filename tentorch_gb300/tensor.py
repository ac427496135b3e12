'''
The block-sparse tensor with the Python surface of the reference's `tentorch.Tensor`
(tentorch/_ext/bindings.cpp:235-327, tentorch/tensors/tensor.h:43-216).

A tensor is a space (its category, legs and charge, interned by the engine) and ONE arena of
device memory holding every block back to back, row major, each block starting on a 16-byte
boundary; `to_tuple()` hands out views of that arena, so the blocks share storage with the tensor
as they do in the reference.  Arena-wide arithmetic (`+=`, `*=`, the scalar products) is one kernel
per call instead of one per block.
'''
from __future__ import annotations

import ctypes
import functools
from typing import Optional

import torch

from tentorch_gb300._lib import check, i32, i64, ints32, lib
from tentorch_gb300.symmetry import FusionCategory, Leg, _label, _render, default_device


class BlockKey(tuple):
    '''(codomain root, domain root, copy) of one block (tentorch/tensors/layout.h:64-79).'''
    __slots__ = ()

    def __new__(cls, codomain, domain, copy = 0):
        return super().__new__(cls, (tuple(codomain), tuple(domain), int(copy)))

    codomain = property(lambda self: self[0])
    domain = property(lambda self: self[1])
    copy = property(lambda self: self[2])

    def __repr__(self) -> str:
        return f'BlockKey({_render(self[0])}, {_render(self[1])}, {self[2]})'


class Space:
    '''The interned shape of a tensor: legs, charge, block keys, shapes and arena offsets.'''
    __slots__ = ('id', 'cat', 'codomain', 'domain', 'qtotal', 'keys', 'shapes', 'offsets', 'size', 'index')

    @staticmethod
    @functools.lru_cache(maxsize = None)
    def of_ids(cat: FusionCategory, codomain_ids: tuple, domain_ids: tuple, qtotal: int) -> 'Space':
        c, nc = ints32(codomain_ids)
        d, nd = ints32(domain_ids)
        out = i32()
        check(lib.tt_space(cat._id, nc, c, nd, d, qtotal, ctypes.byref(out)))
        return Space._load(cat, out.value)

    @staticmethod
    def of(cat: FusionCategory, codomain, domain, qtotal) -> 'Space':
        for leg in list(codomain) + list(domain):
            if leg.cat is not cat:
                raise ValueError('a leg is over a different category')
        return Space.of_ids(cat, tuple(l._id for l in codomain), tuple(l._id for l in domain), _label(qtotal))

    @staticmethod
    @functools.lru_cache(maxsize = None)
    def _load(cat: FusionCategory, space_id: int) -> 'Space':
        s = Space()
        s.id, s.cat = space_id, cat
        nblocks, size = i64(), i64()
        check(lib.tt_space_size(space_id, ctypes.byref(nblocks), ctypes.byref(size)))
        n = nblocks.value
        keys, shapes = (i64 * max(3 * n, 1))(), (i64 * max(3 * n, 1))()
        check(lib.tt_space_blocks(space_id, n, keys, shapes))
        legs, ncod, ndom, q = (i32 * 64)(), i32(), i32(), i64()
        check(lib.tt_space_legs(space_id, 64, legs, ctypes.byref(ncod), ctypes.byref(ndom), ctypes.byref(q)))
        all_legs = [Leg._of(cat, legs[i]) for i in range(ncod.value + ndom.value)]
        s.codomain, s.domain = all_legs[:ncod.value], all_legs[ncod.value:]
        s.qtotal = (q.value,)
        s.keys = [BlockKey((keys[3 * i],), (keys[3 * i + 1],), keys[3 * i + 2]) for i in range(n)]
        s.shapes = [(shapes[3 * i], shapes[3 * i + 1]) for i in range(n)]
        s.offsets = [shapes[3 * i + 2] for i in range(n)]
        s.size = size.value
        s.index = {k: i for i, k in enumerate(s.keys)}
        return s


def _require_device(device):
    device = torch.device(device)
    if device.type == 'cuda' and device.index is None:
        device = torch.device('cuda', torch.cuda.current_device())
    return device


class Tensor:
    '''A map between two graded spaces, one dense matrix per block key
    (tentorch/tensors/tensor.h:43-216).  The scalar type defaults to the category's (complex128),
    the device to CUDA when one is visible.'''
    __slots__ = ('_space', '_data', '__weakref__')

    def __init__(self, cat: FusionCategory, codomain, domain, qtotal, dtype: Optional[torch.dtype] = None,
                 device = None):
        if cat is None:
            raise ValueError('a tensor needs a category')
        self._space = Space.of(cat, list(codomain), list(domain), qtotal)
        dtype = cat.dtype if dtype is None else dtype
        if dtype not in (torch.float64, torch.complex128):
            raise ValueError(f'the engine holds float64 or complex128 blocks, not {dtype}')
        device = default_device() if device is None else _require_device(device)
        self._data = torch.zeros(self._space.size, dtype = dtype, device = device)

    @classmethod
    def _wrap(cls, space: Space, data: torch.Tensor) -> 'Tensor':
        t = cls.__new__(cls)
        t._space, t._data = space, data
        return t

    # -- the reference's read-only surface ------------------------------------------------------
    cat = property(lambda self: self._space.cat)
    codomain = property(lambda self: list(self._space.codomain))
    domain = property(lambda self: list(self._space.domain))
    qtotal = property(lambda self: self._space.qtotal)
    dtype = property(lambda self: self._data.dtype)
    device = property(lambda self: self._data.device)

    @property
    def data(self) -> torch.Tensor:
        '''The arena: every block, back to back (padding entries stay zero).'''
        return self._data

    def nlegs(self) -> int:
        return len(self._space.codomain) + len(self._space.domain)

    def legs(self) -> list:
        return self.codomain + self.domain

    def nblocks(self) -> int:
        return len(self._space.keys)

    def keys(self) -> list:
        return list(self._space.keys)

    def block(self, codomain_root, domain_root, copy: int = 0) -> torch.Tensor:
        key = BlockKey(codomain_root, domain_root, copy)
        at = self._space.index.get(key)
        if at is None:
            raise IndexError(f'the tensor has no block at {_render(key[0])} x {_render(key[1])} of copy {copy}')
        return self._view(at)

    def _view(self, at: int) -> torch.Tensor:
        rows, cols = self._space.shapes[at]
        off = self._space.offsets[at]
        return self._data[off:off + rows * cols].view(rows, cols)

    def to_tuple(self):
        '''(codomain, domain, qtotal, {BlockKey: block}) with blocks sharing storage
        (tentorch/_ext/bindings.cpp:311-323).'''
        return (self.codomain, self.domain, self.qtotal,
                {k: self._view(i) for i, k in enumerate(self._space.keys)})

    @staticmethod
    def from_tuple(cat, codomain, domain, qtotal, blocks = None) -> 'Tensor':
        '''tentorch/_ext/bindings.cpp:131-152'''
        out = Tensor(cat, codomain, domain, qtotal)
        if blocks is None:
            return out
        for key, block in blocks.items():
            key = BlockKey(*key) if not isinstance(key, BlockKey) else key
            mine = out.block(key.codomain, key.domain, key.copy)
            if tuple(block.shape) != tuple(mine.shape):
                raise ValueError(f'the block at {key!r} has shape {block.shape[0]}x{block.shape[1]}, '
                                 f'not {mine.shape[0]}x{mine.shape[1]}')
            mine.copy_(block.to(out.dtype).to(out.device))
        return out

    @staticmethod
    def random(cat, codomain, domain, qtotal) -> 'Tensor':
        '''Standard normal blocks drawn in key order (tentorch/_ext/bindings.cpp:156-164).'''
        out = Tensor(cat, codomain, domain, qtotal)
        for i in range(out.nblocks()):
            out._view(i).normal_()
        return out

    def to(self, device = None, dtype = None) -> 'Tensor':
        data = self._data
        if dtype is not None and dtype != data.dtype:
            if dtype not in (torch.float64, torch.complex128):
                raise ValueError(f'the engine holds float64 or complex128 blocks, not {dtype}')
            data = data.real.to(dtype) if (data.is_complex() and not dtype.is_complex) else data.to(dtype)
        if device is not None:
            data = data.to(_require_device(device))
        return Tensor._wrap(self._space, data if data is not self._data else data.clone())

    def clone(self) -> 'Tensor':
        return Tensor._wrap(self._space, self._data.clone())

    def conj(self) -> 'Tensor':
        '''tentorch/tensors/tensor.cpp:99-107: the bra, blocks conjugate-transposed (one compiled
        pass on the GPU; block by block for a host container).'''
        if self.device.type == 'cuda':
            from tentorch_gb300.linalg import conj
            return conj(self)
        cat = self.cat
        out = Tensor(cat, self.domain, self.codomain, cat.dual(self.qtotal), self.dtype, self.device)
        for i, (r, s, c) in enumerate(self._space.keys):
            out.block(s, r, c).copy_(self._view(i).conj().transpose(0, 1))
        return out

    def place(self, above, below = None) -> 'Tensor':
        '''tentorch/tensors/place.cpp:183-247, compiled once per shape and run on the GPU.'''
        from tentorch_gb300.linalg import place
        return place(self, above, below)

    # -- arithmetic (tentorch/tensors/tensor.cpp:131-180) ----------------------------------------
    def _same_space(self, other: 'Tensor', what: str) -> None:
        if not isinstance(other, Tensor) or other._space is not self._space:
            raise ValueError(f'a {what} needs both tensors with the same legs and the same charge')

    def __iadd__(self, other: 'Tensor') -> 'Tensor':
        self._same_space(other, 'sum')
        self._data.add_(other._data)
        return self

    def __isub__(self, other: 'Tensor') -> 'Tensor':
        self._same_space(other, 'difference')
        self._data.sub_(other._data)
        return self

    def __imul__(self, scalar) -> 'Tensor':
        if isinstance(scalar, complex) and scalar.imag != 0 and not self._data.is_complex():
            raise ValueError(f'a block of real entries cannot take the complex factor {scalar}')
        if isinstance(scalar, complex) and scalar.imag == 0:
            scalar = scalar.real
        self._data.mul_(scalar)
        return self

    def __itruediv__(self, scalar) -> 'Tensor':
        if scalar == 0:
            raise ValueError('a tensor cannot be divided by zero')
        self._data.div_(scalar)
        return self

    def __mul__(self, scalar) -> 'Tensor':
        out = self.clone()
        out *= scalar
        return out

    __rmul__ = __mul__

    def __repr__(self) -> str:
        blocks = ' '.join(f'{_render(k[0])} x {_render(k[1])} {r}x{c}' for k, (r, c) in
                          zip(self._space.keys, self._space.shapes))
        return f'Tensor({self.nlegs()} legs, q = {_render(self.qtotal)}, {self.nblocks()} blocks: {blocks})'


def block_keys(category, codomain, domain, qtotal) -> list:
    '''tentorch/tensors/layout.cpp:34-47, in the order the tensor holds them.'''
    return list(Space.of(category, list(codomain), list(domain), qtotal).keys)


def codomain_legs(tensor: Tensor) -> list:
    return list(range(len(tensor.codomain)))


def domain_legs(tensor: Tensor) -> list:
    above = len(tensor.codomain)
    return list(range(above, above + len(tensor.domain)))
