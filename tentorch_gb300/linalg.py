'''
The contraction path and the linear algebra over block-sparse tensors, with the Python surface of
the reference: `einsum(spec, *tensors, outcharge=None)`, `contract(left, right, left_legs,
right_legs, charge=None)`, `Tensor.place`, `inner`, `norm`, `is_close`, `svd`, `svdvals`, `qr`,
`rq` (tentorch/_ext/bindings.cpp:330-431).

`einsum`, `contract` and `place` compile a plan once per combination of operand spaces (the
engine caches it) and run it on the tensors' CUDA device, on the current torch stream, with no
host synchronisation.  An operand's "prepare" work (the leg moves that depend on it alone) is
cached against the operand's arena and its version counter, so a loop that applies the same
operator to changing vectors (the Lanczos matvec) recouples the operator once.

Block products run in FP64 by default; `precision(k)` switches them to split products on the
tensor cores with k bf16 slices per operand (see gemm_split.cu).
'''
from __future__ import annotations

import contextlib
import ctypes
import math
import weakref
from typing import Optional

import torch

from tentorch_gb300._lib import check, f64, i32, i64, ints32, ints64, lib, pointers, vp
from tentorch_gb300.symmetry import Leg, _label
from tentorch_gb300.tensor import BlockKey, Space, Tensor

_DTYPE = {torch.float64: 0, torch.complex128: 1}
_precision = 0
PER_BLOCK = -1  # the plain per-block FP64 form: one cuBLAS call per block pair


def set_precision(slices: int) -> None:
    '''0: FP64 block products in the grouped kernels; k in 1..8: split products with k bf16 slices
    per operand; PER_BLOCK (-1): the plain per-block FP64 form, one cuBLAS call per block pair, as
    the reference issues its block products on a CUDA device (tentorch/linalg/graded/contract.cpp:148-163).'''
    global _precision
    if not PER_BLOCK <= int(slices) <= 8:
        raise ValueError(f'precision is 0 (FP64), 1..8 slices or -1 (per-block FP64), not {slices}')
    _precision = int(slices)


def get_precision() -> int:
    return _precision


@contextlib.contextmanager
def precision(slices: int):
    '''Run the block products inside the block with `slices` bf16 slices (0: FP64).'''
    old = _precision
    set_precision(slices)
    try:
        yield
    finally:
        set_precision(old)


class Plan:
    '''A compiled program: its output space, workspace and the size of each operand's prepared
    arena.  The engine owns the program; a wholesale clear of the plan caches frees it, and a Plan
    held across that clear compiles its program again on its next use (same key, same result).'''
    __slots__ = ('_handle', 'generation', 'key', 'build', 'cat', 'out_space', 'workspace', 'flops', 'moved', 'n_ops',
                 'prepared', 'sizes', '__weakref__')

    def __init__(self, handle, cat, key = None, build = None):
        self._handle, self.cat, self.key, self.build = handle, cat, key, build
        self.generation = _generation
        space, ws, flops, moved, ops = i32(), i64(), f64(), i64(), i32()
        check(lib.tt_plan_info(handle, ctypes.byref(space), ctypes.byref(ws), ctypes.byref(flops), ctypes.byref(moved),
                               ctypes.byref(ops)))
        self.out_space = Space._load(cat, space.value)
        self.workspace, self.flops, self.moved, self.n_ops = ws.value, flops.value, moved.value, ops.value
        self.prepared = []
        self.sizes = {}

    @property
    def handle(self):
        if self.generation != _generation:
            if self.build is None:
                raise RuntimeError('this plan was freed by clear_plans()')
            fresh = _plan(self.key, self.build, self.cat)
            self._handle, self.generation = fresh._handle, fresh.generation
        return self._handle

    def describe(self) -> str:
        '''The plan's operations and GEMM block shapes, as text.'''
        n = i64()
        check(lib.tt_plan_describe(self.handle, 0, None, ctypes.byref(n)))
        buf = ctypes.create_string_buffer(n.value + 1)
        check(lib.tt_plan_describe(self.handle, n.value + 1, buf, ctypes.byref(n)))
        return buf.value.decode()

    def prepared_size(self, operand: int) -> int:
        size = self.sizes.get(operand)
        if size is None:
            n = i64()
            check(lib.tt_plan_prepared_size(self.handle, operand, ctypes.byref(n)))
            size = self.sizes[operand] = n.value
        return size


_plans = {}
# compiled plans kept before a wholesale clear (the reference clears its plan caches wholesale at a
# budget, tentorch/tensors/cache.cpp:203-217): DMRG compiles new shapes at every window, so without
# a bound the caches would grow with the length of the run
_PLAN_BUDGET = 4096
_generation = 0
# (plan handle, operand) -> (weakref to the operand arena, its version, the prepared arena or None
# when the operand has been seen once and not prepared yet)
_prepared = {}
# (device index, stream, dtype) -> a workspace arena that grows to the largest plan run on it; the
# ops of one stream run in order, so consecutive plans share it
_pools = {}
# workspaces replaced by larger ones after a capture (a captured graph may still address them)
_superseded = []
# set once a plan has run inside a CUDA graph capture: the graph holds the device addresses of its
# tables and workspace, so the automatic clear at the budget no longer runs
_captured = False


def clear_plans() -> None:
    '''Forget every compiled plan, here and in the engine (their device tables are freed): the next
    contraction of each shape compiles again.  Runs by itself when the cache reaches its budget
    (unless a CUDA graph captured plans of this process); by hand, for timing compilation.  A CUDA
    graph captured before a clear launches freed tables: capture it again after one.'''
    global _generation, _captured
    _generation += 1
    _captured = False
    _plans.clear()
    _prepared.clear()
    _pools.clear()
    _batch_pools.clear()
    _superseded.clear()
    check(lib.tt_plan_cache_clear())


def cached_plans() -> int:
    '''How many compiled plans the cache holds.'''
    return len(_plans)


def _note_capture() -> None:
    global _captured
    _captured = True


def _plan(key, build, cat) -> Plan:
    plan = _plans.get(key)
    if plan is None:
        if len(_plans) >= _PLAN_BUDGET and not _captured:
            clear_plans()
        handle = vp()
        check(build(ctypes.byref(handle)))
        plan = Plan(handle, cat, key, build)
        _plans[key] = plan
    return plan


def _uploaded(values, dtype, device) -> torch.Tensor:
    '''A small host table on the device without waiting for the stream's queued work: staged
    through page-locked memory (torch's host cache keeps the staging block until the copy is done),
    so the copy is queued like a kernel and the host returns at once.'''
    if not values:
        return torch.empty(0, dtype = dtype, device = device)
    return torch.tensor(values, dtype = dtype).pin_memory().to(device, non_blocking = True)


def _check_device(tensors) -> None:
    dtype, device = tensors[0].dtype, tensors[0].device
    for t in tensors:
        if t.dtype != dtype:
            raise ValueError('a contraction needs both tensors of one scalar type')
        if t.device != device:
            raise ValueError('a contraction needs every tensor on one device')
    if device.type != 'cuda':
        raise RuntimeError('tentorch_gb300 computes on a CUDA device; these tensors live on the host '
                           '(move them with .to("cuda"))')


def _workspace(plan: Plan, device, dtype, stream) -> Optional[torch.Tensor]:
    if plan.workspace <= 0:
        return None
    key = (device.index, stream, dtype)
    pool = _pools.get(key)
    if pool is None or pool.numel() < plan.workspace:
        if pool is not None and _captured:
            # a CUDA graph captured earlier may hold this pool's address: keep it allocated, so that
            # a replay never writes into memory the caching allocator has handed to another tensor
            _superseded.append(pool)
        # zero: the head of a workspace holds the GEMM tickets, which every execution leaves zero
        pool = _pools[key] = torch.zeros(max(plan.workspace, 1 << 16), dtype = dtype, device = device)
    return pool


def _prepared_arena(plan: Plan, operand: int, tensor: Tensor, ws, stream, force: bool = False) -> Optional[torch.Tensor]:
    """The operand's prepared arena when the same arena (same version) comes back to this plan: the
    first sighting runs the operand's phase inside the plan and only remembers the arena; the
    second prepares it once for every call after (the head and tail of a Lanczos window).  Entries
    are per arena, so windows that share a plan each keep theirs; an entry goes with its arena."""
    size = plan.prepared_size(operand)
    if size <= 0:
        return None
    data = tensor._data
    key = (plan.handle.value, operand, data.data_ptr())
    held = _prepared.get(key)
    seen = held is not None and held[0]() is data and held[1] == data._version
    if seen and held[2] is not None:
        return held[2]
    arena = None
    if force or seen:
        arena = torch.empty(size, dtype = data.dtype, device = data.device)
        check(lib.tt_plan_prepare(plan.handle, _DTYPE[data.dtype], operand, data.data_ptr(), arena.data_ptr(),
                                  ws.data_ptr() if ws is not None else None, stream))
    if held is None or held[0]() is not data:
        def forget(ref, key = key):
            entry = _prepared.get(key)
            if entry is not None and entry[0] is ref:
                del _prepared[key]
        ref = weakref.ref(data, forget)
    else:
        ref = held[0]
    _prepared[key] = (ref, data._version, arena)
    return arena


def _prepare_now(plan: Plan, operand: int, tensor: Tensor, ws, stream) -> Optional[torch.Tensor]:
    '''The operand prepared into a new arena, not cached (the form a CUDA graph captures).'''
    size = plan.prepared_size(operand)
    if size <= 0:
        return None
    data = tensor._data
    arena = torch.empty(size, dtype = data.dtype, device = data.device)
    check(lib.tt_plan_prepare(plan.handle, _DTYPE[data.dtype], operand, data.data_ptr(), arena.data_ptr(),
                              ws.data_ptr() if ws is not None else None, stream))
    return arena


def run(plan: Plan, tensors, out: Optional[Tensor] = None, reuse_prepared: bool = True) -> Tensor:
    """Execute a plan on the operands' device and return the output tensor."""
    _check_device(tensors)
    data0 = tensors[0]._data
    device = data0.device
    if out is None:
        out = Tensor._wrap(plan.out_space, torch.empty(plan.out_space.size, dtype = data0.dtype, device = device))
    stream = torch.cuda.current_stream(device).cuda_stream
    # a captured CUDA graph reads every operand from its own buffer at each replay, never a prepared copy
    if torch.cuda.is_current_stream_capturing():
        _note_capture()
        reuse_prepared = False
    ws = _workspace(plan, device, data0.dtype, stream)
    prepared = [(_prepared_arena(plan, i, t, ws, stream) if reuse_prepared else None) for i, t in enumerate(tensors)]
    inputs = pointers(t._data.data_ptr() for t in tensors)
    prep = pointers((p.data_ptr() if p is not None else None) for p in prepared)
    check(lib.tt_plan_execute(plan.handle, _DTYPE[data0.dtype], _precision, inputs, prep, out._data.data_ptr(),
                              ws.data_ptr() if ws is not None else None, stream))
    return out


def place(tensor: Tensor, above, below = None) -> Tensor:
    '''tentorch/tensors/place.cpp:183-247'''
    total = tensor.nlegs()
    above = [int(a) for a in above]
    if below is None:
        named = set(a for a in above if 0 <= a < total)
        below = [leg for leg in range(total) if leg not in named]
    below = [int(b) for b in below]
    plan = place_plan(tensor._space, above, below)
    if plan.n_ops == 0:
        return tensor
    return run(plan, [tensor], reuse_prepared = False)


def place_plan(space: Space, above, below) -> Plan:
    '''The compiled plan of `place` on a tensor of this space (legs already resolved).'''
    above, below = [int(x) for x in above], [int(x) for x in below]
    a, na = ints32(above)
    b, nb = ints32(below)
    return _plan(('place', space.id, tuple(above), tuple(below)),
                 lambda out: lib.tt_plan_place(space.id, na, a, nb, b, out), space.cat)


def conj(tensor: Tensor) -> Tensor:
    '''tentorch/tensors/tensor.cpp:99-107: the bra of a tensor, one compiled pass.'''
    return run(conj_plan(tensor._space), [tensor], reuse_prepared = False)


def conj_plan(space: Space) -> Plan:
    '''The compiled plan of `conj` on a tensor of this space.'''
    return _plan(('conj', space.id), lambda out: lib.tt_plan_conj(space.id, out), space.cat)


def contract(left: Tensor, right: Tensor, left_legs, right_legs, charge = None) -> Tensor:
    '''tentorch/linalg/graded/contract.cpp:117-175'''
    if left.cat is not right.cat:
        raise ValueError('a contraction needs both tensors over one category')
    if left.dtype != right.dtype:
        raise ValueError('a contraction needs both tensors of one scalar type')
    return run(contract_plan(left._space, right._space, left_legs, right_legs, charge), [left, right])


def contract_plan(left: Space, right: Space, left_legs, right_legs, charge = None) -> Plan:
    '''The compiled plan of `contract` on tensors of these spaces.'''
    left_legs, right_legs = [int(x) for x in left_legs], [int(x) for x in right_legs]
    has = charge is not None
    q = _label(charge) if has else 0
    la, n = ints32(left_legs)
    ra, m = ints32(right_legs)
    if n != m:
        raise ValueError(f'the two legs of a contraction must be given in pairs, got {n} and {m}')
    return _plan(('contract', left.id, right.id, tuple(left_legs), tuple(right_legs), has, q),
                 lambda out: lib.tt_plan_contract(left.id, right.id, n, la, ra, int(has), q, out), left.cat)


def einsum(spec: str, *tensors: Tensor, **options) -> Tensor:
    '''tentorch/linalg/graded/einsum.cpp:444-605 with the binding's keyword handling
    (tentorch/_ext/bindings.cpp:347-361): only `outcharge` is accepted.'''
    for name in options:
        if name != 'outcharge':
            raise ValueError(f"einsum does not take the keyword '{name}'")
    outcharge = options.get('outcharge')
    if not tensors:
        raise ValueError('an einsum needs at least one operand')
    cat = tensors[0].cat
    for t in tensors:
        if t.cat is not cat:
            raise ValueError('an einsum needs every operand over one category')
    return run(einsum_plan(spec, [t._space for t in tensors], outcharge), list(tensors))


# per (device, stream, dtype, window): the workspace of one window of a batch (a batch's windows run
# together, so each needs its own)
_batch_pools = {}
# launches of block products the last einsum_batch made (1 when its windows ran as one launch)
last_batch_launches = 0


def einsum_batch(spec: str, operand_lists, outcharge = None) -> list:
    '''`[einsum(spec, *ops) for ops in operand_lists]` as one call (tt_plan_execute_batch): in FP64
    the two-site matvecs of many windows (different bond dimensions allowed) run as ONE persistent
    launch with their work items dealt together over the SMs; in split precision, or for equations
    that are not a product chain, one window after another.  At most 64 windows per launch (longer
    lists are cut into launches of 64).  Operands are prepared per window as `einsum` prepares them;
    under a CUDA graph capture every operand is read from its buffer (a warm-up call outside the
    capture compiles the plans and deals the batch first).'''
    global last_batch_launches
    operand_lists = [list(ops) for ops in operand_lists]
    if len(operand_lists) > 64:
        return einsum_batch(spec, operand_lists[:64], outcharge) + einsum_batch(spec, operand_lists[64:], outcharge)
    if not operand_lists:
        return []
    first = operand_lists[0][0]
    device, dtype = first._data.device, first._data.dtype
    stream = torch.cuda.current_stream(device).cuda_stream
    # a captured CUDA graph reads every operand from its own buffer at each replay
    capturing = torch.cuda.is_current_stream_capturing()
    if capturing:
        _note_capture()
    handles, outs, keep, inputs, prepared, workspaces = [], [], [], [], [], []
    for w, ops in enumerate(operand_lists):
        _check_device(ops)
        plan = plan_of(spec, *ops, outcharge = outcharge)
        key = (device.index, stream, dtype, w)
        pool = _batch_pools.get(key)
        if pool is None or pool.numel() < plan.workspace:
            if pool is not None and _captured:
                _superseded.append(pool)
            pool = _batch_pools[key] = torch.zeros(max(plan.workspace, 1 << 16), dtype = dtype, device = device)
        prep = [None if capturing else _prepared_arena(plan, i, t, pool, stream) for i, t in enumerate(ops)]
        out = Tensor._wrap(plan.out_space, torch.empty(plan.out_space.size, dtype = dtype, device = device))
        handles.append(plan.handle.value)
        outs.append(out)
        ins = pointers(t._data.data_ptr() for t in ops)
        pre = pointers((p.data_ptr() if p is not None else None) for p in prep)
        keep += [ins, pre, prep]
        inputs.append(ctypes.cast(ins, vp).value)
        prepared.append(ctypes.cast(pre, vp).value)
        workspaces.append(pool.data_ptr())
    launched = i32()
    check(lib.tt_plan_execute_batch(len(handles), pointers(handles), _DTYPE[dtype], _precision, pointers(inputs),
                                    pointers(prepared), pointers(o._data.data_ptr() for o in outs),
                                    pointers(workspaces), stream, ctypes.byref(launched)))
    last_batch_launches = launched.value
    return outs


# the forms a plan's block products run in (tt_autotune): bits of the integer autotune returns
FORM_SEPARATE = 1          # a product chain (the two-site matvec) as separate launches
FORM_NO_TENSOR_CORES = 2   # split products of large blocks on mma.sync instead of tcgen05


def histogram_key(plan: Plan) -> int:
    '''The 64-bit key of a plan's block-size histogram (the autotuner's cache key).'''
    key = ctypes.c_uint64()
    check(lib.tt_plan_histogram(plan.handle, ctypes.byref(key)))
    return key.value


def autotune(spec: str, *operands: Tensor, outcharge = None) -> tuple:
    '''Time every form the einsum's block products can run in on these operands, in the current
    precision, and cache the fastest under the plan's block-size histogram: every later execution
    of a plan with the same histogram (any operands of these shapes, or of others that bin alike)
    runs it.  Returns (forms, milliseconds).  Synchronous; call it outside CUDA graph captures.'''
    _check_device(operands)
    plan = plan_of(spec, *operands, outcharge = outcharge)
    data0 = operands[0]._data
    device = data0.device
    stream = torch.cuda.current_stream(device).cuda_stream
    ws = _workspace(plan, device, data0.dtype, stream)
    prepared = [_prepared_arena(plan, i, t, ws, stream, force = True) for i, t in enumerate(operands)]
    out = torch.empty(plan.out_space.size, dtype = data0.dtype, device = device)
    forms, ms = i32(), ctypes.c_float()
    check(lib.tt_autotune(plan.handle, _DTYPE[data0.dtype], _precision, pointers(t._data.data_ptr() for t in operands),
                          pointers((p.data_ptr() if p is not None else None) for p in prepared), out.data_ptr(),
                          ws.data_ptr() if ws is not None else None, stream, ctypes.byref(forms), ctypes.byref(ms)))
    return forms.value, ms.value


def tuned_forms(plan: Plan, dtype = torch.float64, precision: Optional[int] = None) -> Optional[int]:
    '''The forms cached for the plan's histogram (tt_autotune_lookup), or None.'''
    forms, found = i32(), i32()
    check(lib.tt_autotune_lookup(histogram_key(plan), _DTYPE[dtype], _precision if precision is None else precision,
                                 ctypes.byref(forms), ctypes.byref(found)))
    return forms.value if found.value else None


def store_forms(plan: Plan, forms: int, dtype = torch.float64, precision: Optional[int] = None) -> None:
    '''Cache forms for the plan's histogram by hand (tt_autotune_store): a saved tuning restored.'''
    check(lib.tt_autotune_store(histogram_key(plan), _DTYPE[dtype], _precision if precision is None else precision,
                                int(forms)))


def clear_tuning() -> None:
    '''Forget every cached form choice (tt_autotune_clear).'''
    check(lib.tt_autotune_clear())


def link_copy(dst: torch.Tensor, src: torch.Tensor) -> torch.Tensor:
    '''dst.copy_(src) between a page-locked host tensor and a CUDA tensor (either way round) by a
    kernel that reads or writes the host end over the coherent CPU-GPU link (tt_link_copy), on the
    current stream, without a copy-engine call.  Both contiguous, of one dtype and size; the host
    tensor pinned (`pin_memory=True`), else ValueError.'''
    if dst.dtype != src.dtype or dst.numel() != src.numel() or not dst.is_contiguous() or not src.is_contiguous():
        raise ValueError('link_copy needs two contiguous tensors of one dtype and size')
    if dst.device.type == 'cuda' and src.device.type == 'cpu':
        direction, device = 0, dst.device
    elif dst.device.type == 'cpu' and src.device.type == 'cuda':
        direction, device = 1, src.device
    else:
        raise ValueError('link_copy copies between a host tensor and a CUDA tensor')
    stream = torch.cuda.current_stream(device).cuda_stream
    check(lib.tt_link_copy(dst.data_ptr(), src.data_ptr(), dst.numel() * dst.element_size(), direction, stream))
    # the kernel wrote dst behind torch's back: mark it written, so that no prepared copy of its
    # old contents is reused
    from torch.autograd.graph import increment_version
    increment_version(dst)
    return dst


def plan_of(spec: str, *tensors: Tensor, outcharge = None) -> Plan:
    '''The compiled plan an einsum of these operands runs (for timing and the roofline).'''
    return einsum_plan(spec, [t._space for t in tensors], outcharge)


def einsum_plan(spec: str, spaces, outcharge = None) -> Plan:
    '''The compiled plan of an einsum over operands of these spaces: compiling ahead of the call
    (from spaces a caller expects) fills the cache the call reads.'''
    has = outcharge is not None
    q = _label(outcharge) if has else 0
    ids, n = ints32(s.id for s in spaces)
    return _plan(('einsum', spec, tuple(s.id for s in spaces), has, q),
                 lambda out: lib.tt_plan_einsum(spec.encode(), n, ids, int(has), q, out), spaces[0].cat)


# ---------------------------------------------------------------------------------------------
# scalar products (tentorch/linalg/graded/compare.cpp)
# ---------------------------------------------------------------------------------------------


def _same_legs(a: Tensor, b: Tensor) -> None:
    if a.cat is not b.cat:
        raise ValueError('a scalar product needs both tensors over one category')
    if a._space.codomain != b._space.codomain or a._space.domain != b._space.domain:
        raise ValueError('a scalar product needs both tensors with the same legs')


def inner_device(a: Tensor, b: Tensor) -> torch.Tensor:
    '''<a, b> as a 0-d device tensor, with no host synchronisation (the arena padding is zero).'''
    _same_legs(a, b)
    if a.qtotal != b.qtotal:
        return torch.zeros((), dtype = a.dtype, device = a.device)
    return torch.vdot(a._data, b._data)


def inner(a: Tensor, b: Tensor) -> complex:
    '''tentorch/linalg/graded/compare.cpp:31-43'''
    return complex(inner_device(a, b).item())


def norm(t: Tensor) -> float:
    '''tentorch/linalg/graded/compare.cpp:45'''
    return math.sqrt(abs(inner(t, t)))


def is_close(first: Tensor, second: Tensor, rtol: float = 1e-10, atol: float = 1e-12) -> bool:
    '''tentorch/linalg/graded/compare.cpp:12-29'''
    if first.cat is not second.cat or first.qtotal != second.qtotal:
        return False
    if first._space is not second._space:
        return False
    return bool(torch.allclose(first._data, second._data.to(first.device), rtol = rtol, atol = atol))


# ---------------------------------------------------------------------------------------------
# splittings (tentorch/linalg/graded/svd.cpp)
# ---------------------------------------------------------------------------------------------


# The cuSOLVER method of the per-block SVDs on a CUDA device.  'gesvd' (QR iteration) leaves the
# factors orthonormal to ~4e-15; torch's default for these block sizes (Jacobi, gesvdj) only to
# ~1e-13, which moves a DMRG sweep energy at L = 64, bond 256 by ~1.4e-10.  None picks torch's
# default, which is what the reference's at::linalg_svd (tentorch/linalg/graded/svd.cpp:59) runs
# on a CUDA device.
PER_BLOCK_SVD_DRIVER: Optional[str] = 'gesvd'


# splits whose Jacobi SVD left a block unsettled and were redone per block with cuSOLVER
svd_fallbacks = 0


def _factor_blocks_per_block(arranged: Tensor, present, while_waiting = None):
    '''The thin SVD of each present block by at::linalg_svd, one block at a time (svd.cpp:57-62).'''
    factors = []
    driver = PER_BLOCK_SVD_DRIVER if arranged.device.type == 'cuda' else None
    for i, key in present:
        u, sv, vh = torch.linalg.svd(arranged._view(i), full_matrices = False, driver = driver)
        factors.append([key, u, sv, vh, 0, 0])
    if while_waiting is not None:
        while_waiting()
    host = torch.cat([f[2] for f in factors]).to('cpu', torch.float64).tolist() if factors else []
    return factors, host, None


def _factor_blocks(arranged: Tensor, while_waiting = None):
    """The thin SVD of every non-empty block.  float64 blocks on the GPU go through one launch of
    the engine's Jacobi SVD (tt_svd_blocks), complex blocks, blocks beyond its size and the
    per-block comparison form through at::linalg_svd one block at a time, as svd.cpp:57-62 does.
    Returns [key, u, s, vh, kept, offset] per block (u, s, vh views of packed device arrays in the
    first case) and the host copy of all singular values, block after block."""
    space = arranged._space
    present = [(i, key) for i, key in enumerate(arranged.keys()) if space.shapes[i][0] * space.shapes[i][1] > 0]
    batched = (arranged.dtype == torch.float64 and arranged.device.type == 'cuda' and _precision != PER_BLOCK and
               all(min(space.shapes[i]) <= 1024 for i, _ in present))
    if not batched:
        return _factor_blocks_per_block(arranged, present, while_waiting)
    dims, count = ints64(x for i, _ in present for x in space.shapes[i])
    places, total = (i64 * max(len(present), 1))(), i64()
    check(lib.tt_svd_workspace(len(present), dims, places, ctypes.byref(total)))
    ws_at = total.value
    entries, shapes = [], []
    u_at = s_at = vh_at = 0
    for at, (i, key) in enumerate(present):
        rows, cols = space.shapes[i]
        k = min(rows, cols)
        entries.append([space.offsets[i], rows, cols, u_at, s_at, vh_at, places[at]])
        shapes.append((key, rows, cols, k, u_at, s_at, vh_at))
        u_at, s_at, vh_at = u_at + rows * k, s_at + k, vh_at + k * cols
    # the largest blocks first: the launch's clusters then finish together, small blocks last
    entries.sort(key = lambda e: -min(e[1], e[2]) ** 2 * max(e[1], e[2]))
    table = [x for e in entries for x in e]
    largest = max((min(e[1], e[2]) for e in entries), default = 0)
    device = arranged.device
    # no wait for the stream's queued work (the window's Lanczos): the SVD is queued behind it
    dev_table = _uploaded(table, torch.int64, device)
    u = torch.empty(max(u_at, 1), dtype = torch.float64, device = device)
    sv = torch.empty(max(s_at, 1), dtype = torch.float64, device = device)
    vh = torch.empty(max(vh_at, 1), dtype = torch.float64, device = device)
    ws = torch.empty(max(ws_at, 1), dtype = torch.float64, device = device)
    info = torch.empty(max(len(present), 1), dtype = torch.int32, device = device)
    stream = torch.cuda.current_stream(device).cuda_stream
    check(lib.tt_svd_blocks(len(present), largest, dev_table.data_ptr(), arranged._data.data_ptr(), u.data_ptr(),
                            sv.data_ptr(), vh.data_ptr(), ws.data_ptr(), info.data_ptr(), stream))
    # the values stay on the device: the caller ranks them there and reads the sweep counts
    # (info) with the per-block results in one wait
    factors = [[key, (u_off, rows, k), (s_off, k), (vh_off, k, cols), 0, 0]
               for key, rows, cols, k, u_off, s_off, vh_off in shapes]
    return factors, None, (u, sv, vh, info[:max(len(present), 1)], s_at, present)


def _split_over(tensor: Tensor, left, max_bond, tol, absorb, while_waiting = None):
    '''tentorch/linalg/graded/svd.cpp:41-177: the SVD of every block, the global ranking of the
    singular values, truncation and the +-q pairing of the bond (on the device for the engine's
    batched SVD: one read of each block's kept count), then the two factors.  `while_waiting`, when
    given, runs on the host once the split's device work is queued and before the split reads its
    results (host work of the caller's that needs no device result: it overlaps the SVD).'''
    if absorb not in (0, 1, 2, 3):
        raise ValueError(f'absorb has to be 0, 1, 2 or 3, got {absorb}')
    if max_bond is not None and max_bond < 1:
        raise ValueError(f'a bond needs at least one multiplet, got {max_bond}')
    arranged = tensor.place(left) if left is not None else tensor
    cat = arranged.cat
    factors, host, packed = _factor_blocks(arranged, while_waiting)
    if packed is not None:
        ranked = _rank_on_device(arranged, factors, packed, max_bond, tol, while_waiting)
        if ranked is None:
            # a block the Jacobi sweeps did not settle within their cap: this split's blocks go
            # through cuSOLVER one by one instead (QR iteration, gesvd), as the per-block form runs them
            global svd_fallbacks
            svd_fallbacks += 1
            factors, host, packed = _factor_blocks_per_block(arranged, packed[5])
        else:
            multiplicities = ranked
            return _split_finish(arranged, factors, packed, multiplicities, absorb)
    candidates, at = [], 0
    for fi, f in enumerate(factors):
        for index in range(f[2].numel()):
            candidates.append((host[at], fi, index))
            at += 1
    multiplicities = _rank_candidates(factors, candidates, max_bond, tol, cat)
    return _split_finish(arranged, factors, packed, multiplicities, absorb)


def _rank_on_device(arranged: Tensor, factors, packed, max_bond, tol, while_waiting = None):
    '''The ranking of the split's singular values on the device (tt_svd_rank): per block the values
    it keeps, read with the SVD's sweep counts in one wait.  Returns the bond's multiplets per
    domain sector (the blocks' f[4] set), or None when a block's Jacobi sweeps did not settle.
    Where the values do not fit the ranking kernel, they are read and ranked on the host.'''
    u, sv, vh, info, s_at, present = packed
    cat = arranged.cat
    ids = {}
    for f in factors:
        for sector in (f[0].domain, cat.dual(f[0].domain)):
            ids.setdefault(sector, len(ids))
    sectors = sorted(ids, key = ids.get)
    table = ([f[2][1] for f in factors] + [ids[f[0].domain] for f in factors] +
             [ids[cat.dual(sector)] for sector in sectors])
    device = arranged.device
    dev = _uploaded(table, torch.int32, device)
    kept = torch.zeros(len(factors), dtype = torch.int32, device = device)
    nb, ns = len(factors), len(sectors)
    stream = torch.cuda.current_stream(device).cuda_stream
    try:
        check(lib.tt_svd_rank(sv.data_ptr(), s_at, dev.data_ptr(), dev.data_ptr() + 4 * nb, nb, dev.data_ptr() + 8 * nb, ns,
                              float(tol), -1 if max_bond is None else int(max_bond), kept.data_ptr(), stream))
    except ValueError:
        if while_waiting is not None:
            while_waiting()
        return _rank_on_host(factors, sv[:s_at].cpu().tolist(), info, max_bond, tol, cat)
    if while_waiting is not None:
        while_waiting()
    both = torch.cat([info.to(torch.int32), kept]).cpu()
    if present and int(both[:info.numel()].min()) < 0:
        return None
    multiplicities = {}
    for f, k in zip(factors, both[info.numel():].tolist()):
        f[4] = k
        if k:
            multiplicities[f[0].domain] = multiplicities.get(f[0].domain, 0) + k
    return multiplicities


def _rank_on_host(factors, host, info, max_bond, tol, cat):
    '''The same ranking on the host, for splits too large for the ranking kernel.'''
    if factors and int(info.min()) < 0:
        return None
    candidates, at = [], 0
    for fi, f in enumerate(factors):
        for index in range(f[2][1]):
            candidates.append((host[at], fi, index))
            at += 1
    return _rank_candidates(factors, candidates, max_bond, tol, cat)


def _rank_candidates(factors, candidates, max_bond, tol, cat):
    '''tentorch/linalg/graded/svd.cpp:68-118: the global ranking, truncation and +-q pairing of the
    bond over (value, block, index) candidates; sets each block's kept count f[4] and returns the
    bond's multiplets per domain sector.'''
    candidates.sort(key = lambda c: -c[0])
    cut = next((i for i, c in enumerate(candidates) if c[0] <= tol), len(candidates))
    candidates = candidates[:cut]
    if max_bond is not None and len(candidates) > max_bond:
        candidates = candidates[:max_bond]
    for _, fi, index in candidates:
        factors[fi][4] = max(factors[fi][4], index + 1)
    multiplicities = {}
    for f in factors:
        if f[4]:
            multiplicities[f[0].domain] = multiplicities.get(f[0].domain, 0) + f[4]
    paired = {}
    for sector, count in multiplicities.items():
        other = multiplicities.get(cat.dual(sector))
        if other is not None:
            paired[sector] = min(count, other)
    if paired and paired != multiplicities:
        for f in factors:
            f[4] = 0
        used = {}
        for _, fi, index in candidates:
            f = factors[fi]
            room = paired.get(f[0].domain)
            if room is None or used.get(f[0].domain, 0) >= room:
                continue
            used[f[0].domain] = used.get(f[0].domain, 0) + 1
            f[4] = max(f[4], index + 1)
        multiplicities = paired
    return multiplicities


def _split_finish(arranged: Tensor, factors, packed, multiplicities, absorb):
    '''The bond of the split from its multiplets per domain sector, and the two factors and the
    values written (one launch from the packed factors, else block by block).'''
    cat = arranged.cat
    nxt = {}
    for f in factors:
        f[5] = nxt.get(f[0].domain, 0)
        nxt[f[0].domain] = f[5] + f[4]
    placed, run_at = {}, 0
    for sector in sorted(multiplicities):
        placed[sector] = run_at
        run_at += multiplicities[sector]
    if not multiplicities:
        multiplicities = {cat.trivial(): 1}
    bond = Leg.from_blocks(cat, sorted(multiplicities.items()))[0]
    first = Tensor(cat, arranged.codomain, [bond], arranged.qtotal, arranged.dtype, arranged.device)
    values = torch.zeros(bond.multiplets(), dtype = arranged.dtype, device = arranged.device)
    second = Tensor(cat, [bond], arranged.domain, cat.trivial(), arranged.dtype, arranged.device)
    if packed is not None:
        # one launch writes every kept block of both factors and the values
        u, sv, vh = packed[:3]
        table, count = [], 0
        for key, (u_off, rows, k), (s_off, _), (vh_off, _, cols), kept, offset in factors:
            if kept == 0:
                continue
            fi = first._space.index[BlockKey(key.codomain, key.domain, key.copy)]
            si = second._space.index[BlockKey(key.domain, key.domain, 0)]
            first_ld = first._space.shapes[fi][1]
            table += [u_off, s_off, vh_off, first._space.offsets[fi], second._space.offsets[si],
                      placed[key.domain] + offset, rows | cols << 32, k | kept << 32, first_ld | offset << 32,
                      offset | absorb << 32]
            count += 1
        if count:
            device = arranged.device
            dev_table = _uploaded(table, torch.int64, device)
            stream = torch.cuda.current_stream(device).cuda_stream
            check(lib.tt_svd_keep(count, dev_table.data_ptr(), u.data_ptr(), sv.data_ptr(), vh.data_ptr(),
                                  first._data.data_ptr(), second._data.data_ptr(), values.data_ptr(), stream))
        return first, values, second
    for key, u, s, vh, kept, offset in factors:
        if kept == 0:
            continue
        u, vh, s = u[:, :kept], vh[:kept], s[:kept]
        if absorb == 3:
            u = u * s.sqrt()
            vh = s.sqrt().unsqueeze(1) * vh
        elif absorb == 1:
            u = u * s
        elif absorb == 2:
            vh = s.unsqueeze(1) * vh
        first.block(key.codomain, key.domain, key.copy)[:, offset:offset + kept].copy_(u)
        second.block(key.domain, key.domain)[offset:offset + kept, :].copy_(vh)
        values[placed[key.domain] + offset:placed[key.domain] + offset + kept].copy_(s.to(arranged.dtype))
    return first, values, second


def svd(tensor: Tensor, *args, **kwargs):
    '''svd(tensor, max_bond=None, tol=0.0, absorb=0) or svd(tensor, left, max_bond=None, tol=0.0,
    absorb=0) -> (first, values, second): the two overloads of tentorch/_ext/bindings.cpp:365-382.'''
    left = None
    if args and isinstance(args[0], (list, tuple)):
        left, args = list(args[0]), args[1:]
    elif 'left' in kwargs:
        left = kwargs.pop('left')
    params = {'max_bond': None, 'tol': 0.0, 'absorb': 0}
    for name, value in zip(('max_bond', 'tol', 'absorb'), args):
        params[name] = value
    for name, value in kwargs.items():
        if name not in params:
            raise TypeError(f'svd() got an unexpected keyword argument {name!r}')
        params[name] = value
    return _split_over(tensor, left, params['max_bond'], params['tol'], params['absorb'])


def svdvals(tensor: Tensor, left = None) -> torch.Tensor:
    return _split_over(tensor, left, None, 0.0, 0)[1]


def _split_blocks(tensor: Tensor, pieces):
    '''tentorch/linalg/graded/svd.cpp:203-229'''
    cat = tensor.cat
    multiplicities, nxt, placed = {}, {}, []
    for key, left, right, kept in pieces:
        if kept == 0:
            continue
        offset = nxt.get(key.domain, 0)
        nxt[key.domain] = offset + kept
        multiplicities[key.domain] = multiplicities.get(key.domain, 0) + kept
        placed.append((key, left, right, kept, offset))
    if not multiplicities:
        multiplicities = {cat.trivial(): 1}
    bond = Leg.from_blocks(cat, sorted(multiplicities.items()))[0]
    first = Tensor(cat, tensor.codomain, [bond], tensor.qtotal, tensor.dtype, tensor.device)
    second = Tensor(cat, [bond], tensor.domain, cat.trivial(), tensor.dtype, tensor.device)
    for key, left, right, kept, offset in placed:
        first.block(key.codomain, key.domain, key.copy)[:, offset:offset + kept].copy_(left)
        second.block(key.domain, key.domain)[offset:offset + kept, :].copy_(right)
    return first, second


def qr(tensor: Tensor, left = None):
    '''tentorch/linalg/graded/svd.cpp:233-244'''
    arranged = tensor.place(left) if left is not None else tensor
    pieces = []
    for i, key in enumerate(arranged.keys()):
        matrix = arranged._view(i)
        if matrix.numel() == 0:
            continue
        q, r = torch.linalg.qr(matrix, mode = 'reduced')
        pieces.append((key, q, r, q.shape[1]))
    return _split_blocks(arranged, pieces)


def rq(tensor: Tensor, left = None):
    '''tentorch/linalg/graded/svd.cpp:246-257'''
    arranged = tensor.place(left) if left is not None else tensor
    pieces = []
    for i, key in enumerate(arranged.keys()):
        matrix = arranged._view(i)
        if matrix.numel() == 0:
            continue
        q, r = torch.linalg.qr(matrix.transpose(0, 1), mode = 'reduced')
        pieces.append((key, r.transpose(0, 1), q.transpose(0, 1), q.shape[1]))
    return _split_blocks(arranged, pieces)
