'''
The Lanczos eigensolver of the reference (tentorch/linalg/lanczos.py:8-64) over the engine's
block-sparse tensors, kept on the GPU.

Every Krylov step runs on device-resident scalars: the projections alpha and the norms beta stay
0-d device tensors, and each projection runs against the whole basis at once (one matrix-vector
product for the coefficients and one fused update over the stacked arenas).  The host reads the tridiagonal matrix once, after the last step, and applies the
reference's early stop (a step whose beta falls below `tol` ends the space) to what it reads: the
steps computed after such a stop are discarded, so the result is the reference's.
'''
from __future__ import annotations

import ctypes
from typing import Callable

import numpy as np
import torch

from tentorch_gb300.linalg import norm
from tentorch_gb300.tensor import Tensor


def lanczos(action: Callable[[Tensor], Tensor], start: Tensor, n_iter: int = 5,
            tol: float = 1e-12) -> tuple[float, Tensor]:
    '''
    The lowest eigenpair of a Hermitian action, by Lanczos with full reorthogonalisation (twice).

    Args:
      action: v -> H v on tensors with the legs of `start`.
      start: the starting vector, any normalisation.
      n_iter: the number of Krylov steps.
      tol: the norm below which a step ends the Krylov space.
    Returns:
      The lowest Ritz value and its Ritz vector, normalised.
    Raises:
      ValueError: when `n_iter` is below one or `start` has zero norm.
    '''
    if n_iter < 1:
        raise ValueError(f'Lanczos needs at least one step, not {n_iter}.')
    scale = norm(start)
    if scale == 0.0:
        raise ValueError('Lanczos needs a starting vector of non-zero norm.')
    space = start._space
    data = start.data
    basis = torch.empty((n_iter + 1, data.numel()), dtype = data.dtype, device = data.device)
    basis[0] = data * (1.0 / scale)
    alphas, betas = [], []
    for step in range(n_iter):
        vector = Tensor._wrap(space, basis[step])
        image = action(vector).data
        used = basis[:step + 1]
        # The first projection against every vector so far holds alpha = <v_step, H v_step> as its
        # last coefficient and removes alpha v_step and beta v_{step-1} (the three-term step of
        # the reference) together with the round-off components along the older vectors; then
        # the reference's two full reorthogonalisation passes.  Each pass is one product for the
        # coefficients and one fused update (addmv), so a step launches a handful of kernels and
        # never waits for the host.
        coefficients = torch.mv(used.conj(), image)
        alphas.append(coefficients[step].real)
        image = torch.addmv(image, used.transpose(0, 1), coefficients, alpha = -1)
        for _ in range(2):
            coefficients = torch.mv(used.conj(), image)
            image = torch.addmv(image, used.transpose(0, 1), coefficients, alpha = -1)
        beta = torch.linalg.vector_norm(image)
        betas.append(beta)
        # a beta below tol ends the space on the host afterwards; dividing by it here only fills a
        # row that is then discarded
        torch.div(image, torch.clamp(beta, min = 1e-300), out = basis[step + 1])
    host_alpha = torch.stack(alphas).cpu().numpy().astype(np.float64)
    host_beta = torch.stack(betas).cpu().numpy().astype(np.float64)
    size = n_iter
    for step in range(n_iter):
        if host_beta[step] < tol:
            size = step + 1
            break
    matrix = np.diag(host_alpha[:size])
    for step in range(size - 1):
        matrix[step, step + 1] = matrix[step + 1, step] = host_beta[step]
    values, vectors = np.linalg.eigh(matrix)
    coefficients = torch.as_tensor(vectors[:, 0], dtype = data.dtype, device = data.device)
    result = torch.mv(basis[:size].transpose(0, 1), coefficients)
    result = result / torch.linalg.vector_norm(result)
    return float(values[0]), Tensor._wrap(space, result.contiguous())


def lanczos_einsum(spec: str, tensors, vector: int, start: Tensor, n_iter: int = 5, tol: float = 1e-12,
                   outcharge = None, wait: bool = True):
    '''
    `lanczos(lambda v: einsum(spec, *tensors with v as operand `vector`), start, n_iter, tol)` with
    the whole Krylov loop on the device (tt_lanczos): the einsum's compiled plan runs on each basis
    vector, the projections and norms stay on the GPU, and so does the tridiagonal's eigensolve.
    The operands other than the vector are prepared once for every step (the head and tail of a DMRG
    window).  Same result as `lanczos` up to round-off; block products in the current precision.
    With `wait` False nothing waits for the device (tt_lanczos_async): the energy comes back as a
    0-d device tensor, and the zero-norm check of the start vector is left to the caller.
    '''
    if n_iter < 1:
        raise ValueError(f'Lanczos needs at least one step, not {n_iter}.')
    if wait and norm(start) == 0.0:
        raise ValueError('Lanczos needs a starting vector of non-zero norm.')
    from tentorch_gb300 import linalg
    from tentorch_gb300._lib import check, f64, i32, i64, lib, pointers
    operands = list(tensors)
    operands[vector] = start
    linalg._check_device(operands)
    plan = linalg.plan_of(spec, *operands, outcharge = outcharge)
    if plan.out_space is not start._space:
        raise ValueError('the action has to map the vector to a tensor with the same legs')
    data = start._data
    device = data.device
    stream = torch.cuda.current_stream(device).cuda_stream
    capturing = torch.cuda.is_current_stream_capturing()
    if capturing:
        linalg._note_capture()
    ws = linalg._workspace(plan, device, data.dtype, stream)
    # under a CUDA graph capture the operands are prepared inside the graph (each replay reads the
    # head and tail from their buffers) and the prepared copies are not cached
    prepared = [None if i == vector else
                (linalg._prepare_now(plan, i, t, ws, stream) if capturing else
                 linalg._prepared_arena(plan, i, t, ws, stream, force = True))
                for i, t in enumerate(operands)]
    doubles = i64()
    check(lib.tt_lanczos_scratch(start._space.size, n_iter, linalg._DTYPE[data.dtype], ctypes.byref(doubles)))
    scratch = torch.empty(doubles.value, dtype = torch.float64, device = device)
    result = torch.empty_like(data)
    args = (plan.handle, linalg._DTYPE[data.dtype], linalg.get_precision(), pointers(t._data.data_ptr() for t in operands),
            pointers((p.data_ptr() if p is not None else None) for p in prepared), vector, data.data_ptr(), n_iter, tol,
            ws.data_ptr() if ws is not None else None, scratch.data_ptr(), result.data_ptr())
    if not wait:
        found = torch.empty(2, dtype = torch.float64, device = device)  # the energy, then the size (int32)
        check(lib.tt_lanczos_async(*args, ctypes.cast(found.data_ptr(), ctypes.POINTER(f64)),
                                   ctypes.cast(found.data_ptr() + 8, ctypes.POINTER(i32)), stream))
        return found[0], Tensor._wrap(start._space, result)
    energy, size = f64(), i32()
    check(lib.tt_lanczos(*args, ctypes.byref(energy), ctypes.byref(size), stream))
    return float(energy.value), Tensor._wrap(start._space, result)
