"""Angular-spectrum vacuum step (theory/vacuum.py:5-7 of the reference):
ifft2(exp(i k L) exp(-i pi L lambda f^2) fft2(u)) on the grid of step delta.

Runs the engine's allocation-free vacuum kernel (atm_vacuum_noalloc) on a
complex64 copy of the input on the current CUDA device.  The reference
takes the f^2 grid and its step as arguments; the engine builds the
standard centred grid of the field's own size (f_delta = 1 / (N delta)),
so other grids are refused."""
from __future__ import annotations

import math

import numpy as np

from .. import gpu


def vacuum_propagation(input, length, k, delta, f2=None, f_delta=None):
    import torch
    from ..engine import _lib
    from ..engine.plan import _stream, _tptr
    u = input if isinstance(input, torch.Tensor) else torch.as_tensor(np.asarray(input))
    if u.dim() != 2 or u.shape[0] != u.shape[1]:
        raise ValueError("vacuum_propagation: the field must be a square N x N array")
    N = int(u.shape[0])
    if f_delta is not None and not math.isclose(float(f_delta), 1.0 / (N * float(delta)), rel_tol=1e-6):
        raise ValueError("vacuum_propagation: the engine propagates on the field's own frequency grid "
                         "(f_delta = 1 / (N delta))")
    if f2 is not None and tuple(getattr(f2, "shape", (N, N))) not in ((N, N), (1, N), (N, 1)):
        raise ValueError("vacuum_propagation: f2 must be the field's N x N frequency grid")
    dev = gpu.device()
    field = u.to(dev, torch.complex64).contiguous().clone()
    back = float(length) < 0
    if back:
        # H(-L) = conj(H(L)) and H(f) = H(-f) on the centred grid, so a step
        # back is conj(step forward of conj(u))
        field = field.conj().resolve_conj().contiguous()
    lib = _lib.load()
    _lib.check(lib.atm_vacuum_noalloc(_tptr(field), N, 1, float(delta), 2 * math.pi / float(k), abs(float(length)),
                                      _stream(dev)))
    return field.conj().resolve_conj() if back else field
