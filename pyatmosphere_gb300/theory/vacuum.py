"""Angular-spectrum vacuum step (theory/vacuum.py:5-7 of the reference):
ifft2(exp(i k L) exp(-i pi L lambda f^2) fft2(u)) on the grid of step delta.

Runs the engine's allocation-free vacuum kernel (atm_vacuum_noalloc) on a
complex64 copy of the input on the current CUDA device.  The reference
multiplies by whatever f^2 grid and step it is given; the engine builds the
standard centred grid of the field's own size, f = (j - N/2) / (N delta)
(RectGrid.get_f_grid().get_rho2()), so an f2 or f_delta that is not that
grid is refused with ValueError instead of being silently replaced.

The engine computes in complex64.  The result has the input's complex dtype
(complex128 in, complex128 out, as the reference's numpy path returns), with
complex64 precision (about 1e-6 relative)."""
from __future__ import annotations

import math

import numpy as np

from .. import gpu


def _standard_f2(N: int, delta: float) -> np.ndarray:
    f = (np.arange(N, dtype=np.float32) - np.float32(N // 2)) * np.float32(1.0 / (N * delta))
    return f[None, :] ** 2 + f[:, None] ** 2


def _check_grid(f2, f_delta, N: int, delta: float):
    if f_delta is not None and not math.isclose(float(f_delta), 1.0 / (N * float(delta)), rel_tol=1e-6):
        raise ValueError("vacuum_propagation: the engine propagates on the field's own frequency grid "
                         f"(f_delta = 1 / (N delta) = {1.0 / (N * float(delta)):.6g}, got {float(f_delta):.6g})")
    if f2 is None:
        return
    import torch
    a = f2.detach().cpu().numpy() if isinstance(f2, torch.Tensor) else np.asarray(f2)
    want = _standard_f2(N, float(delta))
    try:
        a = np.broadcast_to(a, (N, N))
    except ValueError:
        raise ValueError(f"vacuum_propagation: f2 must be the field's {N} x {N} frequency grid") from None
    if not np.allclose(a, want, rtol=1e-5, atol=1e-6 * float(want.max())):
        raise ValueError("vacuum_propagation: f2 is not the centred frequency grid of the field "
                         "(RectGrid.get_f_grid().get_rho2()); the engine propagates on that grid only")


def vacuum_propagation(input, length, k, delta, f2=None, f_delta=None):
    import torch
    from ..engine import _lib
    from ..engine.plan import _stream, _tptr
    u = input if isinstance(input, torch.Tensor) else torch.as_tensor(np.asarray(input))
    if u.dim() != 2 or u.shape[0] != u.shape[1]:
        raise ValueError("vacuum_propagation: the field must be a square N x N array")
    N = int(u.shape[0])
    _check_grid(f2, f_delta, N, delta)
    out_dtype = torch.complex128 if u.dtype in (torch.complex128, torch.float64) else torch.complex64
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
    out = field.conj().resolve_conj() if back else field
    return out.to(out_dtype)
