"""FFT phase screens with subharmonics (phase_screens.py:37-67) on the engine.

Host side (FP64): the amplitude grid sqrt(Phi_phi(|f|)) 2 pi df in centred
order with DC = 0, and per subharmonic level s (grid df / 3^(s+1), 3 x 3) the
separable factors X_j(x) = sum_i c_ij exp(i 2 pi f_i x), Y_j(y) =
exp(i 2 pi f_j y) and the mean of their sum.  Device side (atm_fft_screen):
spectrum, unnormalised inverse 2-D FFT by the engine's row and column passes
with (-1)^k factors in place of the centring shifts, subharmonic sum, minus
the mean.
"""
from __future__ import annotations

import numpy as np

from .. import gpu


def _axis(N, step):
    lo = (-N) // 2 + (N % 2)
    return np.arange(lo, lo + N, dtype=np.float64) * step


def screen_amplitude(N, delta, psd_phi_f, k, thickness):
    """sqrt(Phi_phi(|f|)) 2 pi df on the centred frequency grid, DC = 0 (float32)."""
    df = 1.0 / (N * delta)
    ax = _axis(N, df)
    amp = np.sqrt(psd_phi_f(np.sqrt(ax[None, :] ** 2 + ax[:, None] ** 2), k, thickness)) * 2 * np.pi * df
    amp[N // 2, N // 2] = 0.0
    return amp.astype(np.float32)


def subharmonic_factors(N, delta, psd_phi_f, k, thickness, level_normals):
    """Per 3 x 3 subharmonic level s (draws level_normals[s], shape (2, 3, 3)):
    the separable factors X_j(x), Y_j(y) and the mean of sum_j X_j Y_j (FP64)."""
    df = 1.0 / (N * delta)
    x = _axis(N, delta)
    X, Y, mean = [], [], 0j
    for s, nrm in enumerate(level_normals):
        sdf = df / 3 ** (s + 1)
        f3 = np.arange(-1, 2, dtype=np.float64) * sdf
        r3 = np.sqrt(f3[None, :] ** 2 + f3[:, None] ** 2)
        c = (nrm[0] + 1j * nrm[1]).astype(np.complex64) * np.sqrt(psd_phi_f(r3, k, thickness)) * 2 * np.pi * sdf
        c[1, 1] = 0
        ex = np.exp(2j * np.pi * np.outer(f3, x))     # [i][x]
        for j in range(3):
            Xj = (c[:, j, None] * ex).sum(axis=0)
            Yj = ex[j]                                  # y uses the same axis values
            X.append(Xj)
            Y.append(Yj)
            mean += Xj.mean() * Yj.mean()
    return X, Y, mean


def screen_inputs(N, delta, psd_phi_f, k, thickness, normals):
    amp = screen_amplitude(N, delta, psd_phi_f, k, thickness)
    X, Y, mean = subharmonic_factors(N, delta, psd_phi_f, k, thickness, normals[1:])
    return amp, X, Y, mean


def draw_normals(N, subharmonics):
    """The standard normals of one FFTPhaseScreen draw in the reference's order
    (phase_screens.py:46-60): the main grid's real then imaginary part, then
    per subharmonic level a 3 x 3 real then imaginary part."""
    out = [np.stack([np.random.normal(size=(N, N)), np.random.normal(size=(N, N))])]
    for _ in range(subharmonics):
        out.append(np.stack([np.random.normal(size=(3, 3)), np.random.normal(size=(3, 3))]))
    return out


def fft_screen(ps, normals):
    """Complex screen [N, N] (torch complex64) of an FFTPhaseScreen for the
    given draws (list: main grid (2, N, N), then (2, 3, 3) per level)."""
    import ctypes

    import torch

    from ._lib import check
    from .plan import EnginePlan, _stream
    N, delta = ps.grid.N, float(ps.grid.delta)
    dev = gpu.device()
    key = (N, delta, str(dev))
    if getattr(ps, "_fft_plan_key", None) != key:
        ps._fft_plan = EnginePlan(N, delta, float(ps.wvl), 1.0, float("inf"), [], 1.0, batch=1, device=dev)
        ps._fft_plan_key = key
    plan = ps._fft_plan
    amp, X, Y, mean = screen_inputs(N, delta, ps.model.psd_phi_f, 2 * np.pi / ps.wvl, ps.thickness, normals)
    n_sub = len(X)
    t = lambda a, dt: torch.from_numpy(np.ascontiguousarray(a, dtype=dt)).to(dev)
    nrm = t(np.asarray(normals[0], np.float32).reshape(1, 2, N, N), np.float32)
    amp_d = t(amp, np.float32)
    sx = t(np.array(X or [np.zeros(N)]).reshape(1, max(n_sub, 1), N), np.complex64)
    sy = t(np.array(Y or [np.zeros(N)]).reshape(1, max(n_sub, 1), N), np.complex64)
    sm = t(np.array([[mean.real, mean.imag]]), np.float64)
    out = torch.empty((1, N, N), dtype=torch.complex64, device=dev)
    vp = lambda x: ctypes.c_void_p(x.data_ptr())
    with torch.cuda.device(dev):
        check(plan.lib.atm_fft_screen(plan._handle, vp(nrm), vp(amp_d), vp(sx), vp(sy), vp(sm), n_sub, 1, vp(out),
                                      _stream(dev)))
    return out[0]
