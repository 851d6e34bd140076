"""Host-side inputs of the engine: annulus weights of the sparse spectrum
and seeded spectrum draws.

``annulus_psd`` restates SSPhaseScreen._get_psd (phase_screens.py:82-91): the
weight of annulus i is 2 pi * int_{f_{i-1}}^{f_i} (2 pi)^2 f Phi_phi(f) df with
f_{-1} = 0 and Phi_phi the model's phase spectrum (theory/models.py:16-23).
Instead of one adaptive quadrature call per annulus it applies one fixed
64-node Gauss-Legendre rule to all annuli at once (the annuli are narrow and
the integrand smooth, so the two agree to ~1e-12 relative; the result is
rounded to float32 like the reference's).

``draw_spectra`` forms rho / theta / value exactly as grids.py:98-107 and
phase_screens.py:98-103 do from one uniform, P uniforms and 2P normals per
screen, drawn from numpy's default_rng([seed, realisation]).
"""
from __future__ import annotations

from typing import Callable, Sequence

import numpy as np

_GL_X, _GL_W = np.polynomial.legendre.leggauss(64)


def annulus_psd(base: np.ndarray, psd_phi_f: Callable, k: float, thickness: float) -> np.ndarray:
    fb = np.asarray(base, dtype=np.float64)
    a = np.concatenate([[0.0], fb[:-1]])
    mid, half = (a + fb) / 2, (fb - a) / 2
    f = mid[:, None] + half[:, None] * _GL_X[None, :]
    integrand = (2 * np.pi) ** 2 * f * psd_phi_f(f, k, thickness)
    return (2 * np.pi * (integrand * _GL_W[None, :]).sum(axis=1) * half).astype(np.float32)


def draw_spectra(seed: int, realisations: Sequence[int], n_screens: int, base: np.ndarray,
                 psd: np.ndarray):
    base = np.asarray(base, dtype=np.float32)
    P = base.shape[0]
    f_prev = np.insert(base, 0, 0)[:-1]
    span = base ** 2 - f_prev ** 2
    f2 = f_prev ** 2
    sq = np.sqrt(np.asarray(psd, dtype=np.float32))
    R = len(realisations)
    rho = np.empty((R, n_screens, P), np.float32)
    theta = np.empty((R, n_screens, P), np.float32)
    value = np.empty((R, n_screens, P), np.complex64)
    for j, r in enumerate(realisations):
        rng = np.random.default_rng([int(seed), int(r)])
        for i in range(n_screens):
            u = rng.random(1).astype(np.float32)
            t = rng.random(P).astype(np.float32)
            ab = rng.standard_normal((2, P))
            rho[j, i] = np.sqrt(f2 + u * span)
            theta[j, i] = 2 * np.pi * t
            value[j, i] = (ab[0] + 1j * ab[1]).astype(np.complex64) * sq
    return rho, theta, value
