"""numpy restatement of pyAtmosphere's split-step propagation path.

TEST INFRASTRUCTURE ONLY (see ``oracle/__init__.py``): the checker for the
GB300 engine and the timed CPU baseline.  Never imported by the product.

Two precisions are offered for every function that computes:

* ``prec="fp64"`` -- the reference algorithm evaluated in float64 / complex128
  on the injected float32 / complex64 inputs.  This is the truth the engine is
  gated against (field rel-L2 <= 1e-4).
* ``prec="ref"``  -- the same algorithm with the dtypes the reference produces
  under numpy 2 (float32 coordinates, complex64 screen exponentials and GEMM,
  complex64 field between steps).  It reproduces the reference's own outputs to
  FFT round-off and is what pins this restatement against the golden vectors
  made by running the reference itself.

Every function cites the reference lines it restates (paths relative to the
pyAtmosphere source tree).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import List, Optional, Sequence, Tuple

import numpy as np

__all__ = [
    "ChannelSpec", "rect_axis", "f_axis", "logpolar_base", "mvk_psd_n",
    "psd_phi_f", "annulus_psd", "draw_spectra", "ss_screen", "gaussian_source",
    "vacuum", "screen_positions", "propagate", "pupil_mask", "measures",
    "mean_x2_r", "simulate", "fft_screen", "rel_l2",
]


# ----------------------------------------------------------------------------
# channel description used by the oracle (mirrors QuickChannel / Channel args)
# ----------------------------------------------------------------------------
@dataclass
class ChannelSpec:
    N: int = 512
    delta: float = 2e-3
    wvl: float = 808e-9
    w0: float = 0.09
    F0: float = math.inf
    length: float = 10e3
    count: int = 5
    position: str = "middle"
    Cn2: float = 1e-15
    l0: float = 6e-3
    L0: float = 1e3
    points: int = 1024
    f_min: float = 1 / 1e3 / 15
    f_max: float = 2 / 6e-3
    pupil_radius: float = 0.12
    losses_db: float = 0.0

    @property
    def k(self) -> float:
        return 2 * np.pi / self.wvl

    @property
    def thickness(self) -> float:
        return self.length / self.count


def rel_l2(a, b) -> float:
    a = np.asarray(a, dtype=np.complex128)
    b = np.asarray(b, dtype=np.complex128)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


# ----------------------------------------------------------------------------
# grids (grids.py:39-53 bounds, :63-69 get_x/get_y, :82-85 get_f_grid)
# ----------------------------------------------------------------------------
def rect_axis(N: int, delta: float, prec: str = "fp64") -> np.ndarray:
    """Centred coordinates (-N/2 .. N/2-1) * delta; float32 in the reference."""
    lo = (-N) // 2 + (N % 2)
    hi = N // 2 + (N % 2)
    if prec == "ref":
        return np.arange(lo, hi, dtype=np.float32) * np.float32(delta)
    return np.arange(lo, hi, dtype=np.float64) * float(delta)


def f_axis(N: int, delta: float, prec: str = "fp64") -> np.ndarray:
    """Reciprocal-grid axis, spacing 1/(N delta).  In the reference the spacing
    is an np.float64 (np.min(...) * delta), so the axis is float64 even though
    the integer ramp is float32 (grids.py:82-85)."""
    lo = (-N) // 2 + (N % 2)
    hi = N // 2 + (N % 2)
    df = 1.0 / (N * delta)
    return np.arange(lo, hi, dtype=np.float64) * df


def logpolar_base(points: int, f_min: float, f_max: float) -> np.ndarray:
    """Annulus outer radii f_i (grids.py:94-96), float32 as in the reference."""
    return np.exp(np.linspace(np.log(f_min), np.log(f_max), points, dtype=np.float32))


# ----------------------------------------------------------------------------
# turbulence model and annulus weights (theory/models.py:16-23, 80-85;
# phase_screens.py:82-91)
# ----------------------------------------------------------------------------
def mvk_psd_n(kappa, Cn2, l0, L0):
    k0 = 2 * np.pi / L0
    km = 5.92 / l0
    return 0.033 * Cn2 * np.exp(-(kappa / km) ** 2) / (kappa ** 2 + k0 ** 2) ** (11 / 6)


def psd_phi_f(f, k, thickness, Cn2, l0, L0):
    return 2 * np.pi * k ** 2 * thickness * mvk_psd_n(2 * np.pi * f, Cn2, l0, L0)


def annulus_psd(base: np.ndarray, k: float, thickness: float, Cn2: float, l0: float,
                L0: float, use_scipy: bool = True) -> np.ndarray:
    """Per-annulus weight 2*pi * int_{f_{i-1}}^{f_i} (2 pi)^2 f Phi_phi(f) df,
    f_{-1} = 0 (phase_screens.py:82-91).  scipy's quad when present, else a
    64-node Gauss-Legendre rule per annulus (annuli are narrow and the
    integrand smooth, so both agree to ~1e-12 relative)."""
    fb = [float(v) for v in base]

    def integrand(f):
        return (2 * np.pi) ** 2 * f * psd_phi_f(f, k, thickness, Cn2, l0, L0)

    quad = None
    if use_scipy:
        try:
            from scipy.integrate import quad  # noqa: F811
        except ImportError:  # pragma: no cover - the box may lack scipy
            quad = None
    out = np.empty(len(fb), dtype=np.float64)
    if quad is not None:
        for i in range(len(fb)):
            a = fb[i - 1] if i != 0 else 0.0
            out[i] = 2 * np.pi * quad(integrand, a, fb[i])[0]
    else:
        xg, wg = np.polynomial.legendre.leggauss(64)
        a = np.array([0.0] + fb[:-1])
        b = np.array(fb)
        mid, half = (a + b) / 2, (b - a) / 2
        f = mid[:, None] + half[:, None] * xg[None, :]
        out = 2 * np.pi * (integrand(f) * wg[None, :]).sum(axis=1) * half
    return out.astype(np.float32)


# ----------------------------------------------------------------------------
# seeded spectrum draws (grids.py:98-107 and phase_screens.py:98-103)
# ----------------------------------------------------------------------------
def draw_spectra(seed: int, realisations: Sequence[int], n_screens: int,
                 base: np.ndarray, psd: np.ndarray):
    """Per (realisation r, screen i) the reference draws one uniform u for the
    annulus radii, P uniforms for the angles and 2P normals for the complex
    amplitudes.  Here they come from numpy's default_rng([seed, r]) in that
    order, and rho / theta / value are formed with the reference's float32 /
    complex64 arithmetic.  Returns rho, theta (R, n, P) float32 and value
    (R, n, P) complex64."""
    base = np.asarray(base, dtype=np.float32)
    P = base.shape[0]
    f_prev = np.insert(base, 0, 0)[:-1]
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
            rho[j, i] = np.sqrt(f_prev ** 2 + u * (base ** 2 - f_prev ** 2))
            theta[j, i] = 2 * np.pi * t
            value[j, i] = (ab[0] + 1j * ab[1]).astype(np.complex64) * sq
    return rho, theta, value


# ----------------------------------------------------------------------------
# sparse-spectrum screen (phase_screens.py:108-126, :25-28 .real)
# ----------------------------------------------------------------------------
def ss_screen(rho, theta, value, N: int, delta: float, shift=(0.0, 0.0),
              prec: str = "fp64") -> np.ndarray:
    """phi[y, x] = Re sum_p value_p exp(i 2 pi fy_p y) exp(i 2 pi fx_p x)."""
    if prec == "ref":
        rho = np.asarray(rho, np.float32)
        theta = np.asarray(theta, np.float32)
        value = np.asarray(value, np.complex64)
        fx = (rho * np.cos(theta)).reshape((1, -1))
        fy = (rho * np.sin(theta)).reshape((-1, 1))
        x = rect_axis(N, delta, "ref").reshape((1, -1)) + shift[0]
        y = rect_axis(N, delta, "ref").reshape((-1, 1)) + shift[1]
        a = value * np.exp(1j * 2 * np.pi * (y @ fy.T))
        b = np.exp(1j * 2 * np.pi * (fx.T @ x))
        return (a @ b).real
    rho = np.asarray(rho, np.float64)
    theta = np.asarray(theta, np.float64)
    value = np.asarray(value, np.complex128)
    fx = rho * np.cos(theta)
    fy = rho * np.sin(theta)
    x = rect_axis(N, delta, "fp64") + float(shift[0])
    y = rect_axis(N, delta, "fp64") + float(shift[1])
    a = value[None, :] * np.exp(2j * np.pi * np.outer(y, fy))
    b = np.exp(2j * np.pi * np.outer(fx, x))
    return (a @ b).real


# ----------------------------------------------------------------------------
# FFT screen with subharmonics (phase_screens.py:42-67), draws injected
# ----------------------------------------------------------------------------
def fft_screen(normals: Sequence[np.ndarray], N: int, delta: float, k: float,
               thickness: float, Cn2: float, l0: float, L0: float,
               subharmonics: int, prec: str = "fp64") -> np.ndarray:
    """``normals`` holds, per level (0 = main grid, then one per subharmonic
    level), an array (2, n, n) of the standard normals the reference draws
    (real then imaginary part).  Returns the complex screen; ``.real`` is the
    phase used on the path."""
    cdt = np.complex64 if prec == "ref" else np.complex128

    def cn_coeff(level_normals, n, df):
        lo = (-n) // 2 + (n % 2)
        ax = np.arange(lo, lo + n, dtype=np.float64) * df
        rho = np.sqrt(ax[None, :] ** 2 + ax[:, None] ** 2)
        cn = (level_normals[0] + 1j * level_normals[1]).astype(cdt) * \
            np.sqrt(psd_phi_f(rho, k, thickness, Cn2, l0, L0)) * 2 * np.pi * df
        cn[n // 2, n // 2] = 0
        return cn

    df = 1.0 / (N * delta)
    cn = cn_coeff(normals[0], N, df)
    screen = np.fft.ifftshift(np.fft.ifft2(np.fft.ifftshift(cn))) * (N * 1) ** 2
    x = rect_axis(N, delta, prec).reshape((1, -1))
    y = rect_axis(N, delta, prec).reshape((-1, 1))
    for sh in range(subharmonics):
        sdf = df / 3 ** (sh + 1)
        c = cn_coeff(normals[sh + 1], 3, sdf)
        f = np.arange(-1, 2, dtype=np.float64) * sdf
        for i in range(3):
            for j in range(3):
                screen = screen + c[i, j] * np.exp(1j * 2 * np.pi * (f[i] * x + f[j] * y))
    return screen - np.mean(screen)


# ----------------------------------------------------------------------------
# source (sources.py:21-23, theory/sources.py:16-18)
# ----------------------------------------------------------------------------
def gaussian_source(N: int, delta: float, wvl: float, w0: float, F0: float,
                    prec: str = "fp64") -> np.ndarray:
    x = rect_axis(N, delta, prec).reshape((1, -1))
    y = rect_axis(N, delta, prec).reshape((-1, 1))
    r2 = x ** 2 + y ** 2
    c = 1 / w0 ** 2 + 1j * 2 * np.pi / wvl / 2 / F0
    if prec == "ref":
        return np.sqrt(2 / np.pi) / w0 * np.exp(-c * r2)
    return np.sqrt(2 / np.pi) / w0 * np.exp(-complex(c) * r2.astype(np.float64))


# ----------------------------------------------------------------------------
# angular-spectrum vacuum step (theory/vacuum.py:5-7, utils.py:42-50,
# pathes.py:27-40)
# ----------------------------------------------------------------------------
def vacuum(u: np.ndarray, dz: float, k: float, delta: float, prec: str = "fp64") -> np.ndarray:
    if not dz > 0:
        return u
    N = u.shape[0]
    fa = f_axis(N, delta)
    f2 = fa[None, :] ** 2 + fa[:, None] ** 2
    df = 1.0 / (N * delta)
    dz = np.float64(dz)
    H = np.exp(1j * k * dz) * np.exp(-1j * np.pi * dz * (2 * np.pi / k) * f2)
    if prec != "ref":
        u = u.astype(np.complex128)
    U = np.fft.fftshift(np.fft.fft2(np.fft.fftshift(u))) * delta ** 2
    out = np.fft.ifftshift(np.fft.ifft2(np.fft.ifftshift(H * U))) * (N * df) ** 2
    return out.astype(np.complex64) if prec == "ref" else out


# ----------------------------------------------------------------------------
# split-step path (pathes.py:19-24, 61-75, 78-95)
# ----------------------------------------------------------------------------
def screen_positions(length: float, count: int, position: str = "middle") -> np.ndarray:
    thickness = length / count
    if position == "before":
        return np.arange(count) * thickness
    if position == "middle":
        return (np.arange(count) + 1 / 2) * thickness
    if position == "after":
        return (np.arange(count) + 1) * thickness
    raise ValueError(position)


def _loss(u, losses_db):
    return u * 10 ** (-losses_db / 20) if losses_db else u


def propagate(u0: np.ndarray, screens: Sequence[np.ndarray], positions: Sequence[float],
              length: float, k: float, delta: float, losses_db: float = 0.0,
              path_output_loss: bool = True, prec: str = "fp64",
              keep_steps: bool = False):
    """Runs the split-step loop.  ``screens[i]`` is the real phase of screen i.
    The multiply by exp(-i phi) follows each vacuum step.  Loss semantics follow
    the reference literally: a step whose share of the loss is 0 falls back to
    the full path loss (``losses_db or self.losses_db``), and ``Channel.run``
    (``path_output_loss``) applies the full loss once more on exit."""
    u = u0
    steps = []
    for i, phi in enumerate(screens):
        dz = positions[i] - positions[i - 1] if i > 0 else positions[0]
        part = losses_db * dz / length
        v = vacuum(u, dz, k, delta, prec)
        if prec == "ref":
            ph = np.exp(-1j * np.asarray(phi, np.float32))
        else:
            ph = np.exp(-1j * np.asarray(phi, np.float64))
        u = _loss(ph * v, part or losses_db)
        if keep_steps:
            steps.append(u)
    u = vacuum(u, length - positions[-1], k, delta, prec)
    if path_output_loss:
        u = _loss(u, losses_db)
    return (u, steps) if keep_steps else u


# ----------------------------------------------------------------------------
# pupil and measures (pupils.py:8-13, measures.py:1-38, beam.py:26-33)
# ----------------------------------------------------------------------------
def pupil_mask(N: int, delta: float, radius: float, shift=(0.0, 0.0), prec: str = "fp64"):
    x = rect_axis(N, delta, prec).reshape((1, -1))
    y = rect_axis(N, delta, prec).reshape((-1, 1))
    return (x - shift[0]) ** 2 + (y + shift[1]) ** 2 <= radius ** 2


def measures(u: np.ndarray, delta: float, pupil_radii: Sequence[float] = (),
             prec: str = "fp64") -> dict:
    N = u.shape[0]
    x = rect_axis(N, delta, prec).reshape((1, -1))
    y = rect_axis(N, delta, prec).reshape((-1, 1))
    intensity = np.abs(u) ** 2
    if prec != "ref":
        intensity = intensity.astype(np.float64)
    d2 = delta ** 2
    out = {
        "eta_total": float(intensity.sum() * d2),
        "mean_x": float((intensity * x).sum() * d2),
        "mean_y": float((intensity * (-1) * y).sum() * d2),
        "mean_x2": float((intensity * x ** 2).sum() * d2),
        "mean_xy": float((intensity * (-1 * x * y)).sum() * d2),
        "mean_y2": float((intensity * y ** 2).sum() * d2),
    }
    for j, rad in enumerate(pupil_radii):
        out[f"eta_{j}"] = float((intensity * pupil_mask(N, delta, rad, prec=prec)).sum() * d2)
    out["mean_x2_r"] = mean_x2_r(intensity, delta, out["mean_x"], out["mean_y"], prec)
    return out


def mean_x2_r(intensity, delta, mx, my, prec="fp64"):
    """Second moment along the centroid direction (beam.py:26-33)."""
    N = intensity.shape[0]
    x = rect_axis(N, delta, prec).reshape((1, -1))
    y = rect_axis(N, delta, prec).reshape((-1, 1))
    r0 = np.sqrt(mx ** 2 + my ** 2)
    c, s = mx / r0, my / r0
    rot = (x * c + ((-1) * y) * s) ** 2
    return float((intensity * rot).sum() * delta ** 2)


# ----------------------------------------------------------------------------
# Monte-Carlo driver restatement: per-realisation measures for a channel
# ----------------------------------------------------------------------------
def simulate(spec: ChannelSpec, rho, theta, value, pupil_radii=None, prec="fp64",
             return_field=False, mean_intensity=False):
    """Runs R realisations with the injected spectra (R, n, P) and returns a list
    of measure dicts (plus, optionally, the last field and the mean
    intensity)."""
    pupil_radii = [spec.pupil_radius] if pupil_radii is None else list(pupil_radii)
    positions = screen_positions(spec.length, spec.count, spec.position)
    u0 = gaussian_source(spec.N, spec.delta, spec.wvl, spec.w0, spec.F0, prec)
    results = []
    mean_I = np.zeros((spec.N, spec.N)) if mean_intensity else None
    last = None
    for r in range(rho.shape[0]):
        screens = [ss_screen(rho[r, i], theta[r, i], value[r, i], spec.N, spec.delta, prec=prec)
                   for i in range(spec.count)]
        u = propagate(u0, screens, positions, spec.length, spec.k, spec.delta,
                      spec.losses_db, path_output_loss=False, prec=prec)
        results.append(measures(u, spec.delta, pupil_radii, prec))
        if mean_I is not None:
            mean_I += np.abs(u) ** 2
        last = u
    out = [results]
    if return_field:
        out.append(last)
    if mean_intensity:
        out.append(mean_I / rho.shape[0])
    return out[0] if len(out) == 1 else tuple(out)
