"""Maps a channel object graph onto engine plans and spectra.

The channel may be this package's Channel or the reference package's own
(channels.py:17-29): both expose the same attributes, which is all this
module reads -- grid.resolution / delta, source.wvl / w0 / F0,
path.length / losses_db / positions / phase_screens, and per screen
f_grid.base and _get_spectrum.  A plan is built per (geometry, batch,
pupils, screen shift, loss mode) and cached on the channel.  Spectra come
from each screen's ``_get_spectrum`` (numpy's global generator in the
reference's draw order, or an injected spectrum), stacked [batch][n][P].
"""
from __future__ import annotations

import numpy as np

from .. import gpu
from . import _lib


def grid_size(grid) -> int:
    """N of a square grid (RectGrid.resolution is an int or a pair)."""
    res = grid.resolution
    nx, ny = (res, res) if np.ndim(res) == 0 else (res[0], res[1])
    if int(nx) != int(ny):
        raise NotImplementedError(f"the engine propagates square grids only, not {nx} x {ny}")
    return int(nx)


def source_kind(source):
    """('gaussian' | 'plane', wvl, w0, F0) of a GaussianSource / PlaneSource."""
    name = type(source).__name__
    if name == "GaussianSource":
        return "gaussian", float(source.wvl), float(source.w0), float(source.F0)
    if name == "PlaneSource":
        return "plane", float(source.wvl), 0.0, float("inf")
    raise NotImplementedError(f"unsupported source type {name}")


def path_geometry(path):
    """(screen positions, length, losses_db, annulus radii or None) of a
    VacuumPath or a path of sparse-spectrum screens sharing one spectral grid."""
    screens = getattr(path, "phase_screens", None)
    if screens is None:
        if type(path).__name__ != "VacuumPath":
            raise NotImplementedError(f"unsupported path type {type(path).__name__}")
        return [], float(path.length), float(path.losses_db or 0.0), None
    if screen_kind(path) == "fft":
        # FFT screens (atm_run_fft): the plan's spectral grid is a placeholder
        return [float(p) for p in path.positions], float(path.length), float(path.losses_db or 0.0), _FFT_BASE
    if not all(type(s).__name__ == "SSPhaseScreen" for s in screens):
        raise NotImplementedError("the fused engine path takes SSPhaseScreen or FFTPhaseScreen screens")
    bases = [np.asarray(s.f_grid.base, np.float32) for s in screens]
    if any(not np.array_equal(b, bases[0]) for b in bases):
        raise NotImplementedError("all screens of a path must share one RandLogPolarGrid")
    return [float(p) for p in path.positions], float(path.length), float(path.losses_db or 0.0), bases[0]


_FFT_BASE = np.ones(1, np.float32)


def screen_kind(path) -> str:
    """'vacuum', 'fft' (every screen an FFTPhaseScreen with one subharmonic
    count) or 'ss'."""
    screens = getattr(path, "phase_screens", None)
    if screens is None:
        return "vacuum"
    if all(type(s).__name__ == "FFTPhaseScreen" for s in screens) and \
            len({int(s.subharmonics) for s in screens}) == 1:
        return "fft"
    return "ss"


def fusable(channel) -> bool:
    """Whether the fused engine call (atm_run) serves the channel."""
    try:
        source_kind(channel.source)
        path_geometry(channel.path)
        grid_size(channel.grid)
    except NotImplementedError:
        return False
    return True


def get_plan(channel, batch: int = 1, pupils=(), tracked=(), shift=(0.0, 0.0), path_output_loss: bool = False,
             length=None, step_measures: bool = False):
    from .plan import EnginePlan
    gpu.require_engine()
    positions, L, losses, base = path_geometry(channel.path)
    if length is not None:
        L = float(length)
    kind, wvl, w0, F0 = source_kind(channel.source)
    N, delta = grid_size(channel.grid), float(channel.grid.delta)
    key = (N, delta, kind, wvl, w0, F0, tuple(positions), L, losses,
           None if base is None else base.tobytes(), int(batch), tuple(map(tuple, pupils)), tuple(tracked),
           (float(shift[0]), float(shift[1])), bool(path_output_loss), gpu.config.get("cheb_cut", 0.0),
           str(gpu.device()), bool(step_measures))
    cache = channel.__dict__.setdefault("_atm_plans", {})
    plan = cache.get(key)
    if plan is None:
        if len(cache) > 16:
            for p in cache.values():
                p.close()
            cache.clear()
        plan = EnginePlan(N, delta, wvl, w0, F0, positions, L, f_base=base, losses_db=losses,
                          path_output_loss=path_output_loss, shift=shift, pupils=pupils, tracked=tracked,
                          batch=batch, source=kind, cheb_cut=gpu.config.get("cheb_cut", 0.0),
                          device=gpu.device(),
                          flags=(_lib.FLAG_STEP_MEASURES if step_measures else 0) |
                          (_lib.FLAG_FFT_SCREENS if screen_kind(channel.path) == "fft" else 0))
        cache[key] = plan
    return plan


def draw_channel_spectra(channel, realisations: int, wind: bool = False, clear: bool = True):
    """Spectra of `realisations` consecutive realisations, drawn as the
    per-realisation loop draws them (cache_clear, then each screen's
    _get_spectrum in path order).  Returns numpy (rho, theta, value)."""
    screens = channel.path.phase_screens
    n, P = len(screens), screens[0].f_grid.points
    rho = np.empty((realisations, n, P), np.float32)
    theta = np.empty((realisations, n, P), np.float32)
    value = np.empty((realisations, n, P), np.complex64)
    for r in range(realisations):
        for i, ps in enumerate(screens):
            if clear:
                ps.cache_clear()
            sp = ps._get_spectrum(use_cached_spectrum=wind)
            rho[r, i], theta[r, i], value[r, i] = sp.rho, sp.theta, sp.value
    return rho, theta, value


def draw_channel_fft(channel, realisations: int):
    """Inputs of atm_run_fft for `realisations` consecutive realisations of a
    path of FFT screens, drawn as the per-realisation loop draws them (per
    realisation each screen in path order, numpy's global generator):
    (normals [R][n][2][N][N] float32, amp [n][N][N] float32, sub_x, sub_y
    [R][n][n_sub][N] complex64, sub_mean [R][n][2] float64, n_sub)."""
    from .fft_screen import draw_normals, screen_amplitude, subharmonic_factors
    screens = channel.path.phase_screens
    N, delta = grid_size(channel.grid), float(channel.grid.delta)
    n, levels = len(screens), int(screens[0].subharmonics)
    n_sub = 3 * levels
    k = [2 * np.pi / float(_screen_wvl(ps, channel)) for ps in screens]
    amp = np.stack([screen_amplitude(N, delta, ps.model.psd_phi_f, k[i], ps.thickness)
                    for i, ps in enumerate(screens)])
    normals = np.empty((realisations, n, 2, N, N), np.float32)
    sub_x = np.zeros((realisations, n, max(n_sub, 1), N), np.complex64)
    sub_y = np.zeros_like(sub_x)
    sub_mean = np.zeros((realisations, n, 2), np.float64)
    for r in range(realisations):
        for i, ps in enumerate(screens):
            nrm = draw_normals(N, levels)
            normals[r, i] = nrm[0]
            X, Y, mean = subharmonic_factors(N, delta, ps.model.psd_phi_f, k[i], ps.thickness, nrm[1:])
            if n_sub:
                sub_x[r, i], sub_y[r, i] = np.array(X), np.array(Y)
            sub_mean[r, i] = mean.real, mean.imag
    return normals, amp, sub_x, sub_y, sub_mean, n_sub


def run_single(channel, plan, field_out, wind: bool = False, clear: bool = False):
    """One realisation of `channel` on `plan` (batch 1) into field_out, its
    screens drawn as the reference's loop draws them."""
    if plan.n_screens == 0:
        return plan.run(None, None, None, field_out=field_out)
    channel.path.init_phase_screens()
    if screen_kind(channel.path) == "fft":
        normals, amp, sub_x, sub_y, sub_mean, n_sub = draw_channel_fft(channel, 1)
        return plan.run_fft(*to_device(normals, amp, sub_x, sub_y, sub_mean), n_sub, field_out=field_out)
    return plan.run(*to_device(*draw_channel_spectra(channel, 1, wind=wind, clear=clear)), field_out=field_out)


def _screen_wvl(ps, channel):
    try:
        w = ps.wvl
    except Exception:  # a screen whose wavelength defaults to the channel's source
        w = None
    return w if w else channel.source.wvl


def to_device(*arrays):
    import torch
    d = gpu.device()
    return [torch.from_numpy(np.ascontiguousarray(a)).to(d, non_blocking=False) for a in arrays]
