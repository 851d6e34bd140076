"""Maps a Channel object graph to engine plans and spectra.

A plan is built per (geometry, batch, pupils, screen shift, loss mode) and
cached on the channel.  Spectra are taken from each screen's
``_get_spectrum`` (numpy global RNG in the reference's draw order, or an
injected spectrum) and stacked as [batch][n_screens][P].
"""
from __future__ import annotations

from typing import List, Sequence, Tuple

import numpy as np

from .. import gpu
from . import _lib


def _path_geometry(channel):
    from ..pathes import PhaseScreensPath, VacuumPath
    path = channel.path
    if isinstance(path, PhaseScreensPath):
        screens = path.phase_screens
        from ..phase_screens import SSPhaseScreen
        if not all(isinstance(s, SSPhaseScreen) for s in screens):
            raise NotImplementedError("the batched engine path needs SSPhaseScreen screens")
        bases = [np.asarray(s.f_grid.base, np.float32) for s in screens]
        if any(b.shape != bases[0].shape or not np.array_equal(b, bases[0]) for b in bases):
            raise NotImplementedError("all screens of a path must share one RandLogPolarGrid")
        return list(map(float, path.positions)), float(path.length), float(path.losses_db or 0.0), bases[0]
    if isinstance(path, VacuumPath):
        return [], float(path.length), float(path.losses_db or 0.0), None
    raise NotImplementedError(f"unsupported path type {type(path).__name__}")


def _source(channel):
    from ..sources import GaussianSource, PlaneSource
    s = channel.source
    if isinstance(s, GaussianSource):
        return "gaussian", float(s.wvl), float(s.w0), float(s.F0)
    if isinstance(s, PlaneSource):
        return "plane", float(s.wvl), 0.0, float("inf")
    raise NotImplementedError(f"unsupported source type {type(s).__name__}")


def get_plan(channel, batch: int = 1, pupils: Sequence[tuple] = (), tracked: Sequence[float] = (),
             shift=(0.0, 0.0), path_output_loss: bool = False, length=None, step_measures: bool = False):
    from .plan import EnginePlan
    gpu.require_engine()
    positions, L, losses, base = _path_geometry(channel)
    if length is not None:
        L = float(length)
    kind, wvl, w0, F0 = _source(channel)
    N, delta = channel.grid.N, float(channel.grid.delta)
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
                          device=gpu.device(), flags=_lib.FLAG_STEP_MEASURES if step_measures else 0)
        cache[key] = plan
    return plan


def draw_channel_spectra(channel, realisations: int, wind: bool = False, clear: bool = True):
    """Spectra of `realisations` consecutive realisations, drawn like the
    reference's Simulation.iter does (cache_clear, then each screen's
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


def to_device(*arrays):
    import torch
    d = gpu.device()
    return [torch.from_numpy(np.ascontiguousarray(a)).to(d, non_blocking=False) for a in arrays]
