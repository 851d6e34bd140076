"""Phase screens (the reference's phase_screens.py:9-214) on the GB300 engine.

``SSPhaseScreen.generate`` returns the float32 screen computed by the engine
(``atm_screen``: FP64-exact phase wrap, Chebyshev collapse of the low annuli,
FP32 GEMM).  The spectrum is drawn in the reference's order from numpy's
global RNG, or can be injected by replacing ``_get_spectrum``.
"""
from __future__ import annotations

from typing import Tuple

import numpy as np

from . import gpu
from .utils import Default, PolarDiscreteFunction

__all__ = ["PhaseScreen", "SSPhaseScreen", "FFTPhaseScreen", "SUPhaseScreen"]


class PhaseScreen:
    wvl = Default("channel.source.wvl")
    grid = Default("channel.grid")

    def __init__(self, model, thickness=None, wvl=None, grid=None):
        self.model = model
        self.thickness = thickness
        if wvl:
            self.wvl = wvl
        if grid:
            self.grid = grid

    def generate_phase_screen(self, *args, **kwargs):
        raise NotImplementedError

    def generate(self, complex=False, *args, **kwargs):
        ps = self.generate_phase_screen(*args, **kwargs)
        if complex:
            return ps
        return ps.real if hasattr(ps, "is_complex") and ps.is_complex() else ps

    def generator(self, *args, **kwargs):
        while True:
            ps = self.generate(complex=True, *args, **kwargs)
            yield ps.real
            if hasattr(ps, "is_complex") and ps.is_complex():
                yield ps.imag


class SSPhaseScreen(PhaseScreen):
    """Sparse-spectrum screen: sum of random cosines over a RandLogPolarGrid."""

    def __init__(self, f_grid, *args, **kwargs):
        super().__init__(*args, **kwargs)
        self.f_grid = f_grid
        self._psd = None
        self._psd_key = None
        self.cache_clear()

    def cache_clear(self):
        self._cached_spectrum = None
        self._cached_phase_screen = None
        self._cached_phase_screen_shift = 0

    def _get_psd(self):
        """Annulus weights (phase_screens.py:82-91), cached per screen."""
        from .engine.spectra import annulus_psd
        key = (self.wvl, self.thickness, id(self.model), self.model.Cn2, self.model.l0, self.model.L0,
               self.f_grid.points, self.f_grid.f_min, self.f_grid.f_max)
        if self._psd is None or self._psd_key != key:
            self._psd = annulus_psd(self.f_grid.base, self.model.psd_phi_f, 2 * np.pi / self.wvl, self.thickness)
            self._psd_key = key
        return self._psd

    def _get_spectrum(self, use_cached_spectrum):
        if use_cached_spectrum and self._cached_spectrum:
            return self._cached_spectrum
        P = self.f_grid.points
        spectrum = PolarDiscreteFunction(
            rho=self.f_grid.get_rho(),
            theta=self.f_grid.get_theta(),
            value=(np.array([1, 1j]) @ np.random.normal(size=(2, P))).astype(np.complex64)
            * np.sqrt(self._get_psd()))
        if use_cached_spectrum and not self._cached_spectrum:
            self._cached_spectrum = spectrum
        return spectrum

    def _engine_plan(self, shift):
        from .engine.plan import EnginePlan
        N, delta = self.grid.N, float(self.grid.delta)
        key = (N, delta, float(shift[0]), float(shift[1]), self.f_grid.base.tobytes(), str(gpu.device()))
        if getattr(self, "_plan_key", None) != key:
            self._plan = EnginePlan(N, delta, float(self.wvl), 1.0, float("inf"), [0.0], 1.0,
                                    f_base=self.f_grid.base, shift=shift, batch=1,
                                    cheb_cut=gpu.config.get("cheb_cut", 0.0), device=gpu.device())
            self._plan_key = key
        return self._plan

    def generate_with_phasor(self, shift: Tuple[float, float] = (0, 0), wind: bool = False):
        """(phi, exp(-i phi)) of one spectrum draw: the float32 screen the
        reference returns and the phasor the path applies, which the engine
        builds from FP64 phases (more accurate than exp(-i phi) of the float32
        screen, whose piston reaches ~1e3 rad)."""
        import torch
        from .engine.runner import to_device
        sp = self._get_spectrum(use_cached_spectrum=wind)
        plan = self._engine_plan(shift)
        rho, theta, value = to_device(np.asarray(sp.rho, np.float32).reshape(1, 1, -1),
                                      np.asarray(sp.theta, np.float32).reshape(1, 1, -1),
                                      np.asarray(sp.value, np.complex64).reshape(1, 1, -1))
        N = plan.N
        phi = torch.empty((1, N, N), dtype=torch.float32, device=plan.device)
        ph = torch.empty((1, N, N), dtype=torch.complex64, device=plan.device)
        plan.screen(rho, theta, value, 0, phi_out=phi, phasor_out=ph)
        if wind:
            self._cached_phase_screen = phi[0]
            self._cached_phase_screen_shift = shift[0]
        return phi[0], ph[0]

    def generate_phase_screen(self, shift: Tuple[float, float] = (0, 0), wind: bool = False):
        """float32 screen [N, N] (torch, on the engine device)."""
        return self.generate_with_phasor(shift=shift, wind=wind)[0]


class FFTPhaseScreen(PhaseScreen):
    """FFT screen with 3x3 subharmonic levels (phase_screens.py:37-67)."""

    def __init__(self, subharmonics, *args, **kwargs):
        self.subharmonics = subharmonics
        super().__init__(*args, **kwargs)

    def draw_normals(self):
        """Standard normals in the reference's draw order (real then imaginary
        part, main grid then each subharmonic level)."""
        from .engine.fft_screen import draw_normals
        return draw_normals(self.grid.N, self.subharmonics)

    def generate_phase_screen(self, *args, normals=None, **kwargs):
        from .engine.fft_screen import fft_screen
        normals = self.draw_normals() if normals is None else normals
        return fft_screen(self, normals)


class SUPhaseScreen(PhaseScreen):
    """Sparse-uniform screen (phase_screens.py:154-179): the same separable
    sum with amplitudes sqrt(Phi_phi(rho) pi (2 pi)^2 (f_i^2 - f_{i-1}^2))
    evaluated at the drawn radius; runs on the SS engine path."""

    def __init__(self, f_grid, *args, **kwargs):
        self.f_grid = f_grid
        super().__init__(*args, **kwargs)

    def generate_phase_screen(self, shift=(0, 0), wind=False):
        ss = SSPhaseScreen(self.f_grid, self.model, thickness=self.thickness, wvl=self.wvl, grid=self.grid)
        rho = self.f_grid.get_rho()
        theta = self.f_grid.get_theta()
        base = self.f_grid.base
        dk = (2 * np.pi) ** 2 * (base ** 2 - np.insert(base, 0, 0)[:-1] ** 2).astype(np.float32)
        cn = (np.array([1, 1j]) @ np.random.normal(size=(2, self.f_grid.points))).astype(np.complex64) * \
            np.sqrt(self.model.psd_phi_f(rho, 2 * np.pi / self.wvl, self.thickness) * np.pi * dk)
        ss._get_spectrum = lambda use_cached_spectrum: PolarDiscreteFunction(rho, theta, cn.astype(np.complex64))
        return ss.generate_phase_screen(shift=shift)
