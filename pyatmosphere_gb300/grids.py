"""Grids (the reference's grids.py:7-119).

``RectGrid`` coordinates are float32 like the reference's, returned as torch
tensors on the engine's device.  ``RandLogPolarGrid`` draws from numpy's
global RNG in the reference's order, so ``np.random.seed(s)`` reproduces the
reference's spectra.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from . import gpu

__all__ = ["Grid", "RectGrid", "RandLogPolarGrid"]


class Grid:
    def get_array_module(self):
        return gpu.get_xp()


@dataclass
class RectGrid(Grid):
    resolution: tuple
    delta: float

    def __post_init__(self):
        if isinstance(self.resolution, (int, np.integer)):
            self.resolution = (int(self.resolution), int(self.resolution))
        else:
            self.resolution = tuple(self.resolution)

    @property
    def size(self):
        return np.array(self.resolution) * self.delta

    @property
    def extent(self):
        return np.array([self._left_bound, self._right_bound, self._top_bound, self._bottom_bound]) * self.delta

    @property
    def shape(self):
        return self.resolution

    @property
    def origin_index(self):
        return (self.resolution[0] // 2, self.resolution[1] // 2)

    @property
    def _left_bound(self):
        return -self.resolution[0] // 2 + bool(self.resolution[0] % 2)

    @property
    def _right_bound(self):
        return self.resolution[0] // 2 + bool(self.resolution[0] % 2)

    @property
    def _top_bound(self):
        return -self.resolution[1] // 2 + bool(self.resolution[1] % 2)

    @property
    def _bottom_bound(self):
        return self.resolution[1] // 2 + bool(self.resolution[1] % 2)

    def _axis(self, lo, hi):
        import torch
        return torch.arange(lo, hi, dtype=torch.float32, device=gpu.device()) * np.float32(self.delta)

    def get_NxNy(self):
        import torch
        d = gpu.device()
        return (torch.arange(self._top_bound, self._bottom_bound, device=d).reshape(-1, 1),
                torch.arange(self._left_bound, self._right_bound, device=d).reshape(1, -1))

    def get_N2(self):
        Nx, Ny = self.get_NxNy()
        return Nx ** 2 + Ny ** 2

    def get_x(self):
        return self._axis(self._left_bound, self._right_bound).reshape((1, -1))

    def get_y(self):
        return self._axis(self._top_bound, self._bottom_bound).reshape((-1, 1))

    def get_xy(self):
        return self.get_x(), self.get_y()

    def get_rho2(self):
        x, y = self.get_xy()
        return x ** 2 + y ** 2

    def get_rho(self):
        return self.get_rho2().sqrt()

    def get_f_grid(self):
        return RectGrid(resolution=int(np.min(self.resolution)),
                        delta=1 / (np.min(self.resolution) * self.delta))

    # engine helpers ------------------------------------------------------
    @property
    def N(self) -> int:
        if self.resolution[0] != self.resolution[1]:
            raise ValueError("the engine needs a square grid")
        return int(self.resolution[0])


@dataclass
class RandLogPolarGrid(Grid):
    points: int
    f_min: float
    f_max: float

    @property
    def base(self):
        return np.exp(np.linspace(np.log(self.f_min), np.log(self.f_max), self.points, dtype=np.float32))

    def rho_from(self, u):
        """Annulus radii for one uniform draw u (grids.py:98-103)."""
        f = self.base
        f_prev = np.insert(f, 0, 0)[:-1]
        return np.sqrt(f_prev ** 2 + np.asarray(u, np.float32) * (f ** 2 - f_prev ** 2))

    def get_rho(self):
        return self.rho_from(np.random.random(size=(1,)).astype(np.float32))

    def get_theta(self):
        return 2 * np.pi * np.random.random(size=(self.points,)).astype(np.float32)

    def get_x(self, rho, theta):
        return rho * np.cos(theta)

    def get_y(self, rho, theta):
        return rho * np.sin(theta)

    def get_xy(self, rho, theta):
        return (rho * np.cos(theta)).reshape((1, -1)), (rho * np.sin(theta)).reshape((-1, 1))
