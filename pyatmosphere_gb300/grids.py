"""Sample grids of a channel: the spatial grid of the field and the random
log-polar grid of the sparse screen spectrum (the reference's
grids.py:7-119 offers the same classes and methods).

RectGrid puts sample j of an axis of n points at (j - n // 2) * delta, the
x axis along the columns (resolution[0] points) and the y axis down the rows
(resolution[1] points).  Coordinates are float32 products of the index and
delta, the values the reference's float32 aranges produce, returned as torch
tensors on the engine device.

RandLogPolarGrid draws its annulus radii and angles from numpy's global
generator, one uniform for all radii and one uniform per angle, in the order
the reference draws them, so that ``np.random.seed(s)`` gives the reference's
spectra.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from . import gpu

__all__ = ["Grid", "RectGrid", "RandLogPolarGrid"]


class Grid:
    """Base of the grids: the array module their outputs belong to."""

    def get_array_module(self):
        return gpu.get_xp()


def _centred(n: int) -> np.ndarray:
    """Sample indices of an n-point axis, relative to its origin sample n // 2."""
    return np.arange(n, dtype=np.int64) - n // 2


@dataclass
class RectGrid(Grid):
    resolution: tuple
    delta: float

    def __post_init__(self):
        if np.ndim(self.resolution) == 0:
            n = int(self.resolution)
            self.resolution = (n, n)
        else:
            self.resolution = tuple(int(n) for n in self.resolution)

    # ---- geometry in metres and samples ----------------------------------
    @property
    def shape(self):
        return self.resolution

    @property
    def size(self):
        return np.asarray(self.resolution, dtype=float) * self.delta

    @property
    def origin_index(self):
        return tuple(n // 2 for n in self.resolution)

    @property
    def extent(self):
        """(first x, last x + delta, first y, last y + delta): the extent
        matplotlib's imshow takes."""
        edges = []
        for n in self.resolution:
            idx = _centred(n)
            edges += [idx[0], idx[-1] + 1]
        return np.asarray(edges, dtype=float) * self.delta

    # ---- coordinate arrays (torch, engine device) ------------------------
    def _coordinates(self, n: int):
        import torch
        idx = torch.from_numpy(_centred(n).astype(np.float32)).to(gpu.device())
        return idx * self.delta  # one float32 product per sample

    def get_x(self):
        return self._coordinates(self.resolution[0]).reshape(1, -1)

    def get_y(self):
        return self._coordinates(self.resolution[1]).reshape(-1, 1)

    def get_xy(self):
        return self.get_x(), self.get_y()

    def get_rho2(self):
        x, y = self.get_xy()
        return x * x + y * y

    def get_rho(self):
        return self.get_rho2().sqrt()

    def get_NxNy(self):
        """Integer sample indices: a column of y indices and a row of x indices."""
        import torch
        d = gpu.device()
        iy = torch.from_numpy(_centred(self.resolution[1])).to(d).reshape(-1, 1)
        ix = torch.from_numpy(_centred(self.resolution[0])).to(d).reshape(1, -1)
        return iy, ix

    def get_N2(self):
        iy, ix = self.get_NxNy()
        return iy * iy + ix * ix

    def get_f_grid(self):
        """The reciprocal grid of the FFT: the smaller resolution n, step 1 / (n delta)."""
        n = int(min(self.resolution))
        return RectGrid(resolution=n, delta=1 / (n * self.delta))

    # ---- engine helper -----------------------------------------------------
    @property
    def N(self) -> int:
        nx, ny = self.resolution
        if nx != ny:
            raise ValueError(f"the engine propagates square grids only, not {nx} x {ny}")
        return int(nx)


@dataclass
class RandLogPolarGrid(Grid):
    points: int
    f_min: float
    f_max: float

    @property
    def base(self):
        """Outer radii [1/m] of the `points` annuli, log-spaced from f_min to
        f_max, float32."""
        log_lo, log_hi = np.log(self.f_min), np.log(self.f_max)
        return np.exp(np.linspace(log_lo, log_hi, self.points, dtype=np.float32))

    def rho_from(self, u):
        """Annulus radii for one uniform u in [0, 1): radius i sits at the
        fraction u of annulus i's area, in float32."""
        outer = self.base
        inner = np.concatenate([np.zeros(1, np.float32), outer[:-1]])
        inner2, outer2 = inner ** 2, outer ** 2
        return np.sqrt(inner2 + np.asarray(u, np.float32) * (outer2 - inner2))

    def get_rho(self):
        return self.rho_from(np.random.random(size=(1,)).astype(np.float32))

    def get_theta(self):
        return 2 * np.pi * np.random.random(size=(self.points,)).astype(np.float32)

    @staticmethod
    def _components(rho, theta):
        return rho * np.cos(theta), rho * np.sin(theta)

    def get_x(self, rho, theta):
        return self._components(rho, theta)[0]

    def get_y(self, rho, theta):
        return self._components(rho, theta)[1]

    def get_xy(self, rho, theta):
        fx, fy = self._components(rho, theta)
        return fx.reshape(1, -1), fy.reshape(-1, 1)
