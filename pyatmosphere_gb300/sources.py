"""Sources (the reference's sources.py:7-23).  The engine generates the
source field itself from (wvl, w0, F0); ``output()`` materialises it for user
code."""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from .theory.sources import GaussianBeam

__all__ = ["Source", "PlaneSource", "GaussianSource"]


@dataclass
class Source:
    wvl: float

    @property
    def k(self):
        return 2 * np.pi / self.wvl


class PlaneSource(Source):
    kind = "plane"
    w0 = None
    F0 = float("inf")

    def output(self):
        return 1


class GaussianSource(GaussianBeam, Source):
    kind = "gaussian"

    def output(self):
        return self.amplitude(self.channel.grid.get_rho2())
