"""Beam statistics (simulations/beam.py:14-140)."""
from __future__ import annotations

from typing import Sequence, Tuple

import numpy as np

from .. import gpu
from ..measures import I, mean_r, mean_r2, mean_x, mean_x2, mean_xy, mean_y, mean_y2
from .measure import Measure
from .result import Result


class BeamResult(Result):
    def __init__(self, channel, **kwargs):
        measures = [
            Measure(channel, "atmosphere", mean_x),
            Measure(channel, "atmosphere", mean_y),
            Measure(channel, "atmosphere", mean_x2),
            Measure(channel, "atmosphere", mean_xy),
            Measure(channel, "atmosphere", mean_y2),
            Measure(channel, "atmosphere", self.mean_x2_r, name="mean_x2_r"),
        ]
        super().__init__(channel, measures, **kwargs)

    def mean_x2_r(self, channel, output):
        """Second moment along this realisation's centroid direction, from the
        moments (cos^2 mx2 + 2 cos sin mxy + sin^2 my2 with mean_xy weighted by
        -x y, as beam.py:26-33 evaluates it pixel by pixel)."""
        mx, my = self.measures[0].iteration_data, self.measures[1].iteration_data
        r0 = np.sqrt(mx ** 2 + my ** 2)
        c, s = mx / r0, my / r0
        return float(c * c * mean_x2(channel, output=output) + 2 * c * s * mean_xy(channel, output=output)
                     + s * s * mean_y2(channel, output=output))

    @property
    def bw2(self) -> Sequence[float]:
        return np.asarray(self.measures[0]) ** 2

    @property
    def lt2(self) -> Sequence[float]:
        return 4 * np.asarray(self.measures[2])

    @property
    def st2(self) -> Sequence[float]:
        return self.lt2 - 4 * self.bw2

    @staticmethod
    def _stat(x2) -> Tuple[float, float]:
        mean = np.sqrt(x2.mean())
        d2 = x2.std(ddof=1) / np.sqrt(len(x2))
        return mean, d2 / 2 / mean

    @property
    def bw(self):
        return self._stat(self.bw2)

    @property
    def lt(self):
        return self._stat(self.lt2)

    @property
    def st(self):
        return self._stat(self.st2)

    def print_output(self):
        bw, lt, st = self.bw, self.lt, self.st
        print(f"sigma_BW_x = {bw[0]:.1e} +- {bw[1]:.1e}")
        print(f"sigma_LT_x = {lt[0]:.1e} +- {lt[1]:.1e}")
        print(f"W_ST = {st[0]:.1e} +- {st[1]:.1e}")
        print(f"Count of measures: {len(self.measures[0])}")


class BeamPropagationResult(Result):
    """Centroid and width after every screen and at the receiver
    (simulations/beam.py:83-140; uses the restored mean_r / mean_r2).  The
    theory curves of the reference (beam wandering, long-term width) are not
    computed here."""

    def __init__(self, channel, **kwargs):
        measures = [Measure(channel, "propagation", mean_r), Measure(channel, "propagation", mean_r2)]
        super().__init__(channel, measures, **kwargs)

    @property
    def bw2(self):
        return np.asarray(self.measures[0]) ** 2

    @property
    def lt2(self):
        return 2 * np.asarray(self.measures[1])

    @property
    def st2(self):
        return self.lt2 - self.bw2

    @property
    def positions(self):
        return np.array(list(self.channel.path.positions) + [self.channel.path.length])
