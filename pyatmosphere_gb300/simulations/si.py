"""On-axis scintillation index per propagation position (simulations/si.py)."""
from __future__ import annotations

import numpy as np

from .. import gpu
from .measure import Measure
from .result import Result


def intensity_at_center(channel, output):
    i, j = channel.grid.origin_index
    return float(abs(output[i, j]) ** 2)


class SIResult(Result):
    def __init__(self, channel, theoretical_functions=(), *args, **kwargs):
        measures = [Measure(channel, "propagation", intensity_at_center)]
        super().__init__(*args, channel=channel, measures=measures, **kwargs)
        self.theoretical_functions = theoretical_functions

    @property
    def intensities_at_center(self):
        return np.asarray(self.measures[0], dtype=float)

    @property
    def positions(self):
        return np.array(list(self.channel.path.positions) + [self.channel.path.length])

    @property
    def si(self):
        ic = self.intensities_at_center
        return (ic ** 2).mean(axis=0) / ic.mean(axis=0) ** 2 - 1
