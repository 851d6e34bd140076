"""Time coherence under wind shifts (simulations/wind.py:13-66)."""
from __future__ import annotations

from typing import Sequence

import numpy as np

from ..measures import eta, mean_x, mean_y
from .measure import Measure
from .result import Result


class WindResult(Result):
    def load_output(self):
        for measures, col in zip(self.measures, self.csv_columns()):
            measures.data = [[float(v) for v in c[1:-1].split(", ")] for c in col if c.strip()]


class TimeCoherenceResult(WindResult):
    def __init__(self, channel, time, *args, **kwargs):
        measures = [Measure(channel, "pupil", eta, time=time)]
        super().__init__(*args, channel=channel, measures=measures, **kwargs)

    @property
    def tc(self) -> Sequence[float]:
        from scipy.stats import pearsonr
        a = np.asarray(self.measures[0], dtype=float)
        return [pearsonr(a[:, 0], a[:, i])[0] for i in range(len(self.measures[0].time))]


class TimeBWcorrSimulation(WindResult):
    def __init__(self, channel, time, *args, **kwargs):
        measures = [Measure(channel, "atmosphere", mean_x, time=time),
                    Measure(channel, "atmosphere", mean_y, time=time)]
        super().__init__(*args, channel=channel, measures=measures, **kwargs)

    @property
    def xx(self):
        a = np.asarray(self.measures[0], dtype=float)
        return 2 * np.sqrt((a[:, 0, None] * a).mean(axis=0))

    @property
    def yy(self):
        a = np.asarray(self.measures[1], dtype=float)
        return 2 * np.sqrt((a[:, 0, None] * a).mean(axis=0))

    @property
    def xy(self):
        a = np.asarray(self.measures[0], dtype=float)
        b = np.asarray(self.measures[1], dtype=float)
        return 2 * np.sqrt(abs((a[:, 0, None] * b).mean(axis=0)))
