"""Probability distribution of transmittance (the reference's
simulations/pdt.py:11-66 offers the same result classes).

PDTResult measures, per realisation, the power transmitted through each of
its circular pupils: the receiver field times the pupil mask, then ``eta``.
TrackedPDTResult first measures the beam centroid of the realisation and
centres every pupil on it.  The pupil shift convention is CirclePupil's:
(x - sx)^2 + (y + sy)^2 <= R^2 with (sx, sy) = (mean_x, mean_y).
"""
from __future__ import annotations

import numpy as np

from ..measures import eta, mean_x, mean_y
from .measure import Measure
from .result import Result


class PupilStop:
    """Operation of a PDT measure chain: the field behind one pupil of a PDT
    result, displaced by the result's current pupil shift."""

    def __init__(self, result, pupil):
        self.result = result
        self.pupil = pupil
        self.__name__ = f"pupil_{pupil.radius}"

    def __call__(self, channel, output):
        return self.result.append_pupil(self.pupil, channel, output)


class PDTResult(Result):
    def __init__(self, channel, pupils: list = None, **kwargs):
        self.pupil_shift = (0, 0)
        self.pupils = list(pupils) if pupils else [channel.pupil]
        measures = kwargs.pop("measures", None)
        if measures is None:
            measures = [Measure(channel, "atmosphere", PupilStop(self, p), eta, name=f"{p.radius}")
                        for p in self.pupils]
        super().__init__(channel, measures, **kwargs)

    def append_pupil(self, pupil, channel, output):
        """The field behind `pupil` (shifted by pupil_shift) on `channel`'s grid."""
        pupil.channel = channel
        return pupil.output(output, shift=self.pupil_shift)

    def histogram(self, i=0, bins=200, range=(0, 1)):
        return np.histogram(np.asarray(self.measures[i].data, dtype=float), bins=bins, range=range)

    def plot_output(self):
        try:
            from matplotlib import pyplot as plt
        except ImportError:
            self.print_output()
            return
        pdt = [m for m in self.measures if m.operations and m.operations[-1] is eta]
        fig, axes = plt.subplots(1, len(pdt), figsize=(5 * len(pdt), 3), squeeze=False)
        for ax, m in zip(axes[0], pdt):
            ax.hist(np.asarray(m.data, dtype=float), bins=200 if len(pdt) == 1 else 100, range=(0, 1),
                    label=f"R = {m.name} m, {len(m)} realisations")
            ax.legend()
        plt.show()


class TrackedPDTResult(PDTResult):
    def __init__(self, channel, pupils: list = None, **kwargs):
        pupils = list(pupils) if pupils else [channel.pupil]
        centroid = [Measure(channel, "atmosphere", mean_x), Measure(channel, "atmosphere", mean_y)]
        transmitted = [Measure(channel, "atmosphere", self.set_pupil_position, PupilStop(self, p), eta,
                               name=f"{p.radius}") for p in pupils]
        super().__init__(channel, pupils=pupils, measures=centroid + transmitted, **kwargs)

    def set_pupil_position(self, channel, output):
        """Centres the pupils on this realisation's centroid (the values the
        first two measures took in this iteration)."""
        self.pupil_shift = tuple(m.iteration_data for m in self.measures[:2])
        return output
