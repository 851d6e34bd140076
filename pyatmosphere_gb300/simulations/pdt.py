"""Probability distribution of transmittance (simulations/pdt.py:11-66)."""
from __future__ import annotations

from functools import partial

import numpy as np

from ..measures import eta, mean_x, mean_y
from .measure import Measure
from .result import Result


class PDTResult(Result):
    def __init__(self, channel, pupils: list = None, **kwargs):
        self.pupil_shift = (0, 0)
        self.pupils = pupils or [channel.pupil]
        measures = kwargs.pop("measures", [
            Measure(channel, "atmosphere", partial(self.append_pupil, pupil), eta, name=f"{pupil.radius}")
            for pupil in self.pupils])
        super().__init__(channel, measures, **kwargs)

    def append_pupil(self, pupil, channel, output):
        init_pupil = channel.pupil
        channel.pupil = pupil
        output = channel.pupil.output(output, shift=self.pupil_shift)
        channel.pupil = init_pupil
        return output

    def histogram(self, i=0, bins=200, range=(0, 1)):
        return np.histogram(np.asarray(self.measures[i].data, dtype=float), bins=bins, range=range)

    def plot_output(self):
        try:
            from matplotlib import pyplot as plt
        except ImportError:
            self.print_output()
            return
        plt.hist(self.measures[0].data, label=f"Count: {len(self.measures[0])}", bins=200, range=(0, 1))
        plt.legend()
        plt.show()


class TrackedPDTResult(PDTResult):
    def __init__(self, channel, pupils: list = None, **kwargs):
        pupils = pupils or [channel.pupil]
        beam_measures = [Measure(channel, "atmosphere", mean_x), Measure(channel, "atmosphere", mean_y)]
        pdt_measures = [
            Measure(channel, "atmosphere", self.set_pupil_position, partial(self.append_pupil, pupil), eta,
                    name=f"{pupil.radius}")
            for pupil in pupils]
        super().__init__(channel, pupils=pupils, measures=beam_measures + pdt_measures, **kwargs)

    def set_pupil_position(self, channel, output):
        self.pupil_shift = (self.measures[0].iteration_data, self.measures[1].iteration_data)
        return output
