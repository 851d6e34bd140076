"""Measure: the per-realisation values of one operation chain (the
reference's simulations/measure.py:5-38 offers the same container).

A measure applies its operations, in order, to one kind of channel output
(measure_type "atmosphere": the receiver field; "pupil": the field behind the
channel's pupil; "propagation": the field after every screen and at the
receiver; "phase_screen": the first screen) and appends one value per
realisation to ``data``, until ``max_size`` values are stored.  With a
``time`` list the value of a realisation is the list of values at the screen
shifts (0, t).
"""
from __future__ import annotations

from typing import Sequence

import numpy as np


def default_name(operations) -> str:
    """A measure of one named function is called after it; any other chain
    (several operations, a lambda, a partial) is unnamed."""
    if len(operations) == 1:
        name = getattr(operations[0], "__name__", "")
        if name != "<lambda>":
            return name
    return ""


class Measure:
    def __init__(self, channel, measure_type: str, *operations, name: str = "", max_size: int = None,
                 time: Sequence[float] = None, save_path: str = None, save_name: str = None):
        self.operations: tuple = tuple(operations)
        self.channel = channel
        self.measure_type: str = measure_type
        self.name = name or default_name(self.operations)
        self.time: tuple = tuple(time) if time else None
        self.max_size = max_size
        self.iteration_data = None  # this realisation's value, while a Simulation runs
        self.data: list = []

    def __len__(self):
        return len(self.data)

    @property
    def is_done(self):
        return self.max_size is not None and len(self.data) >= self.max_size

    def __array__(self, dtype=None, copy=None):
        a = np.asarray(self.data)
        return a if dtype is None else a.astype(dtype)

    def __repr__(self):
        return self.name
