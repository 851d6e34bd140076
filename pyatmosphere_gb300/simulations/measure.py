"""Per-realisation measure container (simulations/measure.py:5-38)."""
from __future__ import annotations

from typing import Sequence

import numpy as np


class Measure:
    def __init__(self, channel, measure_type: str, *operations, name: str = "", max_size: int = None,
                 time: Sequence[float] = None, save_path: str = None, save_name: str = None):
        self.channel = channel
        self.measure_type: str = measure_type
        self.operations: tuple = tuple(operations)
        self.name = name or (operations[0].__name__ if len(operations) == 1 and
                             getattr(operations[0], "__name__", "<lambda>") != "<lambda>" else "")
        self.max_size = max_size
        self.time: tuple = tuple(time) if time else None
        self.data: list = []
        self.iteration_data = None

    @property
    def is_done(self):
        return self.max_size is not None and len(self) >= self.max_size

    def __len__(self):
        return len(self.data)

    def __array__(self, dtype=None, copy=None):
        a = np.asarray(self.data)
        return a.astype(dtype) if dtype is not None else a

    def __repr__(self):
        return self.name
