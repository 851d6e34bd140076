"""Result base class (simulations/result.py:5-43).  The CSV format is the
reference's (one column per measure, header = measure names, values
'{:.3e}', shorter columns padded with empty cells) written without pandas."""
from __future__ import annotations

import csv
import math

import numpy as np


class Result:
    save_float_format = "{:.3e}".format

    def __init__(self, channel, measures, max_size=None, save_path: str = ""):
        self.channel = channel
        self.measures = measures
        self.set_max_size(max_size)
        self.save_path = save_path
        if self.save_path:
            try:
                self.load_output()
                print(f"Loaded measures from {self.save_path}")
            except FileNotFoundError:
                pass

    def set_max_size(self, max_size):
        for measures in self.measures:
            measures.max_size = max_size

    def print_output(self):
        print(f"Len of the first measures: {len(self.measures[0])}")

    def plot_output(self):
        self.print_output()

    def _format(self, v):
        if isinstance(v, (list, tuple, np.ndarray)):
            return str(list(np.asarray(v).tolist()))
        if v is None or (isinstance(v, float) and math.isnan(v)):
            return ""
        return self.save_float_format(v)

    def save_output(self):
        if not self.save_path:
            return
        cols = [m.data for m in self.measures]
        n = max((len(c) for c in cols), default=0)
        with open(self.save_path, "w", newline="") as f:
            w = csv.writer(f)
            w.writerow([m.name for m in self.measures])
            for i in range(n):
                w.writerow([self._format(c[i]) if i < len(c) else "" for c in cols])

    @staticmethod
    def _parse(cell):
        return float(cell) if cell.strip() != "" else float("nan")

    def _read_columns(self):
        with open(self.save_path, newline="") as f:
            rows = list(csv.reader(f))
        body = rows[1:]
        return [[r[j] if j < len(r) else "" for r in body] for j in range(len(self.measures))]

    def load_output(self):
        for measures, col in zip(self.measures, self._read_columns()):
            measures.data = [self._parse(c) for c in col]
