"""Result: a named set of measures with CSV persistence (the reference's
simulations/result.py:5-43 offers the same base class).

The CSV file has the reference's layout -- one column per measure, the
measure names as the header, values written with '{:.3e}', shorter columns
padded with empty cells -- written and read with the csv module instead of
pandas.  A result whose save_path exists when it is built resumes from it.
"""
from __future__ import annotations

import csv
import math
import os

import numpy as np


class Result:
    save_float_format = "{:.3e}".format

    def __init__(self, channel, measures, max_size=None, save_path: str = ""):
        self.channel = channel
        self.measures = measures
        self.save_path = save_path
        self.set_max_size(max_size)
        if save_path and os.path.exists(save_path):
            self.load_output()
            rows = max((len(m) for m in self.measures), default=0)
            print(f"{type(self).__name__}: resumed {rows} realisations from {save_path}")

    def set_max_size(self, max_size):
        """Realisations each measure collects before it is done (None: no limit)."""
        for m in self.measures:
            m.max_size = max_size

    def print_output(self):
        counts = ", ".join(f"{m.name or i}: {len(m)}" for i, m in enumerate(self.measures))
        print(f"{type(self).__name__} realisations per measure -- {counts}")

    def plot_output(self):
        self.print_output()

    # ---- CSV ------------------------------------------------------------------
    def _cell(self, v):
        if isinstance(v, (list, tuple, np.ndarray)):
            return str(np.asarray(v).tolist())
        if v is None or (isinstance(v, float) and math.isnan(v)):
            return ""
        return self.save_float_format(v)

    def save_output(self):
        if not self.save_path:
            return
        columns = [m.data for m in self.measures]
        depth = max((len(c) for c in columns), default=0)
        with open(self.save_path, "w", newline="") as f:
            out = csv.writer(f)
            out.writerow([m.name for m in self.measures])
            out.writerows([[self._cell(c[i]) if i < len(c) else "" for c in columns] for i in range(depth)])

    def csv_columns(self):
        """The saved file's cells, one list per measure (header dropped)."""
        with open(self.save_path, newline="") as f:
            body = list(csv.reader(f))[1:]
        return [[row[j] if j < len(row) else "" for row in body] for j in range(len(self.measures))]

    def load_output(self):
        for m, cells in zip(self.measures, self.csv_columns()):
            m.data = [float(c) if c.strip() else float("nan") for c in cells]
