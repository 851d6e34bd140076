"""Circular pupil (the reference's pupils.py:4-13)."""
from __future__ import annotations

from dataclasses import dataclass

__all__ = ["CirclePupil"]


@dataclass
class CirclePupil:
    radius: float

    def get_pupil(self, shift=(0, 0)):
        x, y = self.channel.grid.get_xy()
        return (x - shift[0]) ** 2 + (y + shift[1]) ** 2 <= self.radius ** 2

    def output(self, input, **kwargs):
        return input * self.get_pupil(**kwargs)
