"""Descriptors and helpers of the reference's utils.py:7-50."""
from __future__ import annotations

from dataclasses import dataclass
from typing import Sequence


class CrossRef:
    """Attribute that back-links the assigned object to its owner
    (``channel.grid = g`` sets ``g.channel = channel``)."""

    def __init__(self, cross_ref_name):
        self.cross_ref_name = cross_ref_name

    def __set_name__(self, obj, name):
        self.private_name = "_" + name

    def __get__(self, obj, type=None):
        if obj is None:
            return self
        return getattr(obj, self.private_name, None)

    def __set__(self, obj, value):
        if not value:
            return
        setattr(obj, self.private_name, value)
        setattr(value, self.cross_ref_name, obj)


class Default:
    """Attribute whose value is read along a dotted path of the owner
    (``Default("channel.source.wvl")``) unless set on the instance."""

    def __init__(self, default_path):
        self._path = default_path.split(".")

    def __set_name__(self, owner, name):
        self.private_name = "_default_" + name

    def __get__(self, obj, cls):
        if obj is None:
            return self
        if self.private_name in obj.__dict__:
            return obj.__dict__[self.private_name]
        node = obj
        for part in self._path:
            node = getattr(node, part)
        return node

    def __set__(self, obj, value):
        obj.__dict__[self.private_name] = value


@dataclass
class PolarDiscreteFunction:
    rho: Sequence[float]
    theta: Sequence[float]
    value: Sequence[complex]


def fft2(x, delta):
    """Centred 2-D FFT scaled by delta^2 (utils.py:42-44); convenience for user
    code, not used by the engine (which never materialises the shifts)."""
    import torch
    return torch.fft.fftshift(torch.fft.fft2(torch.fft.fftshift(x))) * delta ** 2


def ifft2(x, delta):
    """Centred inverse 2-D FFT scaled by (N delta)^2 (utils.py:47-50)."""
    import torch
    N = x.shape[0]
    return torch.fft.ifftshift(torch.fft.ifft2(torch.fft.ifftshift(x))) * (N * delta) ** 2
