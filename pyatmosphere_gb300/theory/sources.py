"""Gaussian beam (theory/sources.py:6-33 of the reference)."""
from __future__ import annotations

import numpy as np


class GaussianBeam:
    def __init__(self, wvl, w0, F0):
        self.wvl = wvl
        self.w0 = w0
        self.F0 = F0

    @property
    def k(self):
        return 2 * np.pi / self.wvl

    def amplitude(self, r2):
        """sqrt(2/pi)/w0 exp(-(1/w0^2 + i pi/(wvl F0)) r^2) on a tensor or array of r^2."""
        c = 1 / self.w0 ** 2 + 1j * 2 * np.pi / self.wvl / 2 / self.F0
        try:
            import torch
            if isinstance(r2, torch.Tensor):
                return np.sqrt(2 / np.pi) / self.w0 * torch.exp(-c * r2.to(torch.complex64))
        except ImportError:  # pragma: no cover
            pass
        return np.sqrt(2 / np.pi) / self.w0 * np.exp(-c * r2)

    def get_theta0(self, length):
        return 1 - length / self.F0

    def get_Lambda0(self, length):
        return 2 * length / self.k / self.w0 ** 2

    def get_theta(self, length):
        return self.get_theta0(length) / (self.get_theta0(length) ** 2 + self.get_Lambda0(length) ** 2)

    def get_Lambda(self, length):
        return self.get_Lambda0(length) / (self.get_theta0(length) ** 2 + self.get_Lambda0(length) ** 2)

    def get_w(self, length):
        return self.w0 * np.sqrt(self.get_theta0(length) ** 2 + self.get_Lambda0(length) ** 2)
