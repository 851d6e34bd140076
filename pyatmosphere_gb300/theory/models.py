"""Refractive-index turbulence models (theory/models.py of the reference).

Phi_n(kappa) spectra and the phase spectrum Phi_phi(f, k, dz) = 2 pi k^2 dz
Phi_n(2 pi f) (theory/models.py:16-23) used to weight the sparse-spectrum
annuli.  Evaluated with numpy on the host (FP64); the engine only consumes the
per-annulus weights.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from .atmosphere import get_r0

__all__ = ["Model", "MVKModel", "AndrewsModel"]


@dataclass
class Model:
    Cn2: float
    l0: float
    L0: float

    def psd_n_f(self, f):
        return self.psd_n(2 * np.pi * f)

    def psd_phi(self, kappa, k, thickness):
        return 2 * np.pi * k ** 2 * thickness * self.psd_n(kappa)

    def psd_phi_f(self, f, k, thickness):
        return 2 * np.pi * k ** 2 * thickness * self.psd_n_f(f)

    def sf_phi_numeric(self, r, k, thickness):
        """Phase structure function by numerical Hankel integral of the
        spectrum (theory/models.py:25-32), for screen validation."""
        import scipy.integrate
        import scipy.special

        def dsf(f, ri):
            return self.psd_n(2 * np.pi * f) * (1 - scipy.special.jv(0, 2 * np.pi * f * ri)) * 2 * np.pi * f

        phi_coeff = 2 * np.pi * k ** 2 * thickness
        return np.array([phi_coeff * (2 * np.pi) * 2 * scipy.integrate.quad(dsf, 0, np.inf, args=(float(ri),),
                                                                               epsrel=1e-3)[0] * (2 * np.pi)
                         for ri in np.atleast_1d(r)])

    def psd_n(self, kappa):
        raise NotImplementedError


class MVKModel(Model):
    """Modified von Karman spectrum (theory/models.py:80-91)."""

    def psd_n(self, kappa):
        k0 = 2 * np.pi / self.L0
        km = 5.92 / self.l0
        return 0.033 * self.Cn2 * np.exp(-(kappa / km) ** 2) / (kappa ** 2 + k0 ** 2) ** (11 / 6)

    def sf_phi(self, r, k, thickness):
        k0 = 2 * np.pi / self.L0
        r0 = get_r0(self.Cn2, k, thickness)
        return 7.75 * r0 ** (-5 / 3) * self.l0 ** (-1 / 3) * r ** 2 * (
            1 / (1 + 2.03 * r ** 2 / self.l0 ** 2) ** (1 / 6) - 0.72 * (k0 * self.l0) ** (1 / 3))


class AndrewsModel(Model):
    """Andrews spectrum with the high-wavenumber bump (theory/models.py:94-101)."""

    def psd_n(self, kappa):
        kl = 3.3 / self.l0
        k0 = 2 * np.pi / self.L0
        q = kappa / kl
        return 0.033 * self.Cn2 * (1 + 1.802 * q - 0.254 * q ** (7 / 6)) * np.exp(-q ** 2) / \
            (kappa ** 2 + k0 ** 2) ** (11 / 6)
