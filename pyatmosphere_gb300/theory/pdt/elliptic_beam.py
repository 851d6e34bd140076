"""Elliptic-beam model of the PDT (theory/pdt/elliptic_beam.py:7-103 of the
reference; Vasylyev, Semenov and Vogel, PRL 117, 090501, 2016).

A realisation is an elliptic Gaussian beam with semi-axes W1, W2
(theta_i = ln(W_i^2 / W0^2), jointly normal), orientation phi, and
centroid at distance r0 ~ Rayleigh(bw) in direction varphi0 ~ U[0, 2 pi).
Its transmittance through an aperture of radius a is
    eta = eta_0(W1, W2) exp(-(r0 / (a R))^lambda),
where R and lambda come from the effective width W_eff(phi - varphi0)
(a Lambert-W expression) and eta_0 from W1, W2.

The parameters are set directly, or from per-realisation beam moments
(mean_x, mean_x2, mean_y2) through the moment relations of the model.
`pdt()` draws `size` realisations from numpy's global generator in the
reference's order (Rayleigh r0, uniform varphi0, bivariate normal
thetas, uniform phi), so a seeded call gives the reference's samples; the
transmittances are then evaluated for all samples at once.
"""
from __future__ import annotations

from typing import Optional, Tuple

import numpy as np
from scipy.special import ive, lambertw


class EllipticBeamAnalyticalPDT:
    def __init__(self, W0, a, size: int):
        self.W0 = W0
        self.a = a
        self.size = size
        self.bw: Optional[float] = None
        self.theta_mean: Optional[float] = None
        self.theta_cov: Optional[Tuple[float, float]] = None

    def set_params(self, bw: float, theta_mean: float, theta_cov: Tuple[float, float]):
        self.bw = bw
        self.theta_mean = theta_mean
        self.theta_cov = theta_cov
        return self

    def set_params_from_data(self, mean_x, mean_x2, mean_y2):
        mean_x, mean_x2, mean_y2 = (np.asarray(v, dtype=np.float64) for v in (mean_x, mean_x2, mean_y2))
        bw = np.sqrt((mean_x ** 2).mean())
        W2_mean, W2_cov = self._get_mean_W(mean_x, mean_x2, mean_y2)
        theta_mean, theta_cov = self._get_mean_theta(W2_mean, W2_cov)
        return self.set_params(bw, theta_mean, theta_cov)

    def _get_mean_W(self, mean_x, mean_x2, mean_y2):
        """<W^2> and the covariances (<W1^2 W1^2>, <W1^2 W2^2>) - <W^2>^2 from
        the beam moments (centroid term removed)."""
        c2 = (mean_x ** 2).mean()               # <x0^2>
        x2 = mean_x2.mean()                     # <x^2>
        W2_mean = 4 * (x2 - c2)
        same = np.asarray([1, 0])               # Kronecker delta: (i = j, i != j)
        quad_terms = (mean_x2 ** 2).mean() * (4 * same - 1) - (mean_x2 * mean_y2).mean() * (4 * same - 3)
        WiWj = 8 * (quad_terms - 8 * same * c2 ** 2 - c2 * W2_mean)
        return W2_mean, WiWj - W2_mean ** 2

    def _get_mean_theta(self, W2_mean, W2_cov):
        rel = W2_cov / W2_mean ** 2
        theta_mean = np.log(W2_mean / self.W0 ** 2 / np.sqrt(1 + rel[0]))
        return theta_mean, np.log(1 + rel)

    def _get_W_eff(self, chi, W1, W2):
        a2 = self.a ** 2
        expo = a2 / W1 ** 2 * (1 + 2 * np.cos(chi) ** 2) + a2 / W2 ** 2 * (1 + 2 * np.sin(chi) ** 2)
        arg = 4 * a2 / W1 / W2 * np.exp(expo)
        return np.sqrt(4 * a2 / lambertw(arg).real)

    def _get_R_lambda(self, xi):
        """Scale R and shape lambda of the transmittance's fall-off with the
        deflection for inverse width xi (R = inf, lambda = 2 at xi = 0)."""
        xi = np.asarray(xi, dtype=np.float64)
        arg = self.a ** 2 * xi ** 2
        with np.errstate(divide="ignore", invalid="ignore"):
            one_minus = 1 - ive(0, arg)
            log_part = np.log(2 * (1 - np.exp(-arg / 2)) / one_minus)
            lmbd = 2 * arg * ive(1, arg) / one_minus / log_part
            R = log_part ** (-1 / lmbd)
        zero = xi == 0
        R, lmbd = np.where(zero, np.inf, R), np.where(zero, 2.0, lmbd)
        if R.ndim == 0:
            return float(R), float(lmbd)
        return R, lmbd

    def _get_eta0(self, W1, W2):
        W1 = np.asarray(W1, dtype=np.float64)
        W2 = np.asarray(W2, dtype=np.float64)
        a2 = self.a ** 2
        R, lmbd = self._get_R_lambda(1 / W1 - 1 / W2)
        u = a2 * (1 / W1 ** 2 - 1 / W2 ** 2)
        v = a2 * (1 / W1 ** 2 + 1 / W2 ** 2)
        # I_0(u) exp(-v) = ive(0, u) exp(|u| - v)
        centred = ive(0, u) * np.exp(np.abs(u) - v)
        with np.errstate(divide="ignore", invalid="ignore", over="ignore"):
            p3 = 2 * (1 - np.exp(-a2 / 2 * (1 / W1 - 1 / W2) ** 2))
            p4 = np.exp(-((W1 + W2) ** 2 / np.abs(W1 ** 2 - W2 ** 2) / R) ** lmbd)
            edge = np.where(W1 == W2, 0.0, p3 * p4)
        out = 1 - centred - edge
        return float(out) if out.ndim == 0 else out

    def eta(self, r_0, varphi_0, theta_1, theta_2, phi):
        W1 = self.W0 * np.exp(np.asarray(theta_1, dtype=np.float64) / 2)
        W2 = self.W0 * np.exp(np.asarray(theta_2, dtype=np.float64) / 2)
        W_eff = self._get_W_eff(np.asarray(phi) - np.asarray(varphi_0), W1=W1, W2=W2)
        eta_0 = self._get_eta0(W1=W1, W2=W2)
        R, lmbd = self._get_R_lambda(2 / W_eff)
        return eta_0 * np.exp(-(np.asarray(r_0) / self.a / R) ** lmbd)

    def pdt(self):
        if self.bw is None or self.theta_mean is None or self.theta_cov is None:
            raise ValueError(
                'The parametes must be setted via .set_params(...) or .set_params_from_data(...).')
        r_0s = np.random.rayleigh(self.bw, size=self.size)
        varphi_0s = np.random.uniform(0, 2 * np.pi, size=self.size)
        cov = np.asarray(self.theta_cov)
        thetas = np.random.multivariate_normal([self.theta_mean, self.theta_mean], [cov, cov[::-1]],
                                               size=self.size).T
        phis = np.random.uniform(0, np.pi / 2, size=self.size)
        return self.eta(r_0s, varphi_0s, thetas[0], thetas[1], phis).tolist()
