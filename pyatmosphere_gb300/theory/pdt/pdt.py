"""Analytic probability distributions of the transmittance (PDT) eta of a
beam through a circular aperture of radius a (theory/pdt/pdt.py:14-147 of
the reference).

The models take a few moments of the beam or of eta and return a density
on an eta grid, or per-realisation transmittances:
* beam wandering (Vasylyev, Semenov and Vogel, PRL 108, 220501, 2012):
  eta = eta_0 exp(-(r/R)^l) for a beam of short-term width W (st2 = W^2)
  deflected by r ~ Rayleigh(sigma_bw); eta_0, the shape l and the scale R
  follow from a / W through modified Bessel functions;
* log-normal and beta densities fitted by the method of moments to
  <eta> and <eta^2>;
* Bayesian mixtures: a log-normal (or beta) density conditioned on the
  deflection r0, averaged over r0 ~ Rayleigh(sigma_bw) drawn from numpy's
  global generator as the reference does (seed it for repeatable results);
* the elliptic-beam transmittance of per-realisation beam moments on a
  grid (`elliptic_beam_numerical_transmission`).

Every function is vectorised over its eta grid and, where the reference
loops in Python (mixture components, realisations), over those too.
exp(-z) I_n(z) is evaluated as the exponentially scaled Bessel function
(scipy.special.ive): equal to the reference's exp(-z) * iv(n, z) to
rounding where that is finite, and finite where its I_n(z) overflows
(z > ~700).
"""
from __future__ import annotations

import numpy as np
from scipy import special, stats
from scipy.integrate import quad

__all__ = ["bw_eta_0", "bw_shape_l", "bw_scale_R", "bw_pdt", "lognormal_pdt", "beam_wandering_pdt", "beta_pdt",
           "bayesian_pdt", "beta_bayesian_pdt", "elliptic_beam_numerical_transmission"]

# mixture components evaluated together (bounds the (components x eta) work arrays)
_BLOCK = 256


def _scaled_i0_i1(z):
    """exp(-z) I_0(z), exp(-z) I_1(z) for z >= 0."""
    return special.ive(0, z), special.ive(1, z)


def bw_eta_0(a, st2):
    """Maximal transmittance of the undeflected beam: 1 - exp(-2 a^2 / W^2)."""
    return 1 - np.exp(-2 * a ** 2 / st2)


def _bw_log_term(eta_0, a, st2):
    # ln(2 eta_0 / (1 - exp(-z) I_0(z))), z = 4 a^2 / W^2
    g0, _ = _scaled_i0_i1(4 * a ** 2 / st2)
    return np.log(2 * eta_0 / (1 - g0))


def bw_shape_l(eta_0, a, st2):
    """Shape parameter l of the beam-wandering model."""
    z = 4 * a ** 2 / st2
    g0, g1 = _scaled_i0_i1(z)
    return 2 * z * (g1 / (1 - g0)) / _bw_log_term(eta_0, a, st2)


def bw_scale_R(eta_0, a, l, st2):
    """Scale parameter R of the beam-wandering model."""
    return a * _bw_log_term(eta_0, a, st2) ** (-1 / l)


def bw_pdt(eta, eta_0, R, l, bw2):
    """Beam-wandering density of eta (0 where it is undefined: eta >= eta_0
    or eta = 0)."""
    eta = np.asarray(eta, dtype=np.float64)
    with np.errstate(divide="ignore", invalid="ignore", over="ignore"):
        lg = np.log(eta_0 / eta)
        p = R ** 2 / (bw2 * eta * l) * lg ** (2 / l - 1) * np.exp(-(R ** 2 / (2 * bw2)) * lg ** (2 / l))
    return np.where(np.isnan(p), 0.0, p)


def _lognormal_parts(eta_mean, eta2_mean):
    """(mu, sigma) of the log-normal law with the given <eta>, <eta^2>, in
    the parametrisation pdf = exp(-(ln eta + mu)^2 / 2 sigma^2) / (eta sigma sqrt(2 pi))."""
    mu = -np.log(eta_mean ** 2 / np.sqrt(eta2_mean))
    sigma = np.sqrt(np.log(eta2_mean / eta_mean ** 2))
    return mu, sigma


def _truncated_lognormal(eta, mu, sigma):
    """Log-normal density renormalised to eta <= 1 (its CDF at 1 is
    Phi(mu / sigma)); broadcasts over mu."""
    eta = np.asarray(eta, dtype=np.float64)
    pos = eta > 0
    le = np.log(np.where(pos, eta, 1.0))
    pdf = np.exp(-0.5 * ((le + mu) / sigma) ** 2) / (np.where(pos, eta, 1.0) * sigma * np.sqrt(2 * np.pi))
    return np.where(pos, pdf, 0.0) / special.ndtr(mu / sigma)


def lognormal_pdt(eta, eta_mean, eta2_mean):
    """Log-normal density with the given first two moments, truncated to eta <= 1."""
    mu, sigma = _lognormal_parts(eta_mean, eta2_mean)
    return _truncated_lognormal(eta, mu, sigma)


def beam_wandering_pdt(eta, a, st2, bw2, eta_0=None, shape_l=None, scale_R=None):
    """Beam-wandering density; eta_0, l and R follow from a and st2 unless given."""
    eta_0 = eta_0 or bw_eta_0(a, st2)
    shape_l = shape_l or bw_shape_l(eta_0, a, st2)
    scale_R = scale_R or bw_scale_R(eta_0, a, shape_l, st2)
    return bw_pdt(eta, eta_0, scale_R, shape_l, bw2)


def _beta_ab(eta_mean, eta2_mean):
    var = eta2_mean - eta_mean ** 2
    a = (eta_mean ** 2 - eta_mean ** 3 - eta_mean * var) / var
    return a, a * (1 / eta_mean - 1)


def beta_pdt(eta, eta_mean, eta2_mean):
    """Beta density with the given first two moments."""
    a, b = _beta_ab(eta_mean, eta2_mean)
    return stats.beta.pdf(eta, a, b)


def _deflection_moments(eta_mean, eta2_mean, bw, scale_R, shape_l):
    """eta0 and zeta0^2 of the Bayesian models: <eta> and <eta^2> divided by
    the Rayleigh averages of exp(-(r/R)^l) and exp(-2 (r/R)^l)."""
    def avg(k):
        return quad(lambda xi: xi * np.exp(-xi ** 2 / 2) * np.exp(-k * (bw / scale_R * xi) ** shape_l), 0, np.inf)[0]
    return eta_mean / avg(1), eta2_mean / avg(2)


def _bw_params(a, st2, scale_R, shape_l):
    eta_0 = bw_eta_0(a, st2)
    shape_l = shape_l or bw_shape_l(eta_0, a, st2)
    scale_R = scale_R or bw_scale_R(eta_0, a, shape_l, st2)
    return scale_R, shape_l


def bayesian_pdt(eta, eta_mean, eta2_mean, a, st2, bw2, scale_R=None, shape_l=None, r0_size=2000):
    """Average over r0 ~ Rayleigh(sqrt(bw2)) (numpy's global generator) of a
    log-normal density whose log-mean moves with (r0 / R)^l."""
    bw = np.sqrt(bw2)
    scale_R, shape_l = _bw_params(a, st2, scale_R, shape_l)
    eta0, zeta02 = _deflection_moments(eta_mean, eta2_mean, bw, scale_R, shape_l)
    sigma = np.sqrt(np.log(zeta02 / eta0 ** 2))
    mu0 = -np.log(eta0 ** 2 / np.sqrt(zeta02))
    r0 = np.random.rayleigh(bw, size=r0_size)
    eta = np.asarray(eta, dtype=np.float64)
    total = np.zeros_like(eta)
    for s in range(0, r0_size, _BLOCK):
        mu = mu0 + (np.abs(r0[s:s + _BLOCK]) / scale_R) ** shape_l
        mu = mu.reshape((-1,) + (1,) * eta.ndim)
        total = total + _truncated_lognormal(eta[None], mu, sigma).sum(axis=0)
    return total / r0_size


def beta_bayesian_pdt(eta, eta_mean, eta2_mean, a, st2, bw2, scale_R=None, shape_l=None, r0_size=2000):
    """Average over r0 ~ Rayleigh(sqrt(bw2)) (numpy's global generator) of a
    beta density whose moments fall off as exp(-(r0 / R)^l) and exp(-2 (r0 / R)^l)."""
    bw = np.sqrt(bw2)
    scale_R, shape_l = _bw_params(a, st2, scale_R, shape_l)
    eta0, zeta02 = _deflection_moments(eta_mean, eta2_mean, bw, scale_R, shape_l)
    r0 = np.random.rayleigh(bw, size=r0_size)
    eta = np.asarray(eta, dtype=np.float64)
    total = np.zeros_like(eta)
    for s in range(0, r0_size, _BLOCK):
        f = np.exp(-(r0[s:s + _BLOCK] / scale_R) ** shape_l).reshape((-1,) + (1,) * eta.ndim)
        a_r, b_r = _beta_ab(eta0 * f, zeta02 * f ** 2)
        total = total + stats.beta.pdf(eta[None], a_r, b_r).sum(axis=0)
    return total / r0_size


def elliptic_beam_numerical_transmission(beam_params: dict, pupil_radiuses, resolution=2 ** 8, is_tracked=False,
                                         chunk=32):
    """Transmittance of each realisation's elliptic Gaussian beam (centroid
    and second moments from `beam_params`: mean_x, mean_y, mean_x2, mean_y2,
    mean_xy) through each pupil, on a resolution^2 grid spanning 8 long-term
    radii; with `is_tracked` the pupils sit on each beam's centroid.  Returns
    one list of transmittances per pupil."""
    mx = np.asarray(beam_params["mean_x"], dtype=np.float64)
    my = np.asarray(beam_params["mean_y"], dtype=np.float64)
    mx2 = np.asarray(beam_params["mean_x2"], dtype=np.float64)
    my2 = np.asarray(beam_params["mean_y2"], dtype=np.float64)
    mxy = np.asarray(beam_params["mean_xy"], dtype=np.float64)
    lt_mean = np.sqrt(4 * (mx2 + my2).mean())
    delta = 8 * lt_mean / resolution
    n = int(resolution)
    lo = -(n // 2) + (n % 2)
    # grid coordinates as RectGrid.get_x / get_y: float32 indices times delta
    x = np.arange(lo, lo + n, dtype=np.float32) * delta
    y = np.arange(lo, lo + n, dtype=np.float32) * delta
    out = [[] for _ in pupil_radiuses]
    for s in range(0, len(mx), chunk):
        cx, cy = mx[s:s + chunk, None, None], my[s:s + chunk, None, None]
        Sxx = 4 * (mx2[s:s + chunk, None, None] - cx ** 2)
        Syy = 4 * (my2[s:s + chunk, None, None] - cy ** 2)
        Sxy = 4 * (mxy[s:s + chunk, None, None] - cx * cy)
        det = Sxx * Syy - Sxy ** 2
        X = x[None, None, :] - cx
        Y = -y[None, :, None] - cy
        amp = np.sqrt(2 / np.pi / np.sqrt(det)) * np.exp(-(Syy * X ** 2 - 2 * Sxy * X * Y + Sxx * Y ** 2) / det)
        I = amp ** 2
        for i, r in enumerate(pupil_radiuses):
            if is_tracked:
                inside = (x[None, None, :] - cx) ** 2 + (y[None, :, None] + cy) ** 2 <= r ** 2
            else:
                inside = (x[None, None, :] ** 2 + y[None, :, None] ** 2 <= r ** 2)
            out[i].extend((np.where(inside, I, 0.0).sum(axis=(-1, -2)) * delta ** 2).tolist())
    return out
