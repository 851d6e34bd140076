"""The method without the surrogate: analytic PDT models (theory/pdt)
fitted to a parameter point's own simulated realisations, scored with the
same bin-edge KS distance as the network.

For each point the fits get the fresh simulation's own moments, so they
are an upper bound on what the analytic route gives without simulating:
* beta and log-normal: <eta>, <eta^2>;
* beam wandering: aperture a, short-term width^2 and centroid variance per
  axis from the beam moments (simulations/beam.py:26-33 of the reference);
* elliptic beam: the model fitted to (mean_x, mean_x2, mean_y2) and
  sampled (`EllipticBeamAnalyticalPDT.pdt`);
* elliptic numerical: each realisation's elliptic Gaussian through the
  pupil (`elliptic_beam_numerical_transmission`), a per-realisation
  moment closure rather than a PDT model.
"""
from __future__ import annotations

from typing import Dict

import numpy as np

from ..engine import _lib
from ..theory import pdt as P
from ..theory.pdt import EllipticBeamAnalyticalPDT
from .model import N_HIST, ks_binned

MODELS = ("beta", "lognormal", "beam_wandering", "elliptic_beam", "elliptic_numeric")

_SUB = 32  # density samples per bin


def _density_to_probs(pdf) -> np.ndarray:
    """64 bin probabilities of a density on [0, 1] (midpoint rule with
    _SUB points per bin, renormalised; all-zero or non-finite -> uniform)."""
    x = (np.arange(N_HIST * _SUB) + 0.5) / (N_HIST * _SUB)
    with np.errstate(all="ignore"):
        f = np.asarray(pdf(x), dtype=np.float64)
    f = np.where(np.isfinite(f) & (f > 0), f, 0.0)
    p = f.reshape(N_HIST, _SUB).sum(axis=1)
    s = p.sum()
    return p / s if s > 0 else np.full(N_HIST, 1.0 / N_HIST)


def _samples_to_probs(eta) -> np.ndarray:
    eta = np.clip(np.asarray(eta, dtype=np.float64), 0, 1)
    eta = eta[np.isfinite(eta)]
    h = np.histogram(eta, bins=N_HIST, range=(0.0, 1.0))[0].astype(np.float64)
    return h / max(1.0, h.sum())


def analytic_ks(m: np.ndarray, aperture: float, w0: float, seed: int = 0, model_samples: int = 20000,
                numeric_realisations: int = 2048) -> Dict[str, float]:
    """Bin-edge KS of each analytic model against the eta of the
    realisations `m` ([realisations][n_out] engine measures of one point)."""
    m = np.asarray(m, dtype=np.float64)
    eta = np.clip(m[:, _lib.OUT_PUPIL0], 0.0, 1.0)
    mx, my = m[:, _lib.OUT_MEAN_X], m[:, _lib.OUT_MEAN_Y]
    mx2, my2, mxy = m[:, _lib.OUT_MEAN_X2], m[:, _lib.OUT_MEAN_Y2], m[:, _lib.OUT_MEAN_XY]
    e1, e2 = float(eta.mean()), float((eta ** 2).mean())
    a = float(aperture)
    bw2 = float(np.mean(mx ** 2 + my ** 2) / 2)                   # centroid variance per axis
    st2 = float(np.mean(2 * (mx2 + my2) - 2 * (mx ** 2 + my ** 2)))  # 4 x central second moment per axis
    probs = {}
    probs["beta"] = _density_to_probs(lambda x: P.beta_pdt(x, e1, e2))
    probs["lognormal"] = _density_to_probs(lambda x: P.lognormal_pdt(x, e1, e2))
    probs["beam_wandering"] = _density_to_probs(lambda x: P.beam_wandering_pdt(x, a, st2, bw2))
    state = np.random.get_state()
    try:
        np.random.seed(seed)
        eb = EllipticBeamAnalyticalPDT(W0=float(w0), a=a, size=model_samples)
        with np.errstate(all="ignore"):
            eb.set_params_from_data(mx, mx2, my2)
            cov = np.asarray(eb.theta_cov, dtype=np.float64)
            if np.all(np.isfinite(cov)) and np.isfinite(eb.theta_mean):
                # the moment estimate of the theta covariance can come out
                # indefinite (its centroid terms cancel only on average):
                # raise the variance to the nearest valid value
                eb.theta_cov = (max(cov[0], abs(cov[1])), cov[1])
                probs["elliptic_beam"] = _samples_to_probs(eb.pdt())
            else:
                probs["elliptic_beam"] = np.full(N_HIST, 1.0 / N_HIST)
    finally:
        np.random.set_state(state)
    k = min(len(eta), numeric_realisations)
    bp = {"mean_x": mx[:k], "mean_y": my[:k], "mean_x2": mx2[:k], "mean_y2": my2[:k], "mean_xy": mxy[:k]}
    with np.errstate(all="ignore"):
        probs["elliptic_numeric"] = _samples_to_probs(P.elliptic_beam_numerical_transmission(bp, [a], resolution=128)[0])
    return {name: ks_binned(probs[name], eta) for name in MODELS}
