"""The analytic-model baselines of the surrogate check: on realisations
drawn from the beam-wandering model itself the fitted model reproduces the
histogram (KS at sampling noise), and every model gives a KS in [0, 1]."""
import numpy as np

from pyatmosphere_gb300.engine import _lib
from pyatmosphere_gb300.surrogate.baselines import MODELS, analytic_ks
from pyatmosphere_gb300.theory import pdt as P


def _beam_wandering_realisations(n, a, W, sigma, rng):
    x0, y0 = rng.normal(0, sigma, n), rng.normal(0, sigma, n)
    st2 = W ** 2
    e0 = P.bw_eta_0(a, st2)
    l = P.bw_shape_l(e0, a, st2)
    R = P.bw_scale_R(e0, a, l, st2)
    eta = e0 * np.exp(-(np.hypot(x0, y0) / R) ** l)
    m = np.zeros((n, _lib.OUT_PUPIL0 + 1))
    m[:, _lib.OUT_MEAN_X], m[:, _lib.OUT_MEAN_Y] = x0, y0
    m[:, _lib.OUT_MEAN_X2] = x0 ** 2 + st2 / 4
    m[:, _lib.OUT_MEAN_Y2] = y0 ** 2 + st2 / 4
    m[:, _lib.OUT_MEAN_XY] = x0 * y0
    m[:, _lib.OUT_PUPIL0] = eta
    return m


def test_beam_wandering_fit_reproduces_its_own_realisations():
    rng = np.random.default_rng(4)
    m = _beam_wandering_realisations(8192, a=0.1, W=0.08, sigma=0.05, rng=rng)
    ks = analytic_ks(m, aperture=0.1, w0=0.05, seed=1, model_samples=4000, numeric_realisations=256)
    assert set(ks) == set(MODELS)
    assert all(0.0 <= v <= 1.0 for v in ks.values())
    # sampling noise of 8192 realisations is ~0.01
    assert ks["beam_wandering"] < 0.03
    # a round beam with a known centroid: the per-realisation elliptic closure is exact
    # up to the grid (128^2 over 8 long-term radii)
    assert ks["elliptic_numeric"] < 0.1
