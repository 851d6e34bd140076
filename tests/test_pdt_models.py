"""The analytic PDT models (theory/pdt) against golden vectors made by the
reference's own theory/pdt functions (tests/golden/make_golden_pdt.py)."""
import os

import numpy as np
import pytest

from pyatmosphere_gb300.theory import pdt as P
from pyatmosphere_gb300.theory.pdt import EllipticBeamAnalyticalPDT

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def g():
    return np.load(os.path.join(HERE, "golden", "pdt_models.npz"))


def test_beam_wandering_parameters_and_density(g):
    a, eta = float(g["a"]), g["eta"]
    for i, st2 in enumerate(g["st2"]):
        e0 = P.bw_eta_0(a, st2)
        l = P.bw_shape_l(e0, a, st2)
        R = P.bw_scale_R(e0, a, l, st2)
        np.testing.assert_allclose([e0, l, R], g[f"bw_params_{i}"], rtol=1e-12)
        for j, bw2 in enumerate(g["bw2"]):
            np.testing.assert_allclose(P.beam_wandering_pdt(eta, a, st2, bw2), g[f"bw_pdt_{i}_{j}"],
                                       rtol=1e-10, atol=1e-300)


def test_moment_fitted_densities(g):
    eta, (m1, m2) = g["eta"], g["moments"]
    np.testing.assert_allclose(P.lognormal_pdt(eta, m1, m2), g["lognormal"], rtol=1e-12, atol=1e-300)
    np.testing.assert_allclose(P.beta_pdt(eta, m1, m2), g["beta"], rtol=1e-12)


def test_bayesian_mixtures_with_the_same_draws(g):
    eta, (m1, m2), a = g["eta"], g["moments"], float(g["a"])
    np.random.seed(5)
    np.testing.assert_allclose(P.bayesian_pdt(eta, m1, m2, a, 0.01, 1e-3, r0_size=300), g["bayesian"],
                               rtol=1e-10, atol=1e-300)
    np.random.seed(6)
    np.testing.assert_allclose(P.beta_bayesian_pdt(eta, m1, m2, a, 0.01, 1e-3, r0_size=300), g["beta_bayesian"],
                               rtol=1e-10)


def _beam(g):
    return {k: g[f"beam_{k}"] for k in ("mean_x", "mean_y", "mean_x2", "mean_y2", "mean_xy")}


def test_elliptic_beam_numerical_transmission(g):
    bp = _beam(g)
    for tracked in (0, 1):
        got = np.array(P.elliptic_beam_numerical_transmission(bp, [0.05, 0.1], resolution=128, is_tracked=bool(tracked)))
        np.testing.assert_allclose(got, g[f"elliptic_numeric_{tracked}"], rtol=1e-12)


def test_elliptic_beam_model(g):
    bp = _beam(g)
    m = EllipticBeamAnalyticalPDT(W0=0.05, a=float(g["a"]), size=500)
    m.set_params_from_data(bp["mean_x"], bp["mean_x2"], bp["mean_y2"])
    np.testing.assert_allclose([m.bw, m.theta_mean, *m.theta_cov], g["elliptic_params"], rtol=1e-9)
    s = g["elliptic_samples"]
    # all samples at once and one at a time; 1 - exp(-z) I_0(z) cancels for
    # small z, so the scaled Bessel form and the reference's product differ
    # by a few 1e-12
    np.testing.assert_allclose(m.eta(*s), g["elliptic_eta"], rtol=1e-10)
    np.testing.assert_allclose([m.eta(*s[:, i]) for i in range(3)], g["elliptic_eta"][:3], rtol=1e-10)
    np.random.seed(7)
    np.testing.assert_allclose(m.pdt(), g["elliptic_pdt"], rtol=1e-9)


def test_edge_cases():
    m = EllipticBeamAnalyticalPDT(W0=0.05, a=0.1, size=4)
    with pytest.raises(ValueError):
        m.pdt()
    assert m._get_R_lambda(0.0) == (np.inf, 2.0)
    # a round beam: no edge term
    assert m._get_eta0(0.04, 0.04) == pytest.approx(1 - np.exp(-2 * 0.1 ** 2 / 0.04 ** 2), rel=1e-12)
    # beyond eta_0 the beam-wandering density is zero, not NaN
    p = P.beam_wandering_pdt(np.array([0.0, 0.5, 0.9999999]), 0.1, 0.04, 1e-3)
    assert np.all(np.isfinite(p)) and p[0] == 0.0 and p[2] == 0.0
