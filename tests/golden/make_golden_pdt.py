"""Golden vectors of the analytic PDT models, made by running the reference's
own theory/pdt functions (pdt.py, elliptic_beam.py) on fixed and seeded
inputs.

Usage (from the repository root, where the reference tree is available)::

    python tests/golden/make_golden_pdt.py /path/to/pyAtmosphere

Writes ``pdt_models.npz`` beside this script.  The seeded models draw from
numpy's global generator; the inputs record each seed, and the tests seed
the same generator before calling the engine package's functions.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
from make_golden import import_reference  # noqa: E402

A = 0.1
ST2 = (0.003, 0.01, 0.04)
BW2 = (1e-4, 1e-3)
ETA = np.linspace(0.0005, 0.9995, 200)
MOMENTS = (0.6, 0.4)   # <eta>, <eta^2>


def beam_moments(rng, R, bw, W0, theta_std=0.3):
    """Per-realisation beam moments drawn from the elliptic-beam model
    itself: centroid ~ N(0, bw^2) per axis, W_i^2 = W0^2 exp(theta_i) with
    theta_i ~ N(-0.5, theta_std^2), orientation ~ U[0, pi/2)."""
    mx, my = rng.normal(0, bw, R), rng.normal(0, bw, R)
    w1 = W0 ** 2 * np.exp(rng.normal(-0.5, theta_std, R))
    w2 = W0 ** 2 * np.exp(rng.normal(-0.5, theta_std, R))
    phi = rng.uniform(0, np.pi / 2, R)
    c, s = np.cos(phi), np.sin(phi)
    return {"mean_x": mx, "mean_y": my, "mean_x2": mx ** 2 + (w1 * c ** 2 + w2 * s ** 2) / 4,
            "mean_y2": my ** 2 + (w1 * s ** 2 + w2 * c ** 2) / 4, "mean_xy": mx * my + (w1 - w2) * s * c / 4}


def main(path):
    import_reference(path)
    from pyatmosphere.theory.pdt import pdt as P
    from pyatmosphere.theory.pdt import EllipticBeamAnalyticalPDT
    g = {"eta": ETA, "a": A, "st2": np.array(ST2), "bw2": np.array(BW2), "moments": np.array(MOMENTS)}
    for i, st2 in enumerate(ST2):
        e0 = P.bw_eta_0(A, st2)
        l = P.bw_shape_l(e0, A, st2)
        R = P.bw_scale_R(e0, A, l, st2)
        g[f"bw_params_{i}"] = np.array([e0, l, R])
        for j, bw2 in enumerate(BW2):
            g[f"bw_pdt_{i}_{j}"] = P.beam_wandering_pdt(ETA.copy(), A, st2, bw2)
    g["lognormal"] = P.lognormal_pdt(ETA, *MOMENTS)
    g["beta"] = P.beta_pdt(ETA, *MOMENTS)
    np.random.seed(5)
    g["bayesian"] = P.bayesian_pdt(ETA, *MOMENTS, A, 0.01, 1e-3, r0_size=300)
    np.random.seed(6)
    g["beta_bayesian"] = P.beta_bayesian_pdt(ETA, *MOMENTS, A, 0.01, 1e-3, r0_size=300)

    rng = np.random.default_rng(8)
    bp = beam_moments(rng, 256, 0.005, 0.05)
    for k, v in bp.items():
        g[f"beam_{k}"] = v
    for tracked in (False, True):
        out = P.elliptic_beam_numerical_transmission(bp, [0.05, 0.1], resolution=128, is_tracked=tracked)
        g[f"elliptic_numeric_{int(tracked)}"] = np.array(out)

    model = EllipticBeamAnalyticalPDT(W0=0.05, a=A, size=500)
    model.set_params_from_data(bp["mean_x"], bp["mean_x2"], bp["mean_y2"])
    g["elliptic_params"] = np.array([model.bw, model.theta_mean, *model.theta_cov])
    # the transmittance of fixed samples, one scalar call each as the reference evaluates them
    srng = np.random.default_rng(9)
    samples = np.stack([srng.rayleigh(0.02, 50), srng.uniform(0, 2 * np.pi, 50), srng.normal(-0.5, 0.3, 50),
                        srng.normal(-0.5, 0.3, 50), srng.uniform(0, np.pi / 2, 50)])
    g["elliptic_samples"] = samples
    g["elliptic_eta"] = np.array([model.eta(*samples[:, i]) for i in range(samples.shape[1])])
    np.random.seed(7)
    g["elliptic_pdt"] = np.array(model.pdt())
    np.savez_compressed(os.path.join(HERE, "pdt_models.npz"), **g)
    print("wrote", os.path.join(HERE, "pdt_models.npz"), len(g), "arrays")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else os.environ.get("PYATMOSPHERE_REF", "../pyAtmosphere"))
