"""Properties of the FP64 oracle that hold whatever the reference's numbers:
the checker itself is sound, independently of the golden vectors.
- vacuum step: unitary, linear, and two steps equal one step of the summed
  length (the transfer functions multiply);
- SS screen: real, linear in the spectral amplitudes, and a shift of the
  grid equals a phase rotation of the amplitudes;
- Gaussian source: unit energy on a grid much wider than the beam."""
import numpy as np
import pytest

from oracle import atm_oracle as o

N, DELTA, WVL = 128, 4e-3, 1550e-9
K = 2 * np.pi / WVL


def _field(seed):
    rng = np.random.default_rng(seed)
    x = (np.arange(N) - N // 2) * DELTA
    env = np.exp(-(x[None, :] ** 2 + x[:, None] ** 2) / 0.08 ** 2)
    return env * np.exp(1j * rng.uniform(0, 2 * np.pi, (N, N)))


def test_vacuum_is_unitary_linear_and_composes():
    u, w = _field(1), _field(2)
    e = lambda f: float(np.sum(np.abs(f) ** 2))
    vu = o.vacuum(u, 3e3, K, DELTA)
    assert e(vu) == pytest.approx(e(u), rel=1e-12)
    a, b = 0.7 - 0.2j, -1.3 + 0.4j
    np.testing.assert_allclose(o.vacuum(a * u + b * w, 3e3, K, DELTA), a * vu + b * o.vacuum(w, 3e3, K, DELTA),
                               atol=1e-12 * np.max(np.abs(vu)))
    two = o.vacuum(o.vacuum(u, 1.2e3, K, DELTA), 1.8e3, K, DELTA)
    assert o.rel_l2(two, vu) < 1e-12


def test_ss_screen_is_real_linear_and_shift_covariant():
    rng = np.random.default_rng(3)
    P = 64
    rho = rng.uniform(0.1, 20.0, P)
    theta = rng.uniform(0, 2 * np.pi, P)
    v1 = rng.standard_normal(P) + 1j * rng.standard_normal(P)
    v2 = rng.standard_normal(P) + 1j * rng.standard_normal(P)
    phi1 = o.ss_screen(rho, theta, v1, N, DELTA)
    phi2 = o.ss_screen(rho, theta, v2, N, DELTA)
    assert np.isrealobj(phi1)
    np.testing.assert_allclose(o.ss_screen(rho, theta, 2.5 * v1 - v2, N, DELTA), 2.5 * phi1 - phi2, atol=1e-10)
    # moving the grid by (sx, sy) multiplies each amplitude by exp(i 2 pi (fx sx + fy sy))
    sx, sy = 0.013, -0.021
    rot = np.exp(2j * np.pi * (rho * np.cos(theta) * sx + rho * np.sin(theta) * sy))
    np.testing.assert_allclose(o.ss_screen(rho, theta, v1, N, DELTA, shift=(sx, sy)),
                               o.ss_screen(rho, theta, v1 * rot, N, DELTA), atol=1e-9)


def test_gaussian_source_has_unit_energy():
    u = o.gaussian_source(N, DELTA, WVL, 0.05, np.inf)
    assert float(np.sum(np.abs(u) ** 2)) * DELTA ** 2 == pytest.approx(1.0, rel=1e-9)
