"""Pins the CPU oracle against golden vectors made by the reference itself
(tests/golden/make_golden.py).  In reference precision the oracle must
reproduce the reference to FFT / GEMM round-off; in FP64 it must stay within
the reference's own FP32 error of it."""
import numpy as np
import pytest

from oracle import atm_oracle as o

SMALL = dict(N=128, delta=3e-3, w0=0.06, length=5e3, count=3, points=256, Cn2=2e-15,
             pupil_radius=0.08)


@pytest.mark.parametrize("tag,F0", [("inf", np.inf), ("f20000", 20000.0), ("fm6000", -6000.0)])
def test_vacuum_matches_reference(golden, tag, F0):
    for prec, tol in [("ref", 1e-6), ("fp64", 1e-6)]:
        u0 = o.gaussian_source(128, 4e-3, 809e-9, 0.05, F0, prec)
        u = o.vacuum(u0, 4e3, 2 * np.pi / 809e-9, 4e-3, prec)
        assert o.rel_l2(u, golden[f"vac_{tag}_field"]) < tol


def test_ss_screen_matches_reference(golden):
    ref = golden["ss_screen"]
    s = o.ss_screen(golden["ss_rho"], golden["ss_theta"], golden["ss_value"], 64, 2e-3, prec="ref")
    assert np.abs(s - ref).max() <= 1e-6 * np.abs(ref).max() * 10
    s2 = o.ss_screen(golden["ss_rho"], golden["ss_theta"], golden["ss_value"], 64, 2e-3,
                     shift=(0.05, -0.1), prec="ref")
    assert np.abs(s2 - golden["ss_screen_shift"]).max() <= 1e-6 * np.abs(ref).max() * 10
    s64 = o.ss_screen(golden["ss_rho"], golden["ss_theta"], golden["ss_value"], 64, 2e-3)
    # the reference's float32 phase arguments cost it ~1e-3 rad here
    assert np.abs(s64 - ref).max() < 5e-3


@pytest.mark.parametrize("pos,key", [("middle", "small_field"), ("before", "small_before_field")])
def test_small_channel_matches_reference(golden, pos, key):
    spec = o.ChannelSpec(**SMALL, position=pos)
    out = {}
    for prec in ["ref", "fp64"]:
        scr = [o.ss_screen(golden["small_rho"][i], golden["small_theta"][i], golden["small_value"][i],
                           spec.N, spec.delta, prec=prec) for i in range(spec.count)]
        u0 = o.gaussian_source(spec.N, spec.delta, spec.wvl, spec.w0, spec.F0, prec)
        out[prec] = o.propagate(u0, scr, o.screen_positions(spec.length, spec.count, pos),
                                spec.length, spec.k, spec.delta, prec=prec)
    assert o.rel_l2(out["ref"], golden[key]) < 3e-5
    assert o.rel_l2(out["fp64"], golden[key]) < 1e-3
    if pos == "middle":
        m = o.measures(out["ref"], spec.delta, [spec.pupil_radius], "ref")
        for k in ["mean_x", "mean_y", "mean_x2", "mean_xy", "mean_y2"]:
            assert m[k] == pytest.approx(float(golden[f"small_{k}"]), rel=1e-5, abs=1e-9)
        assert m["eta_0"] == pytest.approx(float(golden["small_eta_pupil"]), rel=1e-5)


@pytest.mark.parametrize("cfg", ["c1", "c2"])
def test_psd_matches_reference(golden, cfg):
    spec = o.ChannelSpec() if cfg == "c1" else o.ChannelSpec(
        N=2048, delta=1.5e-3, w0=0.12, length=50e3, Cn2=5e-16, pupil_radius=0.2)
    base = o.logpolar_base(spec.points, spec.f_min, spec.f_max)
    assert np.array_equal(base, golden[f"{cfg}_base"])
    psd = o.annulus_psd(base, spec.k, spec.thickness, spec.Cn2, spec.l0, spec.L0, use_scipy=False)
    np.testing.assert_allclose(psd, golden[f"{cfg}_psd"], rtol=2e-7)


def test_simulation_measures_match_reference(golden):
    """Beam / PDT / tracked-PDT scalars of 4 realisations of the basic channel (512^2, 5 screens,
    1024 spectral points) through the reference's Simulation."""
    spec = o.ChannelSpec()
    base = o.logpolar_base(spec.points, spec.f_min, spec.f_max)
    psd = o.annulus_psd(base, spec.k, spec.thickness, spec.Cn2, spec.l0, spec.L0, use_scipy=False)
    rho, theta, value = o.draw_spectra(1234, range(4), spec.count, base, psd)
    res = o.simulate(spec, rho, theta, value, prec="ref")
    for k in ["mean_x", "mean_y", "mean_x2", "mean_xy", "mean_y2", "mean_x2_r", "eta_0"]:
        got = np.array([r[k] for r in res])
        np.testing.assert_allclose(got, golden[f"c1_{k}"], rtol=1e-4, atol=2e-7)


def test_vacuum_known_answers():
    """itest_vacuum_propagation.ipynb cells 4-7: eta = 1, |sum u| delta^2 =
    sqrt(2 pi) w0, sum I delta^2 = 1 and the analytic waist."""
    N, d, wvl, w0, L = 256, 2e-3, 809e-9, 0.02, 4e3
    u = o.vacuum(o.gaussian_source(N, d, wvl, w0, np.inf), L, 2 * np.pi / wvl, d)
    I = np.abs(u) ** 2
    assert I.sum() * d ** 2 == pytest.approx(1, abs=1e-6)
    assert abs(u.sum()) * d ** 2 == pytest.approx(np.sqrt(2 * np.pi) * w0, abs=1e-7)
    m = o.measures(u, d)
    zR = np.pi * w0 ** 2 / wvl
    assert np.sqrt(2 * (m["mean_x2"] + m["mean_y2"])) == pytest.approx(w0 * np.sqrt(1 + (L / zR) ** 2), abs=1e-7)


def test_fft_screen_matches_reference(golden):
    normals = [golden["fft_normals"][0]] + [golden["fft_sub_normals"][i] for i in range(3)]
    k = 2 * np.pi / 808e-9
    s = o.fft_screen(normals, 64, 2e-3, k, 1e3, 1e-14, 6e-3, 1e3, 3)
    ref = golden["fft_screen"]
    assert o.rel_l2(s, ref) < 1e-5
