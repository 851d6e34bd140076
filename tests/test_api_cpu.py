"""Host-side pieces of the API mirror: spectra drawing, PSD weights, result
CSV persistence, measure classification for the batched path."""
import numpy as np
import pytest

from oracle import atm_oracle as o


def test_spectrum_draws_match_oracle():
    from pyatmosphere_gb300.engine.spectra import draw_spectra
    spec = o.ChannelSpec()
    base = o.logpolar_base(spec.points, spec.f_min, spec.f_max)
    psd = o.annulus_psd(base, spec.k, spec.thickness, spec.Cn2, spec.l0, spec.L0, use_scipy=False)
    a = draw_spectra(9, range(3), 5, base, psd)
    b = o.draw_spectra(9, range(3), 5, base, psd)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)


def test_psd_weights_match_reference(golden):
    from pyatmosphere_gb300.engine.spectra import annulus_psd
    from pyatmosphere_gb300.theory.models import MVKModel
    for cfg, (Cn2, L) in {"c1": (1e-15, 10e3), "c2": (5e-16, 50e3)}.items():
        m = MVKModel(Cn2=Cn2, l0=6e-3, L0=1e3)
        psd = annulus_psd(golden[f"{cfg}_base"], m.psd_phi_f, 2 * np.pi / 808e-9, L / 5)
        np.testing.assert_allclose(psd, golden[f"{cfg}_psd"], rtol=2e-7)


def test_screen_spectrum_follows_reference_rng_order():
    """SSPhaseScreen._get_spectrum draws u, then P uniforms, then 2P normals
    from numpy's global RNG (grids.py:98-107, phase_screens.py:98-103)."""
    import pyatmosphere_gb300 as pa
    fg = pa.RandLogPolarGrid(points=64, f_min=1e-4, f_max=300)
    ps = pa.SSPhaseScreen(fg, pa.MVKModel(1e-15, 6e-3, 1e3), thickness=1e3, wvl=808e-9,
                          grid=pa.RectGrid(128, 2e-3))
    np.random.seed(4)
    sp = ps._get_spectrum(False)
    np.random.seed(4)
    u = np.random.random(size=(1,)).astype(np.float32)
    t = np.random.random(size=(64,)).astype(np.float32)
    ab = np.random.normal(size=(2, 64))
    base = fg.base
    fp = np.insert(base, 0, 0)[:-1]
    assert np.array_equal(sp.rho, np.sqrt(fp ** 2 + u * (base ** 2 - fp ** 2)))
    assert np.array_equal(sp.theta, 2 * np.pi * t)
    assert np.array_equal(sp.value, (ab[0] + 1j * ab[1]).astype(np.complex64) * np.sqrt(ps._get_psd()))


def test_result_csv_round_trip(tmp_path):
    import pyatmosphere_gb300 as pa
    from pyatmosphere_gb300 import simulations
    ch = pa.QuickChannel()
    path = str(tmp_path / "pdt.csv")
    r = simulations.PDTResult(ch, max_size=10, save_path=path)
    r.measures[0].data = [0.123456, 0.5, 1e-7]
    r.save_output()
    text = open(path).read().splitlines()
    assert text[0] == "0.02" and text[1] == "1.235e-01"
    r2 = simulations.PDTResult(ch, max_size=10, save_path=path)
    assert r2.measures[0].data == pytest.approx([0.1235, 0.5, 1e-7], rel=1e-3)


def test_batched_path_classification():
    import pyatmosphere_gb300 as pa
    from pyatmosphere_gb300 import measures, simulations
    ch = pa.QuickChannel()
    sim = simulations.Simulation([simulations.BeamResult(ch, max_size=2), simulations.PDTResult(ch, max_size=2),
                                  simulations.TrackedPDTResult(ch, max_size=2)])
    plans = sim._batch_plan()
    kinds = sorted({k[0] for _, k, _ in plans[ch]})
    assert kinds == ["pupil", "slot", "tracked"]
    sim2 = simulations.Simulation(measures_list=[simulations.Measure(ch, "atmosphere", lambda c, output: 0.0)])
    assert sim2._batch_plan() is None
    # wind (time-shifted), per-step and first-screen structure-function measures are fused too
    sim3 = simulations.Simulation([simulations.TimeCoherenceResult(ch, [0, 1], max_size=2),
                                   simulations.SIResult(ch, max_size=2),
                                   simulations.BeamPropagationResult(ch, max_size=2)])
    plans3 = sim3._batch_plan()
    assert sorted({(k[0], t) for _, k, t in plans3[ch]}) == [("pupil", (0, 1)), ("step", None),
                                                              ("step_mean_r", None), ("step_mean_r2", None)]
    sim4 = simulations.Simulation([simulations.StructureFunctionResult(ch, max_size=2)])
    assert [k for _, k, _ in sim4._batch_plan()[ch]] == [("screen_sf",)]


def test_step_values_resolve_to_screens_then_receiver():
    from pyatmosphere_gb300.engine import _lib
    from pyatmosphere_gb300.simulations.fused import resolve
    n, pupils = 3, [(0.1, 0.0, 0.0)]
    base = _lib.OUT_PUPIL0 + 1
    out = np.zeros((2, base + _lib.STEP_SLOTS * n))
    out[:, _lib.OUT_I_CENTER] = [7.0, 8.0]
    for i in range(n):
        out[:, base + i * _lib.STEP_SLOTS + _lib.OUT_I_CENTER] = [i, 10 + i]
        out[:, base + i * _lib.STEP_SLOTS + _lib.OUT_MEAN_X] = 3.0
        out[:, base + i * _lib.STEP_SLOTS + _lib.OUT_MEAN_Y] = 4.0
    v = resolve(("step", _lib.OUT_I_CENTER), out, pupils, [], n)
    assert v.tolist() == [[0, 1, 2, 7], [10, 11, 12, 8]]
    r = resolve(("step_mean_r",), out, pupils, [], n)
    assert r[:, :3].tolist() == [[5.0] * 3] * 2 and r[:, 3].tolist() == [0.0, 0.0]


def test_theory_vacuum_rejects_other_grids_before_touching_a_device():
    """theory.vacuum.vacuum_propagation runs on the field's own frequency grid
    (f_delta = 1 / (N delta)); other grids and non-square fields are refused."""
    import numpy as np
    import pytest
    from pyatmosphere_gb300.theory.vacuum import vacuum_propagation
    u = np.zeros((64, 64), np.complex64)
    with pytest.raises(ValueError):
        vacuum_propagation(u, 1e3, 2 * np.pi / 1e-6, 1e-3, f_delta=1.0)
    with pytest.raises(ValueError):
        vacuum_propagation(np.zeros((64, 32), np.complex64), 1e3, 2 * np.pi / 1e-6, 1e-3)
    with pytest.raises(ValueError):
        vacuum_propagation(u, 1e3, 2 * np.pi / 1e-6, 1e-3, f2=np.zeros((32, 32)))
    # same shape, other values: a grid the engine would not use is refused too
    with pytest.raises(ValueError):
        vacuum_propagation(u, 1e3, 2 * np.pi / 1e-6, 1e-3, f2=np.ones((64, 64)))


def test_theory_vacuum_accepts_the_reference_f2_grid():
    """The f^2 grid the reference passes (RectGrid.get_f_grid().get_rho2(),
    pathes.py:31-38) is the grid the engine builds."""
    import numpy as np
    from pyatmosphere_gb300.theory import vacuum as V
    for N, delta in ((64, 1e-3), (2048, 1.5e-3), (512, 2e-3)):
        f = (np.arange(N) - N // 2).astype(np.float32) * (1 / (N * delta))  # float32 axis times a python float
        ref_f2 = f.reshape(1, -1) ** 2 + f.reshape(-1, 1) ** 2
        V._check_grid(ref_f2, 1 / (N * delta), N, delta)  # no exception


def test_mixed_workload_sampler_follows_its_distribution():
    """engine.uneven.sample_mixed: N from the size set with N delta = 3 m,
    screen counts on the closed range, log-uniform L and Cn2 inside their
    ranges, F0 either infinity or L; middle-of-slab screen positions."""
    import math
    import numpy as np
    from pyatmosphere_gb300.engine.uneven import sample_mixed
    chans = sample_mixed(400, np.random.default_rng(5))
    assert {c.N for c in chans} == {512, 1024, 2048, 4096}
    assert all(abs(c.N * c.delta - 3.0) < 1e-12 for c in chans)
    counts = [c.n_screens for c in chans]
    assert min(counts) == 3 and max(counts) == 20
    assert all(1e3 <= c.length <= 1e5 and 1e-16 <= c.Cn2 <= 1e-14 and 0.02 <= c.w0 <= 0.2 for c in chans)
    assert {c.wvl for c in chans} == {808e-9, 1550e-9}
    assert {math.isinf(c.F0) for c in chans} == {True, False}
    assert all(c.F0 == c.length for c in chans if not math.isinf(c.F0))
    c = chans[0]
    pos = c.positions()
    np.testing.assert_allclose(np.diff(pos), c.length / c.n_screens)
    assert pos[0] == pytest.approx(0.5 * c.length / c.n_screens)
    b = c.base()
    assert b[0] == pytest.approx(c.f_min, rel=1e-6) and b[-1] == pytest.approx(2 / c.l0, rel=1e-6)
