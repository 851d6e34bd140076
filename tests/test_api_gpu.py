"""The reference-facing Python API on the engine: seeded runs reproduce the
reference's own realisations (same numpy RNG order), the batched Simulation
path agrees with the per-realisation path, and the step-by-step path object
agrees with the fused channel run."""
import numpy as np
import pytest

from oracle import atm_oracle as o

pytestmark = pytest.mark.gpu

# the reference computes screens with float32 phase arguments: ~2-5e-4 field error
REF_TOL = 2e-3


def small_channel(pa):
    return pa.Channel(
        grid=pa.RectGrid(resolution=128, delta=3e-3),
        source=pa.GaussianSource(wvl=808e-9, w0=0.06, F0=np.inf),
        path=pa.IdenticalPhaseScreensPath(
            phase_screen=pa.SSPhaseScreen(model=pa.MVKModel(Cn2=2e-15, l0=6e-3, L0=1e3),
                                          f_grid=pa.RandLogPolarGrid(points=256, f_min=1 / 1e3 / 15,
                                                                     f_max=2 / 6e-3)),
            length=5e3, count=3),
        pupil=pa.CirclePupil(radius=0.08))


def test_seeded_channel_run_reproduces_reference(golden):
    import pyatmosphere_gb300 as pa
    np.random.seed(123)
    u = small_channel(pa).run(pupil=False).cpu().numpy()
    assert o.rel_l2(u, golden["seeded_run_field"]) < REF_TOL


def test_seeded_simulation_reproduces_reference(golden):
    import pyatmosphere_gb300 as pa
    from pyatmosphere_gb300 import simulations
    np.random.seed(321)
    ch = small_channel(pa)
    beam = simulations.BeamResult(ch, max_size=3)
    pdt = simulations.PDTResult(ch, max_size=5)
    tpdt = simulations.TrackedPDTResult(ch, max_size=5)
    sim = simulations.Simulation([beam, pdt, tpdt])
    assert sim._batch_plan() is not None, "Beam / PDT / tracked PDT must take the batched path"
    sim.run()
    np.testing.assert_allclose(pdt.measures[0].data, golden["seeded_sim_eta"], rtol=1e-3)
    np.testing.assert_allclose(tpdt.measures[2].data, golden["seeded_sim_tracked_eta"], rtol=1e-3)
    for i, nm in enumerate(["mean_x", "mean_y", "mean_x2", "mean_xy", "mean_y2", "mean_x2_r"]):
        np.testing.assert_allclose(beam.measures[i].data, golden[f"seeded_sim_{nm}"], rtol=2e-2, atol=2e-5)
    assert len(beam.measures[0]) == 3 and len(pdt.measures[0]) == 5


def test_batched_simulation_equals_per_realisation_path():
    import pyatmosphere_gb300 as pa
    from pyatmosphere_gb300 import gpu, simulations
    results = []
    for batched in (True, False):
        np.random.seed(7)
        ch = small_channel(pa)
        beam = simulations.BeamResult(ch, max_size=4)
        pdt = simulations.PDTResult(ch, max_size=4)
        sim = simulations.Simulation([beam, pdt])
        if batched:
            gpu.config["batch"] = 3     # two engine calls: 3 + 1 realisations
            sim.run()
        else:
            while not sim.is_measures_done():
                sim.iter()
        results.append((np.array(pdt.measures[0].data, float), np.array(beam.measures[0].data, float),
                        np.array(beam.measures[5].data, float)))
    gpu.config["batch"] = 256
    for a, b in zip(*results):
        np.testing.assert_allclose(a, b, rtol=2e-5, atol=1e-8)


def test_path_generator_matches_fused_run():
    import torch
    import pyatmosphere_gb300 as pa
    np.random.seed(11)
    ch = small_channel(pa)
    fused = ch.run(pupil=False)
    np.random.seed(11)
    ch2 = small_channel(pa)
    steps = list(ch2.generator(pupil=False))
    assert len(steps) == 3
    assert tuple(steps[0][1].shape) == (128, 128)
    assert o.rel_l2(ch2.output.cpu().numpy(), fused.cpu().numpy()) < 1e-5


def test_measures_on_field_match_oracle():
    import pyatmosphere_gb300 as pa
    from pyatmosphere_gb300 import measures
    np.random.seed(5)
    ch = small_channel(pa)
    u = ch.run(pupil=False)
    ref = o.measures(u.cpu().numpy().astype(np.complex128), 3e-3, [0.08])
    assert measures.eta(ch, output=u) == pytest.approx(ref["eta_total"], rel=1e-6)
    assert measures.mean_x(ch, output=u) == pytest.approx(ref["mean_x"], rel=1e-5, abs=1e-10)
    assert measures.mean_xy(ch, output=u) == pytest.approx(ref["mean_xy"], rel=1e-5, abs=1e-12)
    assert measures.eta(ch, output=ch.pupil.output(u)) == pytest.approx(ref["eta_0"], rel=1e-5)


def test_vacuum_channel_length_override_and_known_answer():
    """itest_sources: mean_r2(channel, length=L, pupil=False) on a VacuumPath."""
    import pyatmosphere_gb300 as pa
    from pyatmosphere_gb300 import measures
    ch = pa.Channel(grid=pa.RectGrid(512, 5e-3), source=pa.GaussianSource(wvl=809e-9, w0=0.2, F0=np.inf),
                    path=pa.VacuumPath(length=4e3), pupil=pa.CirclePupil(0.1))
    for L in [0.0, 5000.0, 20000.0]:
        w = np.sqrt(2 * measures.mean_r2(ch, length=L, pupil=False))
        assert w == pytest.approx(ch.source.get_w(L), rel=1e-3)


def test_theory_vacuum_propagation_matches_oracle_and_runs_backwards():
    """theory.vacuum.vacuum_propagation (theory/vacuum.py:5-7) on the engine:
    a forward step equals the FP64 oracle's; a step back undoes it."""
    import torch
    from pyatmosphere_gb300.theory.vacuum import vacuum_propagation
    N, delta, wvl, L = 256, 4e-3, 1550e-9, 3e3
    k = 2 * np.pi / wvl
    rng = np.random.default_rng(12)
    x = (np.arange(N) - N // 2) * delta
    u = (np.exp(-(x[None, :] ** 2 + x[:, None] ** 2) / 0.1 ** 2) *
         np.exp(1j * rng.uniform(0, 0.5, (N, N)))).astype(np.complex64)
    got = vacuum_propagation(torch.from_numpy(u), L, k, delta, f_delta=1 / (N * delta))
    assert got.is_cuda and got.dtype == torch.complex64
    ref = o.vacuum(u, L, k, delta)
    g = got.cpu().numpy()
    assert np.linalg.norm(g - ref) / np.linalg.norm(ref) < 2e-5
    back = vacuum_propagation(got, -L, k, delta).cpu().numpy()
    assert np.linalg.norm(back - u) / np.linalg.norm(u) < 2e-5
    with pytest.raises(ValueError):
        vacuum_propagation(torch.from_numpy(u), L, k, delta, f_delta=2 / (N * delta))


def test_screen_generate_matches_oracle():
    import pyatmosphere_gb300 as pa
    ch = small_channel(pa)
    ch.path.init_phase_screens()
    ps = ch.path.phase_screens[0]
    np.random.seed(2)
    phi = ps.generate().cpu().numpy()
    np.random.seed(2)
    sp = ps._get_spectrum(False)
    ref = o.ss_screen(sp.rho, sp.theta, sp.value, 128, 3e-3)
    assert np.abs(phi - ref).max() < 2e-4


def test_fft_screen_matches_oracle():
    """FFTPhaseScreen with 3 subharmonic levels (phase_screens.py:42-67)."""
    import pyatmosphere_gb300 as pa
    N, d = 256, 2e-3
    ps = pa.FFTPhaseScreen(3, model=pa.MVKModel(Cn2=1e-14, l0=6e-3, L0=1e3), thickness=1e3, wvl=808e-9,
                           grid=pa.RectGrid(N, d))
    rng = np.random.default_rng(8)
    normals = [rng.standard_normal((2, N, N))] + [rng.standard_normal((2, 3, 3)) for _ in range(3)]
    got = ps.generate(complex=True, normals=normals).cpu().numpy()
    ref = o.fft_screen(normals, N, d, 2 * np.pi / 808e-9, 1e3, 1e-14, 6e-3, 1e3, 3)
    assert o.rel_l2(got, ref) < 1e-5
    real = ps.generate(normals=normals).cpu().numpy()
    assert np.abs(real - ref.real).max() < 1e-4 * np.abs(ref.real).max()


def test_fft_screen_channel_conserves_energy():
    import pyatmosphere_gb300 as pa
    from pyatmosphere_gb300 import measures
    ch = pa.Channel(grid=pa.RectGrid(256, 4e-3), source=pa.GaussianSource(wvl=808e-9, w0=0.08, F0=np.inf),
                    path=pa.IdenticalPhaseScreensPath(
                        phase_screen=pa.FFTPhaseScreen(2, model=pa.MVKModel(2e-15, 6e-3, 1e3)),
                        length=5e3, count=3),
                    pupil=pa.CirclePupil(0.1))
    np.random.seed(1)
    u = ch.run(pupil=False)
    assert measures.eta(ch, output=u) == pytest.approx(1.0, abs=2e-5)


def test_seeded_wind_results_reproduce_reference(golden):
    """TimeCoherenceResult / TimeBWcorrSimulation (time-shifted screens, one
    spectrum per realisation) on the batched engine path."""
    import pyatmosphere_gb300 as pa
    from pyatmosphere_gb300 import simulations
    np.random.seed(555)
    ch = small_channel(pa)
    times = list(golden["wind_times"])
    tc = simulations.TimeCoherenceResult(ch, times, max_size=4)
    bwc = simulations.TimeBWcorrSimulation(ch, times, max_size=4)
    sim = simulations.Simulation([tc, bwc])
    assert sim._batch_plan() is not None, "wind measures must take the batched path"
    sim.run()
    np.testing.assert_allclose(np.array(tc.measures[0].data), golden["wind_eta"], rtol=1e-3)
    np.testing.assert_allclose(np.array(bwc.measures[0].data), golden["wind_mean_x"], rtol=2e-2, atol=2e-5)
    np.testing.assert_allclose(np.array(bwc.measures[1].data), golden["wind_mean_y"], rtol=2e-2, atol=2e-5)
    assert len(tc.tc) == 3 and tc.tc[0] == pytest.approx(1.0)


def test_seeded_si_result_reproduces_reference(golden):
    """SIResult: on-axis intensity after every screen and at the receiver,
    from the engine's per-step measures."""
    import pyatmosphere_gb300 as pa
    from pyatmosphere_gb300 import simulations
    np.random.seed(777)
    ch = small_channel(pa)
    si = simulations.SIResult(ch, max_size=4)
    sim = simulations.Simulation([si])
    assert sim._batch_plan() is not None, "SIResult must take the batched path"
    sim.run()
    got = np.array(si.measures[0].data, float)
    assert got.shape == golden["si_center"].shape == (4, 4)
    # one pixel of a speckled field: the reference's FP32 screens move it by ~1e-3
    np.testing.assert_allclose(got, golden["si_center"], rtol=5e-3)


def test_batched_propagation_and_wind_equal_per_realisation_path():
    import pyatmosphere_gb300 as pa
    from pyatmosphere_gb300 import gpu, simulations
    results = []
    for batched in (True, False):
        np.random.seed(21)
        ch = small_channel(pa)
        bp = simulations.BeamPropagationResult(ch, max_size=3)
        si = simulations.SIResult(ch, max_size=3)
        tc = simulations.TimeCoherenceResult(ch, [0.0, 0.03], max_size=3)
        sim = simulations.Simulation([bp, si, tc])
        if batched:
            gpu.config["batch"] = 2
            sim.run()
        else:
            while not sim.is_measures_done():
                sim.iter()
        results.append([np.array(m.data, float) for m in (bp.measures[0], bp.measures[1], si.measures[0],
                                                           tc.measures[0])])
    gpu.config["batch"] = 256
    for a, b in zip(*results):
        assert a.shape == b.shape
        np.testing.assert_allclose(a, b, rtol=1e-4, atol=1e-9)


def test_seeded_structure_function_result_reproduces_reference(golden):
    """StructureFunctionResult of the first screen on the batched path
    (atm_screen + atm_structure_function) against the reference's own run."""
    import pyatmosphere_gb300 as pa
    from pyatmosphere_gb300 import simulations
    np.random.seed(888)
    ch = small_channel(pa)
    sfr = simulations.StructureFunctionResult(ch, max_size=2)
    sim = simulations.Simulation([sfr])
    assert sim._batch_plan() is not None
    sim.run()
    got = np.array(sfr.measures[0].data, float)
    ref = golden["sf_seeded"]
    assert got.shape == ref.shape == (2, 127)
    # the reference builds its screens with float32 phase arguments
    np.testing.assert_allclose(got, ref, rtol=1e-2)
    assert sfr.structure_function.shape == (127,)
