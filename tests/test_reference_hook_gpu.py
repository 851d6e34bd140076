"""The stock reference package (installed under baseline/_ref) with its
gpu.config switch set to the engine: the seeded runs of the golden vectors,
made by running the reference itself, come out of the engine.

* Channel.run (channels.py:31-35) runs as one fused atm_run;
* Simulation.run (simulations/simulation.py:127-138) with BeamResult,
  PDTResult and TrackedPDTResult takes the batched engine path;
* a Simulation with a measure the engine does not fuse runs the reference's
  own loop, whose VacuumPath and SSPhaseScreen steps go to atm_vacuum /
  atm_screen, and agrees with the same loop on the reference's numpy path.
The reference computes its screens with float32 phase arguments (2-5e-4
field error against FP64); the engine is within 1e-6 of FP64, so the
comparisons use the reference's own error as the tolerance."""
import numpy as np
import pytest

from oracle import atm_oracle as o

pytestmark = pytest.mark.gpu

REF_TOL = 2e-3


@pytest.fixture
def hooked(stock_reference):
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    from pyatmosphere_gb300 import reference_hook as hook
    ref = stock_reference
    hook.install(ref)
    ref.gpu.config["engine"] = "gb300"
    yield ref
    ref.gpu.config["engine"] = None
    hook.uninstall(ref)


def golden_channel(ref):
    """The channel of the golden seeded runs: 128^2, delta 3 mm, w0 6 cm,
    5 km, 3 screens (MVK Cn2 2e-15, 256 annuli), pupil 8 cm."""
    from pyatmosphere.channels import Channel
    from pyatmosphere.grids import RandLogPolarGrid, RectGrid
    from pyatmosphere.pathes import IdenticalPhaseScreensPath
    from pyatmosphere.phase_screens import SSPhaseScreen
    from pyatmosphere.pupils import CirclePupil
    from pyatmosphere.sources import GaussianSource
    from pyatmosphere.theory.models import MVKModel
    return Channel(
        grid=RectGrid(resolution=128, delta=3e-3), source=GaussianSource(wvl=808e-9, w0=0.06, F0=np.inf),
        path=IdenticalPhaseScreensPath(
            phase_screen=SSPhaseScreen(model=MVKModel(Cn2=2e-15, l0=6e-3, L0=1e3),
                                       f_grid=RandLogPolarGrid(points=256, f_min=1 / 1e3 / 15, f_max=2 / 6e-3)),
            length=5e3, count=3),
        pupil=CirclePupil(radius=0.08))


def test_switch_runs_the_reference_channel_on_the_engine(hooked, golden):
    ref = hooked
    ch = golden_channel(ref)
    np.random.seed(123)
    u = ch.run(pupil=False)
    assert isinstance(u, np.ndarray) and u.dtype == np.complex64
    assert "_atm_plans" in ch.__dict__, "the fused engine call did not run"
    assert o.rel_l2(u, golden["seeded_run_field"]) < REF_TOL


def test_switch_runs_the_reference_simulation_batched(hooked, golden):
    ref = hooked
    from pyatmosphere.simulations import BeamResult, PDTResult, Simulation, TrackedPDTResult
    np.random.seed(321)
    ch = golden_channel(ref)
    beam, pdt, tpdt = BeamResult(ch, max_size=3), PDTResult(ch, max_size=5), TrackedPDTResult(ch, max_size=5)
    sim = Simulation([beam, pdt, tpdt])
    sim.run()
    assert any(k[0] != "vacuum-steps" for k in ch.__dict__.get("_atm_plans", {})), "no batched engine plan"
    np.testing.assert_allclose(pdt.measures[0].data, golden["seeded_sim_eta"], rtol=1e-3)
    np.testing.assert_allclose(tpdt.measures[2].data, golden["seeded_sim_tracked_eta"], rtol=1e-3)
    width = np.sqrt(np.asarray(golden["seeded_sim_mean_x2"], float))
    for i, nm in enumerate(["mean_x", "mean_y", "mean_x2", "mean_xy", "mean_y2", "mean_x2_r"]):
        g = np.asarray(golden[f"seeded_sim_{nm}"], float)
        scale = width if nm in ("mean_x", "mean_y") else np.asarray(golden["seeded_sim_mean_x2"], float)
        assert np.all(np.abs(np.asarray(beam.measures[i].data, float) - g) <= 1e-3 * scale), nm


def test_unfused_measures_run_the_reference_loop_on_engine_steps(hooked):
    ref = hooked
    from pyatmosphere import measures
    from pyatmosphere.simulations import Measure, Simulation

    def run(engine):
        ref.gpu.config["engine"] = "gb300" if engine else None
        np.random.seed(99)
        ch = golden_channel(ref)
        m_eta = Measure(ch, "pupil", measures.eta, max_size=2)
        m_peak = Measure(ch, "atmosphere", lambda c, output: float(np.abs(output).max()), name="peak", max_size=2)
        Simulation(measures_list=[m_eta, m_peak]).run()
        steps = [k for k in ch.__dict__.get("_atm_plans", {}) if k[0] == "vacuum-steps"]
        return np.array(m_eta.data, float), np.array(m_peak.data, float), steps

    eta_e, peak_e, steps_e = run(True)
    eta_r, peak_r, steps_r = run(False)
    assert steps_e and not steps_r, "the engine's vacuum steps did not run"
    np.testing.assert_allclose(eta_e, eta_r, rtol=REF_TOL)
    np.testing.assert_allclose(peak_e, peak_r, rtol=5 * REF_TOL)
