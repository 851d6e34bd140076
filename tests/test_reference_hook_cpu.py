"""The engine behind the stock reference's own gpu.config switch, on CPU:
installing and removing the hook, the switch leaving the reference's own
methods in charge while it is off, and how the hook reads the reference's
object graph (geometry, fusable channels, which Simulation measures take the
batched engine path).  Skipped where the reference is not installed under
baseline/_ref."""
import numpy as np
import pytest


def ref_channel(ref, N=64, screen="ss", count=3):
    from pyatmosphere.channels import Channel
    from pyatmosphere.grids import RandLogPolarGrid, RectGrid
    from pyatmosphere.pathes import IdenticalPhaseScreensPath
    from pyatmosphere.phase_screens import FFTPhaseScreen, SSPhaseScreen
    from pyatmosphere.pupils import CirclePupil
    from pyatmosphere.sources import GaussianSource
    from pyatmosphere.theory.models import MVKModel
    model = MVKModel(Cn2=2e-15, l0=6e-3, L0=1e3)
    ps = (SSPhaseScreen(model=model, f_grid=RandLogPolarGrid(points=128, f_min=1 / 1e3 / 15, f_max=2 / 6e-3))
          if screen == "ss" else FFTPhaseScreen(subharmonics=1, model=model))
    return Channel(grid=RectGrid(resolution=N, delta=4e-3), source=GaussianSource(wvl=808e-9, w0=0.05, F0=np.inf),
                   path=IdenticalPhaseScreensPath(phase_screen=ps, length=4e3, count=count, losses_db=1.5),
                   pupil=CirclePupil(radius=0.06))


def test_install_is_idempotent_and_reversible(stock_reference):
    from pyatmosphere_gb300 import reference_hook as hook
    ref = stock_reference
    run0 = ref.channels.Channel.run
    hook.install(ref)
    hook.install(ref)
    assert hook.installed(ref) and ref.gpu.config.get("engine") is None
    assert ref.channels.Channel.run is not run0
    hook.uninstall(ref)
    assert not hook.installed(ref) and ref.channels.Channel.run is run0


def test_switch_off_leaves_the_reference_in_charge(stock_reference):
    from pyatmosphere_gb300 import reference_hook as hook
    ref = stock_reference
    np.random.seed(5)
    before = ref_channel(ref).run(pupil=False)
    hook.install(ref)
    try:
        ref.gpu.config["engine"] = None
        np.random.seed(5)
        after = ref_channel(ref).run(pupil=False)
    finally:
        hook.uninstall(ref)
    np.testing.assert_array_equal(before, after)


def test_geometry_is_read_from_the_reference_objects(stock_reference):
    from pyatmosphere_gb300.engine import runner
    ref = stock_reference
    ch = ref_channel(ref, count=4)
    pos, L, losses, base = runner.path_geometry(ch.path)
    np.testing.assert_allclose(pos, (np.arange(4) + 0.5) * 1e3)
    assert (L, losses) == (4e3, 1.5)
    np.testing.assert_array_equal(base, ch.path.phase_screens[0].f_grid.base)
    assert runner.source_kind(ch.source) == ("gaussian", 808e-9, 0.05, float("inf"))
    assert runner.grid_size(ch.grid) == 64
    assert runner.fusable(ch)
    fft = ref_channel(ref, screen="fft")
    assert runner.fusable(fft) and runner.screen_kind(fft.path) == "fft"  # atm_run_fft
    assert runner.screen_kind(ch.path) == "ss"


def test_batched_path_takes_the_reference_results(stock_reference):
    from pyatmosphere_gb300 import reference_hook as hook
    ref = stock_reference
    from pyatmosphere.simulations import BeamResult, Measure, PDTResult, Simulation, TrackedPDTResult
    ch = ref_channel(ref)
    sim = Simulation([BeamResult(ch, max_size=2), PDTResult(ch, max_size=2), TrackedPDTResult(ch, max_size=2)])
    plans = hook._batch_plan_reference(ref, sim)
    kinds = [k for _, k, _ in plans[ch]]
    assert ("slot", 1) in kinds and ("slot", 6) in kinds  # mean_x, BeamResult.mean_x2_r
    assert ("pupil", (0.06, 0.0, 0.0)) in kinds and ("tracked", (0.06,)) in kinds
    sim2 = Simulation(measures_list=[Measure(ch, "atmosphere", lambda c, output: 0.0)])
    assert hook._batch_plan_reference(ref, sim2) is None
