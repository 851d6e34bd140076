"""Channels of FFT phase screens (FFTPhaseScreen with subharmonics,
phase_screens.py:37-67) on the batched engine path: atm_run_fft builds every
realisation's screens on the device and propagates the batch, against the FP64
oracle (screens from the same draws, oracle split-step loop and measures),
and the Simulation's batched path against its per-realisation loop."""
import numpy as np
import pytest

from oracle import atm_oracle as o

pytestmark = pytest.mark.gpu

N, DELTA, WVL, W0, L, COUNT, SUB = 256, 4e-3, 808e-9, 0.08, 6e3, 3, 2
CN2, L0_IN, L0_OUT = 3e-15, 6e-3, 1e3


def _channel(pa, pupil=0.1):
    return pa.Channel(grid=pa.RectGrid(N, DELTA), source=pa.GaussianSource(wvl=WVL, w0=W0, F0=np.inf),
                      path=pa.IdenticalPhaseScreensPath(
                          phase_screen=pa.FFTPhaseScreen(SUB, model=pa.MVKModel(CN2, L0_IN, L0_OUT)),
                          length=L, count=COUNT),
                      pupil=pa.CirclePupil(pupil))


def test_batched_fft_run_matches_oracle():
    import torch
    import pyatmosphere_gb300 as pa
    from pyatmosphere_gb300.engine import _lib
    from pyatmosphere_gb300.engine.runner import draw_channel_fft, get_plan, to_device
    ch = _channel(pa)
    R = 3
    np.random.seed(12)
    normals, amp, sub_x, sub_y, sub_mean, n_sub = draw_channel_fft(ch, R)
    assert n_sub == 3 * SUB and normals.shape == (R, COUNT, 2, N, N)
    plan = get_plan(ch, batch=R, pupils=[(0.1, 0.0, 0.0)])
    assert plan.info is not None
    field = torch.empty((R, N, N), dtype=torch.complex64, device="cuda")
    got = plan.run_fft(*to_device(normals, amp, sub_x, sub_y, sub_mean), n_sub, field_out=field).cpu().numpy()
    plan.check()
    field = field.cpu().numpy()
    # the oracle: the same draws in the reference's per-realisation order
    np.random.seed(12)
    k = 2 * np.pi / WVL
    thickness = L / COUNT
    pos = o.screen_positions(L, COUNT)
    u0 = o.gaussian_source(N, DELTA, WVL, W0, np.inf)
    for r in range(R):
        screens = []
        for i in range(COUNT):
            draws = [np.stack([np.random.normal(size=(N, N)), np.random.normal(size=(N, N))])]
            draws += [np.stack([np.random.normal(size=(3, 3)), np.random.normal(size=(3, 3))]) for _ in range(SUB)]
            screens.append(o.fft_screen(draws, N, DELTA, k, thickness, CN2, L0_IN, L0_OUT, SUB).real)
        u = o.propagate(u0, screens, pos, L, k, DELTA, path_output_loss=False)
        ref = o.measures(u, DELTA, [0.1])
        assert o.rel_l2(field[r], u) < 1e-4
        assert got[r, _lib.OUT_ETA_TOTAL] == pytest.approx(ref["eta_total"], rel=1e-5)
        assert got[r, _lib.OUT_PUPIL0] == pytest.approx(ref["eta_0"], rel=2e-5, abs=1e-8)
        for key, slot in (("mean_x", _lib.OUT_MEAN_X), ("mean_y", _lib.OUT_MEAN_Y)):
            assert got[r, slot] == pytest.approx(ref[key], rel=1e-4, abs=1e-8)
        assert got[r, _lib.OUT_MEAN_X2] == pytest.approx(ref["mean_x2"], rel=1e-5)


def test_simulation_takes_the_batched_fft_path():
    """PDTResult / BeamResult over FFT screens: the batched path (one
    atm_run_fft per batch) gives the per-realisation Channel.run values."""
    import pyatmosphere_gb300 as pa
    from pyatmosphere_gb300 import measures, simulations
    # 0.101 m is 25.25 pixels: no pixel centre lies within float32 round-off of the rim, so the
    # mirror's float32 pupil and the fused FP64 pupil mask the same pixels (at 0.1 m = 25 pixels
    # the 20 lattice points on the rim flip between the two predicates)
    ch = _channel(pa, pupil=0.101)
    pdt = simulations.PDTResult(ch, max_size=4)
    beam = simulations.BeamResult(ch, max_size=4)
    sim = simulations.Simulation([pdt, beam])
    assert sim._batch_plan() is not None, "FFT channels must take the batched path"
    np.random.seed(33)
    sim.run()
    eta_batched = np.array(pdt.measures[0].data, dtype=float)
    np.random.seed(33)
    eta_loop = [measures.eta(ch, output=ch.run()) for _ in range(4)]
    # the same draws and engine kernels; the loop's eta sums the masked field on the host side of
    # the mirror (pupil pixels by the mirror's predicate), the batched path's in the fused reduction
    np.testing.assert_allclose(eta_batched.ravel(), np.array(eta_loop, dtype=float), rtol=2e-4, atol=1e-7)
    assert len(beam.measures[0].data) == 4
