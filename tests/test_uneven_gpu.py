"""Mixed workloads (grid size, screen count and geometry varying per channel)
through one re-targeted plan per grid size: every channel gives the bits of
a fresh plan built for it alone, and the FP64 oracle's measures."""
import math

import numpy as np
import pytest

from oracle import atm_oracle as o

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def mix():
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    from pyatmosphere_gb300.engine.uneven import ChannelParams, run_uneven, sample_mixed
    rng = np.random.default_rng(3)
    chans = sample_mixed(6, rng, sizes=(128, 256), screens=(2, 5), length=(1e3, 5e3), Cn2=(1e-15, 1e-14),
                         w0=(0.05, 0.12), extent=1.0, pupil_radius=0.08, points=256)
    # a vacuum-free edge case: the largest screen count first, then fewer screens on the same plan
    chans.append(ChannelParams(N=256, n_screens=1, length=2e3, Cn2=5e-15, w0=0.08, wvl=1550e-9, focused=True,
                               extent=1.0, pupil_radius=0.08, points=256))
    res = run_uneven(chans, realisations=4, seed=9, keep_measures=True)
    return chans, res


def _fresh(c, i, R, seed):
    """Measures and spectra of channel i from a plan built for it alone."""
    import torch
    from pyatmosphere_gb300.engine import EnginePlan
    plan = EnginePlan(c.N, c.delta, c.wvl, c.w0, c.F0, c.positions(), c.length, f_base=c.base(),
                      pupils=[(c.pupil_radius,)], batch=R)
    n, P = c.n_screens, c.points
    rho = torch.empty((R, n, P), dtype=torch.float32, device="cuda")
    theta = torch.empty_like(rho)
    value = torch.empty((R, n, P), dtype=torch.complex64, device="cuda")
    sq = torch.from_numpy(c.sqrt_psd()).cuda().expand(n, -1).contiguous()
    plan.draw_spectra(seed, i * R, sq, rho, theta, value)
    m = plan.run(rho, theta, value).cpu().numpy()
    plan.close()
    return m, rho.cpu().numpy(), theta.cpu().numpy(), value.cpu().numpy()


def test_every_channel_matches_a_fresh_plan(mix):
    chans, res = mix
    assert res.pdt.shape == (len(chans), 64)
    np.testing.assert_allclose(res.pdt.sum(axis=1), 1.0, atol=1e-12)
    assert set(res.groups) == {128, 256}
    for i, c in enumerate(chans):
        m, *_ = _fresh(c, i, 4, 9)
        np.testing.assert_array_equal(res.measures[i], m)


def test_channels_match_the_oracle(mix):
    from pyatmosphere_gb300.engine import _lib
    chans, res = mix
    for i in (0, len(chans) - 1):
        c = chans[i]
        _, rho, theta, value = _fresh(c, i, 4, 9)
        spec = o.ChannelSpec(N=c.N, delta=c.delta, wvl=c.wvl, w0=c.w0, F0=c.F0, length=c.length,
                             count=c.n_screens, position="middle", Cn2=c.Cn2, l0=c.l0, L0=c.L0, points=c.points,
                             pupil_radius=c.pupil_radius)
        ref = o.simulate(spec, rho, theta, value)
        got = res.measures[i]
        for r in range(4):
            assert got[r, _lib.OUT_PUPIL0] == pytest.approx(ref[r]["eta_0"], rel=2e-5, abs=1e-7)
            assert got[r, _lib.OUT_ETA_TOTAL] == pytest.approx(ref[r]["eta_total"], rel=2e-5)
            assert got[r, _lib.OUT_MEAN_X2] == pytest.approx(ref[r]["mean_x2"], rel=1e-4)
