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


def test_graph_mix_matches_the_sequential_run(mix):
    """The whole mix as one CUDA graph launch (channel table sets,
    atm_run_channel, one stream per grid size): every channel's measures and
    PDT equal the re-targeted sequential run's, bit for bit (hence a fresh
    plan's, by the test above)."""
    from pyatmosphere_gb300.engine.uneven import run_uneven_graph
    chans, res = mix
    g = run_uneven_graph(chans, realisations=4, seed=9, keep_measures=True)
    assert g.groups["graph"]["launches"] == 1
    for i in range(len(chans)):
        np.testing.assert_array_equal(g.measures[i], res.measures[i])
    np.testing.assert_array_equal(g.pdt, res.pdt)


def test_channel_table_sets_on_one_plan():
    """atm_run_channel with a table set equals atm_plan_update + atm_run on the
    same plan, and leaves the plan's own channel in place."""
    import torch
    from pyatmosphere_gb300.engine import EnginePlan
    from pyatmosphere_gb300.engine.uneven import ChannelParams
    a = ChannelParams(N=256, n_screens=4, length=4e3, Cn2=2e-15, w0=0.06, wvl=808e-9, extent=1.0, points=256,
                      pupil_radius=0.08)
    b = ChannelParams(N=256, n_screens=2, length=1.5e3, Cn2=8e-15, w0=0.1, wvl=1550e-9, focused=True, extent=1.0,
                      points=256, pupil_radius=0.05)
    R = 3
    plan = EnginePlan(a.N, a.delta, a.wvl, a.w0, a.F0, a.positions(), a.length, f_base=a.base(),
                      pupils=[(a.pupil_radius,)], batch=R)
    ch = plan.channel(b.wvl, b.w0, b.F0, b.positions(), b.length, pupils=[(b.pupil_radius,)])
    rho = torch.empty((R, 2, 256), dtype=torch.float32, device="cuda")
    theta = torch.empty_like(rho)
    value = torch.empty((R, 2, 256), dtype=torch.complex64, device="cuda")
    plan.draw_spectra(4, 0, torch.from_numpy(b.sqrt_psd()).cuda().expand(2, -1).contiguous(), rho, theta, value,
                      channel=ch)
    ra = torch.empty((R, 4, 256), dtype=torch.float32, device="cuda")
    ta = torch.empty_like(ra)
    va = torch.empty((R, 4, 256), dtype=torch.complex64, device="cuda")
    plan.draw_spectra(5, 0, torch.from_numpy(a.sqrt_psd()).cuda().expand(4, -1).contiguous(), ra, ta, va)
    own = plan.run(ra, ta, va).cpu().numpy()
    via_set = plan.run_channel(ch, rho, theta, value).cpu().numpy()
    np.testing.assert_array_equal(plan.run(ra, ta, va).cpu().numpy(), own)  # the plan's own channel is back
    plan.update(b.wvl, b.w0, b.F0, b.positions(), b.length, pupils=[(b.pupil_radius,)])
    np.testing.assert_array_equal(plan.run(rho, theta, value).cpu().numpy(), via_set)
    plan.check()
    ch.close()
    plan.close()
