"""The tiled field layout (ATM_FLAG_TILED: 4 x 4 blocks of 128 bytes between
passes) against the row-major forms and the FP64 oracle.

The tiled row pass (variant 5) and column pass (variant 5) run the same FFT
arithmetic as the row-major bulk-copy row pass (variant 3) and the TMA column
pass with alternating exchanges (variant 4); the product-twiddle forms (tiled
row 6, 8, 9 and 10, column 8 and 9; row-major row 4 and 7, column 2 and 7) share another
arithmetic, with or without the twiddle bases in registers.  The measures reduce one row
per partial in both at N = 2048: there the results are equal bit for bit.  At
N = 512 and 1024 the row-major forms sum several rows per partial, so the
moments agree to FP64 round-off and the field bit for bit."""
import numpy as np
import pytest

from oracle import atm_oracle as o

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda():
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    return torch


def _plans(spec, batch, **kw):
    from pyatmosphere_gb300.engine import EnginePlan, _lib
    base = o.logpolar_base(spec.points, spec.f_min, spec.f_max)
    pos = o.screen_positions(spec.length, spec.count) if spec.count else []
    common = dict(f_base=base, pupils=[(spec.pupil_radius,)], batch=batch, **kw)
    rm = EnginePlan(spec.N, spec.delta, spec.wvl, spec.w0, spec.F0, pos, spec.length, **common)
    rm.set_variants(3, 4, 4)
    tl = EnginePlan(spec.N, spec.delta, spec.wvl, spec.w0, spec.F0, pos, spec.length, flags=_lib.FLAG_TILED,
                    **common)
    assert tl.info["tiled"] == 1 and rm.info["tiled"] == 0
    tl.set_variants(5, 4, 5)  # the table-twiddle tiled forms: rm's arithmetic
    return rm, tl, base


def _spectra(spec, base, seed, R):
    psd = o.annulus_psd(base, spec.k, spec.thickness, spec.Cn2, spec.l0, spec.L0, use_scipy=False)
    return o.draw_spectra(seed, range(R), spec.count, base, psd)


@pytest.mark.parametrize("N", [512, 1024, 2048])
def test_tiled_run_equals_row_major(torch_cuda, N):
    torch = torch_cuda
    spec = o.ChannelSpec(N=N, delta=3.0 / N, w0=0.12, length=20e3, count=3, points=512, Cn2=5e-16,
                         pupil_radius=0.2)
    R = 3
    rm, tl, base = _plans(spec, R)
    dev = [torch.from_numpy(a).cuda() for a in _spectra(spec, base, 11, R)]
    f_rm = torch.empty((R, N, N), dtype=torch.complex64, device="cuda")
    f_tl = torch.empty_like(f_rm)
    m_rm = rm.run(*dev, field_out=f_rm).cpu().numpy()
    m_tl = tl.run(*dev, field_out=f_tl).cpu().numpy()
    tl.check()
    assert torch.equal(f_rm, f_tl), "tiled and row-major fields differ"
    if N == 2048:
        np.testing.assert_array_equal(m_tl, m_rm)
    else:
        np.testing.assert_allclose(m_tl, m_rm, rtol=1e-12, atol=1e-18)
    rm.close()
    tl.close()


@pytest.mark.parametrize("row_variant,col_variant", [(5, 5), (6, 5), (5, 6), (6, 6), (8, 8), (6, 9), (9, 9),
                                                      (10, 8)])
def test_tiled_run_matches_oracle(torch_cuda, row_variant, col_variant):
    torch = torch_cuda
    spec = o.ChannelSpec(N=512, delta=2e-3, w0=0.09, length=10e3, count=5, points=1024, Cn2=1e-15,
                         pupil_radius=0.12)
    _, tl, base = _plans(spec, 2)
    tl.set_variants(row_variant, 4, col_variant)
    rho, theta, value = _spectra(spec, base, 3, 2)
    dev = [torch.from_numpy(a).cuda() for a in (rho, theta, value)]
    field = torch.empty((2, 512, 512), dtype=torch.complex64, device="cuda")
    meas = tl.run(*dev, field_out=field).cpu().numpy()
    field = field.cpu().numpy()
    for b in range(2):
        res, u = o.simulate(spec, rho[b:b + 1], theta[b:b + 1], value[b:b + 1], return_field=True)
        assert o.rel_l2(field[b], u) < 1e-4
        for k, slot in [("eta_total", 0), ("mean_x", 1), ("mean_y", 2), ("mean_x2", 3), ("eta_0", 8)]:
            assert meas[b, slot] == pytest.approx(res[0][k], rel=2e-5, abs=2e-9), k


@pytest.mark.parametrize("N", [512, 2048])
def test_tiled_vacuum_and_measures(torch_cuda, N):
    """atm_vacuum converts the caller's row-major field to the tiled layout and
    back; atm_measures reads the caller's row-major field."""
    torch = torch_cuda
    spec = o.ChannelSpec(N=N, delta=3.0 / N, w0=0.3, count=0, length=2e3, pupil_radius=0.5)
    rm, tl, _ = _plans(spec, 2)
    rng = np.random.default_rng(N)
    u0 = o.gaussian_source(N, spec.delta, spec.wvl, 0.3, float("inf"))
    f = np.stack([u0, u0 * (1 + 0.1 * rng.standard_normal((N, N)))]).astype(np.complex64)
    a = torch.from_numpy(f).cuda()
    b = a.clone()
    rm.vacuum(a, 987.0)
    tl.vacuum(b, 987.0)
    assert torch.equal(a, b)
    # different kernels reduce the moments (their FP32 per-thread sums may contract differently)
    np.testing.assert_allclose(tl.measures(b).cpu().numpy(), rm.measures(a).cpu().numpy(), rtol=1e-6, atol=1e-15)
    tl.check()


def test_tiled_step_measures_and_tracked(torch_cuda):
    from pyatmosphere_gb300.engine import _lib
    torch = torch_cuda
    spec = o.ChannelSpec(N=2048, delta=1.5e-3, w0=0.12, length=20e3, count=2, points=512, Cn2=5e-16,
                         pupil_radius=0.2)
    R = 2
    from pyatmosphere_gb300.engine import EnginePlan
    base = o.logpolar_base(spec.points, spec.f_min, spec.f_max)
    pos = o.screen_positions(spec.length, spec.count)
    kw = dict(f_base=base, pupils=[(0.2,)], tracked=(0.15,), batch=R)
    rm = EnginePlan(spec.N, spec.delta, spec.wvl, spec.w0, spec.F0, pos, spec.length,
                    flags=_lib.FLAG_STEP_MEASURES, **kw)
    rm.set_variants(3, 4, 4)
    tl = EnginePlan(spec.N, spec.delta, spec.wvl, spec.w0, spec.F0, pos, spec.length,
                    flags=_lib.FLAG_STEP_MEASURES | _lib.FLAG_TILED, **kw)
    dev = [torch.from_numpy(a).cuda() for a in _spectra(spec, base, 5, R)]
    np.testing.assert_allclose(tl.run(*dev).cpu().numpy(), rm.run(*dev).cpu().numpy(), rtol=1e-6, atol=1e-15)
    tl.check()


def test_tiled_autotune_keeps_tiled_forms(torch_cuda):
    spec = o.ChannelSpec(N=2048, delta=1.5e-3, count=2, points=256, length=10e3)
    _, tl, _ = _plans(spec, 2)
    choice = tl.autotune(repeats=1)
    # 13: the warp-FFT column groups on whole 128-byte blocks (N = 1024, 2048)
    assert choice["row_variant"] in (5, 6, 8, 9, 10) and choice["col_variant"] in (5, 6, 8, 9, 13)
    assert choice["col_tile"] == 4
    assert tl.info["tiled"] == 1


def test_register_twiddles_give_the_product_twiddle_bits(torch_cuda):
    """Twiddle bases held in registers (row 8 / column 8 tiled, row 7 / column 7
    row-major) form the twiddles as the table product forms do (row 6 / column 9
    tiled, row 4 / column 2 row-major): the runs agree bit for bit."""
    torch = torch_cuda
    spec = o.ChannelSpec(N=2048, delta=1.5e-3, w0=0.12, length=20e3, count=3, points=512, Cn2=5e-16,
                         pupil_radius=0.2)
    R = 2
    rm, tl, base = _plans(spec, R)
    dev = [torch.from_numpy(a).cuda() for a in _spectra(spec, base, 17, R)]
    runs = {}
    for name, plan, v in (("rm table", rm, (4, 4, 2)), ("rm reg", rm, (7, 4, 7)), ("tiled reg", tl, (8, 4, 8)),
                          ("tiled table rows", tl, (6, 4, 8)), ("tiled table", tl, (6, 4, 9)),
                          ("tiled one-row", tl, (9, 4, 9)), ("tiled one-row reg", tl, (10, 4, 8))):
        plan.set_variants(*v)
        f = torch.empty((R, 2048, 2048), dtype=torch.complex64, device="cuda")
        m = plan.run(*dev, field_out=f).cpu().numpy()
        plan.check()
        runs[name] = (m, f)
    for name in ("rm reg", "tiled reg", "tiled table rows", "tiled table", "tiled one-row", "tiled one-row reg"):
        assert torch.equal(runs[name][1], runs["rm table"][1]), name
        # the tiled forms reduce the moments in other kernels: round-off apart
        np.testing.assert_allclose(runs[name][0], runs["rm table"][0], rtol=1e-9, atol=1e-15, err_msg=name)
    np.testing.assert_array_equal(runs["rm reg"][0], runs["rm table"][0])
