"""Parity of the CUDA engine (through the C ABI) with the FP64 oracle.

Tolerances: field rel-L2 <= 1e-4 against FP64 (the engine computes in
complex64 / FP32 with FP64 phase arguments); moments to 1e-5 relative."""
import math

import numpy as np
import pytest

from oracle import atm_oracle as o

pytestmark = pytest.mark.gpu

FIELD_TOL = 1e-4


@pytest.fixture(scope="module")
def torch_cuda():
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    return torch


def make_plan(spec, batch=1, pupils=None, tracked=(), **kw):
    from pyatmosphere_gb300.engine import EnginePlan
    base = o.logpolar_base(spec.points, spec.f_min, spec.f_max)
    positions = o.screen_positions(spec.length, spec.count, spec.position) if spec.count else []
    pupils = [(spec.pupil_radius,)] if pupils is None else pupils
    return EnginePlan(spec.N, spec.delta, spec.wvl, spec.w0, spec.F0, positions, spec.length,
                      f_base=base, losses_db=spec.losses_db, pupils=pupils, tracked=tracked,
                      batch=batch, **kw), base


def spectra(spec, base, seed, R):
    psd = o.annulus_psd(base, spec.k, spec.thickness, spec.Cn2, spec.l0, spec.L0, use_scipy=False)
    return o.draw_spectra(seed, range(R), spec.count, base, psd)


def to_dev(torch, *arrs):
    return [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in arrs]


@pytest.mark.parametrize("N", [128, 256, 512, 1024, 2048, 4096])
def test_vacuum_step_matches_oracle(torch_cuda, N):
    torch = torch_cuda
    d = 3.0 / N
    spec = o.ChannelSpec(N=N, delta=d, w0=0.3, count=0, length=2e3)
    plan, _ = make_plan(spec, batch=2, pupils=[])
    rng = np.random.default_rng(N)
    u0 = o.gaussian_source(N, d, spec.wvl, 0.3, math.inf)
    noise = (rng.standard_normal((N, N)) + 1j * rng.standard_normal((N, N))) * 0.2 * np.abs(u0)
    fields = np.stack([u0, u0 + noise]).astype(np.complex64)
    dev = torch.from_numpy(fields).cuda()
    plan.vacuum(dev, 1234.5)
    got = dev.cpu().numpy()
    for b in range(2):
        ref = o.vacuum(fields[b].astype(np.complex128), 1234.5, spec.k, d)
        assert o.rel_l2(got[b], ref) < 2e-6


@pytest.mark.parametrize("N,P,Cn2", [(128, 256, 1e-14), (512, 1024, 1e-15), (2048, 1024, 5e-16)])
def test_screen_matches_oracle(torch_cuda, N, P, Cn2):
    torch = torch_cuda
    d = 1.0 / N if N < 2048 else 1.5e-3
    spec = o.ChannelSpec(N=N, delta=d, points=P, Cn2=Cn2, count=2, length=10e3)
    plan, base = make_plan(spec, batch=2)
    rho, theta, value = spectra(spec, base, seed=N, R=2)
    r, t, v = to_dev(torch, rho, theta, value)
    phi = torch.empty((2, N, N), dtype=torch.float32, device="cuda")
    ph = torch.empty((2, N, N), dtype=torch.complex64, device="cuda")
    plan.screen(r, t, v, 1, phi_out=phi, phasor_out=ph)
    phi, ph = phi.cpu().numpy(), ph.cpu().numpy()
    for b in range(2):
        ref = o.ss_screen(rho[b, 1], theta[b, 1], value[b, 1], N, d)
        assert o.rel_l2(ph[b], np.exp(-1j * ref)) < 1e-5
        # float32 output of a screen whose piston reaches ~1e3 rad
        assert np.abs(phi[b] - ref).max() < 2e-4 * max(1.0, np.abs(ref).max() / 1e3)


def run_engine(torch, spec, rho, theta, value, pupils=None, tracked=()):
    R = rho.shape[0]
    plan, _ = make_plan(spec, batch=R, pupils=pupils, tracked=tracked)
    r, t, v = to_dev(torch, rho, theta, value)
    field = torch.empty((R, spec.N, spec.N), dtype=torch.complex64, device="cuda")
    meas = plan.run(r, t, v, field_out=field)
    return plan, meas.cpu().numpy(), field.cpu().numpy()


@pytest.mark.parametrize("position", ["middle", "before", "after"])
def test_channel_run_matches_oracle(torch_cuda, position):
    torch = torch_cuda
    spec = o.ChannelSpec(N=256, delta=4e-3, w0=0.08, length=8e3, count=4, points=512, Cn2=2e-15,
                         pupil_radius=0.1, position=position)
    base = o.logpolar_base(spec.points, spec.f_min, spec.f_max)
    rho, theta, value = spectra(spec, base, seed=5, R=3)
    plan, meas, field = run_engine(torch, spec, rho, theta, value)
    for b in range(3):
        res, u = o.simulate(spec, rho[b:b + 1], theta[b:b + 1], value[b:b + 1], return_field=True)
        assert o.rel_l2(field[b], u) < FIELD_TOL
        m = res[0]
        for k, slot in [("eta_total", 0), ("mean_x", 1), ("mean_y", 2), ("mean_x2", 3), ("mean_xy", 4),
                        ("mean_y2", 5), ("mean_x2_r", 6), ("eta_0", 8)]:
            assert meas[b, slot] == pytest.approx(m[k], rel=2e-5, abs=2e-9), k


def test_config1_realisations_match_oracle(torch_cuda):
    """512^2, 5 screens, 1024 spectral points, pupil 0.12 m (config 1 geometry)."""
    torch = torch_cuda
    spec = o.ChannelSpec()
    base = o.logpolar_base(spec.points, spec.f_min, spec.f_max)
    rho, theta, value = spectra(spec, base, seed=1234, R=4)
    plan, meas, field = run_engine(torch, spec, rho, theta, value, tracked=(0.12,))
    res, u = o.simulate(spec, rho[3:4], theta[3:4], value[3:4], return_field=True)
    assert o.rel_l2(field[3], u) < FIELD_TOL
    ref = o.simulate(spec, rho, theta, value)
    for b in range(4):
        assert meas[b, 8] == pytest.approx(ref[b]["eta_0"], rel=1e-5)
        assert meas[b, 1] == pytest.approx(ref[b]["mean_x"], rel=1e-4, abs=1e-8)
        # tracked pupil: mask centred on the engine's own centroid
        I = np.abs(field[b].astype(np.complex128)) ** 2
        mask = o.pupil_mask(spec.N, spec.delta, 0.12, shift=(meas[b, 1], meas[b, 2]))
        assert meas[b, 9] == pytest.approx((I * mask).sum() * spec.delta ** 2, rel=1e-5)


def test_measures_entry_matches_oracle(torch_cuda):
    torch = torch_cuda
    spec = o.ChannelSpec(N=512, delta=2e-3, count=0, length=3e3)
    plan, _ = make_plan(spec, batch=2, pupils=[(0.05,), (0.1, 0.02, -0.01)], tracked=(0.07,))
    rng = np.random.default_rng(3)
    u = o.vacuum(o.gaussian_source(512, 2e-3, spec.wvl, 0.09, math.inf), 3e3, spec.k, 2e-3)
    fields = np.stack([u, u * np.exp(1j * rng.standard_normal((512, 512)) * 0.1)]).astype(np.complex64)
    got = plan.measures(torch.from_numpy(fields).cuda()).cpu().numpy()
    for b in range(2):
        f64 = fields[b].astype(np.complex128)
        m = o.measures(f64, 2e-3, [0.05])
        assert got[b, 0] == pytest.approx(m["eta_total"], rel=1e-6)
        assert got[b, 3] == pytest.approx(m["mean_x2"], rel=1e-5)
        I = np.abs(f64) ** 2
        shifted = o.pupil_mask(512, 2e-3, 0.1, shift=(0.02, -0.01))
        assert got[b, 9] == pytest.approx((I * shifted).sum() * 4e-6, rel=1e-6)


def test_vacuum_known_answers_engine(torch_cuda):
    """itest_vacuum_propagation cells 4-7 through the engine (VacuumPath channel)."""
    torch = torch_cuda
    N, d, wvl, w0, L = 256, 2e-3, 809e-9, 0.02, 4e3
    spec = o.ChannelSpec(N=N, delta=d, wvl=wvl, w0=w0, count=0, length=L)
    plan, _ = make_plan(spec, pupils=[])
    field = torch.empty((1, N, N), dtype=torch.complex64, device="cuda")
    m = plan.run(None, None, None, field_out=field).cpu().numpy()[0]
    u = field.cpu().numpy()[0].astype(np.complex128)
    assert m[0] == pytest.approx(1, abs=1e-6)
    assert abs(u.sum()) * d ** 2 == pytest.approx(np.sqrt(2 * np.pi) * w0, abs=1e-7)
    zR = np.pi * w0 ** 2 / wvl
    assert np.sqrt(2 * (m[3] + m[5])) == pytest.approx(w0 * np.sqrt(1 + (L / zR) ** 2), abs=1e-7)


@pytest.mark.parametrize("F0", [20000.0, 6000.0, -6000.0])
def test_focused_beam_width(torch_cuda, F0):
    """itest_sources cell 4 as assertions: sqrt(2 mean_r2) = GaussianBeam.get_w(L)."""
    torch = torch_cuda
    N, d, wvl, w0 = 512, 5e-3, 809e-9, 0.2
    for L in [2000.0, 4000.0]:
        spec = o.ChannelSpec(N=N, delta=d, wvl=wvl, w0=w0, F0=F0, count=0, length=L)
        plan, _ = make_plan(spec, pupils=[])
        m = plan.run(None, None, None).cpu().numpy()[0]
        width = np.sqrt(2 * (m[3] + m[5]))
        # the sampled grid against the FP64 oracle of the same grid
        u = o.vacuum(o.gaussian_source(N, d, wvl, w0, F0), L, spec.k, d)
        ref = o.measures(u, d)
        assert width == pytest.approx(np.sqrt(2 * (ref["mean_x2"] + ref["mean_y2"])), rel=1e-5)
        # and the continuum beam width GaussianBeam.get_w (sampling error ~4e-4 near focus)
        k = 2 * np.pi / wvl
        theta0, lam0 = 1 - L / F0, 2 * L / k / w0 ** 2
        assert width == pytest.approx(w0 * np.sqrt(theta0 ** 2 + lam0 ** 2), rel=1e-3)


def test_config2_geometry_matches_oracle(torch_cuda):
    """2048^2, delta 1.5 mm, 50 km, 5 screens (config 2), one realisation vs FP64."""
    torch = torch_cuda
    spec = o.ChannelSpec(N=2048, delta=1.5e-3, w0=0.12, length=50e3, Cn2=5e-16, pupil_radius=0.2)
    base = o.logpolar_base(spec.points, spec.f_min, spec.f_max)
    rho, theta, value = spectra(spec, base, seed=99, R=1)
    plan, meas, field = run_engine(torch, spec, rho, theta, value)
    res, u = o.simulate(spec, rho, theta, value, return_field=True)
    assert o.rel_l2(field[0], u) < FIELD_TOL
    assert meas[0, 8] == pytest.approx(res[0]["eta_0"], rel=1e-5)


def test_graph_capture_replays_run(torch_cuda):
    """atm_run captured into a CUDA graph gives the direct run's results, also
    after the inputs are refilled in place."""
    torch = torch_cuda
    spec = o.ChannelSpec(N=256, delta=4e-3, w0=0.08, length=8e3, count=3, points=256, Cn2=2e-15, pupil_radius=0.1)
    plan, base = make_plan(spec, batch=2)
    sp1 = spectra(spec, base, seed=1, R=2)
    sp2 = spectra(spec, base, seed=2, R=2)
    r, t, v = to_dev(torch, *sp1)
    g, out = plan.capture(r, t, v)
    g.replay()
    torch.cuda.synchronize()
    direct = plan.run(*to_dev(torch, *sp1)).cpu().numpy()
    np.testing.assert_array_equal(out.cpu().numpy(), direct)
    for dst, src in zip((r, t, v), to_dev(torch, *sp2)):
        dst.copy_(src)
    g.replay()
    torch.cuda.synchronize()
    direct2 = plan.run(*to_dev(torch, *sp2)).cpu().numpy()
    np.testing.assert_array_equal(out.cpu().numpy(), direct2)
    assert not np.array_equal(direct, direct2)


ROW_FORMS = (0, 1, 2, 3, 4, 7)
COL_FORMS = (0, 1, 2, 3, 4, 7)
PRODUCT_ROW = (4, 7)
PRODUCT_COL = (2, 7)
# the warp-FFT forms (N = 1024 and 2048; column tile 4): their own FP32 round-off
WARP_ROW = (11,)
WARP_COL = (10,)
# the split column forms (two half-length warp FFTs per column; column tile 4): 15 at 2048, 14 at 4096
SPLIT_COL = {2048: (15,), 4096: (14,)}


def _forms(N):
    warp = N in (1024, 2048)
    return ROW_FORMS + (WARP_ROW if warp else ()), COL_FORMS + (WARP_COL if warp else ()) + SPLIT_COL.get(N, ())


@pytest.mark.parametrize("N", [512, 2048])
def test_autotune_keeps_results(torch_cuda, N):
    """atm_autotune changes launch shapes (and, with column variant 2, the
    twiddle rounding): the tuned plan gives the untuned plan's results, and
    its choice is reported in the plan info."""
    torch = torch_cuda
    d = 3.0 / N
    spec = o.ChannelSpec(N=N, delta=d, w0=0.08, length=8e3, count=3, points=256, Cn2=2e-15, pupil_radius=0.1)
    plan, base = make_plan(spec, batch=3)
    sp = to_dev(torch, *spectra(spec, base, seed=5, R=3))
    before = plan.run(*sp).cpu().numpy()
    choice = plan.autotune(repeats=2)
    assert choice["tuned"] == 1
    assert choice["col_tile"] in (2, 4, 8, 16) and choice["col_tile"] * N // 16 <= 512
    row_forms, col_forms = _forms(N)
    assert choice["row_variant"] in row_forms and choice["col_variant"] in col_forms
    after = plan.run(*sp).cpu().numpy()
    rounding = PRODUCT_COL + WARP_COL + (14, 15), PRODUCT_ROW + WARP_ROW
    if choice["col_variant"] in rounding[0] or choice["row_variant"] in rounding[1]:
        np.testing.assert_allclose(after, before, rtol=2e-5, atol=1e-9)
    else:
        np.testing.assert_array_equal(after, before)
    # every launch form computes the same arithmetic, except the product
    # twiddles (row variants 4 and 7, column variants 2 and 7) and the warp
    # FFTs (row 11, columns 10 and 15): FP32 round-off
    product = {}
    for rv in row_forms:
        for ct in (2, 4, 8, 16):
            if ct * N // 16 > 512:
                continue
            for cv in col_forms:
                if cv in WARP_COL + (14, 15) and ct != 4:
                    continue
                plan.set_variants(rv, ct, cv)
                got = plan.run(*sp).cpu().numpy()
                if cv in rounding[0] or rv in rounding[1]:
                    np.testing.assert_allclose(got, before, rtol=2e-5, atol=1e-9, err_msg=f"{rv} {ct} {cv}")
                else:
                    np.testing.assert_array_equal(got, before, err_msg=f"{rv} {ct} {cv}")
                if cv in PRODUCT_COL and rv in PRODUCT_ROW:
                    product[(rv, ct, cv)] = got
    # twiddle bases in registers (row 7, column 7) give the bits of the table product forms (row 4, column 2)
    for (rv, ct, cv), got in product.items():
        ref = product.get((4, ct, 2))
        if ref is not None:
            np.testing.assert_array_equal(got, ref, err_msg=f"{rv} {ct} {cv}")


def test_step_measures_match_oracle(torch_cuda):
    """ATM_FLAG_STEP_MEASURES: moments and centre intensity of the field just
    after every screen (the reference generator's yields) against FP64."""
    torch = torch_cuda
    from pyatmosphere_gb300.engine import _lib
    spec = o.ChannelSpec(N=256, delta=4e-3, w0=0.08, length=8e3, count=3, points=256, Cn2=2e-15, pupil_radius=0.1)
    plan, base = make_plan(spec, batch=2, flags=_lib.FLAG_STEP_MEASURES)
    assert plan.n_out == _lib.OUT_PUPIL0 + 1 + _lib.STEP_SLOTS * 3
    rho, theta, value = spectra(spec, base, seed=13, R=2)
    out = plan.run(*to_dev(torch, rho, theta, value)).cpu().numpy()
    positions = o.screen_positions(spec.length, spec.count, spec.position)
    u0 = o.gaussian_source(spec.N, spec.delta, spec.wvl, spec.w0, spec.F0)
    base_slot = _lib.OUT_PUPIL0 + 1
    for r in range(2):
        screens = [o.ss_screen(rho[r, i], theta[r, i], value[r, i], spec.N, spec.delta) for i in range(3)]
        u, steps = o.propagate(u0, screens, positions, spec.length, spec.k, spec.delta, path_output_loss=False,
                               keep_steps=True)
        ref_final = o.measures(u, spec.delta, [0.1])
        assert out[r, _lib.OUT_ETA_TOTAL] == pytest.approx(ref_final["eta_total"], rel=1e-5)
        for i, ui in enumerate(steps):
            ref = o.measures(ui, spec.delta)
            blk = out[r, base_slot + i * _lib.STEP_SLOTS: base_slot + (i + 1) * _lib.STEP_SLOTS]
            assert blk[_lib.OUT_ETA_TOTAL] == pytest.approx(ref["eta_total"], rel=1e-5)
            assert blk[_lib.OUT_MEAN_X2] == pytest.approx(ref["mean_x2"], rel=1e-4)
            assert blk[_lib.OUT_MEAN_Y2] == pytest.approx(ref["mean_y2"], rel=1e-4)
            assert blk[_lib.OUT_MEAN_X] == pytest.approx(ref["mean_x"], rel=1e-3, abs=1e-7)
            c = spec.N // 2
            assert blk[_lib.OUT_I_CENTER] == pytest.approx(abs(ui[c, c]) ** 2, rel=1e-4)
    # the final measures do not depend on the flag
    plain, _ = make_plan(spec, batch=2)
    np.testing.assert_array_equal(plain.run(*to_dev(torch, rho, theta, value)).cpu().numpy(),
                                  out[:, :plain.n_out])


def test_shifted_screens_match_oracle(torch_cuda):
    """Screens moved by (0, t) (the wind shift of Simulation.iter) through
    atm_plan_update, against FP64 screens evaluated at y + t."""
    torch = torch_cuda
    spec = o.ChannelSpec(N=256, delta=4e-3, w0=0.08, length=8e3, count=2, points=256, Cn2=2e-15, pupil_radius=0.1)
    plan, base = make_plan(spec, batch=1)
    rho, theta, value = spectra(spec, base, seed=4, R=1)
    dev = to_dev(torch, rho, theta, value)
    field = torch.empty((1, spec.N, spec.N), dtype=torch.complex64, device="cuda")
    positions = o.screen_positions(spec.length, spec.count, spec.position)
    u0 = o.gaussian_source(spec.N, spec.delta, spec.wvl, spec.w0, spec.F0)
    for t in (0.0, 0.037, -0.2):
        plan.set_shift((0.0, t))
        plan.run(*dev, field_out=field)
        screens = [o.ss_screen(rho[0, i], theta[0, i], value[0, i], spec.N, spec.delta, shift=(0.0, t))
                   for i in range(2)]
        u = o.propagate(u0, screens, positions, spec.length, spec.k, spec.delta, path_output_loss=False)
        assert o.rel_l2(field.cpu().numpy()[0], u) < FIELD_TOL, t


@pytest.mark.parametrize("N,B", [(100, 2), (1000, 1), (1024, 3)])
def test_structure_function_kernel_matches_numpy(torch_cuda, N, B):
    """atm_structure_function against the FP64 restatement of calculate_sf
    (theory/phase_screens/sf.py:4-8) and its row mean, any N (ragged lag
    chunks and row tails)."""
    torch = torch_cuda
    from pyatmosphere_gb300.engine.plan import structure_function
    rng = np.random.default_rng(N)
    # a rough screen with a large tilt, like a low-frequency phase
    phi = (np.cumsum(rng.standard_normal((B, N, N)), axis=2) * 0.05 + 30.0 * np.linspace(-1, 1, N)).astype(np.float32)
    got = structure_function(torch.from_numpy(phi).cuda()).cpu().numpy()
    s = phi.astype(np.float64)
    ref = np.stack([np.stack([((s[b, :, :-r] - s[b, :, r:]) ** 2).sum(axis=1) / (N - r) for r in range(1, N)]).mean(axis=1)
                    for b in range(B)])
    assert got.shape == (B, N - 1)
    np.testing.assert_allclose(got, ref, rtol=2e-5)


def test_product_twiddle_column_pass_matches_oracle(torch_cuda):
    """Row variant 4 and column variant 2 (twiddles from powers of two) keep
    the FP64 parity bound."""
    torch = torch_cuda
    spec = o.ChannelSpec(N=2048, delta=1.5e-3, w0=0.12, length=50e3, Cn2=5e-16, pupil_radius=0.2)
    plan, base = make_plan(spec, batch=1)
    plan.set_variants(4, 4, 2)
    rho, theta, value = spectra(spec, base, seed=31, R=1)
    field = torch.empty((1, 2048, 2048), dtype=torch.complex64, device="cuda")
    plan.run(*to_dev(torch, rho, theta, value), field_out=field)
    res, u = o.simulate(spec, rho, theta, value, return_field=True)
    assert o.rel_l2(field.cpu().numpy()[0], u) < FIELD_TOL


@pytest.mark.parametrize("N,variants,R", [(1024, (11, 4, 10), 3), (2048, (11, 4, 10), 3), (4096, (4, 4, 10), 2),
                                         (4096, (4, 4, 14), 2), (2048, (4, 4, 15), 3)])
def test_warp_fft_passes_match_oracle(torch_cuda, N, variants, R):
    """The warp-FFT forms (row variant 11 at 1024 and 2048; column variant 10,
    with 64-lane transforms at 4096; column variants 14 at 4096 and 15 at 2048,
    two half-length warp FFTs per column) keep the FP64 parity bound on fields and measures, for
    batches of several realisations (the column pass's two groups on
    neighbouring tiles), and through atm_vacuum on the same plan."""
    torch = torch_cuda
    spec = o.ChannelSpec(N=N, delta=3.0 / N, w0=0.1, length=20e3, count=4, Cn2=1e-15, pupil_radius=0.15)
    plan, base = make_plan(spec, batch=R)
    plan.set_variants(*variants)
    rho, theta, value = spectra(spec, base, seed=77, R=R)
    field = torch.empty((R, N, N), dtype=torch.complex64, device="cuda")
    got = plan.run(*to_dev(torch, rho, theta, value), field_out=field).cpu().numpy()
    plan.check()
    f = field.cpu().numpy()
    for r in range(R):
        res, u = o.simulate(spec, rho[r:r + 1], theta[r:r + 1], value[r:r + 1], return_field=True)
        res = {r: res[0]}
        assert o.rel_l2(f[r], u) < FIELD_TOL
        assert got[r, 0] == pytest.approx(res[r]["eta_total"], rel=1e-5)
        assert got[r, 8] == pytest.approx(res[r]["eta_0"], rel=1e-5)
        assert got[r, 3] == pytest.approx(res[r]["mean_x2"], rel=1e-5)
    # a vacuum step on the same plan (atm_vacuum runs the plan's column form)
    g = o.gaussian_source(N, spec.delta, spec.wvl, spec.w0, spec.F0)
    dev = torch.from_numpy(np.stack([g] * 2).astype(np.complex64)).cuda()
    plan.vacuum(dev, 5e3)
    ref = o.vacuum(g, 5e3, spec.k, spec.delta)
    for r in range(2):
        assert o.rel_l2(dev[r].cpu().numpy(), ref) < FIELD_TOL
    plan.close()


def test_sizes_tool_runs(torch_cuda, capsys):
    """python -m pyatmosphere_gb300.engine.sizes: per-kernel times at one grid size."""
    from pyatmosphere_gb300.engine import sizes
    assert sizes.main(["--N", "256", "--batch", "2", "--warmup", "1", "--runs", "1", "--variants", "3,4,3"]) == 0
    out = capsys.readouterr().out
    assert "row_pass" in out and "col_pass" in out and "GB/s" in out
