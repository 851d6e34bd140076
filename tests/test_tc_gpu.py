"""The tensor-core screen GEMM (tcgen05, FP16 hi/lo slices, FP32 TMEM
accumulation) against an FP64 numpy product."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("variant", [0, 1, 2])
@pytest.mark.parametrize("S,M,N,K", [(1, 128, 256, 64), (2, 256, 512, 200), (1, 512, 512, 768), (3, 2048, 2048, 768)])
def test_tc_gemm_matches_fp64(S, M, N, K, variant):
    """Every form (0: persistent TMA 128 x 128 with double-buffered
    accumulators, 1: cp.async per tile, 2: persistent TMA 128 x 256),
    including more tiles than SMs so the persistent loop wraps."""
    import torch
    from pyatmosphere_gb300.engine import _lib
    lib = _lib.load()
    rng = np.random.default_rng(M + N + K)
    A = rng.standard_normal((S, M, K)).astype(np.float32)
    B = rng.standard_normal((S, N, K)).astype(np.float32)
    Ad, Bd = torch.from_numpy(A).cuda(), torch.from_numpy(B).cuda()
    out = torch.empty((S, M, N), dtype=torch.float32, device="cuda")
    rc = lib.atm_tc_gemm_test(ctypes.c_void_p(Ad.data_ptr()), ctypes.c_void_p(Bd.data_ptr()), S, M, N, K, 0.5,
                              ctypes.c_void_p(out.data_ptr()), variant,
                              ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == 0, lib.atm_last_error()
    ref = 0.5 * np.einsum("smk,snk->smn", A.astype(np.float64), B.astype(np.float64))
    got = out.cpu().numpy().astype(np.float64)
    err = np.linalg.norm(got - ref) / np.linalg.norm(ref)
    assert err < 2e-6, err


@pytest.mark.parametrize("N,P,Cn2,delta", [(256, 512, 1e-14, 4e-3), (2048, 1024, 5e-16, 1.5e-3),
                                           (4096, 256, 1e-15, 3.0 / 4096)])
def test_tc_screen_matches_oracle(N, P, Cn2, delta):
    """Screens through the tensor-core GEMM against the FP64 oracle."""
    import torch
    from oracle import atm_oracle as o
    from pyatmosphere_gb300.engine import EnginePlan, _lib
    spec = o.ChannelSpec(N=N, delta=delta, points=P, Cn2=Cn2, count=2, length=10e3)
    base = o.logpolar_base(P, spec.f_min, spec.f_max)
    plan = EnginePlan(N, delta, spec.wvl, spec.w0, spec.F0, o.screen_positions(spec.length, 2), spec.length,
                      f_base=base, batch=2, flags=_lib.FLAG_TC_GEMM)
    psd = o.annulus_psd(base, spec.k, spec.thickness, Cn2, spec.l0, spec.L0, use_scipy=False)
    rho, theta, value = o.draw_spectra(N, range(2), 2, base, psd)
    r, t, v = [torch.from_numpy(a).cuda() for a in (rho, theta, value)]
    ph = torch.empty((2, N, N), dtype=torch.complex64, device="cuda")
    plan.screen(r, t, v, 1, phasor_out=ph)
    ph = ph.cpu().numpy()
    for b in range(2):
        ref = o.ss_screen(rho[b, 1], theta[b, 1], value[b, 1], N, delta)
        assert o.rel_l2(ph[b], np.exp(-1j * ref)) < 1e-5


def test_tc_channel_config2_matches_oracle():
    import torch
    from oracle import atm_oracle as o
    from pyatmosphere_gb300.engine import EnginePlan, _lib
    spec = o.ChannelSpec(N=2048, delta=1.5e-3, w0=0.12, length=50e3, Cn2=5e-16, pupil_radius=0.2)
    base = o.logpolar_base(spec.points, spec.f_min, spec.f_max)
    psd = o.annulus_psd(base, spec.k, spec.thickness, spec.Cn2, spec.l0, spec.L0, use_scipy=False)
    rho, theta, value = o.draw_spectra(99, range(1), spec.count, base, psd)
    plan = EnginePlan(spec.N, spec.delta, spec.wvl, spec.w0, spec.F0, o.screen_positions(spec.length, spec.count),
                      spec.length, f_base=base, pupils=[(0.2,)], batch=1, flags=_lib.FLAG_TC_GEMM)
    field = torch.empty((1, 2048, 2048), dtype=torch.complex64, device="cuda")
    meas = plan.run(*[torch.from_numpy(a).cuda() for a in (rho, theta, value)], field_out=field).cpu().numpy()
    res, u = o.simulate(spec, rho, theta, value, return_field=True)
    assert o.rel_l2(field.cpu().numpy()[0], u) < 1e-4
    assert meas[0, 8] == pytest.approx(res[0]["eta_0"], rel=1e-5)


def test_tc_channel_4096_matches_oracle():
    """The largest grid: 4096^2, two screens, through the whole run."""
    import torch
    from oracle import atm_oracle as o
    from pyatmosphere_gb300.engine import EnginePlan
    spec = o.ChannelSpec(N=4096, delta=3.0 / 4096, w0=0.1, length=20e3, count=2, points=256, Cn2=2e-15,
                         pupil_radius=0.15)
    base = o.logpolar_base(spec.points, spec.f_min, spec.f_max)
    psd = o.annulus_psd(base, spec.k, spec.thickness, spec.Cn2, spec.l0, spec.L0, use_scipy=False)
    rho, theta, value = o.draw_spectra(41, range(1), spec.count, base, psd)
    plan = EnginePlan(spec.N, spec.delta, spec.wvl, spec.w0, spec.F0, o.screen_positions(spec.length, spec.count),
                      spec.length, f_base=base, pupils=[(0.15,)], batch=1)
    assert plan.info["gemm_k"] % 64 == 0  # the tensor-core layout is in use
    field = torch.empty((1, 4096, 4096), dtype=torch.complex64, device="cuda")
    meas = plan.run(*[torch.from_numpy(a).cuda() for a in (rho, theta, value)], field_out=field).cpu().numpy()
    res, u = o.simulate(spec, rho, theta, value, return_field=True)
    assert o.rel_l2(field.cpu().numpy()[0], u) < 1e-4
    assert meas[0, 8] == pytest.approx(res[0]["eta_0"], rel=1e-5)


def test_tc_forms_agree_on_a_channel():
    """The persistent TMA form with 128 x 256 tiles is the default; its 128 x
    128 form (flag) gives the same measures, the cp.async form (flag) the same
    to FP32 round-off."""
    import torch
    from oracle import atm_oracle as o
    from pyatmosphere_gb300.engine import EnginePlan, _lib
    spec = o.ChannelSpec(N=512, delta=3.0 / 512, w0=0.08, length=10e3, count=3, points=512, Cn2=3e-15,
                         pupil_radius=0.1)
    base = o.logpolar_base(spec.points, spec.f_min, spec.f_max)
    psd = o.annulus_psd(base, spec.k, spec.thickness, spec.Cn2, spec.l0, spec.L0, use_scipy=False)
    sp = [torch.from_numpy(a).cuda() for a in o.draw_spectra(17, range(4), spec.count, base, psd)]
    pos = o.screen_positions(spec.length, spec.count)
    tma = EnginePlan(spec.N, spec.delta, spec.wvl, spec.w0, spec.F0, pos, spec.length, f_base=base,
                     pupils=[(0.1,)], batch=4)
    cpa = EnginePlan(spec.N, spec.delta, spec.wvl, spec.w0, spec.F0, pos, spec.length, f_base=base,
                     pupils=[(0.1,)], batch=4, flags=_lib.FLAG_TC_CPASYNC)
    assert tma.info["gemm_form"] == 3 and cpa.info["gemm_form"] == 1
    t128 = EnginePlan(spec.N, spec.delta, spec.wvl, spec.w0, spec.F0, pos, spec.length, f_base=base,
                      pupils=[(0.1,)], batch=4, flags=_lib.FLAG_TC_N128)
    assert t128.info["gemm_form"] == 2
    np.testing.assert_allclose(t128.run(*sp).cpu().numpy(), tma.run(*sp).cpu().numpy(), rtol=1e-6, atol=1e-12)
    a, b = tma.run(*sp).cpu().numpy(), cpa.run(*sp).cpu().numpy()
    # the TMA form also folds the 1-D phases into the GEMM output (one FP32
    # rounding more): integrated measures to 2e-5, the one-pixel intensity to 1e-4
    cols = [c for c in range(a.shape[1]) if c != _lib.OUT_I_CENTER]
    np.testing.assert_allclose(a[:, cols], b[:, cols], rtol=2e-5, atol=1e-9)
    np.testing.assert_allclose(a[:, _lib.OUT_I_CENTER], b[:, _lib.OUT_I_CENTER], rtol=1e-4)


def test_simt_gemm_path_still_matches_oracle():
    """The FP32 SIMT screen GEMM (ATM_FLAG_SIMT_GEMM) stays covered."""
    import torch
    from oracle import atm_oracle as o
    from pyatmosphere_gb300.engine import EnginePlan, _lib
    N, P, d = 512, 1024, 1.0 / 512
    spec = o.ChannelSpec(N=N, delta=d, points=P, Cn2=1e-15, count=2, length=10e3)
    base = o.logpolar_base(P, spec.f_min, spec.f_max)
    plan = EnginePlan(N, d, spec.wvl, spec.w0, spec.F0, o.screen_positions(spec.length, 2), spec.length,
                      f_base=base, batch=1, flags=_lib.FLAG_SIMT_GEMM)
    psd = o.annulus_psd(base, spec.k, spec.thickness, spec.Cn2, spec.l0, spec.L0, use_scipy=False)
    rho, theta, value = o.draw_spectra(3, range(1), 2, base, psd)
    ph = torch.empty((1, N, N), dtype=torch.complex64, device="cuda")
    plan.screen(*[torch.from_numpy(a).cuda() for a in (rho, theta, value)], 0, phasor_out=ph)
    ref = o.ss_screen(rho[0, 0], theta[0, 0], value[0, 0], N, d)
    assert o.rel_l2(ph.cpu().numpy()[0], np.exp(-1j * ref)) < 1e-5
