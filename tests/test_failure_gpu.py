"""Failure detection without a GPU fault.

Every wait of the TMA-fed FFT passes and of the tensor-core screen GEMM has a
budget (atm_set_wait_budget, 2 s by default).  A budget of a few nanoseconds
is far below the latency of a tile copy, so the first waits run out: the
kernels record it in the plan's status word, drain their copies and MMAs
(their drains keep the 2 s bound), free their TMEM and return.  The measures
of that run are NaN and atm_plan_check reports ATM_ERR_TIMEOUT; the next run
with the default budget gives the bits of a clean run on the same plan.

Injected NaN / infinite spectra are the host-side fault: the spectrum kernel
drops the term, the measures are NaN and atm_plan_check reports
ATM_ERR_NONFINITE.  The reference's only failure handling is the
KeyboardInterrupt flush of Simulation.run (simulations/simulation.py:135-138)."""
import numpy as np
import pytest

from oracle import atm_oracle as o

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda():
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    return torch


def _setup(torch, N, flags=0, variants=None, R=2):
    from pyatmosphere_gb300.engine import EnginePlan
    spec = o.ChannelSpec(N=N, delta=3.0 / N, w0=0.1, length=10e3, count=3, points=512, Cn2=1e-15,
                         pupil_radius=0.2)
    base = o.logpolar_base(spec.points, spec.f_min, spec.f_max)
    plan = EnginePlan(N, spec.delta, spec.wvl, spec.w0, spec.F0, o.screen_positions(spec.length, spec.count),
                      spec.length, f_base=base, pupils=[(0.2,)], batch=R, flags=flags)
    if variants:
        plan.set_variants(*variants)
    psd = o.annulus_psd(base, spec.k, spec.thickness, spec.Cn2, spec.l0, spec.L0, use_scipy=False)
    arrs = o.draw_spectra(21, range(R), spec.count, base, psd)
    return plan, [torch.from_numpy(a).cuda() for a in arrs]


@pytest.mark.parametrize("form", ["row-major TMA forms", "tiled", "warp-FFT column groups", "4096 split columns",
                                  "2048 split columns"])
def test_wait_budget_runs_out_then_recovers(torch_cuda, form):
    from pyatmosphere_gb300.engine import _lib
    from pyatmosphere_gb300.engine.plan import set_wait_budget
    torch = torch_cuda
    if form == "tiled":
        plan, dev = _setup(torch, 512, flags=_lib.FLAG_TILED)
    elif form == "warp-FFT column groups":
        # column variant 10: two groups handing stages to each other through mbarriers
        plan, dev = _setup(torch, 1024, variants=(3, 4, 10))
    elif form == "2048 split columns":
        # column variant 15: two pairs of groups handing unit stages to each other through mbarriers
        plan, dev = _setup(torch, 2048, variants=(3, 4, 15))
    elif form == "4096 split columns":
        # column variant 14: both groups on one tile of two units, CTA-wide handoffs
        plan, dev = _setup(torch, 4096, variants=(3, 4, 14))
    else:
        plan, dev = _setup(torch, 512, variants=(3, 4, 3))  # bulk-copied rows, TMA column tiles
    assert plan.info["gemm_form"] == 3  # persistent TMA tensor-core GEMM
    clean = plan.run(*dev).cpu().numpy()
    plan.check()
    assert np.isfinite(clean).all()
    try:
        set_wait_budget(5)  # 5 ns: every wait that does not find its data already there runs out
        bad = plan.run(*dev).cpu().numpy()
        with pytest.raises(_lib.EngineError) as err:
            plan.check()
        assert err.value.code == _lib.ERR_TIMEOUT
        assert np.isnan(bad[:, :9]).all()
    finally:
        set_wait_budget(2_000_000_000)
    again = plan.run(*dev).cpu().numpy()
    plan.check()  # the record was cleared by the failed check
    np.testing.assert_array_equal(again, clean)
    plan.close()


@pytest.mark.parametrize("which", ["rho", "theta", "value"])
def test_nonfinite_spectra_are_reported(torch_cuda, which):
    from pyatmosphere_gb300.engine import _lib
    torch = torch_cuda
    plan, dev = _setup(torch, 256)
    clean = plan.run(*dev).cpu().numpy()
    plan.check()
    bad = [t.clone() for t in dev]
    k = {"rho": 0, "theta": 1, "value": 2}[which]
    bad[k][1, 0, 3] = float("nan") if which != "rho" else float("inf")  # a low annulus
    bad[k][0, 2, 400] = float("nan")  # a high annulus
    out = plan.run(*bad).cpu().numpy()
    with pytest.raises(_lib.EngineError) as err:
        plan.check()
    assert err.value.code == _lib.ERR_NONFINITE
    assert np.isnan(out[:, :9]).all()
    np.testing.assert_array_equal(plan.run(*dev).cpu().numpy(), clean)
    plan.check()
    plan.close()


def test_mlp_inference_wait_budget_runs_out_then_recovers(torch_cuda):
    """The fused tensor-core inference shares the GEMM's wait budget: with 5 ns
    its waits for the operand and the weights run out, the CTAs drain their
    copies and MMAs and free their TMEM, and atm_mlp_check reports
    ATM_ERR_TIMEOUT; with the default budget the next call gives the clean bits."""
    from pyatmosphere_gb300.engine import _lib
    from pyatmosphere_gb300.engine.plan import set_wait_budget
    from pyatmosphere_gb300.surrogate.mlp import EngineMLP
    torch = torch_cuda
    mlp = EngineMLP([12, 256, 256, 256, 67], max_batch=64)
    mlp.init_params(5)
    assert mlp.infer_form == "tensor cores"
    x = torch.rand((4096, 12), device="cuda")
    clean, _ = mlp.infer(x)
    mlp.check()
    clean = clean.cpu()
    try:
        set_wait_budget(5)
        mlp.infer(x)
        with pytest.raises(_lib.EngineError) as err:
            mlp.check()
        assert err.value.code == _lib.ERR_TIMEOUT
    finally:
        set_wait_budget(2_000_000_000)
    again, _ = mlp.infer(x)
    mlp.check()
    assert torch.equal(again.cpu(), clean)
    mlp.close()
