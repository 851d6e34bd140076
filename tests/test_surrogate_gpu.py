"""The surrogate's hand-written training kernels against the FP64 oracle, and
the data -> train -> query pipeline on a small case."""
import numpy as np
import pytest

from oracle import mlp_oracle as mo

pytestmark = pytest.mark.gpu


def test_mlp_gradients_match_oracle():
    import torch
    from pyatmosphere_gb300.surrogate.mlp import EngineMLP
    widths = [8, 256, 256, 256, 67]
    mlp = EngineMLP(widths, max_batch=64)
    mlp.init_params(3)
    params = mlp.get_params()
    rng = np.random.default_rng(1)
    B = 32
    x = rng.random((B, 8)).astype(np.float32)
    t = np.concatenate([rng.dirichlet(np.ones(64) * 0.3, B), rng.standard_normal((B, 3))], axis=1).astype(np.float32)
    xd, td = torch.from_numpy(x).cuda(), torch.from_numpy(t).cuda()
    mlp.forward(xd)
    loss = mlp.loss_backward(td, 64, 0.5).item()
    _, g = mlp.get_params(with_grads=True)
    ref_loss, ref_g = mo.loss_and_grad(params.astype(np.float64), widths, x.astype(np.float64),
                                       t.astype(np.float64), 64, 0.5)
    assert loss == pytest.approx(ref_loss, rel=1e-5)
    assert np.linalg.norm(g - ref_g) / np.linalg.norm(ref_g) < 1e-4
    # per layer as well
    off = 0
    for i in range(len(widths) - 1):
        n = widths[i + 1] * widths[i] + widths[i + 1]
        a, b = g[off:off + n], ref_g[off:off + n]
        assert np.linalg.norm(a - b) <= 1e-4 * np.linalg.norm(b) + 1e-12
        off += n
    mlp.close()


def test_mlp_training_reduces_loss_on_smooth_target():
    import torch
    from pyatmosphere_gb300.surrogate.mlp import EngineMLP
    rng = np.random.default_rng(2)
    X = rng.random((2048, 8)).astype(np.float32)
    centers = 0.2 + 0.6 * X[:, 0]
    widths_ = 0.05 + 0.1 * X[:, 1]
    grid = (np.arange(64) + 0.5) / 64
    H = np.exp(-0.5 * ((grid[None, :] - centers[:, None]) / widths_[:, None]) ** 2)
    H /= H.sum(axis=1, keepdims=True)
    M = np.stack([X[:, 2], X[:, 3] ** 2, np.sin(3 * X[:, 4])], axis=1)
    Y = np.concatenate([H, M], axis=1).astype(np.float32)
    mlp = EngineMLP([8, 256, 256, 256, 67], max_batch=512)
    mlp.init_params(0)
    Xd, Yd = torch.from_numpy(X).cuda(), torch.from_numpy(Y).cuda()
    first = None
    for s in range(1500):
        idx = torch.randint(0, 2048, (256,), device="cuda")
        mlp.forward(Xd[idx].contiguous())
        loss = mlp.loss_backward(Yd[idx].contiguous(), 64, 1.0)
        mlp.adam(lr=1e-3)
        if s == 0:
            first = loss.item()
    last = loss.item()
    assert last < 0.1 * first, (first, last)
    mlp.close()


def test_surrogate_pipeline_small():
    import torch
    from pyatmosphere_gb300.surrogate import Box, SimConfig, Surrogate, features, ks_hist
    box = Box()
    cfg = SimConfig(N=256, extent=3.0, realisations=64)
    P, X, Y, samples = Surrogate.generate(box, 48, cfg, seed=5, keep_samples=True)
    assert Y.shape == (48, 67) and np.allclose(Y[:, :64].sum(axis=1), 1.0, atol=1e-5)
    assert np.all((Y[:, 64] >= 0) & (Y[:, 64] <= 1))
    s = Surrogate(box, max_batch=1024)
    s.fit(X, Y, steps=300, batch=48)
    probs, mom, oor = s.predict(torch.from_numpy(X).cuda())
    p = probs.cpu().numpy()
    assert np.allclose(p.sum(axis=1), 1.0, atol=1e-4)
    assert not oor.cpu().numpy().any()
    # an out-of-box query falls back to the simulator
    q = {k: v[:2].copy() for k, v in P.items()}
    q["Cn2"][1] = 1e-12
    probs_q, flags = s.query(q, fallback_cfg=SimConfig(N=256, realisations=64))
    assert list(flags) == [False, True]
    assert probs_q[1].sum() == pytest.approx(1.0, abs=1e-5)
    # KS of the fit on its own training points is finite and in [0, 1]
    ks = [ks_hist(p[i], samples[i]) for i in range(8)]
    assert all(0 <= k <= 1 for k in ks)


def _tc_mlp(widths, seed=7, max_batch=64):
    """An engine MLP with random weights and biases (the biases exercise the epilogue)."""
    from pyatmosphere_gb300.surrogate.mlp import EngineMLP
    mlp = EngineMLP(widths, max_batch=max_batch)
    mlp.init_params(seed)
    params = mlp.get_params()
    rng = np.random.default_rng(seed)
    off = 0
    for i in range(len(widths) - 1):
        off += widths[i + 1] * widths[i]
        params[off:off + widths[i + 1]] = 0.3 * rng.standard_normal(widths[i + 1])
        off += widths[i + 1]
    mlp.set_params(params.astype(np.float32))
    return mlp, params


@pytest.mark.parametrize("widths", [[12, 256, 256, 256, 67], [8, 128, 128, 40], [20, 64, 64, 64, 64, 67]])
def test_tc_inference_matches_oracle_and_tile_form(widths):
    """The fused tcgen05 inference against its own arithmetic restated in FP64
    (bf16 input slices, bf16 activations) and against the tile-GEMM form with
    FP32 activations; out-of-box flags bit for bit; a batch of 1000 queries
    (seven full tiles and a partial one) in one launch, beyond max_batch."""
    import torch
    mlp, params = _tc_mlp(widths)
    assert mlp.infer_form == "tensor cores"
    rng = np.random.default_rng(3)
    B, n_hist = 1000, min(64, widths[-1])
    x = rng.random((B, widths[0])).astype(np.float32)
    x[::7, 0] = 1.2  # outside the box
    lo = torch.zeros(widths[0], device="cuda")
    hi = torch.ones(widths[0], device="cuda")
    xd = torch.from_numpy(x).cuda()
    y_tc, oor_tc = mlp.infer(xd, lo, hi, n_hist=n_hist)
    mlp.check()
    y_tc, oor_tc = y_tc.cpu().numpy(), oor_tc.cpu().numpy()
    ref = mo.infer_tc_emulated(params.astype(np.float64), widths, x, n_hist)
    np.testing.assert_array_equal(oor_tc, (x > 1).any(axis=1).astype(np.int32))
    assert np.isfinite(y_tc).all()
    np.testing.assert_allclose(y_tc[:, :n_hist].sum(axis=1), 1.0, atol=1e-5)
    assert np.abs(y_tc[:, :n_hist] - ref[:, :n_hist]).max() < 2e-4
    assert np.abs(np.cumsum(y_tc[:, :n_hist], 1) - np.cumsum(ref[:, :n_hist], 1)).max() < 2e-4
    if widths[-1] > n_hist:
        np.testing.assert_allclose(y_tc[:, n_hist:], ref[:, n_hist:], rtol=2e-3, atol=2e-3)
    mlp.set_infer_form("tile gemm")
    assert mlp.infer_form == "tile gemm"
    y_tile, oor_tile = mlp.infer(xd, lo, hi, n_hist=n_hist)
    y_tile = y_tile.cpu().numpy()
    np.testing.assert_array_equal(oor_tile.cpu().numpy(), oor_tc)
    # bf16 activations against FP32 ones: histogram CDFs within 1e-2
    assert np.abs(np.cumsum(y_tc[:, :n_hist], 1) - np.cumsum(y_tile[:, :n_hist], 1)).max() < 1e-2
    mlp.close()


def test_tc_inference_form_rules():
    from pyatmosphere_gb300.engine import _lib
    from pyatmosphere_gb300.surrogate.mlp import EngineMLP
    odd = EngineMLP([8, 100, 67], max_batch=16)  # hidden width not a multiple of 64
    assert odd.infer_form == "tile gemm"
    with pytest.raises(_lib.EngineError):
        odd.set_infer_form("tensor cores")
    odd.close()
    # training changes the weights: the packed image follows
    import torch
    mlp, _ = _tc_mlp([12, 256, 256, 256, 67])
    x = torch.rand((300, 12), device="cuda")
    t = torch.softmax(torch.randn((300, 67), device="cuda"), dim=1)
    y0, _ = mlp.infer(x)
    mlp.forward(x[:64].contiguous())
    mlp.loss_backward(t[:64].contiguous(), 64, 1.0)
    mlp.adam(lr=1e-2)
    y1, _ = mlp.infer(x)
    mlp.set_infer_form("tile gemm")
    y2, _ = mlp.infer(x)
    assert not torch.equal(y0, y1)
    assert (torch.cumsum(y1[:, :64], 1) - torch.cumsum(y2[:, :64], 1)).abs().max().item() < 1e-2
    mlp.close()
