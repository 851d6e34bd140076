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
