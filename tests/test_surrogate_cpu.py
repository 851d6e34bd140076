"""CPU checks of the surrogate's oracle and host logic."""
import numpy as np

from oracle import mlp_oracle as mo


def test_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    widths = [8, 16, 16, 11]
    n = sum(widths[i + 1] * widths[i] + widths[i + 1] for i in range(3))
    params = mo.bf16_round(rng.standard_normal(n) * 0.3)   # bf16-exact so rounding is the identity
    x = rng.random((5, 8))
    t = np.concatenate([rng.dirichlet(np.ones(8), 5), rng.standard_normal((5, 3))], axis=1)
    loss, g = mo.loss_and_grad(params, widths, x, t, 8, 0.7)

    # the same model without the bf16 rounding, differentiated numerically
    # (the weights are bf16-exact, so both agree at the evaluation point)
    def loss_fp64(p):
        layers = mo.unpack(p, widths)
        a = x
        for l, (W, b) in enumerate(layers):
            z = a @ W.T + b
            a = mo.gelu(z) if l < 2 else z
        h = a[:, :8] - a[:, :8].max(axis=1, keepdims=True)
        logp = h - np.log(np.exp(h).sum(axis=1, keepdims=True))
        kl = (t[:, :8] * (np.log(t[:, :8]) - logp)).sum(axis=1)
        d = a[:, 8:] - t[:, 8:]
        return (kl + 0.7 * (d * d).sum(axis=1) / 3).mean()
    assert abs(loss_fp64(params) - loss) < 1e-12
    for j in rng.choice(n, 25, replace=False):
        e = np.zeros(n)
        e[j] = 1e-6
        fd = (loss_fp64(params + e) - loss_fp64(params - e)) / 2e-6
        assert abs(fd - g[j]) < 1e-6 * max(1.0, abs(fd))


def test_bf16_rounding_is_round_to_nearest_even():
    vals = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -9, -2.5, 3.14159], np.float32)
    r = mo.bf16_round(vals)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0 + 2 ** -7 and r[3] == -2.5
    assert abs(r[4] - 3.140625) < 1e-12


def test_features_and_ks():
    from pyatmosphere_gb300.surrogate.model import Box, features, ks_hist
    box = Box()
    p = box.sample(100, np.random.default_rng(1))
    X = features(p, box)
    assert X.shape == (100, 12) and X[:, :8].min() >= -1e-6 and X[:, :8].max() <= 1 + 1e-6
    assert np.isfinite(X).all() and X[:, 8:].min() > -0.5 and X[:, 8:].max() < 1.5
    assert features(p, box, physics=False).shape == (100, 8)
    samples = np.random.default_rng(2).random(20000)
    assert ks_hist(np.full(64, 1 / 64), samples) < 0.02
    assert ks_hist(np.eye(64)[0], samples) > 0.9


def test_ensemble_gate_helpers():
    """The ensemble's disagreement score and its calibrated threshold."""
    import torch
    from pyatmosphere_gb300.surrogate.ensemble import calibrate_threshold, disagreement
    # two members that agree on query 0 and split on query 1
    p = torch.zeros((2, 2, 64))
    p[:, 0, 10] = 1.0
    p[0, 1, 10] = 1.0
    p[1, 1, 50] = 1.0
    s = disagreement(p)
    assert float(s[0]) == 0.0 and abs(float(s[1]) - 0.5) < 1e-6
    scores = np.array([0.01, 0.02, 0.03, 0.04, 0.05])
    ks = np.array([0.01, 0.015, 0.05, 0.01, 0.09])   # the point at score 0.03 misses the 0.02 gate
    assert calibrate_threshold(scores, ks, target=0.95) == 0.02
    assert calibrate_threshold(scores, ks, target=0.75) == 0.04
    assert calibrate_threshold(np.array([0.1]), np.array([0.5])) == 0.0
