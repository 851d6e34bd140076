"""numpy FP64 restatement of the surrogate MLP's forward pass, loss and
gradients (TEST INFRASTRUCTURE ONLY: the checker for the engine's training
kernels).  The weights are rounded to bfloat16 first, exactly as the
engine's GEMMs see them, so the comparison isolates the kernels' FP32
arithmetic."""
from __future__ import annotations

import numpy as np
from scipy.special import erf


def bf16_round(a):
    """Round-to-nearest-even to bfloat16, returned as float64."""
    a = np.asarray(a, np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(params, widths):
    out, off = [], 0
    for i in range(len(widths) - 1):
        n_w = widths[i + 1] * widths[i]
        W = params[off:off + n_w].reshape(widths[i + 1], widths[i])
        off += n_w
        b = params[off:off + widths[i + 1]]
        off += widths[i + 1]
        out.append((W, b))
    return out


def gelu(z):
    return 0.5 * z * (1 + erf(z / np.sqrt(2)))


def gelu_grad(z):
    return 0.5 * (1 + erf(z / np.sqrt(2))) + z * np.exp(-0.5 * z * z) / np.sqrt(2 * np.pi)


def forward(params, widths, x):
    layers = unpack(np.asarray(params, np.float64), widths)
    acts, pres = [np.asarray(x, np.float64)], [None]
    for l, (W, b) in enumerate(layers):
        z = acts[-1] @ bf16_round(W).T + b
        if l < len(layers) - 1:
            pres.append(z)
            acts.append(gelu(z))
        else:
            acts.append(z)
    return acts, pres


def loss_and_grad(params, widths, x, t, n_hist, w_mse):
    """Mean over the batch of KL(t_hist || softmax(y_hist)) + w_mse * MSE(y_rest, t_rest)."""
    layers = unpack(np.asarray(params, np.float64), widths)
    acts, pres = forward(params, widths, x)
    y = acts[-1]
    B = y.shape[0]
    h = y[:, :n_hist]
    h = h - h.max(axis=1, keepdims=True)
    logp = h - np.log(np.exp(h).sum(axis=1, keepdims=True))
    th = t[:, :n_hist]
    kl = np.where(th > 0, th * (np.log(np.where(th > 0, th, 1)) - logp), 0).sum(axis=1)
    d = y[:, n_hist:] - t[:, n_hist:]
    nm = y.shape[1] - n_hist
    loss = (kl + w_mse * (d * d).sum(axis=1) / nm).mean()
    dy = np.concatenate([np.exp(logp) - th, 2 * w_mse * d / nm], axis=1) / B
    grads = []
    dz = dy
    for l in range(len(layers) - 1, -1, -1):
        W, _ = layers[l]
        gW = dz.T @ acts[l]
        gb = dz.sum(axis=0)
        grads = [gW.ravel(), gb] + grads
        if l > 0:
            dz = (dz @ bf16_round(W)) * gelu_grad(pres[l])
    return loss, np.concatenate(grads)


def infer_tc_emulated(params, widths, x, n_hist):
    """The arithmetic of the engine's fused tensor-core inference in FP64:
    inputs as two bfloat16 slices x = hi + lo (lo = bf16(x - hi) formed in
    FP32), bfloat16 weights, hidden activations rounded to bfloat16 after
    GELU, FP64 sums in place of the tensor cores' FP32 accumulation; a
    softmax over the first n_hist outputs, the rest raw."""
    layers = unpack(np.asarray(params, np.float64), widths)
    x32 = np.asarray(x, np.float32)
    hi = bf16_round(x32)
    lo = bf16_round((x32.astype(np.float64) - hi).astype(np.float32))
    a = hi + lo
    for l, (W, b) in enumerate(layers):
        z = a @ bf16_round(W).T + b
        if l < len(layers) - 1:
            a = bf16_round(gelu(z).astype(np.float32))
        else:
            a = z
    h = a[:, :n_hist] - a[:, :n_hist].max(axis=1, keepdims=True)
    p = np.exp(h)
    p /= p.sum(axis=1, keepdims=True)
    return np.concatenate([p, a[:, n_hist:]], axis=1)
