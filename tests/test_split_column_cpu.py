"""The algebra of the 4096^2 column form (column variant 14), restated on the
host with numpy: a column transform of length N = 2H as two H-point
transforms (a radix-2 split in y), the transfer function taken from the
half table hy[0..H] through hy[K] = hy[N - K], and the combine of the two
inverses.  The kernel's bits are checked against the FP64 oracle on the GPU;
this checks the formulas the kernel is built on, at sizes numpy does at once.

The transfer function of a vacuum step in the unshifted order
(theory/vacuum.py:5-7 with the shifts folded away) is
exp(-i pi lambda dz f_K^2), f_K = K df for K < N/2 and (K - N) df above, so
f_K^2 = f_{N-K}^2 exactly and the half table loses nothing."""
import numpy as np
import pytest


def transfer(N, delta, wvl, dz):
    """The y transfer function of one step in FP64, rounded to complex64 (as
    the plan's tables are)."""
    df = 1.0 / (N * delta)
    k = np.arange(N)
    f = np.where(k < N // 2, k, k - N).astype(np.float64) * df
    arg = (np.pi * dz) * wvl * (f * f)
    return (np.cos(arg) - 1j * np.sin(arg)).astype(np.complex64)


@pytest.mark.parametrize("N", [64, 4096])
def test_half_table_is_exact(N):
    hy = transfer(N, 3.0 / N, 808e-9, 4e3)
    K = np.arange(N // 2 + 1, N)
    assert np.array_equal(hy[K], hy[N - K])  # bitwise: the same FP64 argument


@pytest.mark.parametrize("N,C", [(64, 4), (512, 4)])
def test_split_column_pass_equals_direct(N, C):
    rng = np.random.default_rng(N)
    H = N // 2
    x = rng.normal(size=(N, C)) + 1j * rng.normal(size=(N, C))
    hy = transfer(N, 3.0 / N, 808e-9, 4e3).astype(np.complex128)
    hx = np.exp(1j * rng.uniform(0, 2 * np.pi, size=C))
    # direct: forward transform, H = hy[K] hx, unnormalised inverse
    X = np.fft.fft(x, axis=0)
    want = np.fft.ifft(X * hy[:, None] * hx[None, :], axis=0) * N
    # split: the halves' inputs (group 0: a + b, group 1: (a - b) W_N^n)
    n = np.arange(H)[:, None]
    w = np.exp(-2j * np.pi * n / N)
    a, b = x[:H], x[H:]
    Ef, Of = np.fft.fft(a + b, axis=0), np.fft.fft((a - b) * w, axis=0)
    np.testing.assert_allclose(Ef, X[0::2], rtol=1e-12, atol=1e-10)
    np.testing.assert_allclose(Of, X[1::2], rtol=1e-12, atol=1e-10)
    # the transfer function from the half table: element k of half g is frequency K = 2k + g
    half = hy[:H + 1]
    k = np.arange(H)
    hy_of = [half[np.where(2 * k + g <= H, 2 * k + g, N - (2 * k + g))] for g in (0, 1)]
    E = np.fft.ifft(Ef * hy_of[0][:, None] * hx[None, :], axis=0) * H
    O = np.fft.ifft(Of * hy_of[1][:, None] * hx[None, :], axis=0) * H * np.conj(w)
    got = np.concatenate([E + O, E - O])
    np.testing.assert_allclose(got, want, rtol=1e-10, atol=1e-9 * np.abs(want).max())
