"""Size-independent properties at the benchmark's own size (2048^2 advanced
channel, 5 screens x 1024 annuli, 256 realisations per launch), covering
every realisation of the batch (the FP64 oracle checks 16 of them in
test_bench_parity_gpu.py, about 2.5 s per realisation on the host cores):
- a lossless channel conserves each realisation's energy (unimodular screen
  phasors, unitary vacuum steps);
- two runs of the same batch give the same bits;
- a realisation's result does not depend on the batch it runs in;
and, at 4096^2, a vacuum step is unitary and a step back undoes it."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def advanced():
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    from pyatmosphere_gb300.engine.uneven import ChannelParams
    return ChannelParams(N=2048, n_screens=5, length=50e3, Cn2=5e-16, w0=0.12, wvl=808e-9, extent=2048 * 1.5e-3,
                         pupil_radius=0.2, points=1024)


def _run(c, B, seed=77, first=0):
    import torch
    from pyatmosphere_gb300.engine import EnginePlan
    plan = EnginePlan(c.N, c.delta, c.wvl, c.w0, c.F0, c.positions(), c.length, f_base=c.base(),
                      pupils=[(c.pupil_radius,)], batch=B)
    n, P = c.n_screens, c.points
    rho = torch.empty((B, n, P), dtype=torch.float32, device="cuda")
    theta = torch.empty_like(rho)
    value = torch.empty((B, n, P), dtype=torch.complex64, device="cuda")
    sq = torch.from_numpy(c.sqrt_psd()).cuda().expand(n, -1).contiguous()
    plan.draw_spectra(seed, first, sq, rho, theta, value)
    a = plan.run(rho, theta, value).cpu().numpy()
    b = plan.run(rho, theta, value).cpu().numpy()
    plan.close()
    return a, b


def test_benchmark_batch_conserves_energy_is_deterministic_and_batch_independent(advanced):
    from pyatmosphere_gb300.engine import _lib
    a, b = _run(advanced, 256)
    assert a.shape[0] == 256 and np.all(np.isfinite(a))
    # the source is normalised to unit energy on the grid; every step is unitary
    np.testing.assert_allclose(a[:, _lib.OUT_ETA_TOTAL], 1.0, atol=1e-4)
    assert np.all((a[:, _lib.OUT_PUPIL0] > 0) & (a[:, _lib.OUT_PUPIL0] <= a[:, _lib.OUT_ETA_TOTAL] + 1e-6))
    np.testing.assert_array_equal(a, b)
    # realisations 0..15 of the 256-batch, alone in a 16-batch plan
    s, _ = _run(advanced, 16)
    np.testing.assert_array_equal(s, a[:16])


@pytest.mark.parametrize("N", [4096])
def test_vacuum_step_is_unitary_and_reversible_at_full_size(N):
    import torch
    from pyatmosphere_gb300.theory.vacuum import vacuum_propagation
    delta, wvl, L = 3.0 / N, 1550e-9, 20e3
    k = 2 * math.pi / wvl
    rng = np.random.default_rng(N)
    x = (np.arange(N) - N // 2) * delta
    u = (np.exp(-(x[None, :] ** 2 + x[:, None] ** 2) / 0.2 ** 2) *
         np.exp(1j * rng.uniform(0, 2 * np.pi, (N, N)) * 0.3)).astype(np.complex64)
    ut = torch.from_numpy(u).cuda()
    e0 = float((ut.abs() ** 2).sum())
    v = vacuum_propagation(ut, L, k, delta)
    assert float((v.abs() ** 2).sum()) == pytest.approx(e0, rel=2e-5)
    back = vacuum_propagation(v, -L, k, delta)
    assert float(torch.linalg.vector_norm(back - ut) / torch.linalg.vector_norm(ut)) < 3e-5
