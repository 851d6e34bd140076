"""The allocation-free vacuum step (atm_vacuum_noalloc) against the plan-based
one (atm_vacuum), through the C ABI.

atm_vacuum_noalloc serves callers that cannot allocate device memory where
they propagate a field: a host framework whose caching allocator already owns
the device memory, or a loop that cannot take cudaFree's implicit device
synchronisation.  It keeps its tables in one static device array instead of
a plan's workspace.  This file is collected last so that a run stopping at
the first failure has run every other test first; it also passes on its own
in a fresh process."""
import ctypes

import numpy as np
import pytest

from oracle import atm_oracle as o

pytestmark = pytest.mark.gpu

TOL = 2e-6  # the tolerance of the vacuum-step parity tests


def _lib():
    from pyatmosphere_gb300.engine import _lib
    return _lib.load()


def _field(torch, N, delta, seed, batch):
    rng = np.random.default_rng(seed)
    u0 = o.gaussian_source(N, delta, 808e-9, 0.25, np.inf)
    fields = [u0] + [u0 + (rng.standard_normal((N, N)) + 1j * rng.standard_normal((N, N))) * 0.1 * (k + 1) *
                     np.abs(u0) for k in range(batch - 1)]
    return torch.from_numpy(np.stack(fields).astype(np.complex64)).cuda()


# N = 4096 fills the static table exactly (3 x 4096 complex64)
@pytest.mark.parametrize("N,batch", [(512, 2), (2048, 5), (4096, 3)])
def test_noalloc_matches_plan_vacuum_on_two_calls(N, batch):
    import torch
    from pyatmosphere_gb300.engine import EnginePlan
    assert torch.cuda.is_available()
    lib = _lib()
    delta, wvl = 3.0 / N, 808e-9
    plan = EnginePlan(N, delta, wvl, 0.25, np.inf, [], 1e3, batch=batch)
    ref = _field(torch, N, delta, N, batch)
    got = ref.clone()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    for dz in (1500.0, 3700.0):  # two calls in a row on the same array
        plan.vacuum(ref, dz)
        rc = lib.atm_vacuum_noalloc(ctypes.c_void_p(got.data_ptr()), N, batch, delta, wvl, dz, stream)
        assert rc == 0, lib.atm_last_error()
        torch.cuda.synchronize()
        a, b = got.cpu().numpy(), ref.cpu().numpy()
        for k in range(batch):
            assert o.rel_l2(a[k], b[k]) < TOL
    plan.close()


def test_noalloc_rejects_sizes_beyond_its_table():
    import torch
    lib = _lib()
    buf = torch.zeros(16, dtype=torch.complex64, device="cuda")
    rc = lib.atm_vacuum_noalloc(ctypes.c_void_p(buf.data_ptr()), 8192, 1, 1e-3, 808e-9, 100.0,
                                ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == -2
    assert b"4096" in lib.atm_last_error()
