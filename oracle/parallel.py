"""Realisations of the oracle in parallel worker processes.

TEST INFRASTRUCTURE ONLY, like the rest of ``oracle/``: the checker for the
GB300 engine, never imported by the product.

numpy's FFT is single-threaded, so a batch of independent realisations is
spread over worker processes (one BLAS thread each).  The pool is started with
the ``spawn`` method: a process forked after the parent has touched the GPU
can hang.
"""
from __future__ import annotations

import multiprocessing as mp
import os
from typing import List, Optional

import numpy as np

from . import atm_oracle as o


def _one(args):
    spec, rho, theta, value, prec, want_field = args
    res = o.simulate(spec, rho, theta, value, prec=prec, return_field=want_field)
    if want_field:
        meas, field = res
        return meas[0], field
    return res[0], None


def simulate_parallel(spec: o.ChannelSpec, rho: np.ndarray, theta: np.ndarray, value: np.ndarray,
                      prec: str = "fp64", return_fields: bool = False, processes: Optional[int] = None):
    """o.simulate for every realisation of (R, n, P) spectra, one realisation
    per task.  Returns the list of measure dicts (and the list of final fields
    when return_fields)."""
    R = rho.shape[0]
    try:
        cores = len(os.sched_getaffinity(0))
    except AttributeError:
        cores = os.cpu_count() or 1
    processes = max(1, min(processes or cores, R))
    tasks = [(spec, rho[r:r + 1], theta[r:r + 1], value[r:r + 1], prec, return_fields) for r in range(R)]
    keys = ("OPENBLAS_NUM_THREADS", "OMP_NUM_THREADS", "MKL_NUM_THREADS")
    saved = {k: os.environ.get(k) for k in keys}
    for k in keys:
        os.environ[k] = "1"  # the children read it when they import numpy
    try:
        ctx = mp.get_context("spawn")
        with ctx.Pool(processes) as pool:
            out = pool.map(_one, tasks, chunksize=1)
    finally:
        for k, v in saved.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v
    meas: List[dict] = [m for m, _ in out]
    if return_fields:
        return meas, [f for _, f in out]
    return meas
