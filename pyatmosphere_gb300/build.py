"""Builds the engine's shared libraries in-tree with nvcc for sm_103a.

    python -m pyatmosphere_gb300.build           # incremental
    python -m pyatmosphere_gb300.build --force

Outputs (git-ignored) go to ``pyatmosphere_gb300/_lib/``:
  libatm.so           the engine (kernels + C ABI of include/atm.h)
  libatm_selftest.so  host-only emulation of the FFT / Bessel / phase code
Translation units compile in parallel; nothing is rebuilt when the outputs
are newer than every source.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_lib")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I", CSRC, "-I", INCLUDE]

ENGINE_SOURCES = ["atm_kernels.cu", "atm_abi.cu", "atm_noalloc.cu", "atm_mlp.cu", "atm_tc.cu"]
SELFTEST_SOURCES = ["atm_selftest.cu"]
HEADERS = ["atm_common.cuh", "atm_internal.h"]


def _nvcc() -> str:
    for cand in [shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"]:
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the engine needs the CUDA toolkit to build")


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r


def build(force: bool = False, verbose: bool = False) -> dict:
    nvcc = _nvcc()
    os.makedirs(OUT, exist_ok=True)
    headers = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(INCLUDE, "atm.h")]
    engine_srcs = [s for s in ENGINE_SOURCES if os.path.exists(os.path.join(CSRC, s))]
    jobs = []
    objs = []
    for src in engine_srcs:
        s = os.path.join(CSRC, src)
        o = os.path.join(OUT, src.replace(".cu", ".o"))
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append([nvcc] + ARCH + FLAGS + ["-c", s, "-o", o])
    lib = os.path.join(OUT, "libatm.so")
    st_src = os.path.join(CSRC, SELFTEST_SOURCES[0])
    st_lib = os.path.join(OUT, "libatm_selftest.so")
    if force or _stale(st_lib, [st_src] + headers):
        jobs.append([nvcc] + FLAGS + ["-shared", st_src, "-o", st_lib])
    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 2))) as ex:
        for r in ex.map(_run, jobs):
            if verbose and (r.stdout or r.stderr):
                print(r.stdout + r.stderr)
    if force or _stale(lib, objs):
        _run([nvcc] + ARCH + ["-shared", "-o", lib] + objs)
    return {"libatm": lib, "selftest": st_lib}


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
