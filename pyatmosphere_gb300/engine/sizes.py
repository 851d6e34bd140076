"""Per-kernel device time of the engine at one grid size.

    python -m pyatmosphere_gb300.engine.sizes --N 4096 --batch 64 [--variants 4,4,14] [--runs 3]

Runs a channel of the mixed-size family (N delta = 3 m, 20 km, 5 sparse-spectrum
screens of 1024 annuli, MVK Cn2 1e-15, w0 0.1 m, pupil 0.1 m) for a batch of
seeded realisations drawn on the device, with the launch forms given or those
atm_autotune picks, and prints the run time and each kernel category's time per
launch (CUDA events recorded by the library around every launch).  The FFT
passes also get their bandwidth on 16 bytes per pixel (one complex64 read and
write of the field).
"""
from __future__ import annotations

import argparse
import math

import numpy as np
import torch

from ..theory.models import MVKModel
from .plan import EnginePlan
from .spectra import annulus_psd


def channel_plan(N: int, batch: int, device=None, screens: int = 5, points: int = 1024):
    """A plan of the mixed-size family at grid N, and its device spectra."""
    dev = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
    delta, wvl, length = 3.0 / N, 808e-9, 20e3
    f_min, f_max = 1 / 1e3 / 15, 2 / 6e-3
    base = np.exp(np.linspace(np.log(f_min), np.log(f_max), points)).astype(np.float32)
    positions = (np.arange(screens) + 0.5) * (length / screens)
    plan = EnginePlan(N, delta, wvl, 0.1, math.inf, positions, length, f_base=base, pupils=[(0.1,)], batch=batch,
                      device=dev)
    psd = annulus_psd(base, MVKModel(Cn2=1e-15, l0=6e-3, L0=1e3).psd_phi_f, 2 * np.pi / wvl, length / screens)
    sq = torch.from_numpy(np.sqrt(psd)).to(dev).expand(screens, -1).contiguous()
    rho = torch.empty((batch, screens, points), dtype=torch.float32, device=dev)
    theta = torch.empty_like(rho)
    value = torch.empty((batch, screens, points), dtype=torch.complex64, device=dev)
    plan.draw_spectra(3, 0, sq, rho, theta, value)
    return plan, (rho, theta, value)


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--N", type=int, default=4096)
    ap.add_argument("--batch", type=int, default=64)
    ap.add_argument("--variants", default="", help="row,col_tile,col (default: atm_autotune's choice)")
    ap.add_argument("--warmup", type=int, default=2)
    ap.add_argument("--runs", type=int, default=3)
    a = ap.parse_args(argv)
    plan, sp = channel_plan(a.N, a.batch)
    if a.variants:
        plan.set_variants(*(int(x) for x in a.variants.split(",")))
        forms = a.variants
    else:
        t = plan.autotune(repeats=2)
        forms = f"{t['row_variant']},{t['col_tile']},{t['col_variant']}"
    for _ in range(a.warmup):
        plan.run(*sp)
    torch.cuda.synchronize()
    plan.profile_begin(64 * max(1, a.runs))
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(a.runs):
        plan.run(*sp)
    e1.record()
    torch.cuda.synchronize()
    prof = plan.profile_end()
    plan.check()
    ms = e0.elapsed_time(e1) / max(1, a.runs)
    print(f"N = {a.N}, B = {a.batch}, forms {forms}: {ms:.2f} ms per run, {a.batch / ms * 1e3:.0f} realisations/s")
    for k, v in prof.items():
        if not v["launches"]:
            continue
        per = v["ms"] / v["launches"]
        extra = f", {16 * a.N * a.N * a.batch / (per * 1e-3) / 1e9:.0f} GB/s" if k in ("row_pass", "col_pass") else ""
        print(f"  {k:13s} {v['launches'] // max(1, a.runs):3d} per run, {per:.3f} ms per launch{extra}")
    plan.close()
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
