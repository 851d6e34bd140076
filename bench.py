#!/usr/bin/env python
"""Throughput of the 2048^2 split-step channel Monte Carlo on GB300.

Workload (config 2 of the reference's advanced channel): RectGrid 2048 x 2048,
delta 1.5 mm; Gaussian beam 808 nm, w0 0.12 m, collimated; 50 km path with 5
sparse-spectrum screens (MVK Cn2 5e-16, l0 6 mm, L0 1 km, 1024 log-polar
annuli from 1/15 km^-1 to 2/l0); CirclePupil 0.2 m.  One step = one batch of
256 seeded realisations through the engine (screens, propagation, pupil and
moments).  Synthetic inputs: spectra drawn on the host from numpy's
default_rng([seed, realisation]) exactly as the reference forms them.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Prints one JSON line (rank 0).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "2048² channel samples/s, batched vs plain on GPU; surrogate PDT/s at KS≤0.02"
UNIT = "samples/s"

WORKLOAD = dict(N=2048, delta=1.5e-3, wvl=808e-9, w0=0.12, F0=float("inf"), length=50e3, count=5,
                Cn2=5e-16, l0=6e-3, L0=1e3, points=1024, f_min=1 / 1e3 / 15, f_max=2 / 6e-3,
                pupil_radius=0.2)
WORKLOAD_NAME = ("advanced channel: 2048^2 grid, delta 1.5 mm, 808 nm, w0 0.12 m, 50 km, "
                 "5 SS screens x 1024 annuli, MVK Cn2 5e-16, pupil 0.2 m")


# DRAM bytes (read + write) per launch and realisation of the forms row pass 4
# and column pass 10, from ncu captures of 16-realisation runs of this
# workload, averaged over the launches of a run (traffic grows with the
# realisations); a fixed figure, not measured by this script.  Column pass 15
# (the split form) loads and stores the same 32-byte tile rows once.
TRAFFIC_PER_REALISATION = {"row_pass": 66.98e6, "col_pass": 63.78e6, "screen_gemm": 25.98e6,
                           "screen_table": 8.24e6}


def positions(length, count):
    return (np.arange(count) + 0.5) * (length / count)


def base_and_psd():
    from pyatmosphere_gb300.engine.spectra import annulus_psd
    from pyatmosphere_gb300.theory.models import MVKModel
    w = WORKLOAD
    base = np.exp(np.linspace(np.log(w["f_min"]), np.log(w["f_max"]), w["points"], dtype=np.float32))
    model = MVKModel(Cn2=w["Cn2"], l0=w["l0"], L0=w["L0"])
    psd = annulus_psd(base, model.psd_phi_f, 2 * np.pi / w["wvl"], w["length"] / w["count"])
    return base, psd


# ---------------------------------------------------------------------------
# clocks sampled during the timed region
# ---------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for nm, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------------------------
# CPU baseline: the oracle's restatement of the reference numpy path
# (reference precision), timed on this host's cores
# ---------------------------------------------------------------------------
def cpu_realisations(n_real: int, seed: int = 4242):
    from oracle import atm_oracle as o
    w = WORKLOAD
    spec = o.ChannelSpec(N=w["N"], delta=w["delta"], wvl=w["wvl"], w0=w["w0"], F0=w["F0"], length=w["length"],
                         count=w["count"], Cn2=w["Cn2"], l0=w["l0"], L0=w["L0"], points=w["points"],
                         f_min=w["f_min"], f_max=w["f_max"], pupil_radius=w["pupil_radius"])
    base = o.logpolar_base(spec.points, spec.f_min, spec.f_max)
    psd = o.annulus_psd(base, spec.k, spec.thickness, spec.Cn2, spec.l0, spec.L0, use_scipy=False)
    rho, theta, value = o.draw_spectra(seed, range(n_real), spec.count, base, psd)
    t = time.perf_counter()
    o.simulate(spec, rho, theta, value, prec="ref")
    return n_real / (time.perf_counter() - t)


REF_INSTALL = os.path.join(ROOT, "baseline", "_ref")


def import_stock_reference():
    """The unmodified reference package as installed under baseline/_ref (pip
    --target), or None.  Its plotting and pandas imports are served by empty
    stand-in modules for the import only; the reference keeps its own
    bindings.  Its numpy path is selected (gpu.py:4-20)."""
    import importlib
    import types
    if not os.path.isdir(os.path.join(REF_INSTALL, "pyatmosphere")):
        return None
    added = []
    for name in ("matplotlib", "matplotlib.pyplot", "pandas"):
        if name not in sys.modules:
            sys.modules[name] = types.ModuleType(name)
            added.append(name)
    if "matplotlib.pyplot" in added:
        sys.modules["matplotlib"].pyplot = sys.modules["matplotlib.pyplot"]
    if REF_INSTALL not in sys.path:
        sys.path.append(REF_INSTALL)
    try:
        ref = importlib.import_module("pyatmosphere")
        for sub in ("channels", "grids", "sources", "pathes", "phase_screens", "pupils", "measures",
                    "theory.models", "simulations", "simulations.simulation", "simulations.pdt",
                    "simulations.beam", "utils"):
            importlib.import_module("pyatmosphere." + sub)
    finally:
        for name in added:
            sys.modules.pop(name, None)
    ref.gpu.config["use_gpu"] = False
    return ref


class StockRealisation:
    """One realisation of the workload through the unmodified reference:
    Channel.run (channels.py:31-35; its SSPhaseScreen draws the spectra from
    numpy's global generator, phase_screens.py:93-136) and the measures the
    engine fuses (measures.py:7-38): total and pupil eta, centroid and second
    moments."""

    def __init__(self, ref):
        import importlib
        mod = {n: importlib.import_module("pyatmosphere." + n)
               for n in ("channels", "grids", "pathes", "phase_screens", "pupils", "sources", "theory.models",
                         "measures")}
        w = WORKLOAD
        self.m = mod["measures"]
        self.channel = mod["channels"].Channel(
            grid=mod["grids"].RectGrid(resolution=w["N"], delta=w["delta"]),
            source=mod["sources"].GaussianSource(wvl=w["wvl"], w0=w["w0"], F0=w["F0"]),
            path=mod["pathes"].IdenticalPhaseScreensPath(
                phase_screen=mod["phase_screens"].SSPhaseScreen(
                    model=mod["theory.models"].MVKModel(Cn2=w["Cn2"], l0=w["l0"], L0=w["L0"]),
                    f_grid=mod["grids"].RandLogPolarGrid(points=w["points"], f_min=w["f_min"], f_max=w["f_max"])),
                length=w["length"], count=w["count"]),
            pupil=mod["pupils"].CirclePupil(radius=w["pupil_radius"]))

    def __call__(self, seed: int):
        np.random.seed(seed)
        ch, m = self.channel, self.m
        u = ch.run(pupil=False)
        return [m.eta(ch, output=u), m.eta(ch, output=ch.pupil.output(u))] + \
            [f(ch, output=u) for f in (m.mean_x, m.mean_y, m.mean_x2, m.mean_xy, m.mean_y2)]


def cores():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def run_reference(args, rank, world):
    """The reference arm: the unmodified reference package (baseline/_ref) on
    its numpy path when it is installed, else the oracle's restatement of it
    in the reference's precision; one realisation per step."""
    if rank != 0:
        return 0
    ref = None if args.ref_port else import_stock_reference()
    if ref is not None:
        step = StockRealisation(ref)
        kind = "reference"
        sample = (f"{args.steps} single-realisation steps of the 2048^2 channel through the unmodified reference "
                  "(Channel.run and measures on its numpy path, spectra drawn inside the step)")
    else:
        def step(seed):
            return cpu_realisations(1, seed=seed)
        kind = "port"
        sample = (f"{args.steps} single-realisation steps of the 2048^2 channel, numpy/OpenBLAS restatement of "
                  "the reference path in its own precision")
    for w in range(args.warmup):
        step(1 + w)
    t = time.perf_counter()
    for k in range(args.steps):
        step(100 + k)
    el = time.perf_counter() - t
    val = args.steps / el
    line = {
        "impl": "reference", "metric": METRIC, "value": val, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": el / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c64/f32 (numpy, reference precision)",
        "data": "synthetic (seeded spectra, reference's own formulas)",
        "config": {"workload": WORKLOAD_NAME, "batch": 1, "realisations_per_step": 1},
        "cpu_baseline": {"value": val, "unit": UNIT, "cores": cores(), "kind": kind, "sample": sample},
        "e2e": {"value": val, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------------------
# the reference's GPU algorithm restated on torch: a measurement baseline
# ---------------------------------------------------------------------------
def reference_algorithm_on_torch(dev, host_spectra, n_real):
    """Realisations/s of the reference's own GPU algorithm (its cupy backend,
    gpu.py:4-20) restated on torch, one realisation at a time: the shifted
    2-D FFTs of utils.py:42-50 (cuFFT through torch.fft), the transfer function
    of theory/vacuum.py:5-7, the complex64 screen GEMM of
    phase_screens.py:125-126 (cuBLAS through torch's matmul), the exp(-i phi)
    multiply of pathes.py:72-73 and the pupil and measures of pupils.py:8-13 and
    measures.py:1-38, each measure a separate reduction read back to the host.
    A timing baseline only: nothing of the engine runs here."""
    import torch
    w = WORKLOAD
    N, d, wvl, L, n = w["N"], w["delta"], w["wvl"], w["length"], w["count"]
    k = 2 * math.pi / wvl
    ax = (torch.arange(N, device=dev, dtype=torch.float32) - N // 2) * d
    x, y = ax.reshape(1, N), ax.reshape(N, 1)
    r2 = x * x + y * y
    fa = (torch.arange(N, device=dev, dtype=torch.float32) - N // 2) / (N * d)
    f2 = fa.reshape(1, N) ** 2 + fa.reshape(N, 1) ** 2
    pupil = (r2 <= w["pupil_radius"] ** 2)
    pos = positions(L, n)
    steps = [pos[0]] + [pos[i] - pos[i - 1] for i in range(1, n)] + [L - pos[-1]]
    u0 = (math.sqrt(2 / math.pi) / w["w0"] * torch.exp(-r2 / w["w0"] ** 2)).to(torch.complex64)

    def vac(u, dz):
        U = torch.fft.fftshift(torch.fft.fft2(torch.fft.fftshift(u))) * d * d
        h = torch.exp(torch.tensor(1j * k * dz, dtype=torch.complex64, device=dev)) * \
            torch.exp(-1j * (math.pi * dz * wvl) * f2)
        # (N df)^2 with df = 1 / (N delta)
        return (torch.fft.ifftshift(torch.fft.ifft2(torch.fft.ifftshift(U * h))) / (d * d)).to(torch.complex64)

    rho, theta, value = (torch.from_numpy(a).to(dev) for a in host_spectra)

    def one(r):
        u = u0
        for i in range(n):
            u = vac(u, steps[i])
            fx = (rho[r, i] * torch.cos(theta[r, i])).reshape(1, -1)
            fy = (rho[r, i] * torch.sin(theta[r, i])).reshape(-1, 1)
            a = value[r, i].reshape(1, -1) * torch.exp(2j * math.pi * (y @ fy.T))
            b = torch.exp(2j * math.pi * (fx.T @ x))
            u = torch.exp(-1j * (a @ b).real) * u
        u = vac(u, steps[n])
        I = u.real ** 2 + u.imag ** 2
        out = [float((I * pupil).sum() * d * d)]
        for wgt in (x, -y, x * x, -x * y, y * y):
            out.append(float((I * wgt).sum() * d * d))
        return out

    one(0)
    torch.cuda.synchronize()
    t = time.perf_counter()
    for r in range(n_real):
        one(r % rho.shape[0])
    torch.cuda.synchronize()
    return n_real / (time.perf_counter() - t)


# ---------------------------------------------------------------------------
# GB300 engine
# ---------------------------------------------------------------------------
def bf16_peak():
    """The measured dense bf16 burst peak (TFLOP/s) of MEASURED_PEAKS.json, else None."""
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["bf16_tflops"])
    except (OSError, KeyError, ValueError):
        return None


def surrogate_leg(args, dev):
    """PDT surrogate (the inference configuration): 100,000 seeded queries, 90 %
    inside the training box and 10 % outside it (path length 20-100 km).  The
    shipped ensemble answers a query when it is inside the box and its members
    agree (disagreement at most the calibrated threshold); every other query
    goes to the simulator (N = 1024, 256 realisations).  Reported: the
    network's queries/s (device-resident and end to end from host parameters),
    the fraction it answers, the simulator's queries/s on fallback points, the
    mixed queries/s of the whole query set, and the bin-edge KS of the answered
    held-out points against 8192 fresh realisations each (noise floor 0.0096)."""
    import torch
    from pyatmosphere_gb300.surrogate.ensemble import EnsembleSurrogate
    from pyatmosphere_gb300.surrogate.experiment import load
    from pyatmosphere_gb300.surrogate.model import (N_HIST, Box, PointSimulator, SimConfig, features, ks_binned,
                                                    ks_hist, targets_from_measures)
    here = os.path.join(ROOT, "pyatmosphere_gb300", "surrogate")
    ens_path = os.path.join(here, "pdt_ensemble.npz")
    if os.path.exists(ens_path):
        ens = EnsembleSurrogate.load(ens_path, device=dev)
        weights = "pyatmosphere_gb300/surrogate/pdt_ensemble.npz"
    else:
        ens = EnsembleSurrogate([load(os.path.join(here, "pdt_mlp.npz"), device=dev)])
        weights = "pyatmosphere_gb300/surrogate/pdt_mlp.npz (one network, no gate)"
    box = Box()
    rng = np.random.default_rng(args.seed + 7)
    n_q = 100_000
    n_out = n_q // 10
    params = box.sample(n_q, rng)
    params["L"][:n_out] = np.exp(rng.uniform(np.log(20e3), np.log(100e3), n_out))  # outside the box
    X_host = torch.from_numpy(features(params, box, ens.physics)).pin_memory()
    X = X_host.to(dev)

    def answer(x):
        probs, _, oor, score = ens.predict(x)
        return probs, ens.answered(score, oor)

    for _ in range(3):
        answer(X)
    stream = torch.cuda.current_stream(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    reps = 10
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(reps):
        _, ans = answer(X)
    e1.record(stream)
    torch.cuda.synchronize()
    q_dev = n_q * reps / (e0.elapsed_time(e1) * 1e-3)
    answered = float(ans.float().mean())
    # the networks alone (the fused inference kernels of all members): algorithmic FLOPs / time
    mlps = [m.mlp for m in ens.members]
    widths = mlps[0].widths
    flop_q = 2 * sum(widths[i] * widths[i + 1] for i in range(len(widths) - 1)) * len(mlps)
    e0.record(stream)
    for _ in range(reps):
        for m in mlps:
            m.infer(X, ens.members[0].lo, ens.members[0].hi)
    e1.record(stream)
    torch.cuda.synchronize()
    mlp_s = e0.elapsed_time(e1) * 1e-3 / reps
    mlp_tflops = n_q * flop_q / mlp_s / 1e12
    out_host = torch.empty((n_q, N_HIST), dtype=torch.float32).pin_memory()

    def e2e_query():
        probs, a = answer(X_host.to(dev, non_blocking=True))
        out_host.copy_(probs, non_blocking=True)

    for _ in range(3):
        e2e_query()
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(reps):
        e2e_query()
    e1.record(stream)
    torch.cuda.synchronize()
    q_e2e = n_q * reps / (e0.elapsed_time(e1) * 1e-3)
    # the simulator fallback (N = 1024, 256 realisations) on a few out-of-box points
    fb = PointSimulator(SimConfig(N=1024, realisations=256, seed=args.seed + 10), device=dev)
    fq = [{k: v[i] for k, v in params.items()} for i in range(4)]
    for q in fq:
        q["l0"] = 6e-3  # one spectral grid: the plan is re-targeted, not rebuilt
    fb.run(fq[0], 0)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for i, q in enumerate(fq[1:]):
        targets_from_measures(fb.run(q, 1 + i), q["aperture"])
    torch.cuda.synchronize()
    q_sim = (len(fq) - 1) / (time.perf_counter() - t0)
    fb.plan.close()
    mixed = n_q / (n_q / q_dev + (1 - answered) * n_q / q_sim)
    # quality on held-out in-box points against fresh simulations
    n_pts, n_real = args.surrogate_points, 8192
    pts = box.sample(n_pts, np.random.default_rng(args.seed + 8))
    pts["l0"] = np.round(pts["l0"] * 1e3) / 1e3
    probs, ans_h = answer(torch.from_numpy(features(pts, box, ens.physics)).to(dev))
    probs, ans_h = probs.cpu().numpy(), ans_h.cpu().numpy()
    sim = PointSimulator(SimConfig(N=512, realisations=2048, seed=args.seed + 9), device=dev)
    kb, kc = [], []
    for i in range(n_pts):
        q = {k: v[i] for k, v in pts.items()}
        etas = np.concatenate([targets_from_measures(sim.run(q, 1 + 4 * i + c), q["aperture"])[1]
                               for c in range(n_real // 2048)])
        kb.append(ks_binned(probs[i], etas))
        kc.append(ks_hist(probs[i], etas))
    sim.plan.close()
    kb, kc = np.array(kb), np.array(kc)
    a = ans_h.astype(bool)
    return {"queries_per_s": q_dev, "e2e_queries_per_s": q_e2e, "query_batch": n_q, "out_of_box_frac": 0.1,
            "answered_frac": answered, "simulated_queries_per_s": q_sim, "mixed_queries_per_s": mixed,
            "h2d_bytes_per_batch": int(X_host.numel() * 4), "d2h_bytes_per_batch": int(out_host.numel() * 4),
            "members": len(ens.members), "threshold": ens.threshold,
            "mlp": {"form": mlps[0].infer_form, "widths": list(widths), "ms_per_batch": mlp_s * 1e3,
                    "tflops": mlp_tflops, "flop_per_query": flop_q,
                    "frac_of_bf16_peak": mlp_tflops / bf16_peak() if bf16_peak() else None},
            "heldout_points": n_pts, "heldout_answered_frac": float(a.mean()),
            "frac_ks_le_0.02": float((kb[a] <= 0.02).mean()) if a.any() else None,
            "ks_binned_median": float(np.median(kb[a])) if a.any() else None,
            "ks_continuous_median": float(np.median(kc[a])) if a.any() else None,
            "all_frac_ks_le_0.02": float((kb <= 0.02).mean()),
            "ks_noise_floor": 0.87 / math.sqrt(n_real), "weights": weights}


def mixed_leg(args, dev):
    """Uneven workload: channels of mixed grid size (512..4096), screen count
    (3..20) and geometry, 64 realisations and one 64-bin PDT each, as ONE
    CUDA graph launch (one plan per grid size, one channel table set per
    channel, a stream per grid size).  `seconds` is the device time of that
    launch; set-up (plans, tables, capture) is reported apart."""
    from pyatmosphere_gb300.engine.uneven import run_uneven_graph, sample_mixed
    chans = sample_mixed(args.mixed_channels, np.random.default_rng(args.seed + 11))
    res = run_uneven_graph(chans, realisations=64, seed=args.seed, device=dev, autotune=bool(args.autotune))
    work = {}
    for c in chans:
        work[c.N] = work.get(c.N, 0) + c.N * c.N * c.n_screens * 64
    pix = sum(work.values())
    by_n = {str(k): {"channels": v["channels"], "max_screens": v["max_screens"], "tuned": v["tuned"],
                     "work_share": work[k] / pix}
            for k, v in sorted((k, v) for k, v in res.groups.items() if k != "graph")}
    return {"channels": len(chans), "realisations_per_channel": 64, "graph_launches": 1, "seconds": res.seconds,
            "channels_per_s": res.channels_per_s, "realisations_per_s": res.realisations_per_s,
            "screen_pixel_steps_per_s": pix / res.seconds, "by_N": by_n,
            "setup_s": res.groups["graph"]["setup_s"], "capture_s": res.groups["graph"]["capture_s"],
            "distribution": "N in {512,1024,2048,4096}, N delta = 3 m, n ~ U{3..20}, L log-U[1,100] km, "
                            "Cn2 log-U[1e-16,1e-14], w0 U[0.02,0.2], wvl in {808,1550} nm, F0 in {inf, L}; "
                            "l0 6 mm, L0 1 km, pupil 0.1 m"}


def run_gb300(args, rank, world, local_rank):
    import torch
    import torch.distributed as dist
    from pyatmosphere_gb300.engine import EnginePlan
    from pyatmosphere_gb300.engine.plan import fma_peak_tflops
    from pyatmosphere_gb300.engine.spectra import draw_spectra

    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    w = WORKLOAD
    B = args.batch
    base, psd = base_and_psd()
    pos = positions(w["length"], w["count"])
    from pyatmosphere_gb300.engine import _lib
    flags = {"tc": _lib.FLAG_TC_GEMM, "simt": _lib.FLAG_SIMT_GEMM, "auto": 0,
             "tc-cpasync": _lib.FLAG_TC_GEMM | _lib.FLAG_TC_CPASYNC,
             "tc256": _lib.FLAG_TC_GEMM | _lib.FLAG_TC_N256,
             "tc128": _lib.FLAG_TC_GEMM | _lib.FLAG_TC_N128}[args.gemm]
    flags |= {"auto": 0, "tiled": _lib.FLAG_TILED, "rowmajor": _lib.FLAG_ROWMAJOR}[args.layout]
    plan = EnginePlan(w["N"], w["delta"], w["wvl"], w["w0"], w["F0"], pos, w["length"], f_base=base,
                      pupils=[(w["pupil_radius"],)], batch=B, device=dev, flags=flags, cheb_cut=args.cheb_cut)
    if args.variants:
        rv, ct, cv = (int(v) for v in args.variants.split(","))
        plan.set_variants(rv, ct, cv)
        tuned = {"col_tile": ct, "row_variant": rv, "col_variant": cv, "tuned": 0}
    else:
        tuned = plan.autotune(repeats=2) if args.autotune else None
    n_steps = args.warmup + args.steps
    # distinct seeded inputs per step (weak scaling: each rank its own realisations)
    host = []
    for s in range(n_steps):
        first = (rank * n_steps + s) * B
        host.append(draw_spectra(args.seed, range(first, first + B), w["count"], base, psd))
    pinned = [[torch.from_numpy(a).pin_memory() for a in h] for h in host]
    devin = [[t.to(dev) for t in p] for p in pinned]
    out = torch.empty((n_steps, B, plan.n_out), dtype=torch.float64, device=dev)
    torch.cuda.synchronize()

    def barrier():
        if world > 1:
            dist.barrier()

    for s in range(args.warmup):
        plan.run(*devin[s], out=out[s])
    torch.cuda.synchronize()

    # ---- device-resident timed region: one captured CUDA graph per step (each
    # step's whole launch sequence, its spectra already in HBM), replayed; the
    # engine's event pair around every kernel is captured with it ----
    launches = plan.info["launches_per_run"] * args.steps
    plan.profile_begin(launches + 8)
    stream = torch.cuda.current_stream(dev)
    graphs = []
    if args.graph:
        cap = torch.cuda.Stream(device=dev)
        cap.wait_stream(stream)
        for s in range(args.warmup, n_steps):
            g = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g, stream=cap):
                plan.run(*devin[s], out=out[s])
            graphs.append(g)
        stream.wait_stream(cap)
        torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local_rank) as clocks:
        barrier()
        torch.cuda.synchronize()
        e0.record(stream)
        if graphs:
            for g in graphs:
                g.replay()
        else:
            for s in range(args.warmup, n_steps):
                plan.run(*devin[s], out=out[s])
        e1.record(stream)
        torch.cuda.synchronize()
        barrier()
    kernels_timed = "cuda events inside the timed region" + (" (external event nodes of the graphs)" if graphs else "")
    try:
        prof = plan.profile_end()
    except _lib.EngineError:
        prof = None
    plan.check()
    # the same steps as direct launches: their time beside the graphs', and the
    # per-kernel events if the graph replays could not record them
    plan.profile_begin(launches + 8)
    e6, e7 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e6.record(stream)
    for s in range(args.warmup, n_steps):
        plan.run(*devin[s], out=out[s])
    e7.record(stream)
    torch.cuda.synchronize()
    direct_prof = plan.profile_end()
    direct_ms = e6.elapsed_time(e7) / args.steps
    if prof is None:
        prof = direct_prof
        kernels_timed = "cuda events in a direct-launch pass of the same steps right after the graph-timed region"
    plan.check()
    ms = e0.elapsed_time(e1)
    t_max = torch.tensor([ms], dtype=torch.float64, device=dev)
    if world > 1:
        dist.all_reduce(t_max, op=dist.ReduceOp.MAX)
    ms = float(t_max.item())
    value = B * args.steps * world / (ms * 1e-3)

    # ---- end to end through the C ABI: pinned host spectra in, measures out ----
    meas_host = torch.empty((B, plan.n_out), dtype=torch.float64).pin_memory()
    scratch = [torch.empty_like(t) for t in devin[0]]
    h2d = sum(t.numel() * t.element_size() for t in pinned[0])
    d2h = meas_host.numel() * meas_host.element_size()
    barrier()
    torch.cuda.synchronize()
    e2, e3 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e2.record(stream)
    for s in range(args.warmup, n_steps):
        for d_, h_ in zip(scratch, pinned[s]):
            d_.copy_(h_, non_blocking=True)
        m = plan.run(*scratch, out=out[s])
        meas_host.copy_(m, non_blocking=True)
    e3.record(stream)
    torch.cuda.synchronize()
    barrier()
    ms_e2e = e2.elapsed_time(e3)
    te = torch.tensor([ms_e2e], dtype=torch.float64, device=dev)
    if world > 1:
        dist.all_reduce(te, op=dist.ReduceOp.MAX)
    e2e_value = B * args.steps * world / (float(te.item()) * 1e-3)

    # ---- plain form: one realisation per launch sequence, no batching ----
    plain = None
    if args.plain > 0 and rank == 0:
        p1 = EnginePlan(w["N"], w["delta"], w["wvl"], w["w0"], w["F0"], pos, w["length"], f_base=base,
                        pupils=[(w["pupil_radius"],)], batch=1, device=dev, flags=flags, cheb_cut=args.cheb_cut)
        one = [t[:1].contiguous() for t in devin[0]]
        for _ in range(2):
            p1.run(*one)
        torch.cuda.synchronize()
        e4, e5 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e4.record(stream)
        for i in range(args.plain):
            p1.run(*[t[i:i + 1].contiguous() for t in devin[args.warmup]])
        e5.record(stream)
        torch.cuda.synchronize()
        plain = args.plain / (e4.elapsed_time(e5) * 1e-3)
        p1.close()
    torch_ref = None
    if args.torch_reference > 0 and rank == 0:
        torch_ref = reference_algorithm_on_torch(dev, [a[:16] for a in host[args.warmup]], args.torch_reference)

    # ---- roofline of the dominant kernel, measured in the timed region ----
    N, n = w["N"], w["count"]
    K = plan.info["gemm_k"]
    tc = not (flags & _lib.FLAG_SIMT_GEMM) and w["N"] >= 256
    work = {  # algorithmic work per launch of a B-realisation batch
        # tensor cores: three FP16 MMAs (hi.hi, hi.lo, lo.hi) per FP32 product, against the dense 16-bit peak
        "screen_gemm": ("tensor", 3 * 2.0 * N * N * K * B, "TFLOP/s") if tc else ("fp32", 2.0 * N * N * K * B, "TFLOP/s"),
        "col_pass": ("hbm", 16.0 * N * N * B, "GB/s"),
        # n+1 row launches move 8 (write) + 4 (phi) + (n-1)(16 + 4) + 8 (read) bytes per pixel
        "row_pass": ("hbm", (12.0 + 20.0 * (n - 1) + 8.0) / (n + 1) * N * N * B, "GB/s"),
        # the high-frequency columns of A and B (FP16 hi + lo) are written once and the GEMM reads
        # them back while they are still in L2: the DRAM bytes of the capture, not the table size
        "screen_table": ("hbm", TRAFFIC_PER_REALISATION["screen_table"] * B, "GB/s"),
    }
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            mp = json.load(f)
        peaks["hbm"] = (float(mp["hbm_gbs"]), "measured")
    except (OSError, KeyError, ValueError):
        peaks["hbm"] = (6800.0, "fallback")
    peaks["fp32"] = (fma_peak_tflops(dev), "measured (FMA probe)")
    try:
        peaks["tensor"] = (float(mp["bf16_tflops"]), "measured (cuBLAS bf16 burst; FP16 dense rate is the same)")
    except (NameError, KeyError, ValueError):
        peaks["tensor"] = (1900.0, "fallback")
    kernels = {}
    for kname, st in prof.items():
        if st["launches"] == 0:
            continue
        avg_ms = st["ms"] / st["launches"]
        entry = {"launches": st["launches"], "total_ms": st["ms"], "avg_ms": avg_ms,
                 "share": st["ms"] / max(1e-9, sum(v["ms"] for v in prof.values()))}
        if kname in work:
            bound, amount, unit = work[kname]
            achieved = amount / (avg_ms * 1e-3) / (1e12 if unit == "TFLOP/s" else 1e9)
            pk, src = peaks[bound]
            entry.update({"bound": bound, "achieved": achieved, "peak": pk, "unit": unit,
                          "frac": achieved / pk, "peak_source": src})
        kernels[kname] = entry
    dom = max((k for k in kernels if "bound" in kernels[k]), key=lambda k: kernels[k]["total_ms"])
    hbm_dom = max((k for k in kernels if kernels[k].get("bound") == "hbm"), key=lambda k: kernels[k]["total_ms"])

    def roof(k):
        e = kernels[k]
        t = TRAFFIC_PER_REALISATION.get(k)
        return {"kernel": k, "bound": e["bound"], "achieved": e["achieved"], "peak": e["peak"], "unit": e["unit"],
                "frac": e["frac"], "traffic": t * B if t else None,
                "traffic_unit": "bytes per launch (ncu capture at B = 16, scaled per realisation)",
                "peak_source": e["peak_source"]}

    info = dict(plan.info)
    sur = mixed = None
    if rank == 0 and (args.surrogate_points > 0 or args.mixed_channels > 0):
        plan.close()
        plan = None
        del devin, out, scratch
        torch.cuda.empty_cache()
        if args.surrogate_points > 0:
            sur = surrogate_leg(args, dev)
        if args.mixed_channels > 0:
            mixed = mixed_leg(args, dev)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        n_cpu = args.cpu_realisations
        ref = None if args.ref_port else import_stock_reference()
        if ref is not None:
            stock = StockRealisation(ref)
            t0 = time.perf_counter()
            for k in range(n_cpu):
                stock(4242 + k)
            v = n_cpu / (time.perf_counter() - t0)
            cpu = {"value": v, "unit": UNIT, "cores": cores(), "kind": "reference",
                   "sample": f"{n_cpu} realisations of the same 2048^2 channel through the unmodified reference on "
                             "its numpy path (OpenBLAS threads = cores; numpy FFT single-threaded)"}
        else:
            v = cpu_realisations(n_cpu)
            cpu = {"value": v, "unit": UNIT, "cores": cores(), "kind": "port",
                   "sample": f"{n_cpu} realisations of the same 2048^2 channel through the numpy restatement of "
                             "the reference path in its own precision (OpenBLAS threads = cores; numpy FFT "
                             "single-threaded)"}

    if rank == 0:
        def r3(v):
            return None if v is None else float(f"{v:.4g}")

        # standard keys first; the measured extras last, compact, so that the
        # headline ratios sit at the end of the line
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "fp32 (c64 field; fp64 phase args, accumulators)",
            "data": "synthetic (seeded spectra, reference formulas)",
            "config": {"workload": WORKLOAD_NAME, "batch": B,
                       "realisations_per_step": B, "timed_as": "cuda graph replay" if graphs else "direct launches",
                       "direct_ms_per_step": round(direct_ms, 3), "kernels_timed": kernels_timed,
                       "l2": "inputs > L2 (8.6 GB field batch)", "gemm_k": K,
                       "layout": "tiled" if info.get("tiled") else "row-major", "autotune": tuned,
                       "gemm": ["simt", "tc cp.async", "tc tma 128x128", "tc tma 128x256"][info["gemm_form"]]},
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
            "gpu_launches": sum(v["launches"] for v in prof.values()),
            "roofline": roof(dom),
            "clocks": clocks.summary(),
            "cpu_baseline": cpu,
            "roofline_hbm": roof(hbm_dom),
            "kernels": {k: {"ms": r3(e["avg_ms"]), "n": e["launches"], "share": r3(e["share"]),
                            **({"frac": r3(e["frac"]), "bound": e["bound"]} if "frac" in e else {})}
                        for k, e in kernels.items()},
            "mixed": None if mixed is None else {k: r3(mixed[k]) if isinstance(mixed[k], float) else mixed[k]
                                                 for k in ("channels", "realisations_per_channel", "graph_launches",
                                                           "seconds", "channels_per_s", "realisations_per_s",
                                                           "setup_s", "capture_s")
                                                 if k in mixed},
            "surrogate": None if sur is None else dict(
                {k: r3(sur[k]) if isinstance(sur[k], float) else sur[k]
                 for k in ("queries_per_s", "e2e_queries_per_s", "mixed_queries_per_s", "simulated_queries_per_s",
                           "answered_frac", "heldout_answered_frac", "frac_ks_le_0.02", "ks_binned_median",
                           "ks_continuous_median", "all_frac_ks_le_0.02")
                 if k in sur},
                mlp_tflops=r3(sur["mlp"]["tflops"]), mlp_frac_of_bf16_peak=r3(sur["mlp"]["frac_of_bf16_peak"])),
            "plain": {"value": r3(plain), "batched_over_plain": r3(value / world / plain) if plain else None,
                      "torch_reference_algorithm": r3(torch_ref),
                      "batched_over_torch_reference": r3(value / world / torch_ref) if torch_ref else None},
        }
        print(json.dumps(line), flush=True)
    if plan is not None:
        plan.close()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--ref-port", action="store_true",
                    help="reference arm: time the oracle's restatement even where the stock reference is installed")
    ap.add_argument("--batch", type=int, default=256)
    ap.add_argument("--plain", type=int, default=16, help="realisations timed in the plain form (0: skip)")
    ap.add_argument("--seed", type=int, default=2024)
    ap.add_argument("--cpu-realisations", type=int, default=2)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--autotune", type=int, default=1, help="time the FFT-pass launch variants first (atm_autotune)")
    ap.add_argument("--cheb-cut", type=float, default=0.0,
                    help="annuli below cheb_cut / (N delta) go into the Chebyshev block (0: the engine default)")
    ap.add_argument("--graph", type=int, default=1, help="time the batched steps as captured CUDA graphs (0: direct)")
    ap.add_argument("--torch-reference", type=int, default=16,
                    help="realisations of the reference's GPU algorithm restated on torch (0: skip)")
    ap.add_argument("--layout", choices=["auto", "tiled", "rowmajor"], default="auto",
                    help="field layout between the FFT passes (tiled: 4 x 4 blocks of 128 bytes)")
    ap.add_argument("--variants", default="",
                    help="row_variant,col_tile,col_variant set by hand instead of atm_autotune (e.g. 2,4,0)")
    ap.add_argument("--mixed-channels", type=int, default=16,
                    help="channels of the mixed-size workload leg (0: skip)")
    ap.add_argument("--surrogate-points", type=int, default=32,
                    help="held-out points of the surrogate check (0: skip the surrogate leg)")
    ap.add_argument("--gemm", choices=["auto", "tc", "tc256", "tc128", "tc-cpasync", "simt"], default="auto",
                    help="screen GEMM on tensor cores (tc / tc256: persistent TMA form with 128 x 256 tiles, the "
                         "default at 2048^2; tc128: 128 x 128 tiles with double-buffered accumulators; "
                         "tc-cpasync: one CTA per tile) or FP32 SIMT cores")
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "gb300":
        args.warmup = 3
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        return run_reference(args, rank, world)
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local_rank)
        dist.init_process_group("nccl", device_id=torch.device("cuda", local_rank))
    try:
        return run_gb300(args, rank, world, local_rank)
    finally:
        if world > 1:
            import torch.distributed as dist
            dist.destroy_process_group()


if __name__ == "__main__":
    sys.exit(main())
