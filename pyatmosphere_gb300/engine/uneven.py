"""Uneven workloads: many channels of mixed grid size, screen count and
geometry, each with its own realisations and its own PDT histogram.

The reference runs such a mix as one Channel + Simulation per parameter
point (channels.py:17-44, simulations/simulation.py:89-138, PDTResult in
simulations/pdt.py:11-26).  Here the channels are grouped by grid size N; a
group gets one plan sized for its largest screen count, re-targeted
(atm_plan_update) channel by channel, largest N first so that device memory
peaks once.  Spectra are drawn on the device (Philox keyed by the channel's
index), so per channel only the measures leave the GPU.
"""
from __future__ import annotations

import math
import time
from dataclasses import dataclass, field
from typing import Dict, List, Optional, Sequence

import numpy as np
import torch

from . import _lib
from .plan import EnginePlan
from .spectra import annulus_psd


@dataclass
class ChannelParams:
    """One channel of a mixed workload (a Gaussian beam through `n_screens`
    SS screens placed in the middle of equal slabs)."""
    N: int
    n_screens: int
    length: float
    Cn2: float
    w0: float
    wvl: float
    focused: bool = False
    extent: float = 3.0          # N delta [m]
    l0: float = 6e-3
    L0: float = 1e3
    pupil_radius: float = 0.1
    points: int = 1024
    f_min: float = 1.0 / 15000.0

    @property
    def delta(self) -> float:
        return self.extent / self.N

    @property
    def F0(self) -> float:
        return self.length if self.focused else math.inf

    def positions(self) -> np.ndarray:
        # IdenticalPhaseScreensPath(position_in_slab="middle"), pathes.py:105-118
        return (np.arange(self.n_screens) + 0.5) * (self.length / self.n_screens)

    def base(self) -> np.ndarray:
        # RandLogPolarGrid.base, grids.py:94-99
        return np.exp(np.linspace(np.log(self.f_min), np.log(2.0 / self.l0), self.points)).astype(np.float32)

    def sqrt_psd(self) -> np.ndarray:
        from ..theory.models import MVKModel
        model = MVKModel(Cn2=self.Cn2, l0=self.l0, L0=self.L0)
        k = 2 * np.pi / self.wvl
        return np.sqrt(annulus_psd(self.base(), model.psd_phi_f, k, self.length / self.n_screens))


def sample_mixed(n_channels: int, rng: np.random.Generator, sizes=(512, 1024, 2048, 4096),
                 screens=(3, 20), length=(1e3, 1e5), Cn2=(1e-16, 1e-14), w0=(0.02, 0.2),
                 wvl=(808e-9, 1550e-9), **fixed) -> List[ChannelParams]:
    """Channels drawn like the mixed workload: N uniform over `sizes`
    (N delta = 3 m), screen count uniform on the closed range, L and Cn2
    log-uniform, w0 uniform, wavelength one of two, F0 either infinity or L.
    l0 = 6 mm, L0 = 1 km and a 0.1 m pupil unless given in `fixed`."""
    lu = lambda a, b: float(np.exp(rng.uniform(np.log(a), np.log(b))))
    out = []
    for _ in range(n_channels):
        out.append(ChannelParams(N=int(rng.choice(np.asarray(sizes))), n_screens=int(rng.integers(screens[0], screens[1] + 1)),
                                 length=lu(*length), Cn2=lu(*Cn2), w0=float(rng.uniform(*w0)),
                                 wvl=float(rng.choice(np.asarray(wvl))), focused=bool(rng.integers(0, 2)), **fixed))
    return out


@dataclass
class UnevenResult:
    pdt: np.ndarray                      # [channels][bins] probabilities of eta on [0, 1]
    eta_mean: np.ndarray                 # [channels]
    measures: Optional[List[np.ndarray]]  # per channel [realisations][n_out] (keep_measures)
    seconds: float
    realisations: int
    groups: Dict[int, dict] = field(default_factory=dict)

    @property
    def channels_per_s(self) -> float:
        return len(self.pdt) / self.seconds

    @property
    def realisations_per_s(self) -> float:
        return len(self.pdt) * self.realisations / self.seconds


def _group_key(c: ChannelParams):
    # a plan is shared by channels of one grid, spectral grid and pupil count
    return (c.N, c.extent, c.points, c.l0, c.f_min)


def run_uneven(channels: Sequence[ChannelParams], realisations: int = 64, seed: int = 0, bins: int = 64,
               device=None, keep_measures: bool = False, autotune: bool = False) -> UnevenResult:
    """Runs every channel with `realisations` realisations (spectra drawn on
    the device from (seed, channel index)) and returns each channel's PDT
    histogram.  Channel c's realisation r uses Philox counter c * realisations
    + r, so a channel's result does not depend on the rest of the mix."""
    dev = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
    C = len(channels)
    pdt = np.zeros((C, bins))
    eta_mean = np.zeros(C)
    kept: List[Optional[np.ndarray]] = [None] * C
    groups: Dict[tuple, List[int]] = {}
    for i, c in enumerate(channels):
        groups.setdefault(_group_key(c), []).append(i)
    info = {}
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    for key in sorted(groups, key=lambda k: -k[0]):
        idx = groups[key]
        n_max = max(channels[i].n_screens for i in idx)
        first = channels[idx[0]]
        P = first.points
        base = first.base()
        rho_buf = torch.empty(realisations * n_max * P, dtype=torch.float32, device=dev)
        theta_buf = torch.empty_like(rho_buf)
        value_buf = torch.empty(realisations * n_max * P, dtype=torch.complex64, device=dev)
        sq_buf = torch.empty(n_max * P, dtype=torch.float32, device=dev)
        # the plan is created for the largest screen count of the group
        c_max = max((channels[i] for i in idx), key=lambda c: c.n_screens)
        plan = EnginePlan(c_max.N, c_max.delta, c_max.wvl, c_max.w0, c_max.F0, c_max.positions(), c_max.length,
                          f_base=base, pupils=[(c_max.pupil_radius,)], batch=realisations, device=dev)
        if autotune:
            plan.autotune(repeats=2)
        out = torch.empty((realisations, plan.n_out), dtype=torch.float64, device=dev)
        tg = time.perf_counter()
        for i in sorted(idx, key=lambda j: -channels[j].n_screens):
            c = channels[i]
            n = c.n_screens
            plan.update(c.wvl, c.w0, c.F0, c.positions(), c.length, pupils=[(c.pupil_radius,)])
            rho = rho_buf[:realisations * n * P].view(realisations, n, P)
            theta = theta_buf[:realisations * n * P].view(realisations, n, P)
            value = value_buf[:realisations * n * P].view(realisations, n, P)
            sq = sq_buf[:n * P].view(n, P)
            sq.copy_(torch.from_numpy(c.sqrt_psd()).to(dev).expand(n, -1))
            plan.draw_spectra(seed, i * realisations, sq, rho, theta, value)
            plan.run(rho, theta, value, out=out)
            eta = out[:, _lib.OUT_PUPIL0].clamp(0.0, 1.0)
            h = torch.histc(eta, bins=bins, min=0.0, max=1.0)
            pdt[i] = (h / realisations).cpu().numpy()
            eta_mean[i] = float(eta.mean())
            if keep_measures:
                kept[i] = out.cpu().numpy().copy()
        torch.cuda.synchronize(dev)
        info[key[0]] = {"channels": len(idx), "max_screens": n_max, "seconds": time.perf_counter() - tg,
                        "tuned": {k: plan.info[k] for k in ("col_tile", "row_variant", "col_variant")}}
        plan.close()
        del rho_buf, theta_buf, value_buf
    torch.cuda.synchronize(dev)
    return UnevenResult(pdt=pdt, eta_mean=eta_mean, measures=kept if keep_measures else None,
                        seconds=time.perf_counter() - t0, realisations=realisations, groups=info)


def run_uneven_graph(channels: Sequence[ChannelParams], realisations: int = 64, seed: int = 0, bins: int = 64,
                     device=None, keep_measures: bool = False, autotune: bool = False) -> UnevenResult:
    """The mixed workload as ONE CUDA graph launch.

    Set-up (outside the timed launch): per grid-size group one plan sized for
    the group's largest screen count (tuned by atm_autotune when asked), one
    channel table set per channel (atm_channel_create: source, geometry and
    transfer tables built once), the channels' sqrt(PSD) rows on the device.
    Capture: per group one stream, forked from the capturing stream; on it,
    per channel, the device spectrum draw and atm_run_channel into the
    channel's slice of one measures array; the streams join at the end.  The
    graph is instantiated once and launched once for the whole mix; the
    groups' branches run concurrently on the GPU.  Channel c's realisation r
    uses Philox counter c * realisations + r, as in run_uneven, so every
    channel gives the bits of run_uneven and of a fresh plan with the same
    launch forms."""
    dev = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
    C, R = len(channels), int(realisations)
    groups: Dict[tuple, List[int]] = {}
    for i, c in enumerate(channels):
        groups.setdefault(_group_key(c), []).append(i)
    t_setup = time.perf_counter()
    state = []
    n_out = None
    for key in sorted(groups, key=lambda k: -k[0]):
        idx = groups[key]
        c_max = max((channels[i] for i in idx), key=lambda c: c.n_screens)
        n_max, P = c_max.n_screens, c_max.points
        plan = EnginePlan(c_max.N, c_max.delta, c_max.wvl, c_max.w0, c_max.F0, c_max.positions(), c_max.length,
                          f_base=c_max.base(), pupils=[(c_max.pupil_radius,)], batch=R, device=dev)
        if autotune:
            plan.autotune(repeats=2)
        n_out = plan.n_out if n_out is None else n_out
        chans = {i: plan.channel(channels[i].wvl, channels[i].w0, channels[i].F0, channels[i].positions(),
                                 channels[i].length, pupils=[(channels[i].pupil_radius,)]) for i in idx}
        sq = {i: torch.from_numpy(channels[i].sqrt_psd()).to(dev).expand(channels[i].n_screens, -1).contiguous()
              for i in idx}
        buf = {"rho": torch.empty(R * n_max * P, dtype=torch.float32, device=dev)}
        buf["theta"] = torch.empty_like(buf["rho"])
        buf["value"] = torch.empty(R * n_max * P, dtype=torch.complex64, device=dev)
        state.append((key, idx, plan, chans, sq, buf, P))
    out_all = torch.empty((C, R, n_out), dtype=torch.float64, device=dev)

    def launch_group(idx, plan, chans, sq, buf, P):
        for i in sorted(idx, key=lambda j: -channels[j].n_screens):
            n = channels[i].n_screens
            rho = buf["rho"][:R * n * P].view(R, n, P)
            theta = buf["theta"][:R * n * P].view(R, n, P)
            value = buf["value"][:R * n * P].view(R, n, P)
            plan.draw_spectra(seed, i * R, sq[i], rho, theta, value, channel=chans[i])
            plan.run_channel(chans[i], rho, theta, value, out=out_all[i])

    # warm-up outside the capture: the engine's per-device launch settings get cached
    side = torch.cuda.Stream(device=dev)
    side.wait_stream(torch.cuda.current_stream(dev))
    with torch.cuda.stream(side):
        for key, idx, plan, chans, sq, buf, P in state:
            launch_group(idx[:1], plan, chans, sq, buf, P)
    torch.cuda.synchronize(dev)
    t_capture = time.perf_counter()
    streams = [torch.cuda.Stream(device=dev) for _ in state]
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph, stream=side):
        for s, (key, idx, plan, chans, sq, buf, P) in zip(streams, state):
            s.wait_stream(side)
            with torch.cuda.stream(s):
                launch_group(idx, plan, chans, sq, buf, P)
        for s in streams:
            side.wait_stream(s)
    torch.cuda.synchronize(dev)
    t_ready = time.perf_counter()
    # graph.replay() launches on the current stream: time it there
    cur = torch.cuda.current_stream(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(cur)
    graph.replay()
    e1.record(cur)
    torch.cuda.synchronize(dev)
    seconds = e0.elapsed_time(e1) * 1e-3
    for key, idx, plan, chans, sq, buf, P in state:
        plan.check()
    eta = out_all[:, :, _lib.OUT_PUPIL0].clamp(0.0, 1.0)
    cell = torch.clamp((eta * bins).floor(), max=bins - 1).long()
    counts = torch.zeros((C, bins), dtype=torch.float64, device=dev).scatter_add_(1, cell, torch.ones_like(eta))
    pdt = (counts / R).cpu().numpy()
    eta_mean = eta.mean(dim=1).cpu().numpy()
    kept = [m for m in out_all.cpu().numpy()] if keep_measures else None
    info = {key[0]: {"channels": len(idx), "max_screens": max(channels[i].n_screens for i in idx),
                     "tuned": {k: plan.info[k] for k in ("col_tile", "row_variant", "col_variant")}}
            for key, idx, plan, chans, sq, buf, P in state}
    info["graph"] = {"setup_s": t_capture - t_setup, "capture_s": t_ready - t_capture, "launches": 1}
    del graph
    for key, idx, plan, chans, sq, buf, P in state:
        for ch in chans.values():
            ch.close()
        plan.close()
    return UnevenResult(pdt=pdt, eta_mean=eta_mean, measures=kept, seconds=seconds, realisations=R, groups=info)
