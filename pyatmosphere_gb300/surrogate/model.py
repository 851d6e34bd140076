"""Learned PDT surrogate: channel parameters -> probability distribution of
transmittance (64-bin histogram on [0, 1]) + mean transmittance, beam
wandering variance and long-term beam width.

* Data: parameter points drawn in a box (Cn2, L, w0, wvl, F0, aperture, l0,
  L0), each simulated with the batched engine (one plan re-targeted per
  point with atm_plan_update, seeded spectra drawn on the device).
* Model: MLP 8 -> 256 -> 256 -> 256 -> 67 (GELU), BF16 weights, FP32
  accumulation, Adam; loss = KL on the histogram + MSE on the moments; all
  trained by the engine's own kernels (atm_mlp_*).
* Queries: in-box inputs are answered by the network; out-of-box inputs fall
  back to the simulator.
"""
from __future__ import annotations

import math
import time
from dataclasses import dataclass, field
from typing import Dict, List, Optional

import numpy as np
import torch

from ..engine.plan import EnginePlan
from ..engine.spectra import annulus_psd
from ..theory.models import MVKModel
from .mlp import EngineMLP

N_HIST = 64
N_MOM = 3
FEATURES = ["log10_Cn2", "log10_L", "w0", "wvl_um", "L_over_F0", "aperture", "l0_mm", "log10_L0",
            "log10_rytov", "log10_a_over_W", "log10_a_over_W_LT", "log10_Lambda"]


@dataclass
class Box:
    """Training domain (physical units)."""
    Cn2: tuple = (1e-16, 1e-14)
    L: tuple = (1e3, 2e4)
    w0: tuple = (0.03, 0.15)
    wvl: tuple = (808e-9, 1550e-9)      # two values
    aperture: tuple = (0.05, 0.25)
    l0: tuple = (3e-3, 1e-2)
    L0: tuple = (100.0, 1000.0)

    def features_lo_hi(self):
        lo = np.array([math.log10(self.Cn2[0]), math.log10(self.L[0]), self.w0[0], self.wvl[0] * 1e6, 0.0,
                       self.aperture[0], self.l0[0] * 1e3, math.log10(self.L0[0])], np.float32)
        hi = np.array([math.log10(self.Cn2[1]), math.log10(self.L[1]), self.w0[1], self.wvl[1] * 1e6, 1.0,
                       self.aperture[1], self.l0[1] * 1e3, math.log10(self.L0[1])], np.float32)
        return lo, hi

    def sample(self, n, rng):
        lu = lambda a, b: np.exp(rng.uniform(np.log(a), np.log(b), n))
        return {
            "Cn2": lu(*self.Cn2), "L": lu(*self.L), "w0": rng.uniform(*self.w0, n),
            "wvl": rng.choice(np.array(self.wvl), n), "focused": rng.integers(0, 2, n).astype(float),
            "aperture": rng.uniform(*self.aperture, n), "l0": rng.uniform(*self.l0, n), "L0": lu(*self.L0),
        }


N_RAW = 8
N_PHYS = 4


def physics_features(p: Dict[str, np.ndarray]) -> np.ndarray:
    """Analytic combinations of the raw parameters that the PDT depends on
    smoothly (weak-to-strong turbulence theory of a Gaussian beam):
    plane-wave Rytov variance sigma_R^2 = 1.23 Cn2 k^(7/6) L^(11/6), the
    vacuum beam radius at the receiver W = w0 sqrt(Theta0^2 + Lambda0^2)
    (Theta0 = 1 - L/F0, Lambda0 = 2 L / (k w0^2)), a long-term radius
    W_LT = W sqrt(1 + 1.33 sigma_R^2 Lambda^(5/6)) with the receiver-plane
    Fresnel ratio Lambda = Lambda0 / (Theta0^2 + Lambda0^2), and the aperture
    radius over both radii; each log10 mapped to about [0, 1] over the box."""
    k = 2 * np.pi / p["wvl"]
    L, w0, a = p["L"], p["w0"], p["aperture"]
    theta0 = 1.0 - np.asarray(p["focused"], dtype=np.float64)   # F0 = L when focused, else infinity
    lam0 = 2 * L / (k * w0 ** 2)
    W = w0 * np.sqrt(theta0 ** 2 + lam0 ** 2)
    lam = lam0 / (theta0 ** 2 + lam0 ** 2)
    sr2 = 1.23 * p["Cn2"] * k ** (7 / 6) * L ** (11 / 6)
    wlt = W * np.sqrt(1 + 1.33 * sr2 * lam ** (5 / 6))
    return np.stack([(np.log10(sr2) + 3) / 5, (np.log10(a / W) + 2) / 3, (np.log10(a / wlt) + 2) / 3,
                     (np.log10(lam) + 3) / 4], axis=1)


def features(p: Dict[str, np.ndarray], box: Box, physics: bool = True) -> np.ndarray:
    """Raw features scaled to [0, 1] over the box (outside the box: outside
    [0, 1]), followed by the physics features when `physics`."""
    raw = np.stack([np.log10(p["Cn2"]), np.log10(p["L"]), p["w0"], p["wvl"] * 1e6, p["focused"], p["aperture"],
                    p["l0"] * 1e3, np.log10(p["L0"])], axis=1).astype(np.float64)
    lo, hi = box.features_lo_hi()
    X = (raw - lo) / np.where(hi > lo, hi - lo, 1.0)
    if physics:
        X = np.concatenate([X, physics_features(p)], axis=1)
    return X.astype(np.float32)


@dataclass
class SimConfig:
    N: int = 512
    extent: float = 3.0      # N delta
    n_screens: int = 5
    points: int = 1024
    realisations: int = 256
    seed: int = 77


class PointSimulator:
    """Runs the batched engine for one parameter point at a time."""

    def __init__(self, cfg: SimConfig, device=None):
        self.cfg = cfg
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        self.delta = cfg.extent / cfg.N
        self.f_min = 1 / 1e3 / 15
        self.plan = None
        self.sq = torch.empty((cfg.n_screens, cfg.points), dtype=torch.float32, device=self.device)
        B, n, P = cfg.realisations, cfg.n_screens, cfg.points
        self.rho = torch.empty((B, n, P), dtype=torch.float32, device=self.device)
        self.theta = torch.empty_like(self.rho)
        self.value = torch.empty((B, n, P), dtype=torch.complex64, device=self.device)
        self.out = None
        self._base_key = None
        self._variants = None  # launch forms atm_autotune picked for this size and batch (l0 does not change them)

    def _geometry(self, q):
        cfg = self.cfg
        L = float(q["L"])
        pos = (np.arange(cfg.n_screens) + 0.5) * (L / cfg.n_screens)
        F0 = L if q["focused"] > 0.5 else math.inf
        base = np.exp(np.linspace(np.log(self.f_min), np.log(2 / q["l0"]), cfg.points, dtype=np.float32))
        return L, pos, F0, base

    def run(self, q, index: int) -> np.ndarray:
        """(realisations, n_out) engine measures for point q."""
        import ctypes
        from ..engine import _lib
        cfg = self.cfg
        L, pos, F0, base = self._geometry(q)
        key = base.tobytes()
        kw = dict(f_base=base, pupils=[(float(q["aperture"]),)], batch=cfg.realisations, device=self.device)
        if self.plan is None or key != self._base_key:
            # l0 sets the spectral grid: a new plan when it changes
            if self.plan is not None:
                self.plan.close()
            self.plan = EnginePlan(cfg.N, self.delta, float(q["wvl"]), float(q["w0"]), F0, pos, L, **kw)
            self._base_key = key
            # the FFT-pass launch forms: tuned once, then reused by the plans of later spectral grids
            if self._variants is None:
                t = self.plan.autotune(repeats=2)
                self._variants = (t["row_variant"], t["col_tile"], t["col_variant"])
            else:
                self.plan.set_variants(*self._variants)
        else:
            self.plan.update(float(q["wvl"]), float(q["w0"]), F0, pos, L, pupils=[(float(q["aperture"]),)])
        model = MVKModel(Cn2=float(q["Cn2"]), l0=float(q["l0"]), L0=float(q["L0"]))
        psd = annulus_psd(base, model.psd_phi_f, 2 * np.pi / float(q["wvl"]), L / cfg.n_screens)
        self.sq.copy_(torch.from_numpy(np.sqrt(psd)).to(self.device).expand(cfg.n_screens, -1))
        self.plan.draw_spectra(cfg.seed, index * cfg.realisations, self.sq, self.rho, self.theta, self.value)
        return self.plan.run(self.rho, self.theta, self.value)


def fallback_simulator(owner, cfg: SimConfig, device) -> PointSimulator:
    """The point simulator of `owner` (a surrogate) for this configuration,
    kept across queries: its plan, workspace and tuned launch forms are built
    once, not per query batch.  release_fallback(owner) frees them."""
    sims = owner.__dict__.setdefault("_fallback_sims", {})
    key = (tuple(sorted(vars(cfg).items())), str(device))
    if key not in sims:
        sims[key] = PointSimulator(cfg, device=device)
    return sims[key]


def release_fallback(owner):
    """Frees the point simulators `owner` keeps (their plans' device memory)."""
    for sim in owner.__dict__.pop("_fallback_sims", {}).values():
        if sim.plan is not None:
            sim.plan.close()
            sim.plan = None


def targets_from_measures(m: torch.Tensor, aperture: float) -> np.ndarray:
    """(64 histogram probabilities, mean eta, log10 beam-wandering variance,
    log10 long-term width) of one point's realisations."""
    from ..engine import _lib
    m = m.detach().cpu().numpy()
    eta = np.clip(m[:, _lib.OUT_PUPIL0], 0.0, 1.0)
    hist = np.histogram(eta, bins=N_HIST, range=(0.0, 1.0))[0].astype(np.float64)
    hist /= max(1.0, hist.sum())
    bw2 = np.mean(m[:, _lib.OUT_MEAN_X] ** 2 + m[:, _lib.OUT_MEAN_Y] ** 2)
    lt = np.sqrt(np.mean(2 * (m[:, _lib.OUT_MEAN_X2] + m[:, _lib.OUT_MEAN_Y2])))
    return np.concatenate([hist, [eta.mean(), np.log10(bw2 + 1e-12), np.log10(lt + 1e-12)]]).astype(np.float32), eta


def ks_binned(probs: np.ndarray, samples: np.ndarray) -> float:
    """KS distance at the histogram's own resolution: the two CDFs compared at
    the 65 bin edges on [0, 1]."""
    emp = np.histogram(np.clip(samples, 0, 1), bins=N_HIST, range=(0.0, 1.0))[0] / max(1, len(samples))
    return float(np.max(np.abs(np.cumsum(probs) - np.cumsum(emp))))


def ks_hist(probs: np.ndarray, samples: np.ndarray) -> float:
    """Kolmogorov-Smirnov distance between a 64-bin histogram on [0, 1]
    (CDF linear inside bins) and the empirical CDF of samples."""
    s = np.sort(np.clip(samples, 0, 1))
    cdf_edges = np.concatenate([[0.0], np.cumsum(probs)])
    edges = np.linspace(0, 1, N_HIST + 1)
    F = np.interp(s, edges, cdf_edges)
    n = len(s)
    emp_hi = np.arange(1, n + 1) / n
    emp_lo = np.arange(0, n) / n
    return float(max(np.max(np.abs(F - emp_hi)), np.max(np.abs(F - emp_lo))))


class Surrogate:
    """MLP surrogate of the PDT with simulator fallback outside its box."""

    def __init__(self, box: Optional[Box] = None, widths=None, device=None, max_batch=4096):
        self.box = box or Box()
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        widths = tuple(widths) if widths is not None else (N_RAW + N_PHYS, 256, 256, 256, N_HIST + N_MOM)
        if widths[0] not in (N_RAW, N_RAW + N_PHYS):
            raise ValueError(f"input width {widths[0]} is neither {N_RAW} nor {N_RAW + N_PHYS}")
        self.physics = widths[0] == N_RAW + N_PHYS
        self.mlp = EngineMLP(widths, max_batch=max_batch, device=self.device)
        self.mom_mean = np.zeros(N_MOM, np.float32)
        self.mom_std = np.ones(N_MOM, np.float32)
        # the box in feature space, with a margin for float32 rounding of the edges; the
        # physics features follow from the raw ones and are not range-checked
        lo = np.full(widths[0], -1e30, np.float32)
        hi = np.full(widths[0], 1e30, np.float32)
        lo[:N_RAW], hi[:N_RAW] = -1e-3, 1 + 1e-3
        self.lo = torch.from_numpy(lo).to(self.device)
        self.hi = torch.from_numpy(hi).to(self.device)

    # ---------------------------------------------------------------- data
    @staticmethod
    def generate(box: Box, n_points: int, cfg: SimConfig, seed=0, device=None, keep_samples=False):
        rng = np.random.default_rng(seed)
        P = box.sample(n_points, rng)
        # group by l0 bins so the spectral grid (and the plan) is reused
        P["l0"] = np.round(P["l0"] * 1e3) / 1e3
        order = np.argsort(P["l0"], kind="stable")
        P = {k: v[order] for k, v in P.items()}
        sim = PointSimulator(cfg, device=device)
        Y = np.empty((n_points, N_HIST + N_MOM), np.float32)
        samples = [] if keep_samples else None
        for i in range(n_points):
            q = {k: v[i] for k, v in P.items()}
            t, eta = targets_from_measures(sim.run(q, seed * 1_000_000 + i), q["aperture"])
            Y[i] = t
            if keep_samples:
                samples.append(eta)
        sim.plan.close()
        return P, features(P, box), Y, samples

    # --------------------------------------------------------------- train
    def fit(self, X: np.ndarray, Y: np.ndarray, steps=3000, batch=512, lr=1e-3, w_mse=1.0, seed=0, log_every=0,
            weight_decay=0.0):
        self.mom_mean = Y[:, N_HIST:].mean(axis=0)
        self.mom_std = Y[:, N_HIST:].std(axis=0) + 1e-6
        Yn = Y.copy()
        Yn[:, N_HIST:] = (Y[:, N_HIST:] - self.mom_mean) / self.mom_std
        Xd = torch.from_numpy(np.ascontiguousarray(X)).to(self.device)
        Yd = torch.from_numpy(np.ascontiguousarray(Yn)).to(self.device)
        self.mlp.init_params(seed)
        g = torch.Generator(device=self.device)
        g.manual_seed(seed)
        losses = []
        n = X.shape[0]
        batch = min(batch, n, self.mlp.max_batch)
        for s in range(steps):
            idx = torch.randint(0, n, (batch,), device=self.device, generator=g)
            xb = Xd.index_select(0, idx).contiguous()
            yb = Yd.index_select(0, idx).contiguous()
            self.mlp.forward(xb)
            loss = self.mlp.loss_backward(yb, N_HIST, w_mse)
            self.mlp.adam(lr=lr * (0.5 * (1 + math.cos(math.pi * s / steps))) + 1e-5, weight_decay=weight_decay)
            if log_every and s % log_every == 0:
                losses.append(float(loss.item()))
        return losses

    # --------------------------------------------------------------- query
    def predict(self, X: torch.Tensor):
        """(probabilities [B][64], moments [B][3] in physical form, out_of_range [B])."""
        y, oor = self.mlp.infer(X, self.lo, self.hi, N_HIST)
        mom = y[:, N_HIST:] * torch.from_numpy(self.mom_std).to(self.device) + \
            torch.from_numpy(self.mom_mean).to(self.device)
        return y[:, :N_HIST], mom, oor

    def query(self, params: Dict[str, np.ndarray], fallback_cfg: Optional[SimConfig] = None):
        """PDT histograms for parameter points; out-of-box points are simulated."""
        X = torch.from_numpy(features(params, self.box, self.physics)).to(self.device)
        probs, mom, oor = self.predict(X)
        probs = probs.cpu().numpy()
        oor = oor.cpu().numpy().astype(bool)
        n_fb = int(oor.sum())
        if n_fb:
            sim = fallback_simulator(self, fallback_cfg or SimConfig(N=1024, realisations=256), self.device)
            for i in np.nonzero(oor)[0]:
                q = {k: v[i] for k, v in params.items()}
                t, _ = targets_from_measures(sim.run(q, 10_000_000 + int(i)), q["aperture"])
                probs[i] = t[:N_HIST]
        return probs, oor
