"""An ensemble of PDT surrogates with an in-range error gate.

K networks of the same shape are trained on bootstrap resamples of the same
simulated points (different initialisations and resamples).  A query is
answered by the members' mean histogram; the members' disagreement -- the
largest bin-edge KS distance between a member's CDF and the mean CDF -- is
the gate's score.  Where the members disagree the network is extrapolating
or the PDT is hard to learn, so a query whose score is above the threshold
goes to the simulator, as do queries outside the training box.

The threshold is calibrated on held-out points with fresh simulations: the
largest score at which at least `target` (0.95) of the answered calibration
points have a bin-edge KS <= 0.02 against their fresh realisations.
"""
from __future__ import annotations

from typing import Dict, List, Optional

import numpy as np
import torch

from .model import (N_HIST, N_MOM, Box, SimConfig, Surrogate, fallback_simulator, features, release_fallback,
                    targets_from_measures)


def disagreement(member_probs: torch.Tensor) -> torch.Tensor:
    """[K][B][64] member histograms -> [B] max over members of the bin-edge KS
    distance to the mean histogram."""
    cdf = torch.cumsum(member_probs, dim=-1)
    mean = cdf.mean(dim=0, keepdim=True)
    return (cdf - mean).abs().amax(dim=-1).amax(dim=0)


def calibrate_threshold(scores: np.ndarray, ks: np.ndarray, gate: float = 0.02, target: float = 0.95) -> float:
    """Largest score threshold whose answered points (score <= threshold)
    meet ks <= gate in at least `target` of cases (0 if none does)."""
    order = np.argsort(scores)
    good = np.cumsum(ks[order] <= gate) / np.arange(1, len(order) + 1)
    ok = np.nonzero(good >= target)[0]
    return float(scores[order][ok[-1]]) if len(ok) else 0.0


class EnsembleSurrogate:
    def __init__(self, members: List[Surrogate], threshold: float = float("inf")):
        if not members:
            raise ValueError("an ensemble needs at least one member")
        self.members = members
        self.box = members[0].box
        self.physics = members[0].physics
        self.device = members[0].device
        self.threshold = float(threshold)

    @classmethod
    def train(cls, box: Box, X: np.ndarray, Y: np.ndarray, k: int = 4, seed: int = 0, **fit_kw):
        members = []
        rng = np.random.default_rng(seed)
        for j in range(k):
            idx = rng.integers(0, len(X), len(X)) if k > 1 else np.arange(len(X))  # bootstrap resample
            s = Surrogate(box, widths=(X.shape[1], 256, 256, 256, N_HIST + N_MOM))
            s.fit(X[idx], Y[idx], seed=seed + 17 * j, **fit_kw)
            members.append(s)
        return cls(members)

    def predict(self, X: torch.Tensor):
        """(mean probabilities [B][64], mean moments [B][3], out_of_range [B], score [B])."""
        probs, moms, oor = [], [], None
        for s in self.members:
            p, m, o = s.predict(X)
            probs.append(p)
            moms.append(m)
            oor = o if oor is None else oor
        P = torch.stack(probs)
        return P.mean(dim=0), torch.stack(moms).mean(dim=0), oor, disagreement(P)

    def answered(self, score: torch.Tensor, oor: torch.Tensor) -> torch.Tensor:
        """Queries the network answers: inside the box and below the gate."""
        return (oor == 0) & (score <= self.threshold)

    def query(self, params: Dict[str, np.ndarray], fallback_cfg: Optional[SimConfig] = None):
        """PDT histograms of parameter points.  Returns (probs [B][64], answered
        [B] bool): answered by the network, the rest simulated (config: N = 1024,
        256 realisations unless given)."""
        X = torch.from_numpy(features(params, self.box, self.physics)).to(self.device)
        probs, _, oor, score = self.predict(X)
        ans = self.answered(score, oor).cpu().numpy()
        probs = probs.cpu().numpy()
        todo = np.nonzero(~ans)[0]
        if len(todo):
            sim = fallback_simulator(self, fallback_cfg or SimConfig(N=1024, realisations=256), self.device)
            for i in todo:
                q = {k: v[i] for k, v in params.items()}
                t, _ = targets_from_measures(sim.run(q, 10_000_000 + int(i)), q["aperture"])
                probs[i] = t[:N_HIST]
        return probs, ans

    def close(self):
        """Frees the fallback simulator's plan (kept across queries)."""
        release_fallback(self)

    # ---------------------------------------------------------------- files
    def save(self, path: str, **extra):
        arrays = {"members": np.array(len(self.members)), "threshold": np.array(self.threshold),
                  "widths": np.array(self.members[0].mlp.widths)}
        for j, s in enumerate(self.members):
            arrays[f"params_{j}"] = s.mlp.get_params()
            arrays[f"mom_mean_{j}"] = s.mom_mean
            arrays[f"mom_std_{j}"] = s.mom_std
        arrays.update(extra)
        np.savez_compressed(path, **arrays)

    @classmethod
    def load(cls, path: str, device=None):
        z = np.load(path)
        widths = tuple(int(w) for w in z["widths"])
        members = []
        for j in range(int(z["members"])):
            s = Surrogate(widths=widths, device=device)
            s.mlp.set_params(z[f"params_{j}"])
            s.mom_mean, s.mom_std = z[f"mom_mean_{j}"], z[f"mom_std_{j}"]
            members.append(s)
        return cls(members, threshold=float(z["threshold"]))
