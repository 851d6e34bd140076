"""Trains the PDT surrogate and measures it against fresh simulations.

    python -m pyatmosphere_gb300.surrogate.experiment --points 4000 --realisations 512 \
        --steps 6000 --holdout 100 --eval-realisations 8192 --out model.npz --report report.json

1. Data: `points` parameter points in the Box, each simulated with
   `realisations` realisations at N = 512 (N delta = 3 m, 5 screens).
2. Training on 90 % of the points (engine MLP kernels, Adam).
3. Held-out evaluation: for `holdout` fresh points the surrogate's CDF is
   compared (KS) with the empirical CDF of `eval-realisations` new
   realisations of that point; the same is done for the methods without
   the network: the nearest training point's histogram and the analytic
   PDT models fitted to the fresh realisations' own moments
   (surrogate/baselines.py).
4. Speed: surrogate queries/s on 100,000 feature vectors against simulated
   queries/s (one point = 256 realisations at N = 1024, the fallback).
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np
import torch

from .baselines import MODELS, analytic_ks
from .model import (N_HIST, Box, PointSimulator, SimConfig, Surrogate, features, ks_binned, ks_hist,
                    targets_from_measures)


def save(s: Surrogate, path: str):
    np.savez_compressed(path, params=s.mlp.get_params(), widths=np.array(s.mlp.widths), mom_mean=s.mom_mean,
                        mom_std=s.mom_std)


def load(path: str, device=None) -> Surrogate:
    z = np.load(path)
    s = Surrogate(widths=tuple(int(w) for w in z["widths"]), device=device)
    s.mlp.set_params(z["params"])
    s.mom_mean, s.mom_std = z["mom_mean"], z["mom_std"]
    return s


def evaluate(s: Surrogate, box: Box, n_points: int, n_real: int, seed: int, train=None, N=512, baselines=True):
    """KS of the surrogate against fresh simulations, beside the methods
    without it: the nearest training point's histogram (given `train`) and
    the analytic PDT models fitted to the fresh realisations' own moments
    (`baselines`)."""
    rng = np.random.default_rng(seed)
    P = box.sample(n_points, rng)
    P["l0"] = np.round(P["l0"] * 1e3) / 1e3
    X = features(P, box, s.physics)
    probs, _, oor = s.predict(torch.from_numpy(X).to(s.device))
    probs = probs.cpu().numpy()
    cfg = SimConfig(N=N, realisations=min(n_real, 2048), seed=seed)
    sim = PointSimulator(cfg, device=s.device)
    ks, ks_nn, kb, kb_nn = [], [], [], []
    kb_an = {name: [] for name in MODELS}
    for i in range(n_points):
        q = {k: v[i] for k, v in P.items()}
        etas, ms = [], []
        for c in range(max(1, n_real // cfg.realisations)):
            m = sim.run(q, 50_000_000 + i * 64 + c)
            _, eta = targets_from_measures(m, q["aperture"])
            etas.append(eta)
            if baselines:
                ms.append(m.detach().cpu().numpy())
        eta = np.concatenate(etas)
        ks.append(ks_hist(probs[i], eta))
        kb.append(ks_binned(probs[i], eta))
        if baselines:
            for name, v in analytic_ks(np.concatenate(ms), q["aperture"], q["w0"], seed=seed + i).items():
                kb_an[name].append(v)
        if train is not None:
            Xt, Yt = train
            j = int(np.argmin(((Xt - X[i]) ** 2).sum(axis=1)))
            ks_nn.append(ks_hist(Yt[j, :N_HIST], eta))
            kb_nn.append(ks_binned(Yt[j, :N_HIST], eta))
    sim.plan.close()
    return {"ks": np.array(ks), "ks_binned": np.array(kb), "ks_nn": np.array(ks_nn), "ks_binned_nn": np.array(kb_nn),
            "ks_binned_analytic": {k: np.array(v) for k, v in kb_an.items()}}


def fresh(box: Box, n_points: int, n_real: int, seed: int, N: int = 512, device=None, moments: bool = False):
    """Fresh simulations of n_points parameter points drawn in the box:
    (params, features-free dict of per-point eta samples, per-point measure
    arrays when `moments`), n_real realisations each at N."""
    rng = np.random.default_rng(seed)
    P = box.sample(n_points, rng)
    P["l0"] = np.round(P["l0"] * 1e3) / 1e3
    cfg = SimConfig(N=N, realisations=min(n_real, 2048), seed=seed)
    sim = PointSimulator(cfg, device=device)
    etas, meas = [], []
    for i in range(n_points):
        q = {k: v[i] for k, v in P.items()}
        e, ms = [], []
        for c in range(max(1, n_real // cfg.realisations)):
            m = sim.run(q, 50_000_000 + i * 64 + c)
            e.append(targets_from_measures(m, q["aperture"])[1])
            if moments:
                ms.append(m.detach().cpu().numpy())
        etas.append(np.concatenate(e))
        if moments:
            meas.append(np.concatenate(ms))
    sim.plan.close()
    return P, etas, meas


def ensemble_experiment(a, box, X, Y, tr):
    """Trains a K-member ensemble, calibrates its error gate on fresh points
    and tests it on other fresh points; returns (ensemble, report dict)."""
    from .ensemble import EnsembleSurrogate, calibrate_threshold
    t0 = time.perf_counter()
    ens = EnsembleSurrogate.train(box, X[tr], Y[tr], k=a.members, seed=a.seed, steps=a.steps, batch=a.batch,
                                  lr=a.lr, weight_decay=a.weight_decay)
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t0

    def scored(n, seed, moments=False):
        P, etas, meas = fresh(box, n, a.eval_realisations, seed, moments=moments)
        Xq = torch.from_numpy(features(P, box, ens.physics)).to(ens.device)
        probs, _, oor, score = ens.predict(Xq)
        probs = probs.cpu().numpy()
        kb = np.array([ks_binned(probs[i], etas[i]) for i in range(n)])
        kc = np.array([ks_hist(probs[i], etas[i]) for i in range(n)])
        return P, etas, meas, probs, score.cpu().numpy(), oor.cpu().numpy(), kb, kc

    _, _, _, _, sc_cal, _, kb_cal, _ = scored(a.calibrate, a.seed + 200)
    ens.threshold = calibrate_threshold(sc_cal, kb_cal, gate=0.02, target=0.95)
    P, etas, meas, probs, sc, oor, kb, kc = scored(a.holdout, a.seed + 100, moments=True)
    ans = (oor == 0) & (sc <= ens.threshold)
    Xt = X[tr]
    Xq = features(P, box, ens.physics)
    nn = np.array([int(np.argmin(((Xt - Xq[i]) ** 2).sum(axis=1))) for i in range(len(Xq))])
    kb_nn = np.array([ks_binned(Y[tr][nn[i], :N_HIST], etas[i]) for i in range(len(Xq))])
    an = {name: [] for name in MODELS}
    for i in range(len(Xq)):
        for name, v in analytic_ks(meas[i], P["aperture"][i], P["w0"][i], seed=a.seed + i).items():
            an[name].append(v)
    rep = {
        "members": a.members, "training_s": t_train, "threshold": ens.threshold,
        "calibration_points": a.calibrate, "test_points": a.holdout, "eval_realisations": a.eval_realisations,
        "answered_frac": float(ans.mean()), "fallback_frac": float(1 - ans.mean()),
        "answered_ks_binned_frac_le_0.02": float((kb[ans] <= 0.02).mean()) if ans.any() else None,
        "answered_ks_binned_median": float(np.median(kb[ans])) if ans.any() else None,
        "answered_ks_continuous_median": float(np.median(kc[ans])) if ans.any() else None,
        "all_ks_binned_median": float(np.median(kb)), "all_ks_binned_frac_le_0.02": float((kb <= 0.02).mean()),
        "all_ks_continuous_median": float(np.median(kc)),
        "nearest_train_ks_binned_median": float(np.median(kb_nn)),
        "analytic": {k: {"median": float(np.median(v)), "frac_le_0.02": float((np.array(v) <= 0.02).mean())}
                     for k, v in an.items()},
        "ks_noise_floor": 0.87 / np.sqrt(a.eval_realisations),
    }
    if a.save_heldout:
        n_g = min(64, len(Xq))
        hist = np.stack([np.histogram(np.clip(etas[i], 0, 1), bins=N_HIST, range=(0, 1))[0] / len(etas[i])
                         for i in range(n_g)]).astype(np.float32)
        eta_m = np.array([[e.mean(), (e ** 2).mean()] for e in etas[:n_g]])
        np.savez_compressed(a.save_heldout, **{k: np.asarray(v[:n_g]) for k, v in P.items()},
                            fresh_hist=hist, fresh_eta_moments=eta_m,
                            nearest_train_hist=Y[tr][nn[:n_g], :N_HIST].astype(np.float32),
                            realisations=a.eval_realisations, seed=a.seed + 100)
    return ens, rep


def analytic_report(ev) -> dict:
    """Median / p90 / fraction <= 0.02 of the bin-edge KS per analytic model."""
    out = {}
    for name, v in ev.get("ks_binned_analytic", {}).items():
        if len(v):
            out[name] = {"median": float(np.median(v)), "p90": float(np.quantile(v, 0.9)),
                         "frac_le_0.02": float((v <= 0.02).mean())}
    return out


def speed(s: Surrogate, box: Box, n_queries=100_000, seed=3):
    rng = np.random.default_rng(seed)
    X = torch.from_numpy(features(box.sample(n_queries, rng), box, s.physics)).to(s.device)
    for _ in range(3):
        s.predict(X)
    torch.cuda.synchronize()
    t = time.perf_counter()
    reps = 10
    for _ in range(reps):
        s.predict(X)
    torch.cuda.synchronize()
    q_per_s = n_queries * reps / (time.perf_counter() - t)
    # simulation per query: the fallback configuration (N = 1024, 256 realisations)
    cfg = SimConfig(N=1024, realisations=256)
    sim = PointSimulator(cfg, device=s.device)
    P = box.sample(4, np.random.default_rng(seed + 1))
    P["l0"][:] = 6e-3
    q0 = {k: v[0] for k, v in P.items()}
    sim.run(q0, 0)
    torch.cuda.synchronize()
    t = time.perf_counter()
    for i in range(1, 4):
        m = sim.run({k: v[i] for k, v in P.items()}, i)
        targets_from_measures(m, P["aperture"][i])
    torch.cuda.synchronize()
    sim_q_per_s = 3 / (time.perf_counter() - t)
    sim.plan.close()
    return q_per_s, sim_q_per_s


def recalibrate(a, box):
    """Re-calibrates a saved ensemble's error gate on `calibrate` fresh points
    (a seed no earlier calibration or test used) and tests it on `holdout`
    other fresh points; the members stay as they are.  Returns the report."""
    from .ensemble import EnsembleSurrogate, calibrate_threshold
    ens = EnsembleSurrogate.load(a.recalibrate, device="cuda")
    old = ens.threshold

    def scored(n, seed):
        P, etas, _ = fresh(box, n, a.eval_realisations, seed)
        Xq = torch.from_numpy(features(P, box, ens.physics)).to(ens.device)
        probs, _, oor, score = ens.predict(Xq)
        probs = probs.cpu().numpy()
        kb = np.array([ks_binned(probs[i], etas[i]) for i in range(n)])
        kc = np.array([ks_hist(probs[i], etas[i]) for i in range(n)])
        return score.cpu().numpy(), oor.cpu().numpy() != 0, kb, kc

    t0 = time.perf_counter()
    sc, oor, kb, _ = scored(a.calibrate, a.seed + 300)
    ens.threshold = calibrate_threshold(sc[~oor], kb[~oor], gate=0.02, target=0.95)
    sc_t, oor_t, kb_t, kc_t = scored(a.holdout, a.seed + 400)
    ans = ~oor_t & (sc_t <= ens.threshold)
    ans_old = ~oor_t & (sc_t <= old)
    members = ens.members
    ens.save(a.out, box_note=np.array("Box() defaults"))
    return {
        "recalibrated": a.recalibrate, "members": len(members), "old_threshold": old, "threshold": ens.threshold,
        "calibration_points": a.calibrate, "calibration_good_frac": float((kb[~oor] <= 0.02).mean()),
        "test_points": a.holdout, "eval_realisations": a.eval_realisations,
        "answered_frac": float(ans.mean()), "answered_frac_old_threshold": float(ans_old.mean()),
        "answered_ks_binned_frac_le_0.02": float((kb_t[ans] <= 0.02).mean()) if ans.any() else None,
        "answered_ks_binned_frac_le_0.02_old_threshold": float((kb_t[ans_old] <= 0.02).mean()) if ans_old.any() else None,
        "answered_ks_binned_median": float(np.median(kb_t[ans])) if ans.any() else None,
        "answered_ks_continuous_median": float(np.median(kc_t[ans])) if ans.any() else None,
        "all_ks_binned_frac_le_0.02": float((kb_t <= 0.02).mean()), "all_ks_binned_median": float(np.median(kb_t)),
        "ks_noise_floor": 0.87 / np.sqrt(a.eval_realisations), "seconds": time.perf_counter() - t0,
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--points", type=int, default=4000)
    ap.add_argument("--realisations", type=int, default=512)
    ap.add_argument("--steps", type=int, default=6000)
    ap.add_argument("--batch", type=int, default=512)
    ap.add_argument("--holdout", type=int, default=100)
    ap.add_argument("--eval-realisations", type=int, default=8192)
    ap.add_argument("--out", default="pdt_mlp.npz")
    ap.add_argument("--report", default="surrogate_report.json")
    ap.add_argument("--seed", type=int, default=11)
    ap.add_argument("--weight-decay", type=float, default=1e-4)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--raw-features", action="store_true", help="the 8 raw inputs only (no physics features)")
    ap.add_argument("--eval-only", default="", help="evaluate this saved model (no data generation or training)")
    ap.add_argument("--save-data", default="", help="also write the generated training set (features, targets) here")
    ap.add_argument("--load-data", default="", help="train on a training set written by --save-data instead of "
                                                     "simulating one (--points and --realisations are taken from it)")
    ap.add_argument("--members", type=int, default=1,
                    help="ensemble members (> 1: bootstrap ensemble with the calibrated in-range error gate)")
    ap.add_argument("--calibrate", type=int, default=200, help="fresh points that calibrate the ensemble's gate")
    ap.add_argument("--save-heldout", default="", help="write up to 64 test points with their fresh histograms "
                                                       "and nearest-training-point histograms here")
    ap.add_argument("--recalibrate", default="",
                    help="re-calibrate this saved ensemble's gate on --calibrate fresh points, test it on "
                         "--holdout others, and write it to --out (no data generation or training)")
    a = ap.parse_args()
    box = Box()
    if a.recalibrate:
        rep = recalibrate(a, box)
        with open(a.report, "w") as f:
            json.dump(rep, f, indent=1)
        print(json.dumps(rep))
        return
    if a.eval_only:
        s = load(a.eval_only)
        t0 = time.perf_counter()
        ev = evaluate(s, box, a.holdout, a.eval_realisations, seed=a.seed + 100)
        kb = ev["ks_binned"]
        rep = {"model": a.eval_only, "holdout_points": a.holdout, "eval_realisations": a.eval_realisations,
               "ks_binned_median": float(np.median(kb)), "ks_binned_p90": float(np.quantile(kb, 0.9)),
               "ks_binned_frac_le_0.02": float((kb <= 0.02).mean()), "ks_median": float(np.median(ev["ks"])),
               "analytic": analytic_report(ev), "ks_noise_floor": 0.87 / np.sqrt(a.eval_realisations),
               "per_point": {"surrogate": kb.tolist(), **{k: v.tolist() for k, v in ev["ks_binned_analytic"].items()}},
               "seconds": time.perf_counter() - t0}
        with open(a.report, "w") as f:
            json.dump(rep, f, indent=1)
        print(json.dumps(rep))
        return
    t0 = time.perf_counter()
    if a.load_data:
        z = np.load(a.load_data)
        X, Y = z["X"], z["Y"]
        a.points, a.realisations, a.seed = int(z["points"]), int(z["realisations"]), int(z["seed"])
    else:
        _, X, Y, _ = Surrogate.generate(box, a.points, SimConfig(realisations=a.realisations), seed=a.seed)
        if a.save_data:
            np.savez_compressed(a.save_data, X=X, Y=Y, points=a.points, realisations=a.realisations, seed=a.seed)
    if a.raw_features:
        X = X[:, :8]
    t_gen = time.perf_counter() - t0
    n_tr = int(0.9 * len(X))
    perm = np.random.default_rng(a.seed).permutation(len(X))
    tr, va = perm[:n_tr], perm[n_tr:]
    if a.members > 1:
        ens, rep = ensemble_experiment(a, box, X, Y, tr)
        ens.save(a.out, box_note=np.array("Box() defaults"))
        rep.update({"points": a.points, "realisations_per_point": a.realisations, "generation_s": t_gen,
                    "data": a.load_data or "simulated"})
        with open(a.report, "w") as f:
            json.dump(rep, f, indent=1)
        print(json.dumps(rep))
        return
    s = Surrogate(box, widths=(X.shape[1], 256, 256, 256, N_HIST + 3))
    t0 = time.perf_counter()
    losses = s.fit(X[tr], Y[tr], steps=a.steps, batch=a.batch, log_every=max(1, a.steps // 20), lr=a.lr,
                   weight_decay=a.weight_decay)
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t0
    save(s, a.out)
    # validation split of the generated data (noisy targets, informative only)
    pv, _, _ = s.predict(torch.from_numpy(X[va]).to(s.device))
    kl_val = float(np.mean(np.sum(np.where(Y[va, :N_HIST] > 0, Y[va, :N_HIST] *
                                          (np.log(np.maximum(Y[va, :N_HIST], 1e-30)) -
                                           np.log(np.maximum(pv.cpu().numpy(), 1e-30))), 0), axis=1)))
    ev = evaluate(s, box, a.holdout, a.eval_realisations, seed=a.seed + 100, train=(X[tr], Y[tr]))
    ks, ks_nn, kb, kb_nn = ev["ks"], ev["ks_nn"], ev["ks_binned"], ev["ks_binned_nn"]
    q_s, sim_q_s = speed(s, box)
    rep = {
        "points": a.points, "realisations_per_point": a.realisations, "train_points": n_tr,
        "data": a.load_data or "simulated", "generation_s": t_gen, "training_s": t_train, "steps": a.steps, "loss_curve": losses,
        "val_kl": kl_val, "holdout_points": a.holdout, "eval_realisations": a.eval_realisations,
        "ks_mean": float(ks.mean()), "ks_median": float(np.median(ks)), "ks_p90": float(np.quantile(ks, 0.9)),
        "ks_frac_le_0.02": float((ks <= 0.02).mean()),
        "ks_nearest_train_mean": float(ks_nn.mean()), "ks_nearest_train_median": float(np.median(ks_nn)),
        "ks_binned_mean": float(kb.mean()), "ks_binned_median": float(np.median(kb)),
        "ks_binned_frac_le_0.02": float((kb <= 0.02).mean()), "ks_binned_p90": float(np.quantile(kb, 0.9)),
        "ks_binned_nearest_train_mean": float(kb_nn.mean()), "ks_binned_nearest_train_median": float(np.median(kb_nn)),
        "ks_noise_floor": 0.87 / np.sqrt(a.eval_realisations), "analytic": analytic_report(ev),
        "queries_per_s": q_s, "simulated_queries_per_s": sim_q_s, "speedup": q_s / sim_q_s,
    }
    with open(a.report, "w") as f:
        json.dump(rep, f, indent=1)
    print(json.dumps({k: v for k, v in rep.items() if k != "loss_curve"}))


if __name__ == "__main__":
    main()
