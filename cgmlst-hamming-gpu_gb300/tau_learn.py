"""Training data and training of the learned tau and schedule model.

    python -m tau_learn sweep  [--datasets 200] [--out tau_sweep_gb300.npz]
    python -m tau_learn train  [--sweep tau_sweep_gb300.npz] [--out tau_mlp_gb300.f32]
    python -m tau_learn cv     [--sweep tau_sweep_gb300.npz] [--out tau_cv_gb300.json]

(run from this directory, or ``python cgmlst-hamming-gpu_gb300/tau_learn.py``).

sweep: seeded synthetic profile sets of varied shape (n log-uniform in
[50, 63 005], L from the shapes the configs name, n x L <= 7.2e7): 60 % Zipf
(s in [1.0, 1.4], lognormal distinct-allele counts, 5 % 64-bit ids), 20 %
founder models (3-60 alleles per locus, 0.2-5 % mutations to new ids), 20 % the
batched config's law (n <= 5 000); 0-8 % missing.  For each set
the library's own candidate rows (tch_tau_features: tau x sub-stripe rows x
raster group) and, for each candidate whose tau is near the analytic pick, the
measured device time of one whole-triangle solve under that schedule (rare
counts + tile pass, CUDA events, median of 3).

train: the MLP of csrc/k_mlp.cu on ln(ms), trained on the GPU by the library's
kernels (tch_mlp_train), every fifth profile set held out and the longer sets'
candidates repeated in the training rows (oversample).  Feature
standardisation is folded into the first layer, so the saved model takes the
raw feature rows.  The report compares, on the held-out sets, the measured time
at the learned pick (tau and schedule), at the analytic pick (its tau, the
default schedule) and at the best swept candidate.

cv: the same recipe five times, each fifth of the sets held out once: the
learned picks of all 480 sets against the analytic picks (a single fifth's
total is decided by its two or three longest sets).
"""
from __future__ import annotations

import argparse
import importlib
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
tch = importlib.import_module("cgmlst-hamming-gpu_gb300")
synth = importlib.import_module("cgmlst-hamming-gpu_gb300.synth")

SWEEP_PATH = os.path.join(HERE, "tau_sweep_gb300.npz")
REPORT_PATH = os.path.join(HERE, "tau_mlp_gb300.json")
CV_PATH = os.path.join(HERE, "tau_cv_gb300.json")
LOCI = (500, 1142, 1343, 2000, 2794, 3016)


def dataset_params(seed: int) -> dict:
    """Shape and allele law of profile set `seed`."""
    rng = np.random.default_rng(1000 + seed)
    n = int(np.exp(rng.uniform(np.log(50), np.log(63005))))
    L = int(rng.choice(LOCI))
    while n * L > 7.2e7:
        L = int(rng.choice(LOCI[:3]))
        if n * L > 7.2e7:
            n = int(7.2e7 / L)
    p = dict(seed=seed, n=n, L=L, miss=float(rng.uniform(0.0, 0.08)))
    kind = rng.random()
    if kind < 0.2:  # the batched config's law: Zipf over lognormal(40) distinct ids, n up to 5 000
        p.update(kind="batch", n=min(n, 5000), L=int(rng.choice(LOCI[1:])), s=float(rng.uniform(1.0, 1.4)))
    elif kind < 0.4:
        p.update(kind="founders", founders=int(rng.integers(3, 60)), mut=float(np.exp(rng.uniform(np.log(0.002),
                                                                                                 np.log(0.05)))))
    else:
        p.update(kind="zipf", s=float(rng.uniform(1.0, 1.4)), median=float(np.exp(rng.uniform(np.log(15), np.log(150)))),
                 sigma=float(rng.uniform(0.8, 1.4)))
    return p


def make_dataset(p: dict) -> np.ndarray:
    if p.get("kind") == "batch":
        rng = np.random.default_rng(p["seed"])
        n, L = p["n"], p["L"]
        k = np.clip(np.rint(rng.lognormal(np.log(40.0), 1.0, L)), 2, 500).astype(np.int64)
        a = (rng.zipf(max(p["s"], 1.01), size=(n, L)) - 1) % k[None, :]
        A = (np.arange(L, dtype=np.uint64)[None, :] << np.uint64(20)) + a.astype(np.uint64) + np.uint64(1)
        A[rng.random((n, L)) < p["miss"]] = 0
        return A
    if p.get("kind") == "founders":
        rng = np.random.default_rng(p["seed"])
        n, L = p["n"], p["L"]
        out = np.zeros((L, n), dtype=np.uint64)
        for l in range(L):
            f = rng.integers(1, 2**32, size=p["founders"], dtype=np.uint64)
            col = f[rng.integers(0, p["founders"], n)]
            mut = rng.random(n) < p["mut"]
            col[mut] = rng.integers(2**32, 2**64 - 1, size=int(mut.sum()), dtype=np.uint64)
            col[rng.random(n) < 2 * p["miss"] * rng.random()] = 0
            out[l] = col
        return np.ascontiguousarray(out.T)

    def distinct(rng, L):
        return np.clip(np.rint(rng.lognormal(np.log(p["median"]), p["sigma"], L)), 2, 3000).astype(np.int64)

    def miss(rng, L):
        return rng.uniform(0.0, 2 * p["miss"], L)

    return synth.zipf_profiles(p["n"], p["L"], p["seed"], p["s"], distinct, miss, hashed_frac=0.05)


DEFAULT_GROUP = 8  # the library's raster group when none is set


def time_solve(A: np.ndarray, tau: int, scheds, reps: int = 3, device: int = 0) -> list:
    """Median device ms of one whole-triangle stripe (rare counts + tile
    pass) for each schedule (sub-stripe rows, raster group) in scheds, one
    solver (one encoding) at this tau."""
    import torch

    n = A.shape[0]
    ldo = (n + 7) // 8 * 8
    out = torch.empty((n, ldo), dtype=torch.int16, device=f"cuda:{device}")
    stream = torch.cuda.current_stream(device).cuda_stream
    res = []
    with tch.Solver.from_calls(A, tau=tau, device=device) as s:
        for sub, grp in scheds:
            s.set_schedule(int(sub), int(grp))
            s.stripe(0, n, out.data_ptr(), ldo, stream)  # warm-up
            times = []
            for _ in range(reps):
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record()
                s.stripe(0, n, out.data_ptr(), ldo, stream)
                e1.record()
                torch.cuda.synchronize()
                times.append(e0.elapsed_time(e1))
            res.append(float(np.median(times)))
        s.check()
    del out
    return res


def sweep(n_datasets: int, out: str, span: int = 4, device: int = 0, first: int = 0) -> None:
    rows = dict(ds=[], tau=[], sub=[], group=[], feats=[], est=[], ms=[])
    params = []
    t0 = time.time()
    for d in range(first, first + n_datasets):
        p = dataset_params(d)
        A = make_dataset(p)
        c = tch.tau_features(A, device)
        analytic = int(c["taus"][np.argmin(c["est"])])
        for t in sorted(set(int(x) for x in c["taus"])):
            if t < max(4, analytic // span) or t > analytic * span:
                continue
            idx = np.nonzero(c["taus"] == t)[0]
            ms = time_solve(A, t, [(c["subs"][i], c["groups"][i]) for i in idx], device=device)
            for i, m in zip(idx, ms):
                rows["ds"].append(d)
                rows["tau"].append(t)
                rows["sub"].append(int(c["subs"][i]))
                rows["group"].append(int(c["groups"][i]))
                rows["feats"].append(c["feats"][i])
                rows["est"].append(float(c["est"][i]))
                rows["ms"].append(m)
        params.append(p)
        print(f"[{time.time() - t0:6.1f}s] set {d}: {p['kind']} n={p['n']} L={p['L']} analytic tau={analytic}",
              flush=True)
    np.savez(out, ds=np.array(rows["ds"], np.int32), tau=np.array(rows["tau"], np.int32),
             sub=np.array(rows["sub"], np.int32), group=np.array(rows["group"], np.int32),
             feats=np.array(rows["feats"], np.float32), est=np.array(rows["est"]), ms=np.array(rows["ms"]),
             params=json.dumps(params))


# Sub-stripe rows of the schedules tch_tau_features offers (a sweep taken
# when more were offered keeps those rows; they are left out here).
SCHED_SUBS = (0, 8192)


def offered(data: dict) -> dict:
    """The sweep's rows whose schedule the library still offers."""
    keep = np.isin(data["sub"], SCHED_SUBS)
    return {k: (v[keep] if isinstance(v, np.ndarray) and v.shape[:1] == keep.shape else v) for k, v in data.items()}


def holdout_mask(ds: np.ndarray) -> np.ndarray:
    return ds % 5 == 4


def fold_standardisation(w: np.ndarray, mu: np.ndarray, sd: np.ndarray) -> np.ndarray:
    """Model on (x - mu) / sd -> the same model on raw x."""
    F, H = tch.TAU_FEATURES, tch.MLP_HIDDEN
    w = w.astype(np.float64).copy()
    W1 = w[:F * H].reshape(F, H)
    b1 = w[F * H:F * H + H]
    b1 -= (mu / sd) @ W1
    W1 /= sd[:, None]
    w[:F * H] = W1.ravel()
    w[F * H:F * H + H] = b1
    return w.astype(np.float32)


def evaluate(w: np.ndarray, data, device: int = 0, mask=None) -> dict:
    """Per held-out set (mask: rows of the sets to evaluate; default the
    held-out fifth): measured ms at the solver's pick with the model set (the
    learned candidate: tau and schedule), at the analytic pick (its tau with
    the default schedule) and at the best swept candidate."""
    data = offered(data)
    ds, tau, X, est, ms = data["ds"], data["tau"], data["feats"], data["est"], data["ms"]
    sub, grp = data["sub"], data["group"]
    if mask is None:
        mask = holdout_mask(ds)
    pred = tch.mlp_predict(w, X, device)
    default = (sub == 0) & (grp == DEFAULT_GROUP)
    out = []
    for d in np.unique(ds[mask]):
        m = ds == d
        i_l = np.argmin(np.where(m, pred, np.inf))
        i_a = np.argmin(np.where(m & default, est, np.inf))
        i_b = np.argmin(np.where(m, ms, np.inf))
        out.append(dict(set=int(d), tau_learned=int(tau[i_l]), sub_learned=int(sub[i_l]), group_learned=int(grp[i_l]),
                        tau_analytic=int(tau[i_a]), tau_best=int(tau[i_b]), sub_best=int(sub[i_b]),
                        group_best=int(grp[i_b]), ms_learned=float(ms[i_l]), ms_analytic=float(ms[i_a]),
                        ms_best=float(ms[i_b])))
    return summarise(out)


def summarise(out: list) -> dict:
    tl = sum(r["ms_learned"] for r in out)
    ta = sum(r["ms_analytic"] for r in out)
    tb = sum(r["ms_best"] for r in out)
    return dict(sets=out, total_ms_learned=tl, total_ms_analytic=ta, total_ms_best=tb,
                learned_over_best=tl / tb, analytic_over_best=ta / tb,
                mean_learned_over_best=float(np.mean([r["ms_learned"] / r["ms_best"] for r in out])),
                mean_analytic_over_best=float(np.mean([r["ms_analytic"] / r["ms_best"] for r in out])))


def oversample(ds: np.ndarray, ms: np.ndarray, idx: np.ndarray) -> np.ndarray:
    """Training rows with each profile set's candidates repeated
    round(log2(best ms / 0.2 ms)) times (1 to 8): the squared error in ln(ms)
    weighs every set alike, while a wrong pick costs in proportion to the set's
    time, so the sets that dominate a workload's time get more weight."""
    best = {}
    for d, t in zip(ds, ms):
        best[d] = min(best.get(d, np.inf), t)
    reps = np.array([int(np.clip(np.round(np.log2(best[d] / 0.2)), 1, 8)) for d in ds[idx]])
    return np.repeat(idx, reps)


def fit(data: dict, tr: np.ndarray, steps: int, lr: float, seed: int, device: int):
    """The model trained on the rows of the sets in tr (standardisation folded
    into the first layer); returns (weights, final loss, rows used)."""
    ds = data["ds"]
    X = data["feats"].astype(np.float64)
    y = np.log(data["ms"]).astype(np.float32)
    mu = X[tr].mean(0)
    sd = X[tr].std(0)
    sd[sd < 1e-6] = 1.0
    Xn = ((X - mu) / sd).astype(np.float32)
    idx = oversample(ds, data["ms"], np.nonzero(tr)[0])
    w = tch.mlp_init(seed)
    w, _ = tch.mlp_train(w, Xn[idx], y[idx], steps // 2, lr, device)
    w, loss = tch.mlp_train(w, Xn[idx], y[idx], steps - steps // 2, lr / 5, device)
    return fold_standardisation(w, mu, sd), loss, int(len(idx))


def train(sweep_path: str, out: str, steps: int = 6000, lr: float = 3e-3, seed: int = 7, device: int = 0) -> dict:
    """The shipped model: trained on four fifths of the sets, evaluated on the
    held-out fifth."""
    data = offered(dict(np.load(sweep_path)))
    ds = data["ds"]
    tr = ~holdout_mask(ds)
    t0 = time.time()
    w_raw, loss, rows = fit(data, tr, steps, lr, seed, device)
    secs = time.time() - t0
    rep = evaluate(w_raw, data, device)
    rep.update(train_rows=rows, train_sets=int(len(np.unique(ds[tr]))), holdout_rows=int((~tr).sum()), steps=steps,
               final_train_mse=loss, train_seconds=secs)
    w_raw.astype("<f4").tofile(out)
    return rep


def cross_validate(sweep_path: str, folds: int = 5, steps: int = 6000, lr: float = 3e-3, seed: int = 7,
                   device: int = 0) -> dict:
    """The training recipe, k-fold: for each fold a model trained on the
    other sets picks for the fold's sets; every set is held out once."""
    data = offered(dict(np.load(sweep_path)))
    ds = data["ds"]
    out, per_fold = [], []
    for f in range(folds):
        hold = ds % folds == f
        w_raw, _, _ = fit(data, ~hold, steps, lr, seed, device)
        rep = evaluate(w_raw, data, device, mask=hold)
        out += rep["sets"]
        per_fold.append({k: v for k, v in rep.items() if k != "sets"})
    res = summarise(out)
    res.update(folds=folds, per_fold=per_fold)
    return res


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("cmd", choices=["sweep", "train", "report", "cv"])
    ap.add_argument("--datasets", type=int, default=200)
    ap.add_argument("--first", type=int, default=0, help="sweep: first profile set (seed)")
    ap.add_argument("--sweep", default=SWEEP_PATH)
    ap.add_argument("--out", default=None)
    ap.add_argument("--steps", type=int, default=6000)
    ap.add_argument("--device", type=int, default=0)
    a = ap.parse_args()
    if a.cmd == "sweep":
        sweep(a.datasets, a.out or SWEEP_PATH, device=a.device, first=a.first)
    elif a.cmd == "report":  # the shipped model on the shipped sweep
        rep = evaluate(np.fromfile(a.out or tch.TAU_MLP_PATH, dtype="<f4"), dict(np.load(a.sweep)), a.device)
        with open(REPORT_PATH, "w") as f:
            json.dump(rep, f, indent=1)
        print(json.dumps({k: v for k, v in rep.items() if k != "sets"}, indent=1))
    elif a.cmd == "cv":  # the training recipe, 5-fold, on the shipped sweep
        rep = cross_validate(a.sweep, steps=a.steps, device=a.device)
        with open(a.out or CV_PATH, "w") as f:
            json.dump(rep, f, indent=1)
        print(json.dumps({k: v for k, v in rep.items() if k not in ("sets", "per_fold")}, indent=1))
    else:
        rep = train(a.sweep, a.out or tch.TAU_MLP_PATH, steps=a.steps, device=a.device)
        with open(REPORT_PATH, "w") as f:
            json.dump(rep, f, indent=1)
        print(json.dumps({k: v for k, v in rep.items() if k != "sets"}, indent=1))


if __name__ == "__main__":
    main()
