"""Training and evaluation of the learned cost model.

The model maps a filtered candidate's 24 cell-aggregate features
(colo_result_features) to log1p(instance-table rows).  Training pairs come
from the mining itself: every candidate a mine refines yields (features,
exact row count).  The training set is mined from seeded datasets of the
20M-point workload's generator at 200k-2M points (same density), and the
network is trained on the GPU by the library's own kernels
(colo_model_train).

    python -m colo.costmodel train --out cost_model.npz   # needs a GPU

`heuristic_log_rows` is the presize the method would use without the
network (parent rows times the fraction of the last member's instances that
lie in candidate cells); `evaluate` reports both against the exact counts.
"""
from __future__ import annotations

import argparse
import math
import time

import numpy as np

from . import MODE_BATCHED, Context, Dataset, default_params, init_model
from . import gen

TRAIN_SEEDS = range(20270100, 20270150)     # 50 training datasets
HELDOUT_SEEDS = range(20270200, 20270204)   # never trained on
MARGIN = 1.5                                # capacity = 1.5 x predicted rows + 32 (as colo_mine.cpp)


def dataset_size(seed: int) -> int:
    rng = np.random.default_rng(seed)
    return int(math.exp(rng.uniform(math.log(200_000), math.log(2_000_000))))


THRESHOLDS = (0.15, 0.1, 0.07, 0.05, 0.035)   # the workload's 0.15 and lower ones (more, larger candidates)
PER_MINE_CAP = 20_000                          # samples kept per mine (uniform subsample)


def collect(ctx: Context, seeds, thresholds=THRESHOLDS, log=None, cap=PER_MINE_CAP):
    """(X float32[n, 24], log1p(rows) float32[n], k int[n]) of the refined candidates."""
    xs, ts, ks = [], [], []
    for seed in seeds:
        n = dataset_size(seed)
        wl = gen.config(3, seed=seed, scale=n / 20_000_000)
        ds = Dataset.from_arrays(ctx, wl.x, wl.y, wl.fid, wl.bounds)
        for thr in thresholds:
            res = ctx.mine(ds, default_params(wl.R, thr, MODE_BATCHED, max_size=wl.max_size, features=True))
            mx, mt, mk = [], [], []
            for lev in res.levels:
                sel = lev.passed.astype(bool)
                if not sel.any():
                    continue
                mx.append(lev.features[sel])
                mt.append(np.log1p(lev.rows[sel].astype(np.float64)).astype(np.float32))
                mk.append(np.full(int(sel.sum()), lev.k, np.int32))
            if not mx:
                continue
            mx, mt, mk = np.concatenate(mx), np.concatenate(mt), np.concatenate(mk)
            if cap and len(mt) > cap:
                keep = np.sort(np.random.default_rng(seed * 7 + int(thr * 1000)).choice(len(mt), cap, replace=False))
                mx, mt, mk = mx[keep], mt[keep], mk[keep]
            xs.append(mx)
            ts.append(mt)
            ks.append(mk)
        if log:
            log(f"seed {seed}: {n} points, {sum(len(t) for t in ts)} samples so far")
    if not xs:
        return np.zeros((0, 24), np.float32), np.zeros(0, np.float32), np.zeros(0, np.int32)
    return np.concatenate(xs), np.concatenate(ts), np.concatenate(ks)


def heuristic_log_rows(x: np.ndarray) -> np.ndarray:
    """Presize without the network: log1p(parent rows) + log1p(ub_last) - log1p(n_last)."""
    return x[:, 17] + x[:, 23]


def heuristic_params() -> np.ndarray:
    """The same heuristic written as parameters of the network, so the library can run it in place
    of the trained model: y = relu(x17) - relu(-x23) = x17 + x23 (x17 >= 0, x23 <= 0)."""
    p = np.zeros(32 * 64 + 64 + 64 * 64 + 64 + 64 + 1, np.float32)
    w1, w2, w3 = 0, 32 * 64 + 64, 32 * 64 + 64 + 64 * 64 + 64
    p[w1 + 17 * 64 + 0] = 1.0
    p[w1 + 23 * 64 + 1] = -1.0
    p[w2 + 0 * 64 + 0] = 1.0
    p[w2 + 1 * 64 + 1] = 1.0
    p[w3 + 0] = 1.0
    p[w3 + 1] = -1.0
    return p


def errors(pred_log: np.ndarray, t_log: np.ndarray) -> dict:
    pred = np.expm1(np.clip(pred_log.astype(np.float64), 0, 40))
    true = np.expm1(t_log.astype(np.float64))
    rel = np.abs(pred - true) / np.maximum(true, 1.0)
    cap = np.ceil(pred * MARGIN) + 32
    return {"median_rel_err": float(np.median(rel)), "p95_rel_err": float(np.percentile(rel, 95)),
            "overflow_rate": float(np.mean(true > cap)),
            "alloc_over_needed": float(np.sum(cap) / max(np.sum(true), 1.0))}


def evaluate(ctx: Context, params: np.ndarray, x: np.ndarray, t: np.ndarray) -> dict:
    y = ctx.model_forward(params, x)
    return {"model": errors(y, t), "heuristic": errors(heuristic_log_rows(x), t), "samples": int(len(t))}


SCHEDULE = ((40, 2e-3), (30, 5e-4), (30, 1e-4))   # (epochs, learning rate) phases, Adam restarted per phase


def train(ctx: Context, x: np.ndarray, t: np.ndarray, schedule=SCHEDULE, batch: int = 2048, seed: int = 0):
    """GPU training in phases of decreasing learning rate; returns (parameters, per-epoch loss)."""
    p = init_model(seed)
    p[-1] = float(np.mean(t))        # start the output bias at the mean target
    hist = []
    for i, (epochs, lr) in enumerate(schedule):
        p, h = ctx.model_train(p, x, t, epochs, batch, lr, seed + i)
        hist.extend(h.tolist())
    return p, np.array(hist, np.float32)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("cmd", choices=["train"])
    ap.add_argument("--out", required=True)
    args = ap.parse_args()
    ctx = Context(0)
    t0 = time.time()
    x, t, k = collect(ctx, TRAIN_SEEDS, log=print)
    t_collect = time.time() - t0
    xh, th, kh = collect(ctx, HELDOUT_SEEDS)
    t0 = time.time()
    params, hist = train(ctx, x, t)
    t_train = time.time() - t0
    ev = evaluate(ctx, params, xh, th)
    ev_train = evaluate(ctx, params, x, t)
    print({"samples": len(t), "collect_s": t_collect, "train_s": t_train, "loss": hist.tolist(),
           "heldout": ev, "train": ev_train})
    np.savez(args.out, params=params, loss=hist, samples=len(t), train_seeds=np.array(list(TRAIN_SEEDS)),
             heldout_median_rel_err=ev["model"]["median_rel_err"], heldout_p95_rel_err=ev["model"]["p95_rel_err"])


if __name__ == "__main__":
    main()
