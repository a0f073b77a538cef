"""The learned cost model on the GPU: the tensor-core forward and gradient
kernels against the oracle's restatement (same BF16 rounding points, sums
in double), GPU training, and COLO_MODE_LEARNED mining -- identical results
to the batched form with a trained model and with a useless one (every
table overflows its presize and takes the two-pass fallback).

Tolerances: the kernels accumulate in FP32 in the tensor cores' order; a
sum that lands next to a BF16 rounding boundary can round the other way, so
single values may differ by one BF16 step (2^-8 relative) of one hidden
unit.  Forward outputs: |dy| <= 1e-2 (1 + |y|).  Gradients: relative L2
error per parameter block <= 1e-2.
"""
import numpy as np
import pytest

import colo
import oracle
from colo import gen

pytestmark = pytest.mark.gpu

BLOCKS = {"W1": (0, 24 * 64), "b1": (2048, 2112), "W2": (2112, 6208), "b2": (6208, 6272), "W3": (6272, 6336),
          "b3": (6336, 6337)}


@pytest.fixture(scope="module")
def ctx():
    return colo.Context(0)


def _params(seed):
    p = colo.init_model(seed)
    rng = np.random.default_rng(seed + 100)
    p[2048:2112] = rng.normal(0, 0.2, 64)      # b1
    p[6208:6272] = rng.normal(0, 0.2, 64)      # b2
    p[-1] = 1.5
    return p


def _inputs(n, seed):
    rng = np.random.default_rng(seed)
    x = rng.normal(0, 1.5, (n, colo.MODEL_FEATURES)).astype(np.float32)
    t = rng.normal(3, 2, n).astype(np.float32)
    return x, t


@pytest.mark.parametrize("n", [1, 17, 1000, 70001])
def test_forward_matches_oracle(ctx, n):
    p = _params(1)
    x, _ = _inputs(n, 2)
    y = ctx.model_forward(p, x)
    ref = oracle.mlp_forward(p, x, bf16=True)
    assert np.all(np.abs(y - ref) <= 1e-2 * (1 + np.abs(ref))), np.max(np.abs(y - ref))


@pytest.mark.parametrize("n", [16, 300, 20000])
def test_gradient_matches_oracle(ctx, n):
    p = _params(3)
    x, t = _inputs(n, 4)
    g, loss = ctx.model_grad(p, x, t)
    gref, lref = oracle.mlp_grad(p, x, t, bf16=True)
    assert abs(loss - lref) <= 1e-3 * (1 + abs(lref))
    for name, (a, b) in BLOCKS.items():
        num = np.linalg.norm(g[a:b] - gref[a:b])
        den = np.linalg.norm(gref[a:b]) + 1e-12
        assert num / den <= 1e-2, (name, num / den)
    assert np.all(g[24 * 64:32 * 64] == 0)


def test_training_fits_a_teacher(ctx):
    teacher = _params(7)
    x, _ = _inputs(60000, 8)
    t = oracle.mlp_forward(teacher, x, bf16=False).astype(np.float32)
    p0 = colo.init_model(9)
    p0[-1] = float(t.mean())
    _, l0 = ctx.model_grad(p0, x, t)
    p, hist = ctx.model_train(p0, x, t, epochs=15, batch=1024, lr=2e-3, seed=1)
    _, l1 = ctx.model_grad(p, x, t)
    assert len(hist) == 15 and np.all(np.isfinite(hist))
    assert l1 < 0.1 * l0, (l0, l1, hist)


def _same(a, b):
    assert len(a.levels) == len(b.levels)
    for la, lb in zip(a.levels, b.levels):
        assert np.array_equal(la.cand, lb.cand)
        assert np.array_equal(la.ub, lb.ub) and np.array_equal(la.passed, lb.passed)
        assert np.array_equal(la.rows, lb.rows) and np.array_equal(la.num, lb.num)
        assert np.array_equal(la.pi.view(np.uint32), lb.pi.view(np.uint32))
        assert np.array_equal(la.prevalent, lb.prevalent)
        assert set(la.tables) == set(lb.tables)
        for c, t in lb.tables.items():    # one-pass tables: the same rows in the same order
            assert np.array_equal(la.tables[c], t)


WORKLOADS = [(0, 1.0), (1, 0.02), (3, 0.002), (3, 0.01)]


@pytest.mark.parametrize("cfg,scale", WORKLOADS)
@pytest.mark.parametrize("model", ["trained", "zeros"])
def test_learned_mining_is_identical(ctx, cfg, scale, model):
    wl = gen.config(cfg, scale=scale)
    ds = colo.Dataset.from_arrays(ctx, wl.x, wl.y, wl.fid, wl.bounds)
    ref = ctx.mine(ds, colo.default_params(wl.R, wl.thr, colo.MODE_BATCHED, max_size=wl.max_size,
                                           keep_tables=True))
    p = colo.load_model() if model == "trained" else np.zeros(colo.MODEL_PARAMS, np.float32)
    ctx.set_model(p)
    try:
        # the default policy (single pass for tables presized large) and a single pass for every table
        got = ctx.mine(ds, colo.default_params(wl.R, wl.thr, colo.MODE_LEARNED, max_size=wl.max_size,
                                               keep_tables=True))
        every = ctx.mine(ds, colo.default_params(wl.R, wl.thr, colo.MODE_LEARNED, max_size=wl.max_size,
                                                 keep_tables=True, single_pass=True))
    finally:
        ctx.set_model(None)
    _same(got, ref)
    _same(every, ref)
    c = every.counters
    assert c["single_pass"] == c["refined"]
    assert got.counters["single_pass"] <= c["refined"]
    if model == "zeros" and any(int(r) > 32 for lev in ref.levels for r in lev.rows):
        assert c["single_pass_overflow"] > 0    # the fallback ran


def test_learned_without_model_runs_batched(ctx):
    wl = gen.config(0)
    ds = colo.Dataset.from_arrays(ctx, wl.x, wl.y, wl.fid, wl.bounds)
    ctx.set_model(None)
    got = ctx.mine(ds, colo.default_params(wl.R, wl.thr, colo.MODE_LEARNED, max_size=wl.max_size))
    ref = ctx.mine(ds, colo.default_params(wl.R, wl.thr, colo.MODE_BATCHED, max_size=wl.max_size))
    assert got.patterns() == ref.patterns()
    assert got.counters["single_pass"] == 0


def test_trained_model_beats_the_model_free_presize(ctx):
    """What the network gains over the method without it, on datasets it never saw: prediction
    error, buffer overflows at the 1.5x presize margin, and two-pass fallbacks in real mines."""
    from colo import costmodel
    params = colo.load_model()
    x, t, _ = costmodel.collect(ctx, costmodel.HELDOUT_SEEDS[:2], thresholds=(0.15, 0.07))
    ev = costmodel.evaluate(ctx, params, x, t)
    print("held-out", ev)
    m, h = ev["model"], ev["heuristic"]
    assert m["median_rel_err"] < 0.15 and m["p95_rel_err"] < 0.6
    assert m["median_rel_err"] < h["median_rel_err"] / 3
    assert m["overflow_rate"] < h["overflow_rate"]
    # the same comparison through the library: the heuristic written as network parameters
    hp = costmodel.heuristic_params()
    assert np.allclose(ctx.model_forward(hp, x), costmodel.heuristic_log_rows(x), atol=0.1)
    wl = gen.config(3, seed=costmodel.HELDOUT_SEEDS[0], scale=0.05)
    ds = colo.Dataset.from_arrays(ctx, wl.x, wl.y, wl.fid, wl.bounds)
    out = {}
    for name, p in (("trained", params), ("heuristic", hp)):
        ctx.set_model(p)
        try:
            out[name] = ctx.mine(ds, colo.default_params(wl.R, 0.07, colo.MODE_LEARNED, single_pass=True))
        finally:
            ctx.set_model(None)
    print({k: (v.counters["single_pass"], v.counters["single_pass_overflow"]) for k, v in out.items()})
    assert out["trained"].patterns() == out["heuristic"].patterns()
    assert out["heuristic"].counters["single_pass_overflow"] > 0
    assert out["trained"].counters["single_pass_overflow"] <= 0.25 * out["heuristic"].counters["single_pass_overflow"]
