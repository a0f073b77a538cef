"""GPU parity: the CUDA path through the C ABI against the CPU oracle.

Integer results (neighbour lists, filter bounds, row counts, participation
numerators, pattern sets, instance tables) must be identical; the float PI
must have identical bits.
"""
import numpy as np
import pytest

import colo
import oracle
from colo import gen
from helpers import assert_same_trace, oracle_for, resolve_ambiguous

pytestmark = pytest.mark.gpu

CASES = [(0, 1.0), (1, 0.02), (3, 0.002), (4, 0.0004)]


@pytest.fixture(scope="module")
def ctx():
    return colo.Context(0)


@pytest.fixture(scope="module", params=CASES, ids=lambda c: f"config{c[0]}@{c[1]}")
def workload(request):
    cfg, sc = request.param
    return gen.config(cfg, scale=sc)


def test_neighbor_csr_matches_oracle(ctx, workload):
    wl = workload
    ds = colo.Dataset.from_arrays(ctx, wl.x, wl.y, wl.fid, wl.bounds)
    offs, nbr = ctx.stage_neighbors(ds, wl.R)
    res = resolve_ambiguous(ctx, wl.x, wl.y, wl.fid, wl.R)
    o_offs, o_nbr, unres = oracle.neighbors(wl.x, wl.y, wl.fid, wl.bounds, wl.R, res=res)
    assert unres == 0
    assert np.array_equal(offs, o_offs)
    assert np.array_equal(nbr, o_nbr)   # same order: (feature, neighbour cell, id)


@pytest.mark.parametrize("mode", [colo.MODE_PLAIN, colo.MODE_BATCHED])
def test_mining_trace_matches_oracle(ctx, workload, mode):
    wl = workload
    ds = colo.Dataset.from_arrays(ctx, wl.x, wl.y, wl.fid, wl.bounds)
    got = ctx.mine(ds, colo.default_params(wl.R, wl.thr, mode, max_size=wl.max_size, keep_tables=True))
    ref = oracle_for(ctx, wl, keep_tables=True)
    assert_same_trace(got, ref, tables=True)


def test_planted_patterns_config0(ctx):
    wl = gen.config(0)
    ds = colo.Dataset.from_arrays(ctx, wl.x, wl.y, wl.fid, wl.bounds)
    got = ctx.mine(ds, colo.default_params(wl.R, wl.thr, colo.MODE_BATCHED, max_size=4))
    pats = set(got.patterns())
    # every planted pattern and all of its sub-patterns are prevalent; nothing with F9
    for p in wl.patterns:
        assert tuple(p) in pats
    assert not any(9 in p for p in pats)


def test_filter_stage_matches_dense_literal(ctx):
    wl = gen.config(0)
    ds = colo.Dataset.from_arrays(ctx, wl.x, wl.y, wl.fid, wl.bounds)
    rng = np.random.default_rng(1)
    for k in (2, 3, 4, 5):
        cand = np.array([sorted(rng.choice(10, k, replace=False)) for _ in range(40)], np.uint32)
        ub, pas = ctx.stage_filter(ds, wl.R, wl.thr, cand)
        oub, opas = oracle.filter_dense(wl.x, wl.y, wl.fid, wl.bounds, wl.R, wl.thr, cand)
        assert np.array_equal(ub, oub), k
        assert np.array_equal(pas, opas), k


def test_batch_of_jobs_equals_single_runs(ctx):
    jobs = gen.config2_jobs(6, scale=0.05)
    dss = [colo.Dataset.from_arrays(ctx, w.x, w.y, w.fid, w.bounds) for w in jobs]
    params = [colo.default_params(w.R, w.thr, colo.MODE_BATCHED, max_size=w.max_size) for w in jobs]
    batched = ctx.mine_batch(dss, params)
    for w, ds, p, rb in zip(jobs, dss, params, batched):
        single = ctx.mine(ds, p)
        ref = oracle_for(ctx, w)
        assert_same_trace(rb, ref)
        assert_same_trace(single, ref)
