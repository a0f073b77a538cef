"""The oracle against itself and against hand-derived known answers (no GPU)."""
import ctypes as C

import numpy as np
import pytest

import oracle
from colo import gen


def test_neighbor_cell_rule_equals_geometric_characterisation():
    # The reference's 32-bit rule (Utility_Inline.h:35-53) visits the in-grid
    # 3x3 block for gx >= 3, only the own column for gx == 2, nothing for gx == 1.
    lib = oracle.load()
    for gx_f, gy_f in [(1, 4), (2, 5), (3, 3), (4, 2), (6, 5)]:
        g = oracle.Grid()
        R = 10.0
        assert lib.oracle_make_grid(0, 0, gx_f * R, gy_f * R - R, R, C.byref(g)) == 0
        gx, gy = g.gx, g.gy
        for c in range(gx * gy):
            cx, cy = c % gx, c // gx
            for nb in range(gx * gy):
                nx, ny = nb % gx, nb // gx
                geo = abs(nx - cx) <= 1 and abs(ny - cy) <= 1
                if gx == 1:
                    exp = False
                elif gx == 2:
                    exp = geo and nx == cx
                else:
                    exp = geo
                assert lib.oracle_cell_adjacent(C.byref(g), c, nb) == int(exp), (gx, gy, c, nb)


@pytest.mark.parametrize("cfg,scale", [(0, 1.0), (1, 0.001)])
def test_sparse_filter_equals_literal_dense_filter(cfg, scale):
    # the literal form visits every quad of the grid: keep the candidate count small
    wl = gen.config(cfg, scale=scale)
    r = oracle.mine(wl.x, wl.y, wl.fid, wl.bounds, wl.R, wl.thr, max_k=4)
    rng = np.random.default_rng(0)
    for lev in r.levels:
        pick = np.sort(rng.choice(len(lev.cand), min(len(lev.cand), 24), replace=False))
        ub, pas = oracle.filter_dense(wl.x, wl.y, wl.fid, wl.bounds, wl.R, wl.thr, lev.cand[pick])
        assert np.array_equal(ub, lev.ub[pick])
        assert np.array_equal(pas, lev.passed[pick])


def test_apriori_break_quirk():
    # prevalent {AB, AC, AD, BD} without BC: joining AB with AC fails the
    # subset check (BC) and the reference breaks out of the inner loop, so
    # ABD (AB + AD) is never generated.
    prev = np.array([[0, 1], [0, 2], [0, 3], [1, 3]], np.uint32)
    assert oracle.apriori(prev, 3).tolist() == []
    prev2 = np.array([[0, 1], [0, 2], [0, 3], [1, 2], [1, 3]], np.uint32)
    assert oracle.apriori(prev2, 3).tolist() == [[0, 1, 2], [0, 1, 3]]


def test_participation_window_quirk():
    # Degree-2 bitmap layout overlaps the last instance of the first feature
    # with the first of the second (DeviceProcess_Kernel.h:45-49): only the
    # pair (last A, first B) participates, so num = [0, 1].
    pts = [(0, 100.0, 100.0), (0, 5.0, 5.0), (1, 6.0, 5.0), (1, 200.0, 200.0)]
    fid = np.array([p[0] for p in pts], np.int32)
    x = np.array([p[1] for p in pts], np.float32)
    y = np.array([p[2] for p in pts], np.float32)
    r = oracle.mine(x, y, fid, [0, 0, 300, 300], 10.0, 0.0)
    lev = r.levels[0]
    assert lev.rows.tolist() == [1]
    assert lev.num.tolist() == [[0, 1]]     # the anchor is the last A: excluded from A's window
    assert lev.pi[0] == 0.0


def test_sq_decide_exact_and_midpoint_cases():
    # integer coordinates: the exact sum is a float, no ambiguity
    assert oracle.sq_decide(0, 0, 6, 8, 100.0) == (True, False)
    assert oracle.sq_decide(0, 0, 6, 8.0001, 100.0) == (False, False)
    le, amb, val, near = oracle.sq_decide_batch(np.zeros(3), np.zeros(3), np.array([3, 4, 1.5]),
                                                np.array([4, 3, 2.0]), 25.0)
    assert le.tolist() == [True, True, True] and not amb.any() and not near.any()
    assert val.tolist() == [25.0, 25.0, 6.25]
    # a sum exactly halfway between two floats is near a midpoint: 2^24 + 1
    le, amb, val, near = oracle.sq_decide_batch(np.zeros(1), np.zeros(1), np.array([4096.0]), np.array([1.0]),
                                                16777216.0)
    assert near.all() and amb.all()


def test_parse_params_and_csv(tmp_path):
    p = tmp_path / "parameter.txt"
    p.write_text("10\n0.3\n1")
    assert oracle.parse_params(str(p)) == (10.0, pytest.approx(0.3), 1)
    c = tmp_path / "pts.csv"
    c.write_text("5\n7,1.5,2.25\n7,3,4\n09,5,6\n9,7,8\n7,1,1\n\n0,0,10,10")
    x, y, feat, b, names = oracle.parse_csv(str(c))
    # "09" and "9" are the same feature id; a later "7" starts a new feature
    assert feat.tolist() == [0, 0, 1, 1, 2]
    assert names == ["7", "09", "7"]
    assert b.tolist() == [0, 0, 10, 10]


def test_generator_is_deterministic_and_grouped():
    a = gen.config(1, scale=0.005)
    b = gen.config(1, scale=0.005)
    assert np.array_equal(a.x, b.x) and np.array_equal(a.fid, b.fid)
    assert np.all(np.diff(a.fid) >= 0)
    assert a.x.min() >= 0 and a.x.max() < a.bounds[2]


# ---- the scaled oracle (oracle_mine_fast) against the literal restatement ----

@pytest.mark.parametrize("cfg,scale", [(0, 1.0), (1, 0.02), (3, 0.002), (4, 0.0002)])
def test_fast_oracle_equals_literal_oracle(cfg, scale):
    from helpers import assert_same_trace

    wl = gen.config(cfg, scale=scale)
    lit = oracle.mine(wl.x, wl.y, wl.fid, wl.bounds, wl.R, wl.thr, max_k=wl.max_size, keep_tables=True)
    fast = oracle.mine(wl.x, wl.y, wl.fid, wl.bounds, wl.R, wl.thr, max_k=wl.max_size, keep_tables=True, fast=True)
    assert lit.status == 0 and fast.status == 0
    assert_same_trace(fast, lit, tables=True)


def test_fast_oracle_reproduces_reference_golden():
    from golden_check import CASES, assert_matches_golden, load, paths

    for case in CASES:
        g = load(case)
        csv, par = paths(case)
        x, y, feat, b, names = oracle.parse_csv(str(csv))
        R, thr, _ = oracle.parse_params(str(par))
        res = oracle.mine(x, y, feat.astype(np.int32), b, R, thr, keep_tables=True, fast=True)
        assert res.status == 0 and res.unresolved == 0, case
        assert_matches_golden(res, g)


def _planted_midpoints(n_pairs=600, noise=2400, seed=3):
    """Pairs whose exact squared distance is the midpoint 1 + 2^-24 between
    R^2 = 1 and the next float (dx = 1, dy = 2^-12), among uniform noise."""
    rng = np.random.default_rng(seed)
    bx = rng.integers(1, 500, n_pairs).astype(np.float32)
    by = rng.integers(1, 500, n_pairs).astype(np.float32)
    x = np.concatenate([bx, bx + 1, rng.uniform(0, 500, noise).astype(np.float32)])
    y = np.concatenate([by, by + np.float32(2.0 ** -12), rng.uniform(0, 500, noise).astype(np.float32)])
    f = np.concatenate([np.zeros(n_pairs), np.ones(n_pairs), rng.integers(0, 3, noise)]).astype(np.int32)
    order = np.argsort(f, kind="stable")
    return x[order], y[order], f[order]


def test_ambiguous_pairs_equal_brute_force():
    x, y, f = _planted_midpoints()
    got = oracle.ambiguous_pairs(x, y, f, 1.0)
    n = len(x)
    i, j = np.triu_indices(n, 1)
    keep = f[i] != f[j]
    i, j = i[keep], j[keep]
    _, amb, _, _ = oracle.sq_decide_batch(x[i], y[i], x[j], y[j], np.float32(1.0))
    want = np.sort((i[amb].astype(np.uint64) << np.uint64(32)) | j[amb].astype(np.uint64))
    assert len(want) >= 600
    assert np.array_equal(got, want)


def test_fast_oracle_applies_device_outcomes_of_ambiguous_pairs():
    """Both oracles take the outcome of every ambiguous pair from the caller;
    flipping outcomes changes the trace the same way in both."""
    from helpers import assert_same_trace

    x, y, f = _planted_midpoints(n_pairs=400, noise=600, seed=9)
    keys = oracle.ambiguous_pairs(x, y, f, 1.0)
    bounds = np.array([0, 0, 502, 502], np.float32)
    rng = np.random.default_rng(1)
    for le in (np.ones(len(keys), np.uint8), np.zeros(len(keys), np.uint8),
               rng.integers(0, 2, len(keys)).astype(np.uint8)):
        a = oracle.mine(x, y, f, bounds, 1.0, 0.1, keep_tables=True, res=(keys, le))
        b = oracle.mine(x, y, f, bounds, 1.0, 0.1, keep_tables=True, res=(keys, le), fast=True)
        assert a.unresolved == 0 and b.unresolved == 0
        assert_same_trace(b, a, tables=True)
    rows = [oracle.mine(x, y, f, bounds, 1.0, 0.1, res=(keys, np.full(len(keys), v, np.uint8)), fast=True)
            .levels[0].rows[0] for v in (0, 1)]
    assert rows[1] - rows[0] >= 400   # every planted pair counts only when its outcome says <=
