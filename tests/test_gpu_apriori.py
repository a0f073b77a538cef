"""Candidate generation on the device (colo_apriori.cu) against the oracle's
restatement of candidateColocationGeneral (colocationFinder.cpp:517-557),
including its breaks: the j loop of pattern i stops at the first pattern with
another prefix and at the first candidate with a non-prevalent subset."""
import numpy as np
import pytest

import colo
import oracle
from colo import gen

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    return colo.Context(0)


def _check(ctx, prev, k):
    prev = np.asarray(prev, np.uint32).reshape(-1, k - 1)
    got, par = ctx.stage_apriori(prev, k)
    want = oracle.apriori(prev, k)
    assert got.shape == want.shape and np.array_equal(got, want), (k, got[:5], want[:5])
    if len(got):
        assert np.array_equal(prev[par], got[:, : k - 1])   # parent = the candidate's prefix pattern
    return len(got)


def test_break_on_missing_subset(ctx):
    # prevalent AB, AC, AD, BD (not BC): ABC fails its subset BC, which ends the j loop of AB,
    # so ABD is never generated although all its subsets are prevalent
    assert _check(ctx, [[0, 1], [0, 2], [0, 3], [1, 3]], 3) == 0
    assert _check(ctx, [[0, 1], [0, 2], [0, 3], [1, 2], [1, 3], [2, 3]], 3) == 4


def _random_prevalent(rng, F, km1, n, keep):
    """Lexicographic unique (km1)-patterns: the km1-subsets of a random set of larger
    patterns (so many subsets exist), thinned by `keep` so that some are missing.  At most
    n patterns, after at most 20 n draws (few distinct patterns exist when F is small)."""
    rows = set()
    for _ in range(20 * n):
        if len(rows) >= n:
            break
        big = np.sort(rng.choice(F, km1 + 2, replace=False))
        for drop in range(km1 + 2):
            for drop2 in range(drop + 1, km1 + 2):
                r = tuple(int(v) for t, v in enumerate(big) if t not in (drop, drop2))
                if rng.random() < keep:
                    rows.add(r)
    return np.array(sorted(rows), np.uint32)


@pytest.mark.parametrize("k", [3, 4, 5, 6, 8])
@pytest.mark.parametrize("keep", [1.0, 0.9])
def test_random_levels_match_oracle(ctx, k, keep):
    rng = np.random.default_rng(k * 10 + int(keep * 10))
    prev = _random_prevalent(rng, 24, k - 1, 3000, keep)
    assert len(prev) >= 200
    _check(ctx, prev, k)


def test_many_patterns(ctx):
    rng = np.random.default_rng(7)
    prev = _random_prevalent(rng, 60, 3, 30000, 0.97)
    assert len(prev) >= 30000
    _check(ctx, prev, 4)


def test_empty_and_single(ctx):
    assert _check(ctx, np.zeros((0, 2), np.uint32), 3) == 0
    assert _check(ctx, [[1, 2]], 3) == 0


@pytest.mark.parametrize("cfg,scale", [(1, 0.02), (3, 0.002)])
def test_mining_with_device_candidates_is_identical(ctx, cfg, scale):
    wl = gen.config(cfg, scale=scale)
    ds = colo.Dataset.from_arrays(ctx, wl.x, wl.y, wl.fid, wl.bounds)
    a = ctx.mine(ds, colo.default_params(wl.R, wl.thr, colo.MODE_BATCHED, max_size=wl.max_size))
    b = ctx.mine(ds, colo.default_params(wl.R, wl.thr, colo.MODE_BATCHED, max_size=wl.max_size,
                                         device_apriori=True))
    assert len(a.levels) == len(b.levels) and len(a.levels) >= 2
    for la, lb in zip(a.levels, b.levels):
        assert np.array_equal(la.cand, lb.cand) and np.array_equal(la.num, lb.num)
        assert np.array_equal(la.prevalent, lb.prevalent)


def test_batch_of_jobs_with_device_candidates(ctx):
    jobs = gen.config2_jobs(8, scale=0.05)
    dss = [colo.Dataset.from_arrays(ctx, j.x, j.y, j.fid, j.bounds) for j in jobs]
    pa = [colo.default_params(j.R, j.thr, colo.MODE_BATCHED, max_size=j.max_size) for j in jobs]
    pb = [colo.default_params(j.R, j.thr, colo.MODE_BATCHED, max_size=j.max_size, device_apriori=True)
          for j in jobs]
    ra = ctx.mine_batch(dss, pa)
    rb = ctx.mine_batch(dss, pb)
    for x, y in zip(ra, rb):
        assert x.patterns() == y.patterns()
        for la, lb in zip(x.levels, y.levels):
            assert np.array_equal(la.cand, lb.cand)
