"""Jobs with more than 256 features: the per-cell feature masks take more
than 8 words, padded to 12, 16, 24 or 32 (up to 1024 features per job), and
the pair filter's F x F accumulator no longer fits in shared memory.  Mining
and the level filter against the oracle."""
import numpy as np
import pytest

import colo
import oracle
from colo import gen
from helpers import assert_same_trace, oracle_for

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    return colo.Context(0)


def _wide(nf, n, width, seed):
    s = gen.GenSpec()
    s.seed = seed
    s.seed_frac = 0.6
    s.n, s.nfeat, s.zipf_s, s.width = n, nf, 0.8, width
    s.hot_frac, s.nhot, s.hot_sig_lo, s.hot_sig_hi = 0.6, 60, 30.0, 300.0
    s.npat, s.pat_min, s.pat_max, s.pat_sigma = 12, 2, 5, 15.0
    return gen.generate(s, f"wide{nf}", 40.0, 0.2, 5)


def test_mining_300_features_matches_oracle(ctx):
    wl = _wide(300, 40000, 20000.0, 1077)   # 10 mask words, padded to 12
    ds = colo.Dataset.from_arrays(ctx, wl.x, wl.y, wl.fid, wl.bounds)
    for mode in (colo.MODE_BATCHED, colo.MODE_PLAIN):
        got = ctx.mine(ds, colo.default_params(wl.R, wl.thr, mode, max_size=wl.max_size, keep_tables=True))
        if mode == colo.MODE_BATCHED:
            ref = oracle_for(ctx, wl, keep_tables=True)
            assert len(ref.levels) >= 3
        assert_same_trace(got, ref, tables=True)


@pytest.mark.parametrize("nf", [270, 450, 700, 1000])   # 9, 15, 22, 32 words: padded 12, 16, 24, 32
def test_level_filter_wide_masks_matches_dense_literal(ctx, nf):
    wl = _wide(nf, 30000, 8000.0, 2000 + nf)
    ds = colo.Dataset.from_arrays(ctx, wl.x, wl.y, wl.fid, wl.bounds)
    rng = np.random.default_rng(nf)
    present = np.unique(wl.fid)
    total = 0
    for k in (2, 3, 4, 6):
        cand = np.array([sorted(rng.choice(len(present), k, replace=False)) for _ in range(60)], np.uint32)
        # candidates that share features, so that some quads are full
        cand[:20] = np.sort(np.stack([rng.permutation(8)[:k] for _ in range(20)]), axis=1)
        cand = np.unique(cand, axis=0)
        ub, pas = ctx.stage_filter(ds, wl.R, wl.thr, cand)
        oub, opas = oracle.filter_dense(wl.x, wl.y, wl.fid, wl.bounds, wl.R, wl.thr, cand)
        assert np.array_equal(ub, oub), (nf, k)
        assert np.array_equal(pas, opas), (nf, k)
        total += int(ub.sum())
    assert total > 0   # some quads were full


def test_more_than_1024_features_is_a_clear_error(ctx):
    wl = _wide(1100, 20000, 8000.0, 5)
    ds = colo.Dataset.from_arrays(ctx, wl.x, wl.y, wl.fid, wl.bounds)
    with pytest.raises(colo.ColoError) as e:
        ctx.mine(ds, colo.default_params(wl.R, wl.thr, colo.MODE_BATCHED, max_size=3))
    assert e.value.status == colo.ERR_CAPACITY and "1024 features" in str(e.value)
