"""The join autotuner: it picks one of the lane widths, and the neighbour
lists and mining results do not depend on the width it picks."""
import numpy as np
import pytest

import colo
from colo import gen

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("cfg,scale", [(0, 1.0), (1, 0.02), (3, 0.005)])
def test_autotuned_join_gives_identical_results(cfg, scale):
    wl = gen.config(cfg, scale=scale)
    plain_ctx = colo.Context(0)
    ds0 = colo.Dataset.from_arrays(plain_ctx, wl.x, wl.y, wl.fid, wl.bounds)
    params = colo.default_params(wl.R, wl.thr, colo.MODE_BATCHED, max_size=wl.max_size)
    ref = plain_ctx.mine(ds0, params)
    offs0, nbr0 = plain_ctx.stage_neighbors(ds0, wl.R)

    ctx = colo.Context(0)
    ds = colo.Dataset.from_arrays(ctx, wl.x, wl.y, wl.fid, wl.bounds)
    tuned = ctx.autotune(ds, params)
    assert tuned["join_group"] in colo.JOIN_WIDTHS
    assert sorted(tuned["join_ms"]) == list(colo.JOIN_WIDTHS)
    assert all(v > 0 for v in tuned["join_ms"].values())
    got = ctx.mine(ds, params)
    assert got.patterns() == ref.patterns()
    for la, lb in zip(got.levels, ref.levels):
        assert np.array_equal(la.rows, lb.rows) and np.array_equal(la.num, lb.num)
    offs, nbr = ctx.stage_neighbors(ds, wl.R)
    assert np.array_equal(offs, offs0) and np.array_equal(nbr, nbr0)


@pytest.mark.parametrize("width", colo.JOIN_WIDTHS)
def test_every_join_width_writes_the_same_lists(width):
    wl = gen.config(3, scale=0.005)
    ctx0 = colo.Context(0)
    ds0 = colo.Dataset.from_arrays(ctx0, wl.x, wl.y, wl.fid, wl.bounds)
    offs0, nbr0 = ctx0.stage_neighbors(ds0, wl.R)
    params = colo.default_params(wl.R, wl.thr, colo.MODE_BATCHED, max_size=wl.max_size)
    ref = ctx0.mine(ds0, params)
    ctx = colo.Context(0)
    ctx.set_join_group(width)
    ds = colo.Dataset.from_arrays(ctx, wl.x, wl.y, wl.fid, wl.bounds)
    offs, nbr = ctx.stage_neighbors(ds, wl.R)
    assert np.array_equal(offs, offs0) and np.array_equal(nbr, nbr0)
    got = ctx.mine(ds, params)
    assert got.patterns() == ref.patterns()
    for la, lb in zip(got.levels, ref.levels):
        assert np.array_equal(la.rows, lb.rows) and np.array_equal(la.num, lb.num)
