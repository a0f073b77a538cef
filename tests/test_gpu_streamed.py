"""A mine of a dataset that is not on the device reads its page-locked host
arrays over the host link in the cell-key pass (no device copy is kept); an
uploaded dataset is read from its device copy.  Both give the same results."""
import numpy as np
import pytest

import colo
from colo import gen

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("cfg,scale", [(0, 1.0), (1, 0.02), (3, 0.005)])
def test_streamed_and_uploaded_mines_agree(cfg, scale):
    wl = gen.config(cfg, scale=scale)
    ctx = colo.Context(0)
    ds = colo.Dataset.from_arrays(ctx, wl.x, wl.y, wl.fid, wl.bounds)
    params = colo.default_params(wl.R, wl.thr, colo.MODE_BATCHED, max_size=wl.max_size)
    streamed = ctx.mine(ds, params)
    ds.upload()
    uploaded = ctx.mine(ds, params)
    ds.evict()
    again = ctx.mine(ds, params)
    assert streamed.patterns() == uploaded.patterns() == again.patterns()
    for a, b, c in zip(streamed.levels, uploaded.levels, again.levels):
        assert np.array_equal(a.rows, b.rows) and np.array_equal(a.rows, c.rows)
        assert np.array_equal(a.num, b.num) and np.array_equal(a.num, c.num)
