"""Instance tables placed in pinned host memory (mapped into the device, read
and written by the level kernels over the host link) give the same result as
device-resident tables, in both table-building forms."""
import numpy as np
import pytest

import colo
from colo import gen

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = colo.Context(0)
    yield c
    c.set_model(None)


@pytest.mark.parametrize("mode", [colo.MODE_BATCHED, colo.MODE_LEARNED, colo.MODE_PLAIN])
def test_host_tables_are_identical(ctx, mode):
    wl = gen.config(1, scale=0.02)
    ds = colo.Dataset.from_arrays(ctx, wl.x, wl.y, wl.fid, wl.bounds)
    ctx.set_model(colo.load_model() if mode == colo.MODE_LEARNED else None)
    a = ctx.mine(ds, colo.default_params(wl.R, wl.thr, mode, max_size=wl.max_size, keep_tables=True))
    b = ctx.mine(ds, colo.default_params(wl.R, wl.thr, mode, max_size=wl.max_size, keep_tables=True,
                                         host_tables=True))
    assert a.counters["host_table_bytes"] == 0
    assert b.counters["host_table_bytes"] > 0
    assert len(a.levels) == len(b.levels) >= 3
    for la, lb in zip(a.levels, b.levels):
        assert np.array_equal(la.cand, lb.cand) and np.array_equal(la.rows, lb.rows)
        assert np.array_equal(la.num, lb.num) and np.array_equal(la.prevalent, lb.prevalent)
        assert np.array_equal(la.pi.view(np.uint32), lb.pi.view(np.uint32))
        assert set(la.tables) == set(lb.tables)
        for c, t in la.tables.items():
            u = lb.tables[c]
            assert np.array_equal(u[np.lexsort(u.T[::-1])], t[np.lexsort(t.T[::-1])])
