"""Repeated mines on one context reach a steady device-memory footprint.

After a mine that used more of the stream-ordered pool than any before it,
the library gives the pool one free block of twice that peak, so that later
mines find free blocks instead of mapping memory mid-step.  The block must
not count as a mine's own use, or every mine would grow the pool again: here
the device's free memory, read between mines, stops changing after the first
few.
"""
import pytest

import colo
from colo import gen

pytestmark = pytest.mark.gpu


def test_repeated_mines_keep_a_steady_pool():
    torch = pytest.importorskip("torch")
    ctx = colo.Context(0)
    wl = gen.config(3, scale=0.05)            # 1,000,000 points
    ds = colo.Dataset.from_arrays(ctx, wl.x, wl.y, wl.fid, wl.bounds)
    params = colo.default_params(wl.R, wl.thr, colo.MODE_BATCHED, max_size=wl.max_size)
    free = []
    first = None
    for _ in range(7):
        res = ctx.mine(ds, params)
        patterns = res.num_candidates()
        first = patterns if first is None else first
        assert patterns == first
        torch.cuda.synchronize()
        free.append(torch.cuda.mem_get_info(0)[0])
    # the first mine sets the peak and grows the pool once; from then on nothing moves
    assert len(set(free[3:])) == 1, [f >> 20 for f in free]
