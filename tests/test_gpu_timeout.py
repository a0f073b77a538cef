"""The bounded-wait failure path, made to happen without a GPU fault.

The bucketing sort's decoupled look-back waits, with a poll limit, for each
tile's predecessors.  colo_params.reserved[1] (a test knob) makes the first
tile of the first digit pass withhold its counts and lowers the limit to a
few polls, so tile 1's wait runs out: the kernel sets the timeout flag and
finishes, the mine returns COLO_ERR_TIMEOUT, and the context keeps working --
the next mine on it matches the oracle.  No wait is unbounded and nothing
faults.
"""
import pytest

import colo
from colo import gen
from helpers import assert_same_trace, oracle_for

pytestmark = pytest.mark.gpu

COLO_ERR_TIMEOUT = 7


@pytest.mark.parametrize("polls", [1, 64])
def test_sort_wait_that_runs_out_returns_timeout_and_context_survives(polls):
    ctx = colo.Context(0)
    wl = gen.config(3, scale=0.01)          # 200,000 points: ~100 sort tiles
    ds = colo.Dataset.from_arrays(ctx, wl.x, wl.y, wl.fid, wl.bounds)
    bad = colo.default_params(wl.R, wl.thr, colo.MODE_BATCHED, max_size=wl.max_size)
    bad.reserved[1] = polls
    with pytest.raises(colo.ColoError) as e:
        ctx.mine(ds, bad)
    assert e.value.status == COLO_ERR_TIMEOUT, e.value
    for mode in (colo.MODE_BATCHED, colo.MODE_PLAIN):
        got = ctx.mine(ds, colo.default_params(wl.R, wl.thr, mode, max_size=wl.max_size))
        assert_same_trace(got, oracle_for(ctx, wl))
