"""Cells whose neighbourhood run lists hold more than 512 entries (a dense 3x3
block with many features) are filled by the warp-per-cell list kernel; the
neighbour lists the join builds from them match the oracle."""
import numpy as np
import pytest

import colo
import oracle
from helpers import resolve_ambiguous

pytestmark = pytest.mark.gpu


def dense_block(F, per, seed):
    """Every feature has `per` points in a 30 x 30 square (a 3x3 block of
    R = 10 cells) and two uniform points elsewhere; points grouped by feature."""
    rng = np.random.default_rng(seed)
    xs, ys, fs = [], [], []
    for f in range(F):
        x = np.concatenate([100.0 + rng.uniform(0.0, 30.0, per), rng.uniform(0.0, 400.0, 2)])
        y = np.concatenate([100.0 + rng.uniform(0.0, 30.0, per), rng.uniform(0.0, 400.0, 2)])
        xs.append(x)
        ys.append(y)
        fs.append(np.full(per + 2, f))
    x = np.concatenate(xs).astype(np.float32)
    y = np.concatenate(ys).astype(np.float32)
    fid = np.concatenate(fs).astype(np.int32)
    return x, y, fid, np.array([0.0, 0.0, 400.0, 400.0], np.float32)


@pytest.mark.parametrize("F,per", [(100, 9), (700, 4)])
def test_long_lists_match_oracle(F, per):
    x, y, fid, bounds = dense_block(F, per, seed=F)
    R = 10.0
    ctx = colo.Context(0)
    ds = colo.Dataset.from_arrays(ctx, x, y, fid, bounds)
    offs, nbr = ctx.stage_neighbors(ds, R)
    res = resolve_ambiguous(ctx, x, y, fid, R)
    o_offs, o_nbr, unres = oracle.neighbors(x, y, fid, bounds, R, res=res)
    assert unres == 0
    assert np.array_equal(offs, o_offs)
    assert np.array_equal(nbr, o_nbr)
    assert nbr.size > 0
