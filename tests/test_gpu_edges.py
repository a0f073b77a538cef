"""GPU parity on hand-built edge cases of the reference's semantics."""
import numpy as np
import pytest

import colo
from colo.gen import Workload
from helpers import assert_same_trace, oracle_for

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    return colo.Context(0)


def _wl(name, pts, bounds, R, thr, max_size=0):
    pts = sorted(pts, key=lambda p: p[0])   # grouped by feature, stable
    fid = np.array([p[0] for p in pts], np.int32)
    x = np.array([p[1] for p in pts], np.float32)
    y = np.array([p[2] for p in pts], np.float32)
    return Workload(name, x, y, fid, np.array(bounds, np.float32), R, thr, [], max_size)


def _check(ctx, wl, modes=(colo.MODE_PLAIN, colo.MODE_BATCHED)):
    ds = colo.Dataset.from_arrays(ctx, wl.x, wl.y, wl.fid, wl.bounds)
    ref = oracle_for(ctx, wl, keep_tables=True)
    for m in modes:
        got = ctx.mine(ds, colo.default_params(wl.R, wl.thr, m, max_size=wl.max_size, keep_tables=True))
        assert_same_trace(got, ref, tables=True)
    return ref


def _cluster_points(rng, nfeat, nclusters, spread, width, per=1):
    pts = []
    for _ in range(nclusters):
        cx, cy = rng.uniform(0, width, 2)
        for f in range(nfeat):
            for _ in range(per):
                pts.append((f, cx + rng.uniform(-spread, spread), cy + rng.uniform(-spread, spread)))
    return pts


def test_tiny_dataset(ctx):
    wl = _wl("tiny", [(1, 1.0, 1.0), (1, 50.0, 50.0), (2, 2.0, 2.0), (3, 3.0, 1.0), (3, 90.0, 90.0)],
             [0, 0, 100, 100], 10.0, 0.3)
    ref = _check(ctx, wl)
    assert ref.levels[0].prevalent.any()


def test_single_column_grid_has_no_neighbours(ctx):
    # gx = 1: the reference's neighbour-cell rule drops every cell
    rng = np.random.default_rng(3)
    pts = [(f, rng.uniform(0, 5), rng.uniform(0, 100)) for f in range(3) for _ in range(30)]
    wl = _wl("gx1", pts, [0, 0, 5, 100], 10.0, 0.1)
    ref = _check(ctx, wl)
    assert all(r == 0 for r in ref.levels[0].rows)


def test_two_column_grid(ctx):
    # gx = 2: only same-column neighbours are visited
    rng = np.random.default_rng(4)
    pts = [(f, rng.uniform(0, 15), rng.uniform(0, 200)) for f in range(4) for _ in range(60)]
    _check(ctx, _wl("gx2", pts, [0, 0, 15, 200], 10.0, 0.1))


def test_points_on_max_bound_wrap_to_next_row(ctx):
    # x == maxX with (maxX-minX)/R integral: the cell index equals gx and wraps
    pts = [(0, 100.0, 35.0), (1, 99.0, 35.0), (1, 100.0, 45.0), (2, 0.5, 45.0), (0, 3.0, 3.0), (2, 5.0, 5.0)]
    _check(ctx, _wl("wrap", pts, [0, 0, 100, 100], 10.0, 0.1))


def test_points_below_min_are_clamped(ctx):
    pts = [(0, -3.0, 5.0), (1, 2.0, 5.0), (0, 15.0, -2.0), (1, 15.0, 3.0), (2, 1.0, 1.0)]
    _check(ctx, _wl("clamp", pts, [0, 0, 50, 50], 10.0, 0.1))


def test_duplicates_singletons_and_exact_distances(ctx):
    pts = [(0, 10.0, 10.0), (1, 10.0, 10.0), (2, 16.0, 18.0), (3, 40.0, 40.0), (4, 46.0, 48.0),
           (4, 10.0, 20.0), (5, 20.0, 10.0)]
    _check(ctx, _wl("dups", pts, [0, 0, 60, 60], 10.0, 0.2))


def test_large_patterns_generic_kernel_path(ctx):
    # thr = 0: everything passes; sizes above 8 use the runtime-size kernels and
    # the filter's zero bound for members j >= 8
    rng = np.random.default_rng(5)
    pts = _cluster_points(rng, 10, 6, 1.0, 300.0)
    _check(ctx, _wl("k10", pts, [0, 0, 300, 300], 5.0, 0.0))


def test_dense_cells_and_skewed_sizes(ctx):
    # one blob where every point neighbours every other: the level-5 table is
    # the product of the five feature counts (8*16*24*32*40 = 3.9e6 rows)
    rng = np.random.default_rng(6)
    pts = _cluster_points(rng, 5, 20, 4.0, 200.0, per=2)
    pts += [(f, rng.normal(100, 1), rng.normal(100, 1)) for f in range(5) for _ in range(8 * (f + 1))]
    _check(ctx, _wl("dense", pts, [0, 0, 200, 200], 6.0, 0.2))


def test_out_of_grid_point_is_an_error(ctx):
    pts = [(0, 1.0, 1.0), (1, 2.0, 1.0), (1, 5.0, 5000.0)]
    wl = _wl("out", pts, [0, 0, 100, 100], 10.0, 0.1)
    ds = colo.Dataset.from_arrays(ctx, wl.x, wl.y, wl.fid, wl.bounds)
    with pytest.raises(colo.ColoError) as e:
        ctx.mine(ds, colo.default_params(wl.R, wl.thr))
    assert e.value.status == 4
