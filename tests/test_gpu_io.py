"""Datasets loaded by the parallel CSV reader and from binary point files
mine exactly as the reference's golden vectors say, whatever the number of
parser threads."""
import numpy as np
import pytest

import colo
from colo import gen
from golden_check import CASES, assert_matches_golden, load, paths

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    return colo.Context(0)


def _mine(ctx, ds, par):
    p = colo.read_params(str(par))
    p.mode = colo.MODE_BATCHED
    p.keep_tables = 1
    return ctx.mine(ds, p)


@pytest.mark.parametrize("case", CASES)
def test_threaded_and_binary_loads_match_golden(ctx, case, tmp_path):
    g = load(case)
    csv, par = paths(case)
    colo.csv_to_binary(str(csv), tmp_path / "a.colo", 3)
    loads = {
        "threads=1": colo.Dataset.from_csv(ctx, str(csv), threads=1),
        "threads=5": colo.Dataset.from_csv(ctx, str(csv), threads=5),
        "binary": colo.Dataset.from_binary(ctx, tmp_path / "a.colo"),
    }
    ds = loads["threads=5"]
    ds.write_binary(tmp_path / "b.colo")
    loads["binary from dataset"] = colo.Dataset.from_binary(ctx, tmp_path / "b.colo")
    assert (tmp_path / "a.colo").read_bytes() == (tmp_path / "b.colo").read_bytes()
    for name, d in loads.items():
        assert d.names() == g["features"], name
        assert_matches_golden(_mine(ctx, d, par), g)


def test_binary_round_trip_of_host_arrays(ctx, tmp_path):
    wl = gen.config(1, scale=0.02)
    a = colo.Dataset.from_arrays(ctx, wl.x, wl.y, wl.fid, wl.bounds)
    a.write_binary(tmp_path / "w.colo")
    b = colo.Dataset.from_binary(ctx, tmp_path / "w.colo")
    x, y, raw, names, bounds = colo.read_binary(tmp_path / "w.colo")
    assert np.array_equal(x, wl.x) and np.array_equal(y, wl.y) and np.array_equal(raw, wl.fid)
    assert b.names() == a.names() == names
    p = colo.default_params(wl.R, wl.thr, colo.MODE_BATCHED, max_size=wl.max_size)
    ra, rb = ctx.mine(a, p), ctx.mine(b, p)
    assert ra.patterns() == rb.patterns()
    for la, lb in zip(ra.levels, rb.levels):
        assert np.array_equal(la.rows, lb.rows) and np.array_equal(la.num, lb.num)


def test_corrupt_binary_is_rejected(ctx, tmp_path):
    wl = gen.config(0)
    colo.Dataset.from_arrays(ctx, wl.x, wl.y, wl.fid, wl.bounds).write_binary(tmp_path / "c.colo")
    data = (tmp_path / "c.colo").read_bytes()
    (tmp_path / "t.colo").write_bytes(data[:-3])
    with pytest.raises(colo.ColoError) as e:
        colo.Dataset.from_binary(ctx, tmp_path / "t.colo")
    assert e.value.status == colo.ERR_PARSE
    (tmp_path / "m.colo").write_bytes(b"NOTCOLO!" + data[8:])
    with pytest.raises(colo.ColoError):
        colo.Dataset.from_binary(ctx, tmp_path / "m.colo")
