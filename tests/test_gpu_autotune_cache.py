"""The widened autotuner: join lanes per anchor, candidates per level-filter
unit, level-kernel threads per block and the level queue (one warp per
chunk, or a persistent grid taking chunks by ticket), kept in a cache file keyed by the
dataset's shape.  Every setting of every knob gives identical traces, and a
second tuning of the same shape reads the cache instead of timing."""
import itertools

import pytest

import colo
from colo import gen
from helpers import assert_same_trace, oracle_for

pytestmark = pytest.mark.gpu


def test_every_tuned_setting_gives_identical_traces():
    ctx = colo.Context(0)
    wl = gen.config(3, scale=0.01)
    ds = colo.Dataset.from_arrays(ctx, wl.x, wl.y, wl.fid, wl.bounds)
    ref = oracle_for(ctx, wl, keep_tables=True)
    ctx.set_model(colo.load_model())
    for fu, lb, lq in itertools.product(colo.FILTER_UNITS, colo.LEVEL_BLOCKS, (0, 1)):
        ctx.set_tuning(join_group=4, filter_unit=fu, level_block=lb, level_queue=lq)
        assert ctx.tuning()["filter_unit"] == fu and ctx.tuning()["level_block"] == lb
        for mode in (colo.MODE_BATCHED, colo.MODE_LEARNED):
            got = ctx.mine(ds, colo.default_params(wl.R, wl.thr, mode, max_size=wl.max_size, keep_tables=True,
                                                   single_pass=mode == colo.MODE_LEARNED))
            assert_same_trace(got, ref, tables=True)
    with pytest.raises(colo.ColoError):
        ctx.set_tuning(filter_unit=12)


def test_tuning_cache_round_trips(tmp_path):
    cache = tmp_path / "tuning.txt"
    ctx = colo.Context(0)
    wl = gen.config(3, scale=0.02)
    ds = colo.Dataset.from_arrays(ctx, wl.x, wl.y, wl.fid, wl.bounds)
    prm = colo.default_params(wl.R, wl.thr, colo.MODE_BATCHED, max_size=wl.max_size)
    first = ctx.autotune_all(ds, prm, cache=str(cache))
    assert not first["from_cache"]
    assert first["join_group"] in colo.JOIN_WIDTHS and first["filter_unit"] in colo.FILTER_UNITS
    assert first["level_block"] in colo.LEVEL_BLOCKS
    assert cache.read_text().count("colo-tune 2 ") == 1
    ctx2 = colo.Context(0)
    ds2 = colo.Dataset.from_arrays(ctx2, wl.x, wl.y, wl.fid, wl.bounds)
    second = ctx2.autotune_all(ds2, prm, cache=str(cache))
    assert second["from_cache"]
    keys = ("join_group", "filter_unit", "level_block", "level_queue")
    assert {k: second[k] for k in keys} == {k: first[k] for k in keys}
    assert ctx2.tuning()["filter_unit"] == first["filter_unit"]
    # another R is another shape: tuned and appended
    prm2 = colo.default_params(wl.R * 0.5, wl.thr, colo.MODE_BATCHED, max_size=wl.max_size)
    third = ctx2.autotune_all(ds2, prm2, cache=str(cache))
    assert not third["from_cache"]
    assert cache.read_text().count("colo-tune 2 ") == 2
