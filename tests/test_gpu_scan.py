"""The device-wide exclusive scan behind every offset array of the mining
kernels (one pass, decoupled look-back over 4096-item tiles), against numpy's
cumulative sum: empty and one-item inputs, sizes at and around the tile
boundaries, tens of millions of items, and 64-bit values whose sums pass 2^32."""
import numpy as np
import pytest

import colo

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    return colo.Context(0)


def _expect(v):
    """Exclusive prefix sums in uint64 (a plain [0] would promote the concatenation to float64)."""
    if len(v) == 0:
        return np.zeros(0, np.uint64), 0
    c = np.cumsum(v.astype(np.uint64), dtype=np.uint64)
    return np.concatenate([np.zeros(1, np.uint64), c[:-1]]), int(c[-1])


@pytest.mark.parametrize("n", [0, 1, 31, 4095, 4096, 4097, 8192 + 5, 1_000_003, 20_000_000])
def test_scan_u32_matches_cumsum(ctx, n):
    rng = np.random.default_rng(n)
    v = rng.integers(0, 50, n, dtype=np.uint32)
    v[rng.random(n) < 0.5] = 0           # runs of zeros, as the per-cell counts have
    got, tot = ctx.stage_scan(v)
    want, wtot = _expect(v)
    assert tot == wtot
    assert np.array_equal(got, want)


@pytest.mark.parametrize("n", [1, 4097, 3_000_001])
def test_scan_u64_wide_values(ctx, n):
    rng = np.random.default_rng(7 + n)
    v = rng.integers(0, 1 << 40, n, dtype=np.uint64)
    got, tot = ctx.stage_scan(v)
    want, wtot = _expect(v)
    assert tot == wtot
    assert n == 1 or tot > (1 << 32)
    assert np.array_equal(got, want)


def test_scan_u32_sum_past_2_32(ctx):
    v = np.full(3_000_000, 4_000, np.uint32)      # 1.2e10 in total: offsets are 64-bit
    got, tot = ctx.stage_scan(v)
    assert tot == 12_000_000_000
    assert got[-1] == 4_000 * (len(v) - 1)
