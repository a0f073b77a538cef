"""Pin of the float neighbour predicate.

The reference compares pow(x2-x1, 2) + pow(y2-y1, 2) <= R*R with the result
stored in a float (Codes/Utility_Inline.h:25-33).  The product kernels
evaluate that expression with the same compiler; colo_stage_sqdist runs it
in a standalone kernel.  The oracle's host model -- the correctly rounded
float of the exact dx^2 + dy^2, undecided only within a few double ulps of a
float rounding midpoint -- is checked against the device on adversarial
pairs at distance ~R: every pair away from a midpoint must get the same float
bits, and every pair the oracle calls certain the same decision.
"""
import numpy as np
import pytest

import colo
import oracle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    return colo.Context(0)


def _pairs(rng, n, scale, R, decimals=None):
    x1 = rng.uniform(0, scale, n)
    y1 = rng.uniform(0, scale, n)
    ang = rng.uniform(0, 2 * np.pi, n)
    r = R * rng.uniform(0.98, 1.02, n)
    x2 = x1 + r * np.cos(ang)
    y2 = y1 + r * np.sin(ang)
    if decimals is not None:   # CSV-like coordinates: few significant digits, many exact ties
        x1, y1, x2, y2 = (np.round(v, decimals) for v in (x1, y1, x2, y2))
    return [v.astype(np.float32) for v in (x1, y1, x2, y2)]


@pytest.mark.parametrize("scale,R,dec", [(1e6, 10.0, None), (1e6, 100.0, None), (16011.3, 10.0, 2),
                                         (1e4, 20.0, 1), (1000.0, 50.0, None), (1.0, 0.37, None),
                                         (24902.3, 10.0, 1), (2e6, 3.3, 3)])
def test_device_squared_distance_matches_oracle_model(ctx, scale, R, dec):
    rng = np.random.default_rng(int(scale) + int(R * 100))
    n = 2_000_000
    x1, y1, x2, y2 = _pairs(rng, n, scale, R, dec)
    R2 = np.float32(R) * np.float32(R)
    dev = ctx.stage_sqdist(x1, y1, x2, y2)
    le, amb, val, near = oracle.sq_decide_batch(x1, y1, x2, y2, float(R2))
    certain = ~amb
    assert np.array_equal((dev <= R2)[certain], le[certain])
    clean = ~near
    assert np.array_equal(dev[clean].view(np.uint32), val[clean].view(np.uint32))
    # at a midpoint the device returns one of the two neighbours
    nb = np.abs(dev[near].astype(np.float64) - val[near].astype(np.float64))
    assert np.all(nb <= np.abs(np.spacing(val[near])) * 1.0001)
    assert amb.mean() < 1e-3


@pytest.mark.parametrize("scale,R,dec", [(1e6, 10.0, None), (16011.3, 10.0, 2), (1e4, 20.0, 1), (1.0, 0.37, None),
                                         (2e6, 3.3, 3), (600.0, 10.0, 0)])
def test_kernel_decision_equals_reference_expression(ctx, scale, R, dec):
    # the join and level kernels decide sq <= R2 with FMAs and fall back to the
    # reference expression near the boundary: identical decisions everywhere
    rng = np.random.default_rng(int(scale) + 7)
    x1, y1, x2, y2 = _pairs(rng, 2_000_000, scale, R, dec)
    R2 = float(np.float32(R) * np.float32(R))
    sq, within = ctx.stage_within(x1, y1, x2, y2, R2)
    assert np.array_equal(within, sq <= np.float32(R2))


def test_symmetric(ctx):
    rng = np.random.default_rng(7)
    x1, y1, x2, y2 = _pairs(rng, 500_000, 1e5, 25.0, 2)
    a = ctx.stage_sqdist(x1, y1, x2, y2)
    b = ctx.stage_sqdist(x2, y2, x1, y1)
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
