"""Shared helpers of the test suite: oracle-vs-product comparison."""
from __future__ import annotations

import numpy as np

import oracle

FIELDS = ("cand", "ub", "passed", "rows", "num", "prevalent", "argmin")


def resolve_ambiguous(ctx, x, y, fid, R):
    """Device outcomes of every pair whose comparison an exact tie could flip.

    The reference's pow(float, 2) is CUDA's device function; the host oracle
    decides every other pair itself and takes these from the device
    evaluation of the reference expression.
    """
    amb = oracle.ambiguous_pairs(x, y, fid, R)
    if len(amb) == 0:
        return None
    a = (amb >> np.uint64(32)).astype(np.int64)
    b = (amb & np.uint64(0xFFFFFFFF)).astype(np.int64)
    sq = ctx.stage_sqdist(x[a], y[a], x[b], y[b])
    return amb, (sq <= np.float32(R) * np.float32(R)).astype(np.uint8)


def oracle_for(ctx, wl, keep_tables=False, max_k=None):
    res = resolve_ambiguous(ctx, wl.x, wl.y, wl.fid, wl.R) if ctx is not None else None
    out = oracle.mine(wl.x, wl.y, wl.fid, wl.bounds, wl.R, wl.thr,
                      max_k=wl.max_size if max_k is None else max_k, keep_tables=keep_tables, res=res)
    assert out.status == 0, out.status
    assert out.unresolved == 0, out.unresolved
    return out


def assert_same_trace(got, ref, tables=False, sorted_tables=False):
    assert len(got.levels) == len(ref.levels), ([l.k for l in got.levels], [l.k for l in ref.levels])
    for lg, lo in zip(got.levels, ref.levels):
        assert lg.k == lo.k
        for f in FIELDS:
            a, b = getattr(lg, f), getattr(lo, f)
            assert np.array_equal(np.asarray(a).astype(np.uint64), np.asarray(b).astype(np.uint64)), \
                f"level {lg.k} field {f} differs at {np.argwhere(np.asarray(a) != np.asarray(b))[:5].tolist()}"
        # float PI must be the same bits
        assert np.array_equal(lg.pi.view(np.uint32), lo.pi.view(np.uint32)), f"level {lg.k} PI bits differ"
        if tables:
            assert set(lg.tables) == set(lo.tables), f"level {lg.k}: tables built for different candidates"
            for c, t in lo.tables.items():
                g = lg.tables[c]
                if sorted_tables:
                    g = g[np.lexsort(g.T[::-1])]
                    t = t[np.lexsort(t.T[::-1])]
                assert np.array_equal(g, t), f"level {lg.k} candidate {c}: instance table differs"
