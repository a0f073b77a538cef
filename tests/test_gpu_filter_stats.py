"""The level filter's per-candidate statistics -- full quads and cells in
U_c, two of the cost model's inputs -- against a brute-force count.

A quad is a 2x2 block of grid cells with lower corner (bx, by),
0 <= bx <= gx-2, 0 <= by <= gy-2; it is full for a candidate when each of
its first min(k, 8) members has a point in one of the quad's cells
(DeviceProcess_Kernel.h:469-509).  U_c is the set of occupied cells of full
quads.  The counts reach the features as log1p(count) in float; for counts
below 10^5 expm1 of that float rounds back to the count."""
import numpy as np
import pytest

import colo
from colo import gen

pytestmark = pytest.mark.gpu


def _brute_stats(cell_of, fid_local, gx, gy, cands, nfeat):
    occ_id, inv = np.unique(cell_of.astype(np.int64), return_inverse=True)
    cf = np.zeros((len(occ_id), nfeat), bool)
    cf[inv, fid_local] = True
    ci, cj = occ_id % gx, occ_id // gx
    pos = {int(c): n for n, c in enumerate(occ_id.tolist())}
    # every valid quad with an occupied cell
    qs = set()
    for i, j in zip(ci.tolist(), cj.tolist()):
        for bx in (i - 1, i):
            for by in (j - 1, j):
                if 0 <= bx <= gx - 2 and 0 <= by <= gy - 2:
                    qs.add((bx, by))
    qs = np.array(sorted(qs), np.int64).reshape(-1, 2)
    members = np.full((len(qs), 4), -1, np.int64)
    for e, (ex, ey) in enumerate(((0, 0), (1, 0), (0, 1), (1, 1))):
        ids = (qs[:, 1] + ey) * gx + qs[:, 0] + ex
        members[:, e] = [pos.get(int(v), -1) for v in ids.tolist()]
    qf = np.zeros((len(qs), nfeat), bool)
    for e in range(4):
        ok = members[:, e] >= 0
        qf[ok] |= cf[members[ok, e]]
    out = []
    for mem in cands:
        m = mem[: min(len(mem), 8)]
        full = qf[:, m].all(axis=1)
        cells = np.unique(members[full].ravel())
        out.append((int(full.sum()), int((cells >= 0).sum())))
    return np.array(out, np.int64).reshape(-1, 2)


@pytest.mark.parametrize("cfg,scale,thr", [(3, 0.004, 0.1), (1, 0.02, None)])
def test_filter_statistics_match_brute_force(cfg, scale, thr):
    ctx = colo.Context(0)
    wl = gen.config(cfg, scale=scale)
    thr = wl.thr if thr is None else thr
    ds = colo.Dataset.from_arrays(ctx, wl.x, wl.y, wl.fid, wl.bounds)
    res = ctx.mine(ds, colo.default_params(wl.R, thr, colo.MODE_BATCHED, max_size=wl.max_size, features=True))
    cell_of, _, _, _ = ctx.stage_cells(ds, wl.R)
    R = np.float32(wl.R)
    b = np.asarray(wl.bounds, np.float32)
    gx = int(np.ceil((b[2] - b[0]) / R))
    gy = int(np.ceil(((b[3] + R) - b[1]) / R))
    starts = np.ones(len(wl.fid), bool)
    starts[1:] = wl.fid[1:] != wl.fid[:-1]
    fid_local = np.cumsum(starts) - 1
    checked = 0
    for lev in res.levels:
        if lev.k < 3 or len(lev.cand) == 0:
            continue
        want = _brute_stats(cell_of, fid_local, gx, gy, lev.cand.astype(np.int64), int(fid_local.max()) + 1)
        got_quads = np.rint(np.expm1(lev.features[:, 19].astype(np.float64))).astype(np.int64)
        got_cells = np.rint(np.expm1(lev.features[:, 18].astype(np.float64))).astype(np.int64)
        assert want[:, 1].max() < 100_000
        assert np.array_equal(got_quads, want[:, 0]), lev.k
        assert np.array_equal(got_cells, want[:, 1]), lev.k
        checked += len(lev.cand)
    assert checked > 0
