"""Full-size parity fixtures: the oracle's mining trace of the benchmark's
own workloads, for the GPU test tests/test_gpu_fulltrace.py.

    python tests/golden/make_full_traces.py [case ...]

Cases: config3 (20,000,000 points, the workload bench.py times), config1
(1,000,000 points), config4 at scale 0.005 (500,000 points with the dense
sigma = 5 hotspot at full density: levels up to 8, 2.8e9 rows in all) and the
reference's real-data fixture Seattle2012
(seattle2012.csv.gz beside this script, copied from the reference's
TestCase/Data/) at R = 10 with PI 0.3 (its parameter.txt) and 0.55 (its
experiment log).  The trace is the scaled oracle's (oracle_mine_fast, equal
to the literal restatement and to the reference's golden vectors in
tests/test_cpu_oracle.py): per level the candidates, filter bounds and
verdicts, row counts, participation numerators, PI bits, prevalence and
argmin, plus the SHA-256 of every instance table built (row-major u32 in the
reference's row order).  The synthetic datasets are recorded by digest, the
generator's output being the same bits on every platform.  Pairs whose
comparison with R^2 a float tie could flip are listed with the outcome the
trace assumed; the GPU test checks the device evaluates them the same way.
"""
from __future__ import annotations

import gzip
import hashlib
import json
import shutil
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
for p in (ROOT / "gpu-colocationmininig_gb300", ROOT / "oracle"):
    sys.path.insert(0, str(p))

import oracle  # noqa: E402

SEATTLE = HERE / "seattle2012.csv.gz"
CASES = {
    "config3": ("gen", 3, 1.0),
    "config1": ("gen", 1, 1.0),
    "config4_0.005": ("gen", 4, 0.005),
    "seattle_pi0.3": ("csv", SEATTLE, 0.3),
    "seattle_pi0.55": ("csv", SEATTLE, 0.55),
}


def dataset_digest(x, y, fid, bounds) -> str:
    h = hashlib.sha256()
    for a, t in ((x, "<f4"), (y, "<f4"), (fid, "<i4"), (bounds, "<f4")):
        h.update(np.ascontiguousarray(a).astype(t).tobytes())
    return h.hexdigest()


def table_digest(t: np.ndarray) -> bytes:
    return hashlib.sha256(np.ascontiguousarray(t, np.uint32).reshape(-1).astype("<u4").tobytes()).digest()


def read_seattle():
    """x, y, raw ids, bounds of the gzipped Seattle2012 CSV (parsed by the oracle's reader)."""
    with tempfile.TemporaryDirectory() as d:
        csv = Path(d) / "Seattle2012.csv"
        with gzip.open(SEATTLE, "rb") as src, open(csv, "wb") as dst:
            shutil.copyfileobj(src, dst)
        x, y, feat, b, names = oracle.parse_csv(str(csv))
    return x, y, feat.astype(np.int32), b, names


def load_case(name):
    kind, src, arg = CASES[name]
    if kind == "gen":
        from colo import gen

        wl = gen.config(src, scale=arg)
        return wl.x, wl.y, wl.fid, wl.bounds, wl.R, wl.thr, wl.max_size
    x, y, fid, b, _ = read_seattle()
    return x, y, fid, b, 10.0, arg, 0


def trace(name):
    x, y, fid, b, R, thr, max_k = load_case(name)
    t0 = time.time()
    amb = oracle.ambiguous_pairs(x, y, fid, R)
    le = np.zeros(len(amb), np.uint8)
    if len(amb):
        a = (amb >> np.uint64(32)).astype(np.int64)
        c = (amb & np.uint64(0xFFFFFFFF)).astype(np.int64)
        le, _, _, _ = oracle.sq_decide_batch(x[a], y[a], x[c], y[c], np.float32(R) * np.float32(R))
        le = le.astype(np.uint8)
    res = oracle.mine(x, y, fid, b, R, thr, max_k=max_k, keep_tables=True,
                      res=(amb, le) if len(amb) else None, fast=True)
    assert res.status == 0 and res.unresolved == 0, (res.status, res.unresolved)
    kind, src, arg = CASES[name]
    out = {"meta": np.frombuffer(json.dumps({
        "case": name, "config": src if kind == "gen" else None, "scale": arg if kind == "gen" else None,
        "points": int(len(x)), "digest": dataset_digest(x, y, fid, b), "R": float(R),
        "thr": float(thr), "max_size": int(max_k), "levels": [int(l.k) for l in res.levels],
        "candidates": res.num_candidates(), "prevalent": len(res.patterns())}).encode(), np.uint8),
        "amb_keys": amb.astype(np.uint64), "amb_le": le}
    for li, lev in enumerate(res.levels):
        p = f"L{li}_"
        out[p + "cand"] = lev.cand
        out[p + "ub"] = lev.ub
        out[p + "pass"] = lev.passed
        out[p + "rows"] = lev.rows
        out[p + "num"] = lev.num
        out[p + "pi"] = lev.pi.view(np.uint32)
        out[p + "prevalent"] = lev.prevalent
        out[p + "argmin"] = lev.argmin
        keys = np.array(sorted(lev.tables), np.int64)
        out[p + "tab_cand"] = keys
        out[p + "tab_rows"] = np.array([lev.tables[c].shape[0] for c in keys], np.uint64)
        out[p + "tab_sha"] = np.frombuffer(b"".join(table_digest(lev.tables[c]) for c in keys), np.uint8)
    np.savez_compressed(HERE / f"full_{name}.trace.npz", **out)
    print(f"{name}: {len(x)} points, levels {[l.k for l in res.levels]}, {res.num_candidates()} candidates, "
          f"{len(res.patterns())} prevalent, {len(amb)} ambiguous pairs, {time.time() - t0:.1f} s", flush=True)


if __name__ == "__main__":
    for name in sys.argv[1:] or list(CASES):
        trace(name)
