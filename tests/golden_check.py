"""Comparison of a mining trace with a golden vector produced by the reference."""
from __future__ import annotations

import gzip
import hashlib
import json
from pathlib import Path

import numpy as np

GOLDEN = Path(__file__).resolve().parent / "golden"
CASES = sorted(p.name[: -len(".golden.json.gz")] for p in GOLDEN.glob("*.golden.json.gz"))


def load(case: str) -> dict:
    with gzip.open(GOLDEN / f"{case}.golden.json.gz", "rt") as f:
        return json.load(f)


def paths(case: str):
    return GOLDEN / f"{case}.csv", GOLDEN / f"{case}.param.txt"


def assert_matches_golden(trace, golden: dict):
    """trace: levels with cand, ub, passed, rows, num, pi, tables (row-major)."""
    gl = golden["levels"]
    assert [l.k for l in trace.levels] == [l["k"] for l in gl]
    for lev, g in zip(trace.levels, gl):
        k = g["k"]
        C = len(g["cand"]) // k
        assert np.array_equal(lev.cand, np.array(g["cand"]).reshape(C, k)), f"level {k}: candidates"
        assert np.array_equal(lev.ub, np.array(g["ub"]).reshape(C, k)), f"level {k}: filter bounds"
        assert np.array_equal(lev.passed.astype(int), np.array(g["pass"])), f"level {k}: filter verdicts"
        refined = {int(c): v for c, v in g["refined"].items()}
        for c in range(C):
            if c in refined:
                r = refined[c]
                assert int(lev.rows[c]) == r["rows"], f"level {k} cand {c}: rows"
                assert lev.num[c].tolist() == r["num"], f"level {k} cand {c}: window sums"
                assert int(lev.pi[c:c + 1].view(np.uint32)[0]) == r["pi_bits"], f"level {k} cand {c}: PI bits"
            else:
                assert int(lev.rows[c]) == 0 and not lev.prevalent[c]
        # instance tables, in the reference's row order
        mine = {tuple(int(v) for v in lev.cand[c]): t for c, t in lev.tables.items()}
        built = [t for t in g["tables"] if t["nrows"] > 0]
        for t in built:
            key = tuple(t["members"])
            assert key in mine, f"level {k}: table {key} not built"
            rows = np.ascontiguousarray(mine[key], np.uint32)
            assert rows.shape[0] == t["nrows"], f"level {k} table {key}: rows"
            digest = hashlib.sha256(rows.reshape(-1).astype("<u4").tobytes()).hexdigest()
            assert digest == t["sha256"], f"level {k} table {key}: row content or order"
