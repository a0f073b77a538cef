"""The oracle against golden vectors produced by the reference itself (no GPU).

tests/golden/*.golden.json.gz were recorded by running the reference's own
Begin() (its Codes/ sources compiled for the CPU, see
tests/golden/make_golden.py); the oracle must reproduce every level's
candidates, filter bounds and verdicts, row counts, participation window
sums, PI bits and instance tables (contents and row order).
"""
from pathlib import Path

import numpy as np
import pytest

import oracle
from golden_check import CASES, assert_matches_golden, load, paths


@pytest.mark.parametrize("case", CASES)
def test_oracle_reproduces_reference_golden(case):
    g = load(case)
    csv, par = paths(case)
    x, y, feat, b, names = oracle.parse_csv(str(csv))
    assert names == g["features"]
    R, thr, _ = oracle.parse_params(str(par))
    res = oracle.mine(x, y, feat.astype(np.int32), b, R, thr, keep_tables=True)
    assert res.status == 0 and res.unresolved == 0
    assert_matches_golden(res, g)


def test_golden_cases_cover_the_quirks():
    assert {"small", "levels", "apriori_break", "narrow_gx2", "wrap", "singletons", "dense"} <= set(CASES)
    # the Apriori break leaves no level-3 candidate although AB, AD and BD are prevalent
    g = load("apriori_break")
    assert [l["k"] for l in g["levels"]] == [2]


SEATTLE = Path(__file__).resolve().parent / "golden" / "seattle2012.csv.gz"


def _seattle(tmp_path):
    """The reference's real-data fixture (TestCase/Data/Seattle2012.csv, committed gzipped)."""
    import gzip
    import shutil

    p = tmp_path / "Seattle2012.csv"
    with gzip.open(SEATTLE, "rb") as src, open(p, "wb") as dst:
        shutil.copyfileobj(src, dst)
    return oracle.parse_csv(str(p))


@pytest.mark.parametrize("fast", [False, True], ids=["literal", "scaled"])
def test_seattle_experiment_log_counts(tmp_path, fast):
    # TestCase/ExperimentLog/ExperimentLog1.csv:1-2 of the reference logs, for
    # Seattle2012 with PI 0.55 and R 10: "70,83,0.843373" -- 83 candidates in
    # all levels, 70 of them pruned by the filter.
    x, y, feat, b, names = _seattle(tmp_path)
    assert len(x) == 165458 and len(names) == 13
    r = oracle.mine(x, y, feat.astype(np.int32), b, 10.0, 0.55, fast=fast)
    total = sum(len(l.cand) for l in r.levels)
    pruned = sum(int((l.passed == 0).sum()) for l in r.levels)
    assert (pruned, total) == (70, 83)
    assert f"{pruned / total:.6f}" == "0.843373"
