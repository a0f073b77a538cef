"""The drop-in command line, `GPU-Colocation <config.txt>` (Codes/main.cpp:8-48):
the five-line config file (colocationFinder.cpp:1077-1092), the pattern files
in the savetoFileGen format (cpp:979-997), the per-pattern report and the
reference's stdout summary line (cpp:1144)."""
import subprocess
from pathlib import Path

import numpy as np
import pytest

import colo
import oracle
from colo import _build
from helpers import resolve_ambiguous

GOLDEN = Path(__file__).resolve().parent / "golden"


def _cli():
    colo.load()
    return _build.lib_path("GPU-Colocation")


def _config(tmp_path, case):
    cfg = tmp_path / "config.txt"
    out = tmp_path / "out"
    out.mkdir()
    cfg.write_text(f"{out}/\n{GOLDEN / (case + '.param.txt')}\n{GOLDEN / (case + '.csv')}\n{out}/\nreport.txt\n")
    return cfg, out


def test_cli_is_built_and_reports_a_missing_config():
    cli = _cli()
    assert cli.exists()
    r = subprocess.run([str(cli)], capture_output=True, text=True, timeout=120)
    # without a device the constructor reports it (as the reference does); with one, the missing config
    assert r.returncode != 0
    assert "Configuration file missing" in r.stdout or "no device supporting CUDA" in (r.stdout + r.stderr)


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["small", "levels"])
def test_cli_writes_the_oracles_patterns(tmp_path, case):
    cfg, out = _config(tmp_path, case)
    r = subprocess.run([str(_cli()), str(cfg)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    # stdout: the reference's summary line, 10 comma-separated fields
    last = [l for l in r.stdout.splitlines() if l.strip()][-1]
    fields = [f.strip() for f in last.split(",")]
    assert len(fields) == 10 and fields[0].endswith(case + ".csv")
    # the oracle on the same files
    x, y, feat, bounds, names = oracle.parse_csv(GOLDEN / (case + ".csv"))
    R, thr, _ = oracle.parse_params(GOLDEN / (case + ".param.txt"))
    fid = np.asarray(feat, np.int32)
    ctx = colo.Context(0)
    res = resolve_ambiguous(ctx, x, y, fid, R)
    ref = oracle.mine(x, y, fid, bounds, R, thr, res=res)
    counts = np.bincount(oracle.feature_index(fid), minlength=len(names))
    report = {}
    for line in (out / "report.txt").read_text().splitlines()[1:]:
        k, pat, rows, nums, cnts, pi = line.split("\t")
        report[tuple(pat.split("|"))] = (int(rows), [int(v) for v in nums.split(",")],
                                         [int(v) for v in cnts.split(",")], float(pi))
    for lev in ref.levels:
        f = out / f"ColocationDegree_{lev.k}.txt"
        assert f.exists()
        want = ["( " + " | ".join(names[m] for m in lev.cand[c]) + " )" for c in np.nonzero(lev.prevalent)[0]]
        assert f.read_text().splitlines() == want
        for c in np.nonzero(lev.prevalent)[0]:
            key = tuple(names[m] for m in lev.cand[c])
            rows, nums, cnts, pi = report[key]
            assert rows == int(lev.rows[c]) and nums == [int(v) for v in lev.num[c]]
            assert cnts == [int(counts[m]) for m in lev.cand[c]]
            assert np.float32(pi) == np.float32(lev.pi[c])


@pytest.mark.gpu
def test_cli_reads_a_binary_point_file(tmp_path):
    """A config whose dataset line names a .colo file gives the same pattern files as the CSV."""
    outs = {}
    for form in ("csv", "colo"):
        d = tmp_path / form
        d.mkdir()
        data = GOLDEN / "levels.csv"
        if form == "colo":
            data = d / "levels.colo"
            colo.csv_to_binary(GOLDEN / "levels.csv", data)
        out = d / "out"
        out.mkdir()
        cfg = d / "config.txt"
        cfg.write_text(f"{out}/\n{GOLDEN / 'levels.param.txt'}\n{data}\n{out}/\nreport.txt\n")
        r = subprocess.run([str(_cli()), str(cfg)], capture_output=True, text=True, timeout=300)
        assert r.returncode == 0, r.stdout + r.stderr
        outs[form] = {f.name: f.read_text() for f in sorted(out.glob("ColocationDegree_*.txt"))}
        outs[form]["report"] = (out / "report.txt").read_text()
    assert outs["csv"] and outs["csv"] == outs["colo"]
