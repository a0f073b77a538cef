"""Generate the golden vectors in tests/golden/ from the reference itself.

Run where the reference tree is available:
    python tests/golden/make_golden.py /path/to/reference/Codes
or with COLO_REFERENCE_ROOT set to the reference project's root.

Each case is a small seeded point set written in the reference's CSV format
(<name>.csv) with its parameter file; oracle/ref_emu/build_ref.py compiles
the reference's own Codes/ sources for the CPU and its harness runs the
reference's Begin() on the case, recording every level's candidates, filter
bounds and verdicts, row counts, participation window sums, PI bits and
instance tables (<name>.golden.json.gz).

Coordinates are integers below 4096, so every squared coordinate difference
is exact in float and no square is a rounding tie: the CPU build's squares
equal the device's bit for bit.  Point counts satisfy the reference's
bucketing launch (N/1000 blocks of 1024 threads must cover every point).
"""
from __future__ import annotations

import gzip
import hashlib
import json
import shutil
import subprocess
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT / "oracle" / "ref_emu"))


def pad_to_launch_cover(fid, x, y, bounds, rng):
    """Add isolated points of one extra feature (far corner, no neighbours)
    until N/1000 blocks of 1024 threads cover every point."""
    n = len(x)
    target = max(1000, n)
    while (target // 1000) * 1024 < target:
        target += 1
    extra = target - n
    if extra:
        fid = np.concatenate([fid, np.full(extra, int(fid.max()) + 1)])
        x = np.concatenate([x, np.full(extra, float(bounds[2]) - 1.0)])
        y = np.concatenate([y, np.full(extra, float(bounds[3]) - 1.0)])
    return fid, x, y


def write_case(name, fid, x, y, bounds, R, thr):
    fid, x, y = pad_to_launch_cover(fid, x, y, bounds, None)
    order = np.argsort(fid, kind="stable")
    fid, x, y = fid[order], x[order], y[order]
    n = len(x)
    assert n >= 1000 and (n // 1000) * 1024 >= n, n
    with open(HERE / f"{name}.csv", "w") as f:
        f.write(f"{n}\n")
        for i in range(n):
            f.write(f"{int(fid[i])},{x[i]:.9g},{y[i]:.9g}\n")
        f.write("\n" + ",".join(f"{v:.9g}" for v in bounds))
    (HERE / f"{name}.param.txt").write_text(f"{R:g}\n{thr:g}\n1\n")


def planted(rng, groups, seeds, sigma, width, pad_feats=(), pad_n=0, ids=None):
    fid, xs, ys = [], [], []
    for g, ns in zip(groups, seeds):
        for _ in range(ns):
            cx, cy = rng.integers(0, width, 2)
            for f in g:
                fid.append(f)
                xs.append(cx + round(rng.normal(0, sigma)))
                ys.append(cy + round(rng.normal(0, sigma)))
    for f in pad_feats:
        for _ in range(pad_n):
            fid.append(f)
            xs.append(rng.integers(0, width))
            ys.append(rng.integers(0, width))
    fid = np.array(fid)
    x = np.clip(np.array(xs, float), 0, width - 1)
    y = np.clip(np.array(ys, float), 0, width - 1)
    if ids is not None:
        fid = np.array([ids[f] for f in fid])
    return fid, x, y


def cases():
    rng = np.random.default_rng(20260101)
    out = []
    # planted pairs/triples among uniform noise
    f, x, y = planted(rng, [(0, 1), (2, 3, 4)], [300, 250], 3.0, 600, pad_feats=range(6), pad_n=250)
    out.append(("small", f, x, y, [0, 0, 600, 600], 10.0, 0.3))
    # deep levels: a 5-pattern and a 3-pattern with tight clusters
    f, x, y = planted(rng, [(0, 1, 2, 3, 4), (5, 6, 7)], [300, 300], 1.5, 500, pad_feats=range(8), pad_n=80)
    out.append(("levels", f, x, y, [0, 0, 500, 500], 10.0, 0.25))
    # Apriori break: AB, AC, AD, BD prevalent, BC not -> ABD is never generated
    f, x, y = planted(rng, [(0, 1, 3), (0, 2)], [350, 350], 1.0, 600, pad_feats=(4,), pad_n=300)
    out.append(("apriori_break", f, x, y, [0, 0, 600, 600], 10.0, 0.3))
    # two grid columns: only same-column neighbour cells are visited
    g = rng.integers(0, 4, 1000)
    out.append(("narrow_gx2", g, rng.integers(0, 15, 1000).astype(float), rng.integers(0, 600, 1000).astype(float),
                [0, 0, 15, 600], 10.0, 0.1))
    # points on x == maxX with an integral width: cell index gx wraps to the next row
    g = rng.integers(0, 4, 1000)
    xx = np.where(rng.random(1000) < 0.3, 100.0, rng.integers(90, 100, 1000).astype(float))
    out.append(("wrap", g, xx, rng.integers(0, 100, 1000).astype(float), [0, 0, 100, 100], 10.0, 0.1))
    # (points below the lower bounds are not a case here: the reference converts
    # a negative float to unsigned, which saturates to 0 on the device but is
    # undefined in a CPU build)
    rng.integers(0, 4, 1000)
    rng.integers(0, 120, 1000)
    rng.integers(0, 120, 1000)
    # single- and double-instance features next to common ones (window quirks)
    fs = np.array([7] * 1 + [9] * 2 + [11] * 497 + [13] * 500)
    cx = rng.integers(0, 60, 1000).astype(float)
    cy = rng.integers(0, 60, 1000).astype(float)
    cx[:3] = [20, 21, 20]
    cy[:3] = [20, 20, 21]
    out.append(("singletons", fs, cx, cy, [0, 0, 60, 60], 10.0, 0.001))
    # dense cells: many instances of several features per cell
    f, x, y = planted(rng, [(0, 1, 2)], [120], 4.0, 60, pad_feats=range(5), pad_n=150)
    out.append(("dense", f, x, y, [0, 0, 60, 60], 10.0, 0.2))
    return out


def main(codes: str):
    import build_ref

    exe = build_ref.build(codes)
    work = ROOT / "oracle" / "_ref" / "run"
    work.mkdir(parents=True, exist_ok=True)
    for name, fid, x, y, bounds, R, thr in cases():
        write_case(name, fid, x, y, bounds, R, thr)
        shutil.copy(HERE / f"{name}.csv", work / "pts.csv")
        shutil.copy(HERE / f"{name}.param.txt", work / "parameter.txt")
        (work / "config.txt").write_text("./\n./parameter.txt\n./pts.csv\n./\nout.txt\n")
        r = subprocess.run([str(exe), "config.txt", "golden.json"], cwd=work, capture_output=True, text=True,
                           timeout=1800)
        if r.returncode:
            raise RuntimeError(f"{name}: reference harness failed\n{r.stdout[-2000:]}\n{r.stderr[-2000:]}")
        data = json.loads((work / "golden.json").read_text())
        for lev in data["levels"]:   # large tables: row count + digest of the rows in order
            for t in lev["tables"]:
                rows = np.asarray(t["rows"], np.uint32)
                t["nrows"] = len(rows) // lev["k"]
                t["sha256"] = hashlib.sha256(rows.astype("<u4").tobytes()).hexdigest()
                if len(rows) > 20000:
                    del t["rows"]
        data["case"] = name
        data["R"] = R
        data["thr"] = thr
        with gzip.open(HERE / f"{name}.golden.json.gz", "wt") as f:
            json.dump(data, f)
        print(name, [(l["k"], len(l["cand"]) // l["k"], len(l["refined"]), len(l["tables"])) for l in data["levels"]])


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else None)
