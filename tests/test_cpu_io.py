"""The parallel CSV reader and the binary point file, on the host.

colo_csv_to_binary parses a dataset with a chosen number of threads and
writes the binary point file; read_binary reads that file back with numpy.
Whatever the thread count, the result must be the serial reading of
populateData (colocationFinder.cpp:139-254) as the oracle restates it: the
same points (bit for bit), the same feature grouping (a change of id starts
a feature) and names (the id token at each group start), the same bounds,
and on malformed input the same verdict and the same line number.
"""
import numpy as np
import pytest

import colo
import oracle

THREADS = [1, 2, 3, 7, 16, 0]


def _groups(raw):
    start = np.ones(len(raw), bool)
    start[1:] = raw[1:] != raw[:-1]
    return np.cumsum(start) - 1


def _check_same(path, tmp_path, threads):
    x, y, feat, b, names = oracle.parse_csv(path)
    out = tmp_path / f"t{threads}.colo"
    colo.csv_to_binary(path, out, threads)
    gx, gy, raw, gnames, gb = colo.read_binary(out)
    assert np.array_equal(gx.view(np.uint32), x.view(np.uint32))
    assert np.array_equal(gy.view(np.uint32), y.view(np.uint32))
    assert np.array_equal(_groups(raw), feat)
    assert gnames == names
    assert np.array_equal(gb.view(np.uint32), b.view(np.uint32))


def _write(path, text):
    path.write_bytes(text.encode() if isinstance(text, str) else text)
    return str(path)


def _dataset(n, seed, crlf=False, quote_every=0, pad_names=False, trailer=""):
    rng = np.random.default_rng(seed)
    fid = np.sort(rng.integers(0, max(2, n // 50), n))
    fid[n // 3:n // 2] = fid[n // 3]                  # a long group across thread cuts
    if n > 10:
        fid[-5:] = fid[0]                             # an id that comes back: a new feature
    xs = rng.uniform(-1000, 1000, n).astype(np.float32).tolist()
    ys = rng.uniform(-1000, 1000, n).astype(np.float32).tolist()
    nl = "\r\n" if crlf else "\n"
    lines = [str(n)]
    for i in range(n):
        tok = f"{fid[i]:04d}" if pad_names else str(fid[i])
        if quote_every and i % quote_every == 0:
            lines.append(f'"{tok}",{xs[i]!r},"{ys[i]!r}"')
        else:
            lines.append(f"{tok},{xs[i]!r},{ys[i]!r}")
    lines.append("")
    lines.append("-1000,-1000,1000,1000" + trailer)
    return nl.join(lines) + nl


@pytest.mark.parametrize("threads", THREADS)
@pytest.mark.parametrize("form", ["plain", "crlf", "quoted", "names"])
def test_parallel_parse_matches_serial(tmp_path, threads, form):
    text = _dataset(5000, 11, crlf=form == "crlf", quote_every=7 if form == "quoted" else 0,
                    pad_names=form == "names")
    _check_same(_write(tmp_path / "d.csv", text), tmp_path, threads)


@pytest.mark.parametrize("threads", [1, 4, 0])
def test_golden_fixtures(tmp_path, threads):
    from pathlib import Path
    for csv in sorted((Path(__file__).parent / "golden").glob("*.csv")):
        _check_same(str(csv), tmp_path, threads)


@pytest.mark.parametrize("threads", [1, 5, 64])
def test_text_after_the_empty_line(tmp_path, threads):
    """Everything after the bounds line is ignored, and a malformed point after the empty line
    is not an error (the serial reading stops at the empty line)."""
    text = _dataset(300, 3) + "garbage\n1,2\n\n\n7,7,7\n"
    _check_same(_write(tmp_path / "d.csv", text), tmp_path, threads)


@pytest.mark.parametrize("threads", [1, 2, 9])
def test_small_and_edge_files(tmp_path, threads):
    cases = {
        "one": "1\n5,1.5,2.5\n\n0,0,10,10\n",
        "no_newline_at_end": "2\n5,1,2\n6,3,4\n\n0,0,10,10",
        "spaces": "3\n 12 ,  1.5, 2\n12,1e1,-0\n+13,0x10,inf\n\n0,0,10,10\n",
        "extra_fields": "2\n4,1,2,zz\n4,3,4,\n\n0,0,10,10,9\n",
        "empty_cr_line": "2\n4,1,2\n4,3,4\n\r\n0,0,10,10\n",
        "zero_points": "0\n\n0,0,1,1\n",
    }
    for name, text in cases.items():
        _check_same(_write(tmp_path / f"{name}.csv", text), tmp_path, threads)


def _expect_error(tmp_path, text, threads, status, line=None):
    p = _write(tmp_path / "bad.csv", text)
    with pytest.raises(colo.ColoError) as e:
        colo.csv_to_binary(p, tmp_path / "bad.colo", threads)
    assert e.value.status == status, str(e.value)
    if line is not None:
        assert f"line {line}" in str(e.value), str(e.value)
    with pytest.raises(RuntimeError):
        oracle.parse_csv(p)                       # the serial restatement rejects it too


@pytest.mark.parametrize("threads", [1, 3, 8, 0])
def test_errors_name_the_serial_line(tmp_path, threads):
    base = _dataset(2000, 5).split("\n")
    for bad_at in (1, 2, 700, 1333, 2000):              # index into the point lines (line bad_at + 1)
        lines = list(base)
        lines[bad_at] = "12,notanumber,3"
        # a second bad line later: only the first one is reported
        lines[min(bad_at + 400, 2000)] = "12,1"
        _expect_error(tmp_path, "\n".join(lines), threads, colo.ERR_PARSE, bad_at + 1)
    lines = list(base)
    lines[900] = "-1,1,2"
    _expect_error(tmp_path, "\n".join(lines), threads, colo.ERR_PARSE, 901)


@pytest.mark.parametrize("threads", [1, 4])
def test_structural_errors(tmp_path, threads):
    cases = [
        ("", None),                                   # no count line
        ("x\n1,1,1\n\n0,0,1,1\n", None),              # count not a number
        ("-3\n\n0,0,1,1\n", None),                    # negative count
        ("3\n1,1,1\n1,2,2\n\n0,0,1,1\n", None),       # count mismatch
        ("2\n1,1,1\n1,2,2\n", None),                  # no empty line, no bounds
        ("2\n1,1,1\n1,2,2\n\n", None),                # empty line, no bounds
        ("2\n1,1,1\n1,2,2\n\n0,0,1\n", None),         # short bounds
        ("2\n1,1,1\n1,2,2\n\n0,0,q,1\n", None),       # bad bounds
        ("2\n1,1,1\n99999999999,2,2\n\n0,0,1,1\n", 3),  # id beyond int
    ]
    for text, line in cases:
        _expect_error(tmp_path, text, threads, colo.ERR_PARSE, line)


def test_missing_file(tmp_path):
    with pytest.raises(colo.ColoError) as e:
        colo.csv_to_binary(tmp_path / "absent.csv", tmp_path / "x.colo")
    assert e.value.status == colo.ERR_IO


def test_large_parallel_parse(tmp_path):
    """A file big enough for the automatic thread count to split it."""
    text = _dataset(400_000, 21, quote_every=9973)
    p = _write(tmp_path / "big.csv", text)
    _check_same(p, tmp_path, 0)
    colo.csv_to_binary(p, tmp_path / "serial.colo", 1)
    assert (tmp_path / "serial.colo").read_bytes() == (tmp_path / "t0.colo").read_bytes()
