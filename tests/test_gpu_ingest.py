"""The CSV parsed on the device (colo_dataset_from_csv_device) against the
host reader (the serial populateData rules, pinned to the oracle by
test_cpu_io.py): identical binary point files -- coordinates bit for bit,
ids, names, bounds -- and the same verdict and line number on malformed
input.  Mining from the device-parsed dataset gives the golden results."""
import numpy as np
import pytest

import colo
from golden_check import CASES, assert_matches_golden, load, paths
from test_cpu_io import _dataset, _write

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    return colo.Context(0)


def _msg(e):
    """The reader's message without the binding's call prefix."""
    return str(e).split("dataset: ", 1)[-1]


def _same_as_host(ctx, path, tmp_path):
    colo.csv_to_binary(path, tmp_path / "host.colo", 1)
    ds = colo.Dataset.from_csv(ctx, path, device=True)
    ds.write_binary(tmp_path / "dev.colo")
    assert (tmp_path / "dev.colo").read_bytes() == (tmp_path / "host.colo").read_bytes()
    return ds


@pytest.mark.parametrize("form", ["plain", "crlf", "quoted", "names"])
def test_device_parse_matches_host(ctx, tmp_path, form):
    text = _dataset(20000, 11, crlf=form == "crlf", quote_every=7 if form == "quoted" else 0,
                    pad_names=form == "names")
    _same_as_host(ctx, _write(tmp_path / "d.csv", text), tmp_path)


def test_number_forms(ctx, tmp_path):
    rng = np.random.default_rng(3)
    forms = ["{:.9g}", "{:.17g}", "{:.3f}", "{:e}", "{:.25f}", "  {:.6g}", "{:.9g}xyz", "{:.12E}"]
    lines = []
    for i in range(6000):
        v = float(rng.uniform(-1e4, 1e4)) * (10.0 ** int(rng.integers(-8, 8)))
        f = forms[i % len(forms)]
        lines.append(f"{i // 600},{f.format(v)},{forms[(i + 3) % len(forms)].format(-v / 3)}")
    lines += ["77,0x1p3,1", "77,+5,2", "77,inf,3", "77,-0,-0.0", "77,1e-40,5", "77,1e38,3.4e38", "77,1e-38,2",
              "77,12345678901234567890123,7", "77,.5,5.", "77,0.000000000000000000000000001,1"]
    text = f"{len(lines)}\n" + "\n".join(lines) + "\n\n0,0,10,10\n"
    _same_as_host(ctx, _write(tmp_path / "forms.csv", text), tmp_path)


def test_edge_files(ctx, tmp_path):
    for name, text in {
        "one": "1\n5,1.5,2.5\n\n0,0,10,10\n",
        "no_newline_at_end": "2\n5,1,2\n6,3,4\n\n0,0,10,10",
        "spaces": "3\n 12 ,  1.5, 2\n12,1e1,-0\n+13,0x10,inf\n\n0,0,10,10\n",
        "extra_fields": "2\n4,1,2,zz\n4,3,4,\n\n0,0,10,10,9\n",
        "after_empty": "2\n4,1,2\n4,3,4\n\r\n0,0,10,10\ngarbage\n1,2\n",
        "zero_points": "0\n\n0,0,1,1\n",
    }.items():
        _same_as_host(ctx, _write(tmp_path / f"{name}.csv", text), tmp_path)


@pytest.mark.parametrize("bad_at", [1, 2, 700, 1999])
def test_errors_name_the_serial_line(ctx, tmp_path, bad_at):
    base = _dataset(2000, 5).split("\n")
    for repl in ("12,notanumber,3", "12,1", "-1,1,2", "-1,+q,2", '"12",zz,1', "12,3.5e38,1", "12,1,-"):
        lines = list(base)
        lines[bad_at] = repl
        lines[min(bad_at + 300, 2000)] = "12,1"
        p = _write(tmp_path / "bad.csv", "\n".join(lines))
        with pytest.raises(colo.ColoError) as eh:
            colo.csv_to_binary(p, tmp_path / "x.colo", 1)
        with pytest.raises(colo.ColoError) as ed:
            colo.Dataset.from_csv(ctx, p, device=True)
        assert ed.value.status == eh.value.status == colo.ERR_PARSE
        assert _msg(ed.value) == _msg(eh.value), (str(ed.value), str(eh.value))


def test_structural_errors(ctx, tmp_path):
    for text in ("", "x\n1,1,1\n\n0,0,1,1\n", "3\n1,1,1\n1,2,2\n\n0,0,1,1\n", "2\n1,1,1\n1,2,2\n",
                 "2\n1,1,1\n1,2,2\n\n", "2\n1,1,1\n1,2,2\n\n0,0,q,1\n"):
        p = _write(tmp_path / "s.csv", text)
        with pytest.raises(colo.ColoError) as eh:
            colo.csv_to_binary(p, tmp_path / "x.colo", 1)
        with pytest.raises(colo.ColoError) as ed:
            colo.Dataset.from_csv(ctx, p, device=True)
        assert ed.value.status == eh.value.status
        assert _msg(ed.value) == _msg(eh.value), (str(ed.value), str(eh.value))


@pytest.mark.parametrize("case", CASES)
def test_golden_from_device_parse(ctx, case):
    g = load(case)
    csv, par = paths(case)
    ds = colo.Dataset.from_csv(ctx, str(csv), device=True)
    assert ds.names() == g["features"]
    p = colo.read_params(str(par))
    p.mode = colo.MODE_BATCHED
    p.keep_tables = 1
    assert_matches_golden(ctx.mine(ds, p), g)
