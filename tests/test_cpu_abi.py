"""The C-ABI library builds, loads and exports every declared symbol (no GPU)."""
import ctypes as C
import re
from pathlib import Path

import pytest

import colo
from colo import _build

ROOT = Path(__file__).resolve().parent.parent


def _declared(header: Path):
    text = header.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(colo_[a-z0-9_]+)\s*\(", text)))


def test_every_declared_symbol_is_exported():
    lib = colo.load()
    names = _declared(ROOT / "include" / "colo.h")
    assert names, "no declarations found"
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    assert sorted(colo.EXPORTS) == names


def test_status_strings_and_defaults_without_gpu():
    lib = colo.load()
    assert lib.colo_status_string(0) == b"ok"
    assert b"CUDA" in lib.colo_status_string(5)
    p = colo.Params()
    lib.colo_params_default(C.byref(p))
    assert p.mode == colo.MODE_BATCHED and p.max_size == 0


def test_null_arguments_are_rejected():
    lib = colo.load()
    assert lib.colo_create(None, 0) == 1
    assert lib.colo_mine(None, None, None, None) == 1
    assert lib.colo_destroy(None) == 1


def test_read_params_and_config(tmp_path):
    pf = tmp_path / "parameter.txt"
    pf.write_text("10\n0.3\n1\n")
    p = colo.read_params(str(pf))
    assert p.distance == pytest.approx(10.0) and p.pi_threshold == pytest.approx(0.3) and p.filter_flag == 1
    cf = tmp_path / "config.txt"
    cf.write_text("./\n./Data/parameter.txt\n./Data/points.csv\n./out/\nresult.txt\n")
    assert colo.read_config(str(cf)) == ["./", "./Data/parameter.txt", "./Data/points.csv", "./out/", "result.txt"]
    with pytest.raises(colo.ColoError):
        colo.read_params(str(tmp_path / "missing.txt"))


def test_build_outputs_are_in_tree():
    out = _build.build()
    for p in out.values():
        assert Path(p).exists()
        assert str(Path(p).resolve()).startswith(str(ROOT))
