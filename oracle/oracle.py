"""ctypes wrapper of the CPU oracle (oracle/colo_oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU legs, never by the product package.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from dataclasses import dataclass, field
from pathlib import Path
from typing import List, Optional

import numpy as np

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
SRC = HERE / "colo_oracle.cpp"
LIB = BUILD / "liboracle.so"

_u64p = C.POINTER(C.c_uint64)
_u32p = C.POINTER(C.c_uint32)
_u8p = C.POINTER(C.c_uint8)
_f32p = C.POINTER(C.c_float)
_f64p = C.POINTER(C.c_double)
_lib = None


def build(force: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    deps = [SRC, HERE / "colo_oracle.h"]
    if force or not LIB.exists() or any(d.stat().st_mtime > LIB.stat().st_mtime for d in deps):
        cmd = ["g++", "-O2", "-std=c++17", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared", "-o", str(LIB),
               str(SRC)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)
    return LIB


def _p(a, t):
    return None if a is None else a.ctypes.data_as(t)


def load():
    global _lib
    if _lib is not None:
        return _lib
    build()
    lib = C.CDLL(str(LIB))
    V = C.c_void_p
    sig = {
        "oracle_mine": (C.c_int, [_f32p, _f32p, _u32p, C.c_uint64, C.c_uint32, _f32p, C.c_float, C.c_float,
                                  C.c_uint32, C.c_int, C.c_int, _u64p, _u8p, C.c_uint64, C.POINTER(V)]),
        "oracle_mine_fast": (C.c_int, [_f32p, _f32p, _u32p, C.c_uint64, C.c_uint32, _f32p, C.c_float, C.c_float,
                                       C.c_uint32, C.c_int, C.c_int, _u64p, _u8p, C.c_uint64, C.POINTER(V)]),
        "oracle_free": (None, [V]),
        "oracle_phase_ms": (None, [V, _f64p]),
        "oracle_status": (C.c_int, [V]),
        "oracle_unresolved": (C.c_uint64, [V]),
        "oracle_num_levels": (C.c_uint32, [V]),
        "oracle_level_k": (C.c_uint32, [V, C.c_uint32]),
        "oracle_level_ncand": (C.c_uint64, [V, C.c_uint32]),
        "oracle_level_get": (None, [V, C.c_uint32, _u32p, _u64p, _u8p, _u64p, _u64p, _f32p, _u8p, _u32p]),
        "oracle_table": (C.c_uint64, [V, C.c_uint32, C.c_uint64, _u32p]),
        "oracle_neighbors": (C.c_uint64, [_f32p, _f32p, _u32p, C.c_uint64, C.c_uint32, _f32p, C.c_float, _u64p, _u8p,
                                          C.c_uint64, _u64p, _u32p, _u64p]),
        "oracle_filter_dense": (C.c_int, [_f32p, _f32p, _u32p, C.c_uint64, C.c_uint32, _f32p, C.c_float, C.c_float,
                                          _u32p, C.c_uint64, C.c_uint32, _u64p, _u8p]),
        "oracle_apriori": (C.c_uint64, [_u32p, C.c_uint64, C.c_uint32, _u32p, C.c_uint64]),
        "oracle_parse_csv": (C.c_int, [C.c_char_p, _u64p, _u32p, _f32p, _f32p, _u32p, _f32p, C.c_char_p,
                                       C.c_uint64]),
        "oracle_parse_params": (C.c_int, [C.c_char_p, _f32p, _f32p, _u32p]),
        "oracle_sq_decide": (C.c_int, [C.c_float, C.c_float, C.c_float, C.c_float, C.c_float, C.POINTER(C.c_int)]),
        "oracle_sqdist": (C.c_float, [C.c_float, C.c_float, C.c_float, C.c_float]),
        "oracle_sq_decide_batch": (None, [_f32p, _f32p, _f32p, _f32p, C.c_uint64, C.c_float, _u8p, _u8p, _f32p,
                                          _u8p]),
        "oracle_mlp_forward": (None, [_f32p, _f32p, C.c_uint64, C.c_int, _f64p]),
        "oracle_mlp_grad": (None, [_f32p, _f32p, _f32p, C.c_uint64, C.c_int, _f64p, _f64p]),
        "oracle_ambiguous_pairs": (C.c_uint64, [_f32p, _f32p, _u32p, C.c_uint64, C.c_float, _u64p, C.c_uint64]),
        "oracle_cell_adjacent": (C.c_int, [V, C.c_uint64, C.c_uint64]),
        "oracle_make_grid": (C.c_int, [C.c_float, C.c_float, C.c_float, C.c_float, C.c_float, V]),
        "oracle_cell_ids": (C.c_uint64, [V, _f32p, _f32p, C.c_uint64, _u64p]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


class Grid(C.Structure):
    _fields_ = [("min_x", C.c_float), ("min_y", C.c_float), ("max_x", C.c_float), ("max_y_ext", C.c_float),
                ("cell_width", C.c_float), ("gx", C.c_uint32), ("gy", C.c_uint32), ("total_cells", C.c_uint64),
                ("compat32", C.c_int32)]


@dataclass
class OLevel:
    k: int
    cand: np.ndarray
    ub: np.ndarray
    passed: np.ndarray
    rows: np.ndarray
    num: np.ndarray
    pi: np.ndarray
    prevalent: np.ndarray
    argmin: np.ndarray
    tables: dict = field(default_factory=dict)

    def patterns(self):
        return [tuple(int(v) for v in self.cand[c]) for c in np.nonzero(self.prevalent)[0]]


@dataclass
class OResult:
    status: int
    unresolved: int
    levels: List[OLevel]
    phase_ms: Optional[dict] = None

    def patterns(self):
        out = []
        for l in self.levels:
            out.extend(l.patterns())
        return out

    def num_candidates(self):
        return int(sum(len(l.cand) for l in self.levels))


def feature_index(fid: np.ndarray) -> np.ndarray:
    """populateData's grouping: a change of raw id starts a new feature."""
    fid = np.asarray(fid)
    if len(fid) == 0:
        return np.zeros(0, np.uint32)
    change = np.concatenate([[0], (fid[1:] != fid[:-1]).astype(np.int64)])
    return np.cumsum(change).astype(np.uint32)


def resolutions(res) -> tuple:
    if res is None:
        return None, None, 0
    keys = np.ascontiguousarray(res[0], np.uint64)
    le = np.ascontiguousarray(res[1], np.uint8)
    return keys, le, len(keys)


def mine(x, y, fid, bounds, R, thr, max_k=0, threads=0, keep_tables=False, res=None, fast=False) -> OResult:
    """Full mining run.  fast=False: the literal restatement (oracle_mine);
    fast=True: oracle_mine_fast, the same results organised for 10^7-10^8
    points (neighbour lists once, bitset quad tests, parallel sort)."""
    lib = load()
    x = np.ascontiguousarray(x, np.float32)
    y = np.ascontiguousarray(y, np.float32)
    feat = feature_index(fid)
    nf = int(feat.max()) + 1 if len(feat) else 0
    b = np.ascontiguousarray(bounds, np.float32)
    keys, le, nres = resolutions(res)
    h = C.c_void_p()
    fn = lib.oracle_mine_fast if fast else lib.oracle_mine
    fn(_p(x, _f32p), _p(y, _f32p), _p(feat, _u32p), len(x), nf, _p(b, _f32p), R, thr, max_k, threads,
       1 if keep_tables else 0, _p(keys, _u64p), _p(le, _u8p), nres, C.byref(h))
    try:
        st = lib.oracle_status(h)
        unres = lib.oracle_unresolved(h)
        levels = []
        for li in range(lib.oracle_num_levels(h)):
            k = lib.oracle_level_k(h, li)
            n = lib.oracle_level_ncand(h, li)
            cand = np.zeros((n, k), np.uint32)
            ub = np.zeros((n, k), np.uint64)
            pas = np.zeros(n, np.uint8)
            rows = np.zeros(n, np.uint64)
            num = np.zeros((n, k), np.uint64)
            pi = np.zeros(n, np.float32)
            prev = np.zeros(n, np.uint8)
            am = np.zeros(n, np.uint32)
            lib.oracle_level_get(h, li, _p(cand, _u32p), _p(ub, _u64p), _p(pas, _u8p), _p(rows, _u64p),
                                 _p(num, _u64p), _p(pi, _f32p), _p(prev, _u8p), _p(am, _u32p))
            lev = OLevel(k, cand, ub, pas, rows, num, pi, prev, am)
            if keep_tables:
                for c in range(n):
                    r = lib.oracle_table(h, li, c, None)
                    if r != 2 ** 64 - 1:
                        t = np.zeros((r, k), np.uint32)
                        lib.oracle_table(h, li, c, _p(t, _u32p))
                        lev.tables[c] = t
            levels.append(lev)
        ph = np.zeros(6, np.float64)
        lib.oracle_phase_ms(h, _p(ph, _f64p))
        names = ("bucket", "join", "filter", "refine", "fill", "apriori")
        return OResult(st, unres, levels, {k: round(float(v), 2) for k, v in zip(names, ph)})
    finally:
        lib.oracle_free(h)


def neighbors(x, y, fid, bounds, R, res=None):
    lib = load()
    x = np.ascontiguousarray(x, np.float32)
    y = np.ascontiguousarray(y, np.float32)
    feat = feature_index(fid)
    nf = int(feat.max()) + 1 if len(feat) else 0
    b = np.ascontiguousarray(bounds, np.float32)
    keys, le, nres = resolutions(res)
    n = len(x)
    offs = np.zeros(n + 1, np.uint64)
    unres = C.c_uint64(0)
    tot = lib.oracle_neighbors(_p(x, _f32p), _p(y, _f32p), _p(feat, _u32p), n, nf, _p(b, _f32p), R,
                               _p(keys, _u64p), _p(le, _u8p), nres, _p(offs, _u64p), None, C.byref(unres))
    nbr = np.zeros(max(int(tot), 1), np.uint32)
    lib.oracle_neighbors(_p(x, _f32p), _p(y, _f32p), _p(feat, _u32p), n, nf, _p(b, _f32p), R, _p(keys, _u64p),
                         _p(le, _u8p), nres, _p(offs, _u64p), _p(nbr, _u32p), C.byref(unres))
    return offs, nbr[: int(tot)], int(unres.value)


def ambiguous_pairs(x, y, fid, R) -> np.ndarray:
    lib = load()
    x = np.ascontiguousarray(x, np.float32)
    y = np.ascontiguousarray(y, np.float32)
    feat = feature_index(fid)
    n = lib.oracle_ambiguous_pairs(_p(x, _f32p), _p(y, _f32p), _p(feat, _u32p), len(x), R, None, 0)
    keys = np.zeros(max(int(n), 1), np.uint64)
    lib.oracle_ambiguous_pairs(_p(x, _f32p), _p(y, _f32p), _p(feat, _u32p), len(x), R, _p(keys, _u64p), len(keys))
    return keys[: int(n)]


def filter_dense(x, y, fid, bounds, R, thr, cand):
    lib = load()
    x = np.ascontiguousarray(x, np.float32)
    y = np.ascontiguousarray(y, np.float32)
    feat = feature_index(fid)
    nf = int(feat.max()) + 1
    b = np.ascontiguousarray(bounds, np.float32)
    cand = np.ascontiguousarray(cand, np.uint32)
    n, k = cand.shape
    ub = np.zeros((n, k), np.uint64)
    pas = np.zeros(n, np.uint8)
    st = lib.oracle_filter_dense(_p(x, _f32p), _p(y, _f32p), _p(feat, _u32p), len(x), nf, _p(b, _f32p), R, thr,
                                 _p(cand, _u32p), n, k, _p(ub, _u64p), _p(pas, _u8p))
    if st:
        raise RuntimeError(f"oracle_filter_dense status {st}")
    return ub, pas


def apriori(prev: np.ndarray, k: int) -> np.ndarray:
    lib = load()
    prev = np.ascontiguousarray(prev, np.uint32)
    n = lib.oracle_apriori(_p(prev, _u32p), len(prev), k, None, 0)
    out = np.zeros((max(int(n), 1), k), np.uint32)
    lib.oracle_apriori(_p(prev, _u32p), len(prev), k, _p(out, _u32p), n)
    return out[: int(n)]


def parse_csv(path):
    lib = load()
    n = C.c_uint64(0)
    nf = C.c_uint32(0)
    b = np.zeros(4, np.float32)
    st = lib.oracle_parse_csv(str(path).encode(), C.byref(n), C.byref(nf), None, None, None, _p(b, _f32p), None, 0)
    if st:
        raise RuntimeError(f"oracle_parse_csv status {st}")
    x = np.zeros(n.value, np.float32)
    y = np.zeros(n.value, np.float32)
    feat = np.zeros(n.value, np.uint32)
    names = C.create_string_buffer(1 << 20)
    lib.oracle_parse_csv(str(path).encode(), C.byref(n), C.byref(nf), _p(x, _f32p), _p(y, _f32p), _p(feat, _u32p),
                         _p(b, _f32p), names, len(names))
    return x, y, feat, b, names.value.decode().split("\n") if nf.value else []


def parse_params(path):
    lib = load()
    R = C.c_float()
    t = C.c_float()
    f = C.c_uint32()
    st = lib.oracle_parse_params(str(path).encode(), C.byref(R), C.byref(t), C.byref(f))
    if st:
        raise RuntimeError(f"oracle_parse_params status {st}")
    return R.value, t.value, f.value


def sq_decide(x1, y1, x2, y2, R2):
    amb = C.c_int(0)
    le = load().oracle_sq_decide(x1, y1, x2, y2, R2, C.byref(amb))
    return bool(le), bool(amb.value)


def sq_decide_batch(x1, y1, x2, y2, R2):
    """(le, ambiguous, value, near_mid) for arrays of point pairs."""
    a = [np.ascontiguousarray(v, np.float32) for v in (x1, y1, x2, y2)]
    n = len(a[0])
    le = np.zeros(n, np.uint8)
    amb = np.zeros(n, np.uint8)
    val = np.zeros(n, np.float32)
    near = np.zeros(n, np.uint8)
    load().oracle_sq_decide_batch(*[_p(v, _f32p) for v in a], n, R2, _p(le, _u8p), _p(amb, _u8p), _p(val, _f32p),
                                  _p(near, _u8p))
    return le.astype(bool), amb.astype(bool), val, near.astype(bool)


def mlp_forward(params, x, bf16=True) -> np.ndarray:
    """Cost-model predictions (float64) with the kernels' BF16 rounding points (bf16) or exactly."""
    lib = load()
    p = np.ascontiguousarray(params, np.float32)
    x = np.ascontiguousarray(x, np.float32).reshape(-1, 24)
    y = np.zeros(len(x), np.float64)
    lib.oracle_mlp_forward(_p(p, _f32p), _p(x, _f32p), len(x), int(bool(bf16)), _p(y, _f64p))
    return y


def mlp_grad(params, x, t, bf16=True):
    """(gradient float64[6337], loss) of mean 0.5*(y - t)^2."""
    lib = load()
    p = np.ascontiguousarray(params, np.float32)
    x = np.ascontiguousarray(x, np.float32).reshape(-1, 24)
    t = np.ascontiguousarray(t, np.float32)
    g = np.zeros(p.size, np.float64)
    loss = C.c_double(0)
    lib.oracle_mlp_grad(_p(p, _f32p), _p(x, _f32p), _p(t, _f32p), len(x), int(bool(bf16)), _p(g, _f64p),
                        C.byref(loss))
    return g, float(loss.value)
