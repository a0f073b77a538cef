"""Python binding of libcolo (ctypes over the C ABI in include/colo.h).

The product path is libcolo.so: hand-written sm_103a CUDA kernels plus the
C++ level loop.  There is no CPU fallback -- importing works without a GPU,
but every mining call fails with ColoError(COLO_ERR_NO_DEVICE) when no CUDA
device is present.

Mirrors the reference's colocationFinder entry points
(Codes/colocationFinder.h:138-183): LoadParameter -> read_params,
populateData -> Dataset.from_csv, Begin's level loop -> Context.mine.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field
from pathlib import Path
from typing import List, Optional, Sequence

import numpy as np

from . import _build

OK = 0
STATUS = {0: "COLO_OK", 1: "COLO_ERR_ARG", 2: "COLO_ERR_IO", 3: "COLO_ERR_PARSE", 4: "COLO_ERR_INPUT",
          5: "COLO_ERR_CUDA", 6: "COLO_ERR_NOMEM", 7: "COLO_ERR_TIMEOUT", 8: "COLO_ERR_CAPACITY",
          9: "COLO_ERR_NO_DEVICE", 10: "COLO_ERR_INTERNAL"}
ERR_ARG, ERR_IO, ERR_PARSE, ERR_INPUT, ERR_CAPACITY = 1, 2, 3, 4, 8
MODE_PLAIN, MODE_BATCHED, MODE_LEARNED = 0, 1, 2
COUNTERS = ["launches", "active_anchors", "neighbors", "rows_written", "join_pairs", "points", "cells", "runs",
            "count_items", "count_parent_words", "fill_words", "bitmap_words", "h2d_bytes", "d2h_bytes",
            "nrl_entries", "refined", "filter_items", "single_pass", "single_pass_overflow", "filter_cell_members",
            "filter_full_quads", "filter_cells", "pairs_model_us", "level_filter_wait_us", "host_table_bytes"]

# Every symbol declared in include/colo.h (checked by the CPU tests).
EXPORTS = [
    "colo_status_string", "colo_create", "colo_destroy", "colo_last_error", "colo_params_default",
    "colo_read_params", "colo_read_config", "colo_dataset_from_csv", "colo_dataset_from_host",
    "colo_dataset_write_csv", "colo_dataset_upload", "colo_dataset_evict", "colo_dataset_num_points",
    "colo_dataset_num_features", "colo_dataset_feature_name", "colo_dataset_feature_count", "colo_dataset_free", "colo_mine",
    "colo_mine_batch", "colo_result_num_levels", "colo_result_level_size", "colo_result_level_candidates",
    "colo_result_level", "colo_result_table", "colo_result_write_patterns", "colo_result_times",
    "colo_result_counters", "colo_result_free", "colo_stage_cells", "colo_stage_neighbors",
    "colo_stage_filter", "colo_stage_sqdist", "colo_result_num_kernels", "colo_result_kernel", "colo_ctx_stream",
    "colo_stage_within", "colo_stage_scan", "colo_table_pi_static", "colo_model_forward", "colo_model_grad", "colo_model_train",
    "colo_ctx_set_model", "colo_result_features", "colo_autotune", "colo_dataset_from_csv_threads",
    "colo_dataset_write_binary", "colo_dataset_from_binary", "colo_csv_to_binary", "colo_stage_apriori",
    "colo_dataset_from_csv_device", "colo_set_join_group", "colo_autotune_all", "colo_set_tuning",
    "colo_get_tuning",
]
MODEL_FEATURES = 24
MODEL_PARAMS = 32 * 64 + 64 + 64 * 64 + 64 + 64 + 1
MODEL_FILE = Path(__file__).resolve().parent / "cost_model.npz"


class ColoError(RuntimeError):
    def __init__(self, status: int, msg: str = ""):
        self.status = status
        super().__init__(f"{STATUS.get(status, status)}: {msg}")


class Params(C.Structure):
    _fields_ = [("distance", C.c_float), ("pi_threshold", C.c_float), ("filter_flag", C.c_uint32),
                ("max_size", C.c_uint32), ("mode", C.c_int32), ("keep_tables", C.c_int32),
                ("reserved", C.c_int32 * 6)]


_P = C.c_void_p
_u64p = C.POINTER(C.c_uint64)
_u32p = C.POINTER(C.c_uint32)
_u8p = C.POINTER(C.c_uint8)
_f32p = C.POINTER(C.c_float)
_i32p = C.POINTER(C.c_int32)
_lib = None


def _ptr(a: Optional[np.ndarray], t):
    return None if a is None else a.ctypes.data_as(t)


def load(build: bool = True) -> C.CDLL:
    """Load libcolo.so (building it first when sources changed)."""
    global _lib
    if _lib is not None:
        return _lib
    if build:
        _build.build()
    path = _build.lib_path("libcolo.so")
    if not path.exists():
        raise ColoError(9, f"{path} is missing: run __graft_entry__.build()")
    lib = C.CDLL(str(path))
    sig = {
        "colo_status_string": (C.c_char_p, [C.c_int]),
        "colo_create": (C.c_int, [C.POINTER(_P), C.c_int]),
        "colo_destroy": (C.c_int, [_P]),
        "colo_last_error": (C.c_char_p, [_P]),
        "colo_params_default": (None, [C.POINTER(Params)]),
        "colo_read_params": (C.c_int, [C.c_char_p, C.POINTER(Params)]),
        "colo_read_config": (C.c_int, [C.c_char_p, C.c_char_p, C.c_char_p, C.c_char_p, C.c_char_p, C.c_char_p,
                                       C.c_size_t]),
        "colo_dataset_from_csv": (C.c_int, [_P, C.c_char_p, C.POINTER(_P)]),
        "colo_dataset_from_host": (C.c_int, [_P, _f32p, _f32p, _i32p, C.c_uint64, _f32p, C.POINTER(_P)]),
        "colo_dataset_write_csv": (C.c_int, [_P, C.c_char_p]),
        "colo_dataset_from_csv_threads": (C.c_int, [_P, C.c_char_p, C.c_uint32, C.POINTER(_P)]),
        "colo_dataset_write_binary": (C.c_int, [_P, C.c_char_p]),
        "colo_dataset_from_binary": (C.c_int, [_P, C.c_char_p, C.POINTER(_P)]),
        "colo_dataset_from_csv_device": (C.c_int, [_P, C.c_char_p, C.POINTER(_P)]),
        "colo_csv_to_binary": (C.c_int, [C.c_char_p, C.c_char_p, C.c_uint32, C.c_char_p, C.c_size_t]),
        "colo_dataset_upload": (C.c_int, [_P]),
        "colo_dataset_evict": (C.c_int, [_P]),
        "colo_dataset_num_points": (C.c_uint64, [_P]),
        "colo_dataset_num_features": (C.c_uint32, [_P]),
        "colo_dataset_feature_name": (C.c_char_p, [_P, C.c_uint32]),
        "colo_dataset_feature_count": (C.c_uint64, [_P, C.c_uint32]),
        "colo_dataset_free": (None, [_P]),
        "colo_mine": (C.c_int, [_P, _P, C.POINTER(Params), C.POINTER(_P)]),
        "colo_mine_batch": (C.c_int, [_P, C.POINTER(_P), C.POINTER(Params), C.c_uint32, C.POINTER(_P)]),
        "colo_result_num_levels": (C.c_uint32, [_P]),
        "colo_result_level_size": (C.c_uint32, [_P, C.c_uint32]),
        "colo_result_level_candidates": (C.c_uint64, [_P, C.c_uint32]),
        "colo_result_level": (C.c_int, [_P, C.c_uint32, _u32p, _u64p, _u8p, _u64p, _u64p, _f32p, _u8p, _u32p]),
        "colo_result_table": (C.c_uint64, [_P, C.c_uint32, C.c_uint64, _u32p]),
        "colo_result_write_patterns": (C.c_int, [_P, _P, C.c_char_p]),
        "colo_result_times": (C.c_int, [_P, C.POINTER(C.c_double)]),
        "colo_result_counters": (C.c_int, [_P, _u64p, C.c_uint32]),
        "colo_result_num_kernels": (C.c_uint32, [_P]),
        "colo_result_kernel": (C.c_int, [_P, C.c_uint32, C.c_char_p, C.c_size_t, _u64p, C.POINTER(C.c_double)]),
        "colo_ctx_stream": (C.c_void_p, [_P]),
        "colo_result_free": (None, [_P]),
        "colo_stage_cells": (C.c_int, [_P, _P, C.c_float, _u64p, _u64p, _u32p, _u32p, _u64p]),
        "colo_stage_neighbors": (C.c_int, [_P, _P, C.c_float, _u64p, _u32p, _u64p]),
        "colo_stage_filter": (C.c_int, [_P, _P, C.c_float, C.c_float, _u32p, C.c_uint64, C.c_uint32, _u64p, _u8p]),
        "colo_stage_sqdist": (C.c_int, [_P, _f32p, _f32p, _f32p, _f32p, C.c_uint64, _f32p]),
        "colo_stage_within": (C.c_int, [_P, _f32p, _f32p, _f32p, _f32p, C.c_uint64, C.c_float, _f32p, _u8p]),
        "colo_stage_scan": (C.c_int, [_P, _P, C.c_uint64, C.c_int, _u64p, _u64p]),
        "colo_table_pi_static": (C.c_int, [_P, C.c_uint64, C.c_uint32, _u32p, _u32p, _P, _P, _P]),
        "colo_stage_apriori": (C.c_int, [_P, _u32p, C.c_uint64, C.c_uint32, _u32p, _u32p, C.c_uint64, _u64p]),
        "colo_model_forward": (C.c_int, [_P, _f32p, _f32p, C.c_uint64, _f32p]),
        "colo_model_grad": (C.c_int, [_P, _f32p, _f32p, _f32p, C.c_uint64, _f32p, _f32p]),
        "colo_model_train": (C.c_int, [_P, _f32p, _f32p, _f32p, C.c_uint64, C.c_uint32, C.c_uint32, C.c_float,
                                       C.c_uint64, _f32p]),
        "colo_ctx_set_model": (C.c_int, [_P, _f32p]),
        "colo_autotune": (C.c_int, [_P, _P, C.POINTER(Params), _i32p, C.POINTER(C.c_double)]),
        "colo_set_join_group": (C.c_int, [_P, C.c_int32]),
        "colo_autotune_all": (C.c_int, [_P, _P, C.POINTER(Params), C.c_char_p, C.POINTER(Tuning)]),
        "colo_set_tuning": (C.c_int, [_P, C.POINTER(Tuning)]),
        "colo_get_tuning": (C.c_int, [_P, C.POINTER(Tuning)]),
        "colo_result_features": (C.c_int, [_P, C.c_uint32, _f32p]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def default_params(distance: float, pi_threshold: float, mode: int = MODE_BATCHED, max_size: int = 0,
                   keep_tables: bool = False, profile: bool = False, features: bool = False,
                   device_apriori: bool = False, host_tables: bool = False, single_pass: bool = False) -> Params:
    """Mining parameters; `profile` times every kernel, `features` records the cost-model
    features of every candidate (training data), `device_apriori` generates every level's
    candidates on the device (by default only levels with many prevalent patterns), `host_tables`
    keeps the instance tables in pinned host memory (by default only tables too large for the
    device), `single_pass` (COLO_MODE_LEARNED) writes every refined candidate's table while counting
    it (by default only tables presized at 2^20 rows or more)."""
    p = Params()
    load().colo_params_default(C.byref(p))
    p.distance = distance
    p.pi_threshold = pi_threshold
    p.mode = mode
    p.max_size = max_size
    p.keep_tables = 1 if keep_tables else 0
    p.reserved[0] = ((1 if profile else 0) | (2 if features else 0) | (4 if device_apriori else 0) |
                     (8 if host_tables else 0) | (16 if single_pass else 0))
    return p


def read_params(path: str) -> Params:
    """LoadParameter (colocationFinder.cpp:57-74)."""
    p = Params()
    lib = load()
    lib.colo_params_default(C.byref(p))
    st = lib.colo_read_params(str(path).encode(), C.byref(p))
    if st != OK:
        raise ColoError(st, str(path))
    return p


def read_config(path: str) -> List[str]:
    """Begin's five-line config file (colocationFinder.cpp:1077-1092)."""
    bufs = [C.create_string_buffer(4096) for _ in range(5)]
    st = load().colo_read_config(str(path).encode(), *bufs, 4096)
    if st != OK:
        raise ColoError(st, str(path))
    return [b.value.decode() for b in bufs]


def csv_to_binary(csv_path: str, bin_path: str, threads: int = 0) -> None:
    """Parse a CSV dataset on the host (`threads` parser threads, 0: automatic) and write it as a
    binary point file.  Needs no GPU."""
    err = C.create_string_buffer(512)
    st = load().colo_csv_to_binary(str(csv_path).encode(), str(bin_path).encode(), threads, err, len(err))
    if st:
        raise ColoError(st, err.value.decode(errors="replace"))


BINARY_MAGIC = b"COLOPTS1"
# lanes per anchor that the join autotuner times (colo_autotune, in this order)
JOIN_WIDTHS = (1, 2, 4, 8, 16, 32)
# the other tuned launch shapes (colo_autotune_all)
FILTER_UNITS = (8, 16, 32)
LEVEL_BLOCKS = (64, 128, 256)


class Tuning(C.Structure):
    _fields_ = [("join_group", C.c_int32), ("filter_unit", C.c_int32), ("level_block", C.c_int32),
                ("level_queue", C.c_int32), ("from_cache", C.c_int32)]

    def as_dict(self) -> dict:
        return {"join_group": self.join_group, "filter_unit": self.filter_unit, "level_block": self.level_block,
                "level_queue": self.level_queue, "from_cache": bool(self.from_cache)}


def read_binary(path: str):
    """(x, y, raw_id, names, bounds) of a binary point file, read with numpy (no library call)."""
    buf = np.fromfile(path, np.uint8)
    if len(buf) < 64 or bytes(buf[:8]) != BINARY_MAGIC:
        raise ValueError(f"{path}: not a binary point file")
    ver, hb = np.frombuffer(buf[8:16], np.uint32)
    n, nf, nb = (int(v) for v in np.frombuffer(buf[16:40], np.uint64))
    bounds = np.frombuffer(buf[40:56], np.float32).copy()
    if ver != 1 or hb != 64 or len(buf) != 64 + 12 * n + 4 * nf + nb:
        raise ValueError(f"{path}: bad header")
    x = np.frombuffer(buf[64:64 + 4 * n], np.float32).copy()
    y = np.frombuffer(buf[64 + 4 * n:64 + 8 * n], np.float32).copy()
    raw = np.frombuffer(buf[64 + 8 * n:64 + 12 * n], np.int32).copy()
    lens = np.frombuffer(buf[64 + 12 * n:64 + 12 * n + 4 * nf], np.uint32)
    text = bytes(buf[64 + 12 * n + 4 * nf:])
    ends = np.cumsum(lens)
    names = [text[e - ln:e].decode(errors="surrogateescape") for e, ln in zip(ends.tolist(), lens.tolist())]
    return x, y, raw, names, bounds


@dataclass
class Level:
    k: int
    cand: np.ndarray        # (C, k) feature indices
    ub: np.ndarray          # (C, k) filter upper bounds
    passed: np.ndarray      # (C,) filter verdict
    rows: np.ndarray        # (C,) instance-table rows
    num: np.ndarray         # (C, k) participation numerators
    pi: np.ndarray          # (C,) float PI (-1: not refined)
    prevalent: np.ndarray   # (C,)
    argmin: np.ndarray      # (C,)
    features: np.ndarray = None   # (C, 24) cost-model inputs
    tables: dict = field(default_factory=dict)

    def patterns(self):
        return [tuple(int(v) for v in self.cand[c]) for c in np.nonzero(self.prevalent)[0]]


class Result:
    def __init__(self, lib, handle):
        self._lib = lib
        self.h = handle
        self._levels = None          # parsed on first access
        t = (C.c_double * 8)()
        lib.colo_result_times(handle, t)
        self.times = dict(zip(["total", "upload", "bucket", "join", "filter", "refine", "fill", "apriori"], list(t)))
        c = np.zeros(len(COUNTERS), np.uint64)
        lib.colo_result_counters(handle, _ptr(c, _u64p), len(COUNTERS))
        self.counters = dict(zip(COUNTERS, c.tolist()))
        self.kernels = {}
        for i in range(lib.colo_result_num_kernels(handle)):
            name = C.create_string_buffer(64)
            nl = C.c_uint64()
            ms = C.c_double()
            lib.colo_result_kernel(handle, i, name, 64, C.byref(nl), C.byref(ms))
            self.kernels[name.value.decode()] = (int(nl.value), float(ms.value))

    @property
    def levels(self) -> List[Level]:
        if self._levels is None:
            self._levels = self._parse_levels()
        return self._levels

    def _parse_levels(self) -> List[Level]:
        lib, handle = self._lib, self.h
        levels = []
        for li in range(lib.colo_result_num_levels(handle)):
            k = lib.colo_result_level_size(handle, li)
            n = lib.colo_result_level_candidates(handle, li)
            cand = np.zeros((n, k), np.uint32)
            ub = np.zeros((n, k), np.uint64)
            pas = np.zeros(n, np.uint8)
            rows = np.zeros(n, np.uint64)
            num = np.zeros((n, k), np.uint64)
            pi = np.zeros(n, np.float32)
            prev = np.zeros(n, np.uint8)
            am = np.zeros(n, np.uint32)
            lib.colo_result_level(handle, li, _ptr(cand, _u32p), _ptr(ub, _u64p), _ptr(pas, _u8p), _ptr(rows, _u64p),
                                  _ptr(num, _u64p), _ptr(pi, _f32p), _ptr(prev, _u8p), _ptr(am, _u32p))
            feat = np.zeros((n, MODEL_FEATURES), np.float32)
            lib.colo_result_features(handle, li, _ptr(feat, _f32p))
            lev = Level(k, cand, ub, pas, rows, num, pi, prev, am, feat)
            for c in range(n):
                r = lib.colo_result_table(handle, li, c, None)
                if r != 2 ** 64 - 1:
                    t = np.zeros((r, k), np.uint32)
                    lib.colo_result_table(handle, li, c, _ptr(t, _u32p))
                    lev.tables[c] = t
            levels.append(lev)
        return levels

    def patterns(self):
        out = []
        for lev in self.levels:
            out.extend(lev.patterns())
        return out

    def num_candidates(self) -> int:
        lib, h = self._lib, self.h
        return int(sum(lib.colo_result_level_candidates(h, li) for li in range(lib.colo_result_num_levels(h))))

    def write_patterns(self, ds: "Dataset", location: str):
        st = self._lib.colo_result_write_patterns(self.h, ds.h, str(location).encode())
        if st != OK:
            raise ColoError(st, location)

    def __del__(self):
        if getattr(self, "h", None):
            self._lib.colo_result_free(self.h)
            self.h = None


class Context:
    def __init__(self, device: int = 0):
        self.lib = load()
        h = _P()
        st = self.lib.colo_create(C.byref(h), device)
        if st != OK:
            raise ColoError(st, "colo_create")
        self.h = h

    def error(self) -> str:
        return self.lib.colo_last_error(self.h).decode()

    def check(self, st: int, what: str):
        if st != OK:
            raise ColoError(st, f"{what}: {self.error()}")

    def dataset(self, x, y, fid, bounds) -> "Dataset":
        return Dataset.from_arrays(self, x, y, fid, bounds)

    def mine(self, ds: "Dataset", params: Params) -> Result:
        out = _P()
        self.check(self.lib.colo_mine(self.h, ds.h, C.byref(params), C.byref(out)), "colo_mine")
        return Result(self.lib, out)

    def mine_batch(self, dss: Sequence["Dataset"], params: Sequence[Params]) -> List[Result]:
        n = len(dss)
        hs = (_P * n)(*[d.h for d in dss])
        ps = (Params * n)(*params)
        outs = (_P * n)()
        self.check(self.lib.colo_mine_batch(self.h, hs, ps, n, outs), "colo_mine_batch")
        return [Result(self.lib, outs[i]) for i in range(n)]

    def stage_neighbors(self, ds: "Dataset", R: float):
        tot = C.c_uint64(0)
        self.check(self.lib.colo_stage_neighbors(self.h, ds.h, R, None, None, C.byref(tot)), "stage_neighbors")
        offs = np.zeros(ds.n + 1, np.uint64)
        nbr = np.zeros(max(int(tot.value), 1), np.uint32)
        tot2 = C.c_uint64(len(nbr))
        self.check(self.lib.colo_stage_neighbors(self.h, ds.h, R, _ptr(offs, _u64p), _ptr(nbr, _u32p),
                                                 C.byref(tot2)), "stage_neighbors")
        return offs, nbr[: int(tot2.value)]

    def stage_cells(self, ds: "Dataset", R: float):
        nr = C.c_uint64(0)
        self.check(self.lib.colo_stage_cells(self.h, ds.h, R, None, None, None, None, C.byref(nr)), "stage_cells")
        cell = np.zeros(ds.n, np.uint64)
        rc = np.zeros(max(nr.value, 1), np.uint64)
        rf = np.zeros(max(nr.value, 1), np.uint32)
        rn = np.zeros(max(nr.value, 1), np.uint32)
        nr2 = C.c_uint64(len(rc))
        self.check(self.lib.colo_stage_cells(self.h, ds.h, R, _ptr(cell, _u64p), _ptr(rc, _u64p), _ptr(rf, _u32p),
                                             _ptr(rn, _u32p), C.byref(nr2)), "stage_cells")
        n = int(nr2.value)
        return cell, rc[:n], rf[:n], rn[:n]

    def stage_filter(self, ds: "Dataset", R: float, thr: float, cand: np.ndarray):
        cand = np.ascontiguousarray(cand, np.uint32)
        n, k = cand.shape
        ub = np.zeros((n, k), np.uint64)
        pas = np.zeros(n, np.uint8)
        self.check(self.lib.colo_stage_filter(self.h, ds.h, R, thr, _ptr(cand, _u32p), n, k, _ptr(ub, _u64p),
                                              _ptr(pas, _u8p)), "stage_filter")
        return ub, pas

    def stage_apriori(self, prev: np.ndarray, k: int):
        """Level-k candidates of the prevalent (k-1)-patterns `prev` on the device: (candidates, parent)."""
        prev = np.ascontiguousarray(prev, np.uint32).reshape(-1, k - 1)
        n = C.c_uint64(0)
        self.check(self.lib.colo_stage_apriori(self.h, _ptr(prev, _u32p), len(prev), k, None, None, 0, C.byref(n)),
                   "stage_apriori")
        out = np.zeros((max(n.value, 1), k), np.uint32)
        par = np.zeros(max(n.value, 1), np.uint32)
        self.check(self.lib.colo_stage_apriori(self.h, _ptr(prev, _u32p), len(prev), k, _ptr(out, _u32p),
                                               _ptr(par, _u32p), n.value, C.byref(n)), "stage_apriori")
        return out[: n.value], par[: n.value]

    def stage_sqdist(self, x1, y1, x2, y2) -> np.ndarray:
        a = [np.ascontiguousarray(v, np.float32) for v in (x1, y1, x2, y2)]
        out = np.zeros(len(a[0]), np.float32)
        self.check(self.lib.colo_stage_sqdist(self.h, *[_ptr(v, _f32p) for v in a], len(out), _ptr(out, _f32p)),
                   "stage_sqdist")
        return out

    def stage_scan(self, values) -> tuple[np.ndarray, int]:
        """Exclusive scan of uint32 or uint64 values on the device: (offsets as uint64, total)."""
        v = np.ascontiguousarray(values)
        if v.dtype not in (np.uint32, np.uint64):
            raise TypeError("stage_scan takes uint32 or uint64 values")
        out = np.zeros(max(len(v), 1), np.uint64)
        tot = C.c_uint64(0)
        self.check(self.lib.colo_stage_scan(self.h, v.ctypes.data_as(_P) if len(v) else None, len(v),
                                            1 if v.dtype == np.uint64 else 0, _ptr(out, _u64p), C.byref(tot)),
                   "stage_scan")
        return out[: len(v)], int(tot.value)

    def stream(self) -> int:
        return int(self.lib.colo_ctx_stream(self.h) or 0)

    def stage_within(self, x1, y1, x2, y2, R2: float):
        """(reference squared distance, kernels' decision sq <= R2) per pair."""
        a = [np.ascontiguousarray(v, np.float32) for v in (x1, y1, x2, y2)]
        out = np.zeros(len(a[0]), np.float32)
        w = np.zeros(len(a[0]), np.uint8)
        self.check(self.lib.colo_stage_within(self.h, *[_ptr(v, _f32p) for v in a], len(out), R2, _ptr(out, _f32p),
                                              _ptr(w, _u8p)), "stage_within")
        return out, w.astype(bool)

    def autotune(self, ds: "Dataset", params: Params) -> dict:
        """Pick the join's lanes per anchor for this dataset (kept for later mines)."""
        jg = C.c_int32(0)
        ms = (C.c_double * len(JOIN_WIDTHS))()
        self.check(self.lib.colo_autotune(self.h, ds.h, C.byref(params), C.byref(jg), ms), "autotune")
        return {"join_group": int(jg.value), "join_ms": dict(zip(JOIN_WIDTHS, list(ms)))}

    def set_join_group(self, width: int) -> None:
        """Pin the join's lanes per anchor (one of JOIN_WIDTHS; 0 for the default)."""
        self.check(self.lib.colo_set_join_group(self.h, int(width)), "set_join_group")

    def autotune_all(self, ds: "Dataset", params: Params, cache: Optional[str] = None) -> dict:
        """Tune the join width, the filter unit and the level block size for this dataset (kept for
        later mines); `cache` is a text file of tuned shapes read before and appended after tuning."""
        t = Tuning()
        self.check(self.lib.colo_autotune_all(self.h, ds.h, C.byref(params), None if cache is None else
                                              str(cache).encode(), C.byref(t)), "autotune_all")
        return t.as_dict()

    def set_tuning(self, join_group: int = 0, filter_unit: int = 0, level_block: int = 0,
                   level_queue: int = 0) -> None:
        t = Tuning(join_group, filter_unit, level_block, level_queue, 0)
        self.check(self.lib.colo_set_tuning(self.h, C.byref(t)), "set_tuning")

    def tuning(self) -> dict:
        t = Tuning()
        self.check(self.lib.colo_get_tuning(self.h, C.byref(t)), "get_tuning")
        return t.as_dict()

    # ---- learned cost model -------------------------------------------------
    def model_forward(self, params: np.ndarray, x: np.ndarray) -> np.ndarray:
        p = np.ascontiguousarray(params, np.float32)
        x = np.ascontiguousarray(x, np.float32).reshape(-1, MODEL_FEATURES)
        y = np.zeros(len(x), np.float32)
        self.check(self.lib.colo_model_forward(self.h, _ptr(p, _f32p), _ptr(x, _f32p), len(x), _ptr(y, _f32p)),
                   "model_forward")
        return y

    def model_grad(self, params: np.ndarray, x: np.ndarray, t: np.ndarray):
        p = np.ascontiguousarray(params, np.float32)
        x = np.ascontiguousarray(x, np.float32).reshape(-1, MODEL_FEATURES)
        t = np.ascontiguousarray(t, np.float32)
        g = np.zeros(MODEL_PARAMS, np.float32)
        loss = C.c_float(0)
        self.check(self.lib.colo_model_grad(self.h, _ptr(p, _f32p), _ptr(x, _f32p), _ptr(t, _f32p), len(x),
                                            _ptr(g, _f32p), C.byref(loss)), "model_grad")
        return g, float(loss.value)

    def model_train(self, params: np.ndarray, x: np.ndarray, t: np.ndarray, epochs: int, batch: int = 4096,
                    lr: float = 1e-3, seed: int = 0):
        """GPU training (Adam); returns (trained parameters, per-epoch loss)."""
        p = np.array(params, np.float32, copy=True)
        x = np.ascontiguousarray(x, np.float32).reshape(-1, MODEL_FEATURES)
        t = np.ascontiguousarray(t, np.float32)
        hist = np.zeros(max(epochs, 1), np.float32)
        self.check(self.lib.colo_model_train(self.h, _ptr(p, _f32p), _ptr(x, _f32p), _ptr(t, _f32p), len(x), epochs,
                                             batch, lr, seed, _ptr(hist, _f32p)), "model_train")
        return p, hist[:epochs]

    def set_model(self, params: Optional[np.ndarray]):
        """Install cost-model parameters for MODE_LEARNED mines (None: remove)."""
        if params is None:
            self.check(self.lib.colo_ctx_set_model(self.h, None), "set_model")
            return
        p = np.ascontiguousarray(params, np.float32)
        if p.size != MODEL_PARAMS:
            raise ValueError(f"expected {MODEL_PARAMS} parameters, got {p.size}")
        self._model = p
        self.check(self.lib.colo_ctx_set_model(self.h, _ptr(p, _f32p)), "set_model")

    def close(self):
        if getattr(self, "h", None):
            self.lib.colo_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()


def load_model(path=None) -> np.ndarray:
    """The committed trained cost model (parameters as float32)."""
    with np.load(path or MODEL_FILE) as z:
        return np.ascontiguousarray(z["params"], np.float32)


def init_model(seed: int = 0) -> np.ndarray:
    """He-initialised parameters (input rows 24..31 of W1 zero)."""
    rng = np.random.default_rng(seed)
    w1 = np.zeros((32, 64), np.float32)
    w1[:MODEL_FEATURES] = rng.normal(0, np.sqrt(2.0 / MODEL_FEATURES), (MODEL_FEATURES, 64))
    w2 = rng.normal(0, np.sqrt(2.0 / 64), (64, 64)).astype(np.float32)
    w3 = rng.normal(0, np.sqrt(1.0 / 64), 64).astype(np.float32)
    return np.concatenate([w1.ravel(), np.zeros(64, np.float32), w2.ravel(), np.zeros(64, np.float32), w3,
                           np.zeros(1, np.float32)]).astype(np.float32)


class Dataset:
    def __init__(self, ctx: Context, handle):
        self.ctx = ctx
        self.h = handle
        self.n = int(ctx.lib.colo_dataset_num_points(handle))
        self.nfeat = int(ctx.lib.colo_dataset_num_features(handle))

    @classmethod
    def from_csv(cls, ctx: Context, path: str, threads: int = 0, device: bool = False) -> "Dataset":
        """populateData's CSV, parsed by `threads` host threads (0: automatic), or on the device."""
        h = _P()
        if device:
            ctx.check(ctx.lib.colo_dataset_from_csv_device(ctx.h, str(path).encode(), C.byref(h)),
                      "dataset_from_csv_device")
        else:
            ctx.check(ctx.lib.colo_dataset_from_csv_threads(ctx.h, str(path).encode(), threads, C.byref(h)),
                      "dataset_from_csv")
        return cls(ctx, h)

    @classmethod
    def from_binary(cls, ctx: Context, path: str) -> "Dataset":
        """A binary point file written by write_binary or csv_to_binary."""
        h = _P()
        ctx.check(ctx.lib.colo_dataset_from_binary(ctx.h, str(path).encode(), C.byref(h)), "dataset_from_binary")
        return cls(ctx, h)

    def write_binary(self, path: str):
        self.ctx.check(self.ctx.lib.colo_dataset_write_binary(self.h, str(path).encode()), "dataset_write_binary")

    @classmethod
    def from_arrays(cls, ctx: Context, x, y, fid, bounds) -> "Dataset":
        x = np.ascontiguousarray(x, np.float32)
        y = np.ascontiguousarray(y, np.float32)
        fid = np.ascontiguousarray(fid, np.int32)
        b = np.ascontiguousarray(bounds, np.float32)
        h = _P()
        ctx.check(ctx.lib.colo_dataset_from_host(ctx.h, _ptr(x, _f32p), _ptr(y, _f32p), _ptr(fid, _i32p), len(x),
                                                 _ptr(b, _f32p), C.byref(h)), "dataset_from_host")
        return cls(ctx, h)

    def names(self) -> List[str]:
        return [self.ctx.lib.colo_dataset_feature_name(self.h, f).decode() for f in range(self.nfeat)]

    def upload(self):
        self.ctx.check(self.ctx.lib.colo_dataset_upload(self.h), "dataset_upload")

    def evict(self):
        self.ctx.lib.colo_dataset_evict(self.h)

    def write_csv(self, path: str):
        self.ctx.check(self.ctx.lib.colo_dataset_write_csv(self.h, str(path).encode()), "dataset_write_csv")

    def __del__(self):
        if getattr(self, "h", None):
            self.ctx.lib.colo_dataset_free(self.h)
            self.h = None
