"""Seeded synthetic workloads of the benchmark configurations.

config0  plain small: 20,000 points, 10 features x 2,000, planted {0,1},{2,3,4},{5..8}
         (1,200 seeds each, sigma 15), R=50, PI 0.3, domain 10,000
config1  plain at scale: 1e6 points, 40 features Zipf(1.0), 70% in 500 hotspots
         (sigma log-U[50,2000]), 12 planted patterns of size 2-6, R=100, PI 0.2
config2  512 independent jobs of config1's generator (N log-U[2k,400k], F U[8,32],
         2-8 patterns, R = 3 x mean NN spacing x U[0.5,2], PI in {0.1,0.2,0.3})
config3  2e7 points, 100 features Zipf(1.2), 75% in 5,000 hotspots (sigma
         log-U[5,500]), 30 planted patterns of size 2-7, R=20, PI 0.15
config4  1e8 points, 200 features Zipf(1.3), +2% in 50 dense hotspots (sigma 5),
         60 planted patterns of size 2-8, R=10, PI 0.1

Planted offsets use sigma = 0.3 R (config 0's ratio 15/50) and 0.6 x the
smallest member count of seeds per pattern (config 0's 1,200/2,000), shared
between the patterns a feature belongs to.  With Zipf-sized features a
planted pattern can only be prevalent if its members have similar counts
(PI is the smallest participation ratio), so members are a window of
consecutive size ranks outside the Zipf head.  Hotspots each belong to one
feature.  `scale` shrinks N and the domain at constant density (tests).
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass

import numpy as np

from . import _build


class GenSpec(C.Structure):
    _fields_ = [("n", C.c_uint64), ("nfeat", C.c_uint32), ("zipf_s", C.c_double), ("width", C.c_double),
                ("hot_frac", C.c_double), ("nhot", C.c_uint32), ("hot_sig_lo", C.c_double),
                ("hot_sig_hi", C.c_double), ("dense_frac", C.c_double), ("ndense", C.c_uint32),
                ("dense_sigma", C.c_double), ("npat", C.c_uint32), ("pat_min", C.c_uint32),
                ("pat_max", C.c_uint32), ("pat_sigma", C.c_double), ("seed_frac", C.c_double),
                ("seed", C.c_uint64), ("config0", C.c_int32), ("pad", C.c_int32)]


_gen = None


def _lib():
    global _gen
    if _gen is None:
        _build.build()
        _gen = C.CDLL(str(_build.lib_path("libcologen.so")))
        _gen.colo_gen_points.restype = C.c_int
        _gen.colo_gen_points.argtypes = [C.POINTER(GenSpec), C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                         C.c_void_p]
    return _gen


@dataclass
class Workload:
    name: str
    x: np.ndarray
    y: np.ndarray
    fid: np.ndarray
    bounds: np.ndarray
    R: float
    thr: float
    patterns: list
    max_size: int = 0

    @property
    def n(self):
        return len(self.x)

    @property
    def nfeat(self):
        return int(self.fid.max()) + 1 if len(self.fid) else 0


def generate(spec: GenSpec, name: str, R: float, thr: float, max_size: int = 0) -> Workload:
    n = int(spec.n)
    x = np.zeros(n, np.float32)
    y = np.zeros(n, np.float32)
    fid = np.zeros(n, np.int32)
    b = np.zeros(4, np.float32)
    pm = np.full(max(spec.npat, 3) * max(spec.pat_max, 4), -1, np.int32)
    npat = _lib().colo_gen_points(C.byref(spec), x.ctypes.data, y.ctypes.data, fid.ctypes.data, b.ctypes.data,
                                  pm.ctypes.data)
    if npat < 0:
        raise ValueError("bad generator spec")
    width = max(spec.pat_max, 4)
    pats = [tuple(int(v) for v in pm[p * width:(p + 1) * width] if v >= 0) for p in range(npat)]
    return Workload(name, x, y, fid, b, R, thr, pats, max_size)


def spec_config(cfg: int, seed: int = None, scale: float = 1.0) -> tuple:
    """(GenSpec, R, thr, max_size) of configuration cfg (0, 1, 3 or 4).

    scale < 1 gives a smaller case of the same density: N, the domain area
    and the hotspot counts shrink by `scale`; R and all sigmas stay.
    """
    s = GenSpec()
    s.seed = 20260101 + cfg if seed is None else seed
    s.seed_frac = 0.6
    if cfg == 0:
        s.n, s.nfeat, s.zipf_s, s.width = 20000, 10, 0.0, 10000.0
        s.config0, s.npat, s.pat_min, s.pat_max, s.pat_sigma = 1, 3, 2, 4, 15.0
        return s, 50.0, 0.3, 4
    if cfg == 1:
        R = 100.0
        s.n, s.nfeat, s.zipf_s, s.width = int(1_000_000 * scale), 40, 1.0, 1e6
        s.hot_frac, s.nhot, s.hot_sig_lo, s.hot_sig_hi = 0.7, 500, 50.0, 2000.0
        s.npat, s.pat_min, s.pat_max, s.pat_sigma = 12, 2, 6, 0.3 * R
        return s, R, 0.2, 6
    if cfg == 3:
        R = 20.0
        s.n, s.nfeat, s.zipf_s, s.width = int(20_000_000 * scale), 100, 1.2, 1e6
        s.hot_frac, s.nhot, s.hot_sig_lo, s.hot_sig_hi = 0.75, 5000, 5.0, 500.0
        s.npat, s.pat_min, s.pat_max, s.pat_sigma = 30, 2, 7, 0.3 * R
        return s, R, 0.15, 0
    if cfg == 4:
        R = 10.0
        s.n, s.nfeat, s.zipf_s, s.width = int(100_000_000 * scale), 200, 1.3, 1e6
        s.hot_frac, s.nhot, s.hot_sig_lo, s.hot_sig_hi = 0.75, 5000, 5.0, 500.0
        s.dense_frac, s.ndense, s.dense_sigma = 0.02, 50, 5.0
        s.npat, s.pat_min, s.pat_max, s.pat_sigma = 60, 2, 8, 0.3 * R
        return s, R, 0.1, 0
    raise ValueError(cfg)


def config(cfg: int, seed: int = None, scale: float = 1.0) -> Workload:
    s, R, thr, ms = spec_config(cfg, seed, scale)
    if scale != 1.0 and cfg != 0:
        s.width = s.width * math.sqrt(scale)
        s.nhot = max(1, int(round(s.nhot * scale)))
        s.ndense = max(1, int(round(s.ndense * scale))) if s.ndense else 0
    return generate(s, f"config{cfg}" + (f"@{scale:g}" if scale != 1.0 else ""), R, thr, ms)


def config2_jobs(njobs: int = 512, seed: int = 20260103, scale: float = 1.0):
    """The batched form's independent jobs (config 1's generator per job)."""
    rng = np.random.default_rng(seed)
    jobs = []
    for j in range(njobs):
        n = int(math.exp(rng.uniform(math.log(2000), math.log(400000))) * scale)
        nf = int(rng.integers(8, 33))
        n = max(n, nf * 4)
        spacing = 0.5 * 1e6 / math.sqrt(n)
        R = float(np.float32(3.0 * spacing * rng.uniform(0.5, 2.0)))
        thr = float(np.float32(rng.choice([0.1, 0.2, 0.3])))
        s = GenSpec()
        s.seed = seed * 1000 + j
        s.seed_frac = 0.6
        s.n, s.nfeat, s.zipf_s, s.width = n, nf, 1.0, 1e6
        s.hot_frac, s.nhot, s.hot_sig_lo, s.hot_sig_hi = 0.7, 500, 50.0, 2000.0
        s.npat, s.pat_min, s.pat_max, s.pat_sigma = int(rng.integers(2, 9)), 2, 6, 0.3 * R
        jobs.append(generate(s, f"config2.job{j}", R, thr, 6))
    return jobs
