"""Build recipe for libcolo.so, libcologen.so and the GPU-Colocation CLI.

Everything is compiled in-tree into ``gpu-colocationmininig_gb300/lib`` with
nvcc for sm_103a only (one ``-gencode``); translation units are compiled in
parallel, then linked.  A target is rebuilt when any of its sources is newer.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
from pathlib import Path

PKG = Path(__file__).resolve().parent.parent          # gpu-colocationmininig_gb300/
ROOT = PKG.parent                                       # repository root
CSRC = PKG / "csrc"
FINDER = PKG / "finder"
INCLUDE = ROOT / "include"
LIBDIR = PKG / "lib"
OBJDIR = LIBDIR / "obj"

GENCODE = ["-gencode", "arch=compute_103a,code=sm_103a"]
CUDA_SOURCES = ["colo_prims.cu", "colo_bucket.cu", "colo_join.cu", "colo_filter.cu", "colo_level.cu",
                "colo_static.cu", "colo_mlp.cu", "colo_apriori.cu", "colo_ingest.cu"]
HOST_SOURCES = ["colo_mine.cpp", "colo_stage.cpp", "colo_io.cpp", "colo_model.cpp"]
HEADERS = ["colo_internal.h", "colo_batch.h", "colo_device.cuh", "colo_host.h", "colo_mlp.h"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _newer(target: Path, deps) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(Path(d).stat().st_mtime > t for d in deps)


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: " + " ".join(map(str, cmd)) + "\n" + r.stdout + r.stderr)
    return r


def lib_path(name: str) -> Path:
    return LIBDIR / name


def build(force: bool = False, verbose: bool = False) -> dict:
    """Compile all native targets; returns {target: path}."""
    LIBDIR.mkdir(exist_ok=True)
    OBJDIR.mkdir(exist_ok=True)
    nv = nvcc()
    headers = [CSRC / h for h in HEADERS] + [INCLUDE / "colo.h"]
    common = ["-O3", "-std=c++17", "-lineinfo", "-I", str(INCLUDE), "-I", str(CSRC),
              "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off"]
    jobs = []
    objs = []
    for src in CUDA_SOURCES + HOST_SOURCES:
        s = CSRC / src
        o = OBJDIR / (s.stem + ".o")
        objs.append(o)
        if force or _newer(o, [s] + headers):
            lang = [] if src.endswith(".cu") else ["-x", "cu"]
            jobs.append([nv] + GENCODE + common + lang + ["-c", str(s), "-o", str(o)])
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        for r in ex.map(_run, jobs):
            if verbose:
                print(r.stdout + r.stderr)
    out = {}
    so = lib_path("libcolo.so")
    if force or _newer(so, objs):
        _run([nv] + GENCODE + ["-shared", "-o", str(so)] + [str(o) for o in objs])
    out["libcolo"] = so
    gen_src = CSRC / "colo_gen.cpp"
    gen = lib_path("libcologen.so")
    if force or _newer(gen, [gen_src]):
        _run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-o", str(gen), str(gen_src)])
    out["libcologen"] = gen
    # drop-in C++ layer: colocationFinder class + GPU-Colocation CLI
    fsrc = [FINDER / "colocationFinder.cpp", FINDER / "main.cpp"]
    if all(p.exists() for p in fsrc):
        cli = lib_path("GPU-Colocation")
        if force or _newer(cli, fsrc + [FINDER / "colocationFinder.h", so]):
            _run(["g++", "-O2", "-std=c++17", "-I", str(INCLUDE), "-I", str(FINDER)] + [str(p) for p in fsrc]
                 + ["-L", str(LIBDIR), "-lcolo", "-Wl,-rpath,$ORIGIN", "-o", str(cli)])
        out["cli"] = cli
    return out
