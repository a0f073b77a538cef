"""Build the reference's own sources for the CPU (golden-vector harness).

TEST INFRASTRUCTURE.  Compiles, from where they lie under the reference tree
(the project's Codes/ directory, given as an argument or as
$COLO_REFERENCE_ROOT/Codes), colocationFinder.cpp and DeviceProcess.cu
with g++ against the project-written stand-ins in shim/ (CUDA runtime and
kernel execution model, the Thrust calls used, Boost's tokenizer) and links
them with ref_harness.cpp into oracle/_ref/ref_harness.

The only source transformation is done in memory on DeviceProcess.cu (the
translation unit is fed to g++ on stdin; no copy is written):
  * kernel launches `k<<<g, b, ...>>>(args);` become colo_emu_launch(...)
    calls (kernels containing __syncthreads run as fibers);
  * before each threshold_Kernel launch, a hook snapshots the filter bounds;
  * the extern "C" functions the harness wraps are renamed colo_ref_<name>.
Nothing here runs on the GPU machine: the golden vectors it produces are
committed under tests/golden/.
"""
from __future__ import annotations

import os
import re
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE.parent / "_ref"
SHIM = HERE / "shim"
WRAPPED = ["degree2InstanceTableSlotCounter", "degree2InstanceTableGenerator", "generalInstanceTableSlotCounter",
           "calcInstanceTableGeneral", "getParticipationIndex", "filter2", "filter2_2"]


def split_top(s: str):
    out, depth, cur = [], 0, ""
    for ch in s:
        if ch in "([{":
            depth += 1
        elif ch in ")]}":
            depth -= 1
        if ch == "," and depth == 0:
            out.append(cur.strip())
            cur = ""
        else:
            cur += ch
    if cur.strip():
        out.append(cur.strip())
    return out


def kernels_with_barriers(kernel_header: str):
    names = set()
    for m in re.finditer(r"__global__[^(]*?\b(\w+)\s*\(", kernel_header):
        start = kernel_header.index("{", m.end())
        depth, i = 0, start
        while True:
            if kernel_header[i] == "{":
                depth += 1
            elif kernel_header[i] == "}":
                depth -= 1
                if depth == 0:
                    break
            i += 1
        if "__syncthreads" in kernel_header[start:i]:
            names.add(m.group(1))
    return names


def transform(cu: str, barrier_kernels) -> str:
    launch = re.compile(r"(\w+)\s*<<\s*<\s*(.*?)\s*>>\s*>\s*\((.*?)\)\s*;", re.S)

    def rep(m):
        name, cfg, args = m.group(1), split_top(m.group(2)), m.group(3)
        sync = "true" if name in barrier_kernels else "false"
        pre = ""
        if name == "threshold_Kernel":
            a = split_top(args)
            pre = (f"if (colo_emu_hook_threshold) colo_emu_hook_threshold((const unsigned int*)({a[0]}), "
                   f"(unsigned)({a[4]}), (unsigned)({a[5]})); ")
        return f'{pre}colo_emu_launch("{name}", dim3({cfg[0]}), dim3({cfg[1]}), {sync}, [&]{{ {name}({args}); }});'

    out = launch.sub(rep, cu)
    for w in WRAPPED:
        out = re.sub(r"(\b(?:StatusType|Real|void)\s+)" + w + r"\s*\(", r"\1colo_ref_" + w + "(", out)
    return out


def reference_codes(arg: str = None) -> Path:
    """The reference's Codes/ directory: the argument, else $COLO_REFERENCE_ROOT/Codes; None when neither is set."""
    if arg:
        return Path(arg)
    root = os.environ.get("COLO_REFERENCE_ROOT")
    return Path(root) / "Codes" if root else None


def build(ref_codes: str = None) -> Path:
    codes = reference_codes(ref_codes)
    if codes is None:
        raise FileNotFoundError("no reference tree: pass its Codes/ directory or set COLO_REFERENCE_ROOT")
    if not (codes / "DeviceProcess.cu").exists():
        raise FileNotFoundError(f"reference sources not found under {codes}")
    OUT.mkdir(exist_ok=True)
    cu = (codes / "DeviceProcess.cu").read_text()
    hdr = (codes / "DeviceProcess_Kernel.h").read_text()
    src = transform(cu, kernels_with_barriers(hdr))
    common = ["g++", "-std=c++14", "-O1", "-w", "-ffp-contract=off", "-fno-strict-aliasing", "-DCOLO_EMU_OPEN_CLASSES",
              "-I", str(SHIM), "-I", str(codes), "-include", str(SHIM / "colo_emu.h")]
    objs = []
    dev_o = OUT / "DeviceProcess.o"
    r = subprocess.run(common + ["-x", "c++", "-c", "-", "-o", str(dev_o)], input=src, text=True, capture_output=True)
    if r.returncode:
        raise RuntimeError("DeviceProcess.cu (emulated) failed:\n" + r.stderr[-4000:])
    objs.append(dev_o)
    for name, path in [("colocationFinder", codes / "colocationFinder.cpp"), ("colo_emu", HERE / "colo_emu.cpp"),
                       ("ref_harness", HERE / "ref_harness.cpp")]:
        o = OUT / f"{name}.o"
        r = subprocess.run(common + ["-c", str(path), "-o", str(o)], text=True, capture_output=True)
        if r.returncode:
            raise RuntimeError(f"{path} failed:\n" + r.stderr[-4000:])
        objs.append(o)
    exe = OUT / "ref_harness"
    r = subprocess.run(["g++", "-o", str(exe)] + [str(o) for o in objs], text=True, capture_output=True)
    if r.returncode:
        raise RuntimeError("link failed:\n" + r.stderr[-4000:])
    return exe


if __name__ == "__main__":
    print(build(sys.argv[1] if len(sys.argv) > 1 else None))
