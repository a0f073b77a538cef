#!/usr/bin/env python
"""Benchmark: end-to-end colocation mining on one GB300 (per rank).

Workload: the 20,000,000-point configuration (100 features, Zipf 1.2 sizes,
75% in 5,000 Gaussian hotspots, 30 planted colocations, R = 20, PI 0.15),
generated with a fixed seed.  A step is one full mining run (all levels)
over that dataset.

  value   candidates/s of the headline form (batched; learned when enabled)
          with the points resident in HBM when the timed region starts
  e2e     the same through the C ABI from host buffers: every step moves the
          points host->device (the cell-key pass reads the page-locked host
          arrays over the host link) and the per-level results device->host
  plain   the project's plain two-pass form (per-candidate launches) on the
          same resident data, for the batched-vs-plain ratio

With --impl reference the CPU oracle (the reference's semantics restated in
C++/OpenMP, scaled form; the reference itself has no CPU path) mines the same
workload in full, every step, on all host cores.  Under torchrun every rank runs an
independent replica (the path does not exchange data between GPUs).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
for p in (ROOT / "gpu-colocationmininig_gb300", ROOT / "oracle"):
    sys.path.insert(0, str(p))

import numpy as np  # noqa: E402

METRIC = "end-to-end mining s & candidates/s, batched+learned vs plain on 1 GB300, bit-exact PI"
WORKLOAD = ("config3: 20,000,000 points, 100 features (Zipf s=1.2), 75% in 5,000 hotspots "
            "(sigma log-U[5,500]), 30 planted colocations of size 2-7, R=20, PI 0.15")
WORKLOADS = {
    0: "config0: 20,000 points, 10 features x 2,000, planted {0,1},{2,3,4},{5..8}, R=50, PI 0.3, sizes <= 4",
    1: ("config1: 1,000,000 points, 40 features (Zipf s=1.0), 70% in 500 hotspots (sigma log-U[50,2000]), "
        "12 planted colocations of size 2-6, R=100, PI 0.2, sizes <= 6"),
    3: WORKLOAD,
    4: ("config4: 200 features (Zipf s=1.3), 2% of every feature in sigma=5 dense hotspots, the rest as config3, "
        "60 planted colocations of size 2-8, R=10, PI 0.1, no size cap"),
}


def workload_name(cfg: int, scale: float, n: int) -> str:
    w = WORKLOADS.get(cfg, f"config{cfg}")
    return w if scale == 1.0 else f"{w}; at scale {scale:g} ({n:,} points, same density)"


JOBS_WORKLOAD = ("512 independent jobs, 2k-400k points each (log-uniform), 8-32 features, "
                 "R = 3 x mean spacing x U[0.5, 2], PI in {0.1, 0.2, 0.3}")
PEAKS = ROOT / "MEASURED_PEAKS.json"
L2_BYTES = 129 * 1000 * 1000   # GB300 L2


def l2_note(input_bytes: int) -> str:
    """How the timed steps treat L2 (StepTimer's rule), for the JSON line's config."""
    if input_bytes < L2_BYTES:
        return f"inputs (x, y f32: {input_bytes / 1e6:.1f} MB) fit in L2 (129 MB): 256 MB written between timed steps"
    return f"inputs (x, y f32: {input_bytes / 1e6:.0f} MB) larger than L2 (129 MB); no flush"


class StepTimer:
    """Per-step CUDA events on the library's stream, summed over the timed steps.  When a step's
    inputs fit in L2 (`input_bytes` < 129 MB) a 256 MB device write between steps, outside the
    events, flushes L2 so no step starts on inputs the previous one left cached."""

    def __init__(self, torch, dev, stream, input_bytes: int):
        self.torch, self.stream = torch, stream
        self.flush = input_bytes < L2_BYTES
        self.buf = torch.empty(256 << 20, dtype=torch.uint8, device=dev) if self.flush else None
        self.pairs = []


    def step(self, fn):
        """Runs fn() as one timed step; returns its result."""
        torch = self.torch
        if self.flush:
            with torch.cuda.stream(self.stream):
                self.buf.fill_(len(self.pairs) & 0xFF)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(self.stream)
        out = fn()
        e1.record(self.stream)
        self.pairs.append((e0, e1))
        return out

    def ms(self) -> float:
        """Total of the steps' times (after a synchronize)."""
        return sum(a.elapsed_time(b) for a, b in self.pairs)

    def spread(self) -> dict:
        """Fastest, median and slowest step (ms), to show a step that stalled."""
        t = sorted(a.elapsed_time(b) for a, b in self.pairs)
        return {"min": round(t[0], 3), "median": round(statistics.median(t), 3), "max": round(t[-1], 3)} if t else {}


def dist_env():
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


class ClockSampler:
    """nvidia-smi samples during the timed region (clocks and throttle reasons).

    nvidia-smi starts before the timed steps and the steps begin only after its first sample
    (its start-up then stalls no timed step); every 20 ms a sample, and the summary keeps the
    samples that arrived while the steps ran (`mark_start`/`mark_end`), or all of them when the
    steps were shorter than one interval."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.rows = []
        self.proc = None
        self.t0 = self.t1 = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits", "-lms", "20",
                 "-i", str(self.device)], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
            deadline = time.monotonic() + 5.0
            while not self.rows and time.monotonic() < deadline and self.proc.poll() is None:
                time.sleep(0.01)
        except (OSError, ValueError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append((time.monotonic(), [v.strip() for v in line.split(",")]))

    def mark_start(self):
        self.t0 = time.monotonic()

    def mark_end(self):
        self.t1 = time.monotonic()

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        rows = [r for t, r in self.rows
                if self.t0 is not None and self.t1 is not None and self.t0 - 0.02 <= t <= self.t1 + 0.02]
        for r in rows or [r for _, r in self.rows]:
            try:
                sm.append(float(r[1]))
                mx = float(r[2])
            except (ValueError, IndexError):
                continue
            for name, v in zip(names, r[5:9]):
                if v.strip().lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def measured_peak_gbs():
    try:
        return float(json.loads(PEAKS.read_text())["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def algorithmic_bytes(name: str, c: dict, launches: float, words: int) -> float:
    """Algorithmic bytes of all launches (per step) of one kernel family.

    `launches` = launches per step, `words` = 32-bit mask words per cell.
    """
    N, E, M, Rn = c["points"], c["neighbors"], c["cells"], c["runs"]
    kb = 4.0 if c.get("key_bits", 64) <= 32 else 8.0   # cell keys are 32-bit when every key fits
    if name == "radix_sort":       # per digit pass over the points: read and write the key and the 4 B id
        return 2.0 * (kb + 4.0) * N * launches
    if name == "radix_hist":       # one read of the keys for every pass's digit histogram
        return kb * N
    if name == "run_sort":         # per digit pass over the runs
        return 24.0 * Rn * launches
    if name == "cell_keys":        # read x, y, feature; write key, id
        return 24.0 * N
    if name == "gather_sorted":    # read the sorted ids and keys, gather x, y, write x, y, feature in cell order
        return (28.0 + kb) * N
    if name == "cell_neighbours":  # read the key, write 9 neighbour indices
        return 44.0 * M
    if name == "quad_masks":       # read 9 indices + masks, write 4 quad masks + the 3x3 union
        return 36.0 * M + 4.0 * words * M * 6
    if name == "nrl_fill":         # write the run per list entry + per-run suffix and count
        return 4.0 * c["nrl_entries"] + 12.0 * Rn
    if name == "join":             # B_b = 12 N + 4 E + 8 (N + 1): points once, lists and offsets written
        return 12.0 * N + 4.0 * E + 8.0 * (N + 1)
    if name in ("join_count", "join_fill"):   # the same split over the two-pass layout
        return 12.0 * N + 4.0 * N if name == "join_count" else 4.0 * E + 8.0 * (N + 1)
    if name == "level_count":      # parent rows once + candidate slices once
        return 4.0 * c["count_parent_words"] + 4.0 * c["count_items"]
    if name in ("level_fill", "level_single"):
        return 4.0 * c["fill_words"]
    if name == "level_pi":
        return 4.0 * c["bitmap_words"]
    if name == "filter_pairs":
        return 8.0 * Rn + 4.0 * words * M
    if name == "filter_level":     # B_c: a 4-byte count per (cell of U_c, member) run read
        return 4.0 * c["filter_cell_members"]
    return 0.0


def cell_key_bits(grids) -> int:
    """Bits of the batch's cell keys: the sum of the jobs' grid sizes, each grid set as setGrid
    does (colocationFinder.cpp:102-126) in float."""
    total = 0
    for bounds, R in grids:
        b = np.asarray(bounds, np.float32)
        R = np.float32(R)
        gx = int(np.ceil((b[2] - b[0]) / R))
        gy = int(np.ceil(((b[3] + R) - b[1]) / R))
        total += gx * gy
    bits = 1
    while bits < 64 and (1 << bits) < total:
        bits += 1
    return bits


def measure_io(ctx, wl, ds, params, patterns):
    """End to end including input I/O: the workload written once (untimed) as the reference's CSV and
    as a binary point file, then each loaded through the public API -- the CSV by the host reader and
    by the device reader -- and mined (one cold mine: page locking and upload included).  Times in
    ms from the load call to the result."""
    import shutil
    import tempfile

    import colo
    d = tempfile.mkdtemp(prefix="colo_io_")
    try:
        csv, binp = os.path.join(d, "points.csv"), os.path.join(d, "points.colo")
        ds.write_csv(csv)
        ds.write_binary(binp)
        out = {"csv_bytes": os.path.getsize(csv), "binary_bytes": os.path.getsize(binp)}
        for name, load in (("csv", lambda: colo.Dataset.from_csv(ctx, csv)),
                           ("csv_device", lambda: colo.Dataset.from_csv(ctx, csv, device=True)),
                           ("binary", lambda: colo.Dataset.from_binary(ctx, binp))):
            t0 = time.perf_counter()
            dl = load()
            t1 = time.perf_counter()
            r = ctx.mine(dl, params)
            t2 = time.perf_counter()
            out[f"{name}_load_ms"] = round((t1 - t0) * 1e3, 2)
            out[f"e2e_with_{name}_ms"] = round((t2 - t0) * 1e3, 2)
            out[f"{name}_identical"] = r.patterns() == patterns
            del dl, r
        return out
    finally:
        shutil.rmtree(d, ignore_errors=True)


def load_traffic(kernel: str):
    """Per-launch DRAM bytes of `kernel` from the committed ncu summary (or None)."""
    f = ROOT / "profiles" / "traffic.json"
    try:
        d = json.loads(f.read_text())
        return d.get(kernel)
    except (OSError, ValueError):
        return None


def cpu_model() -> str:
    """The host CPU's model name (lscpu, else /proc/cpuinfo)."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    try:
        for line in Path("/proc/cpuinfo").read_text().splitlines():
            if line.lower().startswith(("model name", "cpu part")):
                return line.split(":", 1)[1].strip()
    except OSError:
        pass
    return "unknown"


def run_cpu(workloads, steps: int, warmup: int):
    """The CPU oracle (the reference's semantics restated in C++/OpenMP, scaled form) mining every
    workload in full, every step, on all host cores.  Returns (candidates/s, cores, sample, s/step,
    phase ms of the last step)."""
    import oracle

    times, cands, phases = [], 0, None
    for i in range(warmup + steps):
        t = time.perf_counter()
        c = 0
        for wl in workloads:
            r = oracle.mine(wl.x, wl.y, wl.fid, wl.bounds, wl.R, wl.thr, max_k=wl.max_size, fast=True)
            if r.status != 0:
                raise RuntimeError(f"oracle status {r.status}")
            c += r.num_candidates()
            phases = r.phase_ms
        el = time.perf_counter() - t
        if i >= warmup:
            times.append(el)
            cands = c
    cores = os.cpu_count()
    value = cands * len(times) / sum(times) if times else 0.0
    npts = sum(wl.n for wl in workloads)
    sample = (f"the full workload every step: all {npts} points, every level (oracle_mine_fast, "
              f"OpenMP on {cores} threads of a {cpu_model()})")
    return value, cores, sample, sum(times) / max(len(times), 1), phases


def bench_jobs(args, rank, world, local, dist):
    """The 512-job batched workload: every job's level-k candidates in one launch per phase
    (colo_mine_batch) against the plain form mining the jobs one at a time."""
    import torch
    import colo
    from colo import gen, replicas

    dev = torch.device("cuda", local)
    jobs = gen.config2_jobs(512, scale=args.scale)
    ctx = colo.Context(local)
    dss = [colo.Dataset.from_arrays(ctx, w.x, w.y, w.fid, w.bounds) for w in jobs]
    for d in dss:
        d.upload()
    model = None
    try:
        model = colo.load_model()
    except OSError:
        pass
    ctx.set_model(model)
    mode = colo.MODE_LEARNED if model is not None else colo.MODE_BATCHED
    stream = torch.cuda.ExternalStream(ctx.stream(), device=dev)

    def run(form):
        if form == "plain":
            ps = [colo.default_params(w.R, w.thr, colo.MODE_PLAIN, max_size=w.max_size) for w in jobs]
            return [ctx.mine(d, p) for d, p in zip(dss, ps)]
        ps = [colo.default_params(w.R, w.thr, mode, max_size=w.max_size) for w in jobs]
        return ctx.mine_batch(dss, ps)

    out = {}
    in_bytes = 8 * int(sum(w.n for w in jobs))
    for form in ("batched", "plain"):
        for _ in range(args.warmup):
            run(form)
        if dist:
            dist.barrier()
        torch.cuda.synchronize(dev)
        tm = StepTimer(torch, dev, stream, in_bytes)
        res = None
        for _ in range(args.steps):
            res = tm.step(lambda: run(form))
        torch.cuda.synchronize(dev)
        ms = tm.ms()
        total, ms = replicas.aggregate(dist, sum(r.num_candidates() for r in res) * args.steps, ms, dev)
        out[form] = (ms, res, total)
    cands = sum(r.num_candidates() for r in out["batched"][1])
    same = all(a.patterns() == b.patterns() for a, b in zip(out["batched"][1], out["plain"][1]))
    if rank == 0:
        ms_b, ms_p = out["batched"][0], out["plain"][0]
        print(json.dumps({
            "metric": METRIC, "value": out["batched"][2] / (ms_b / 1e3), "unit": "candidates/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_b / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded generator)",
            "config": {"workload": JOBS_WORKLOAD,
                       "points": int(sum(w.n for w in jobs)), "jobs": len(jobs), "candidates_per_step": cands,
                       "form": "batched+learned" if mode == colo.MODE_LEARNED else "batched",
                       "l2": l2_note(in_bytes)},
            "plain": {"value": out["plain"][2] / (ms_p / 1e3), "unit": "candidates/s",
                      "ms_per_step": ms_p / args.steps},
            "headline_vs_plain": ms_p / ms_b, "identical_patterns_all_forms": same,
        }), flush=True)


def side_configs(ctx, dev, stream, head_mode, steps: int = 3, warmup: int = 1, cpu: bool = True):
    """The other configurations, each timed in the plain two-pass form and in the headline form on
    resident points (CUDA events on the library's stream), with the CPU oracle's time beside them:
    config0 (20,000 points), config1 (1,000,000 points) and config2 (512 independent jobs; batched:
    one colo_mine_batch call, plain: the jobs mined one at a time).  Fewer steps than the headline
    line: these are the reported numbers for the configurations the headline does not cover."""
    import torch
    import colo
    import oracle
    from colo import gen

    def timed(run, in_bytes):
        for _ in range(warmup):
            run()
        torch.cuda.synchronize(dev)
        tm = StepTimer(torch, dev, stream, in_bytes)
        res = None
        for _ in range(steps):
            res = tm.step(run)
        torch.cuda.synchronize(dev)
        return tm.ms() / steps, res

    out = {}
    for cfg in (0, 1):
        wl = gen.config(cfg)
        ds = colo.Dataset.from_arrays(ctx, wl.x, wl.y, wl.fid, wl.bounds)
        ds.upload()
        r = {"workload": f"config{cfg}", "points": wl.n, "l2": l2_note(8 * wl.n)}
        pats = None
        same = True
        for name, mode in (("headline", head_mode), ("plain", colo.MODE_PLAIN)):
            prm = colo.default_params(wl.R, wl.thr, mode, max_size=wl.max_size)
            ms, res = timed(lambda: ctx.mine(ds, prm), 8 * wl.n)
            c = res.num_candidates()
            r[name] = {"ms_per_step": round(ms, 4), "candidates_per_s": c / (ms / 1e3), "candidates": c}
            same &= pats is None or res.patterns() == pats
            pats = res.patterns()
        r["headline_vs_plain"] = r["plain"]["ms_per_step"] / r["headline"]["ms_per_step"]
        r["identical_patterns"] = same
        if cpu:
            t = time.perf_counter()
            o = oracle.mine(wl.x, wl.y, wl.fid, wl.bounds, wl.R, wl.thr, max_k=wl.max_size, fast=True)
            sec = time.perf_counter() - t
            r["cpu_oracle"] = {"ms_per_step": round(sec * 1e3, 2), "candidates_per_s": o.num_candidates() / sec,
                               "identical_patterns": o.patterns() == pats}
        out[f"config{cfg}"] = r
        del ds
    jobs = gen.config2_jobs(512)
    dss = [colo.Dataset.from_arrays(ctx, w.x, w.y, w.fid, w.bounds) for w in jobs]
    for d in dss:
        d.upload()
    hp = [colo.default_params(w.R, w.thr, head_mode, max_size=w.max_size) for w in jobs]
    pp = [colo.default_params(w.R, w.thr, colo.MODE_PLAIN, max_size=w.max_size) for w in jobs]
    jb = 8 * int(sum(w.n for w in jobs))
    ms_b, rb = timed(lambda: ctx.mine_batch(dss, hp), jb)
    ms_p, rp = timed(lambda: [ctx.mine(d, p) for d, p in zip(dss, pp)], jb)
    cands = sum(x.num_candidates() for x in rb)
    out["config2"] = {"workload": JOBS_WORKLOAD, "points": int(sum(w.n for w in jobs)), "jobs": len(jobs),
                      "l2": l2_note(jb),
                      "headline": {"ms_per_step": round(ms_b, 3), "candidates_per_s": cands / (ms_b / 1e3),
                                   "candidates": cands},
                      "plain": {"ms_per_step": round(ms_p, 3), "candidates_per_s": cands / (ms_p / 1e3)},
                      "headline_vs_plain": ms_p / ms_b,
                      "identical_patterns": all(a.patterns() == b.patterns() for a, b in zip(rb, rp)),
                      "steps": steps, "warmup": warmup}
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--config", type=int, default=3)
    ap.add_argument("--scale", type=float, default=1.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-side", action="store_true",
                    help="skip the other configurations (config0, config1, config2) reported beside the headline")
    ap.add_argument("--join-group", type=int, default=0,
                    help="pin the join's lanes per anchor instead of autotuning (profiling runs: "
                         "ncu serialises launches and distorts the autotuner's timings)")
    ap.add_argument("--forms", default="batched,e2e,plain",
                    help="comma list of batched (resident), e2e (host buffers), plain; the headline form "
                         "(batched+learned) always runs")
    args = ap.parse_args()
    rank, world, local = dist_env()
    from colo import gen

    if args.impl == "reference":
        if rank != 0:
            return
        if args.config == 2:
            wls, workload = gen.config2_jobs(512, scale=args.scale), JOBS_WORKLOAD
        else:
            wls = [gen.config(args.config, scale=args.scale)]
            workload = workload_name(args.config, args.scale, wls[0].n)
        value, cores, sample, sec, phases = run_cpu(wls, args.steps, args.warmup)
        print(json.dumps({
            "impl": "reference", "metric": METRIC, "value": value, "unit": "candidates/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": sec * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded generator)",
            "config": {"workload": workload, "points": int(sum(w.n for w in wls)), "sample": sample},
            "cpu_baseline": {"value": value, "unit": "candidates/s", "cores": cores, "kind": "port",
                             "sample": sample, "phase_ms_last_step": phases},
            "e2e": {"value": value, "unit": "candidates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        }), flush=True)
        return

    import torch
    import colo
    from colo import replicas

    dist = None
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    dev = torch.device("cuda", local)
    if args.config == 2:
        return bench_jobs(args, rank, world, local, dist)
    wl = gen.config(args.config, scale=args.scale)
    ctx = colo.Context(local)
    ds = colo.Dataset.from_arrays(ctx, wl.x, wl.y, wl.fid, wl.bounds)
    stream = torch.cuda.ExternalStream(ctx.stream(), device=dev)

    def barrier_sync():
        if dist:
            dist.barrier()
        torch.cuda.synchronize(dev)

    spreads = {}

    def timed(mode, resident, profile=False):
        params = colo.default_params(wl.R, wl.thr, mode, max_size=wl.max_size, profile=profile)
        if resident:
            ds.upload()
        for _ in range(args.warmup):
            if not resident:
                ds.evict()
            ctx.mine(ds, params)
        results = []
        barrier_sync()
        tm = StepTimer(torch, dev, stream, 8 * wl.n)
        with ClockSampler(local) as clk:
            clk.mark_start()
            for _ in range(args.steps):
                if not resident:
                    ds.evict()
                results.append(tm.step(lambda: ctx.mine(ds, params)))
            barrier_sync()
            clk.mark_end()
        ms = tm.ms()
        spreads[(mode, resident, profile)] = tm.spread()
        units = sum(r.num_candidates() for r in results)
        total, ms = replicas.aggregate(dist, units, ms, dev)   # all ranks' candidates, slowest rank's time
        return ms, results, clk.summary(), total

    forms = set(args.forms.split(","))
    # headline form: batched + learned presizing (the committed trained cost model)
    model = None
    try:
        model = colo.load_model()
    except OSError:
        pass
    head_mode = colo.MODE_LEARNED if model is not None else colo.MODE_BATCHED
    ctx.set_model(model)
    # launch shapes for this dataset (untimed; kept by the context): the join's lanes per anchor, the
    # level filter's candidates per unit, the level kernels' threads per block
    if args.join_group:
        ctx.set_join_group(args.join_group)
        tuned = {"join_group": args.join_group, "filter_unit": None, "level_block": None}
    else:
        tuned = ctx.autotune_all(ds, colo.default_params(wl.R, wl.thr, head_mode, max_size=wl.max_size))
    ms_b, res_b, clocks, tot_b = timed(head_mode, True)
    cands = res_b[0].num_candidates()
    value = tot_b / (ms_b / 1e3)
    ms_e, res_e, ms_p, res_p, tot_e, tot_p = ms_b, res_b, ms_b, res_b, tot_b, tot_b
    if "e2e" in forms:
        ms_e, res_e, _, tot_e = timed(head_mode, False)
    e2e = tot_e / (ms_e / 1e3)
    ms_bt, res_bt, tot_bt = ms_b, res_b, tot_b
    if "batched" in forms and head_mode != colo.MODE_BATCHED:
        ms_bt, res_bt, _, tot_bt = timed(colo.MODE_BATCHED, True)
    if "plain" in forms:
        ms_p, res_p, _, tot_p = timed(colo.MODE_PLAIN, True)
    plain = tot_p / (ms_p / 1e3)
    # every form mined the same patterns
    same = all(r.patterns() == res_b[0].patterns() for r in res_b + res_e + res_p + res_bt)

    # per-kernel CUDA-event times (a separate profiled pass, so `value` carries no event overhead)
    ms_k, res_k, _, _ = timed(head_mode, True, profile=True)
    kern, gaps, hosts, parts = {}, {}, {}, {}
    for r in res_k:
        for name, (nl, kms) in r.kernels.items():
            # "gap X": stream time between the previous timed scope and X (the GPU waiting for the host);
            # "host X": host time from the last wait's return to X's launch
            # "part X": host time of one part of the level loop (between two marks)
            a = (gaps if name.startswith("gap ") else hosts if name.startswith("host ")
                 else parts if name.startswith("part ") else kern).setdefault(name, [0, 0.0])
            a[0] += nl
            a[1] += kms
    counters = dict(res_b[0].counters)
    counters["key_bits"] = cell_key_bits([(wl.bounds, wl.R)])
    words = (wl.nfeat + 31) // 32
    peak, peak_kind = measured_peak_gbs()
    roof = None
    if kern:
        top = max(kern, key=lambda k: kern[k][1])
        nl, kms = kern[top]
        per_step_launches = nl / args.steps
        bytes_per_launch = algorithmic_bytes(top, counters, per_step_launches, words) / max(per_step_launches, 1)
        achieved = bytes_per_launch / (kms / nl / 1e3) / 1e9 if kms > 0 else 0.0
        tr = load_traffic(top)
        roof = {"kernel": top, "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "peak_source": f"{peak_kind} hbm_gbs (burst)",
                "traffic": tr, "avg_launch_ms": kms / nl, "launches_per_step": per_step_launches,
                "algorithmic_bytes_per_launch": bytes_per_launch, "share_of_step": kms / ms_k}
    per_kernel = {}
    for name, (nl, kms) in sorted(kern.items(), key=lambda kv: -kv[1][1]):
        ab = algorithmic_bytes(name, counters, nl / args.steps, words)
        per_kernel[name] = {"ms": round(kms / args.steps, 3), "launches": round(nl / args.steps, 1),
                            "gbs": round(ab / (kms / args.steps / 1e3) / 1e9, 1) if kms > 0 and ab else None}
    gaps_per_step = {name[4:]: round(kms / args.steps, 3)
                     for name, (nl, kms) in sorted(gaps.items(), key=lambda kv: -kv[1][1])}
    host_per_step = {name[5:]: round(kms / args.steps, 3)
                     for name, (nl, kms) in sorted(hosts.items(), key=lambda kv: -kv[1][1])}
    parts_per_step = {name[5:]: round(kms / args.steps, 3)
                      for name, (nl, kms) in sorted(parts.items(), key=lambda kv: -kv[1][1])}
    phases = {k: round(statistics.mean(r.times[k] for r in res_b), 3)
              for k in ("bucket", "join", "filter", "refine", "fill", "apriori", "total")}
    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return
    cpu = None
    io = None
    side = None
    if not args.no_side and world == 1 and args.config == 3 and args.scale == 1.0:
        side = side_configs(ctx, dev, stream, head_mode, cpu=not args.no_cpu)
    if not args.no_cpu and world == 1:
        v, cores, sample, sec, phases = run_cpu([wl], 1, 0)
        cpu = {"value": v, "unit": "candidates/s", "cores": cores, "kind": "port", "sample": sample,
               "s_per_step": round(sec, 3), "phase_ms": phases}
        io = measure_io(ctx, wl, ds, colo.default_params(wl.R, wl.thr, head_mode, max_size=wl.max_size),
                        res_b[0].patterns())
    line = {
        "metric": METRIC, "value": value, "unit": "candidates/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_b / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded generator; no public dataset exists)",
        "config": {"workload": workload_name(args.config, args.scale, wl.n), "points": wl.n, "features": wl.nfeat,
                   "candidates_per_step": cands,
                   "join_active_anchors": int(counters["active_anchors"]), "join_pairs": int(counters["join_pairs"]),
                   "neighbor_entries": int(counters["neighbors"]), "cells": int(counters["cells"]),
                   "runs": int(counters["runs"]), "nrl_entries": int(counters["nrl_entries"]),
                   "filter_items": int(counters["filter_items"]), "filter_full_quads": int(counters["filter_full_quads"]),
                   "filter_cells": int(counters["filter_cells"]),
                   "form": "batched+learned" if head_mode == colo.MODE_LEARNED else "batched",
                   "l2": l2_note(8 * wl.n),
                   "parallelism": f"replicas x{world}", "autotuned": tuned},
        "e2e": {"value": e2e, "unit": "candidates/s", "ms_per_step": ms_e / args.steps,
                "h2d_bytes_per_step": int(res_e[0].counters["h2d_bytes"]),
                "d2h_bytes_per_step": int(res_e[0].counters["d2h_bytes"])},
        "plain": {"value": plain, "unit": "candidates/s", "ms_per_step": ms_p / args.steps},
        "batched": {"value": tot_bt / (ms_bt / 1e3), "unit": "candidates/s",
                    "ms_per_step": ms_bt / args.steps,
                    "host_phase_ms": {k: round(statistics.mean(r.times[k] for r in res_bt), 3)
                                      for k in ("bucket", "join", "filter", "refine", "fill", "apriori", "total")},
                    "level_filter_wait_us": int(res_bt[0].counters["level_filter_wait_us"])},
        "pairs_model_us": int(res_b[0].counters["pairs_model_us"]),
        "level_filter_wait_us": int(res_b[0].counters["level_filter_wait_us"]),
        "headline_vs_plain": (ms_p / ms_b),
        "learned_presize": ({"single_pass": int(res_b[0].counters["single_pass"]),
                             "overflow_fallback": int(res_b[0].counters["single_pass_overflow"])}
                            if head_mode == colo.MODE_LEARNED else None),
        "identical_patterns_all_forms": same,
        "step_ms_spread": {"headline": spreads.get((head_mode, True, False)), "e2e": spreads.get((head_mode, False, False)),
                           "batched": spreads.get((colo.MODE_BATCHED, True, False)),
                           "plain": spreads.get((colo.MODE_PLAIN, True, False))},
        "gpu_launches": int(sum(r.counters["launches"] for r in res_b)),
        "clocks": clocks, "roofline": roof, "cpu_baseline": cpu, "kernels_per_step": per_kernel,
        "idle_before_kernel_per_step": gaps_per_step, "host_after_wait_per_step": host_per_step,
        "level_loop_host_ms_per_step": parts_per_step,
        "host_phase_ms": phases,
        "io": io,
        "side_configs": side,
    }
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
