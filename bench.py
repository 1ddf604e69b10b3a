#!/usr/bin/env python3
"""Benchmark of sandengine's Margolus grid update on GB300.

Workload (default, the 16384^2 world): 16384 x 16384 cells (u32 ids, 1 GiB per buffer),
the bundled twelve-material rule set (fire ignites wood p=1/16 and burns out p=1/32, acid
eats stone p=1/8, lava, water, steam, ...), seed-2 fill in 64x64 material patches.  One
step = 60 frames whose first frame carries 32 circle edits (radius 8-64, uniform
positions, EMPTY or sand), i.e. one edit period.  Metric: cell-updates/s (one cell
advanced one frame = one update).  Inputs are larger than L2 (129 MB), so no flush is
needed between steps.

    python bench.py [--steps K] [--warmup W] [--gpus N] [--impl ours|reference]
                    [--workload world16384|world4096|world256] [--k FRAMES_PER_LAUNCH]

--impl reference times the reference's own compute shader compiled for the CPU
(oracle/_ref, the reference's shaders/compute/falling_sand.glsl with the rule set's
generated GLSL) on all host cores, on a bounded band of the same world; without that
build it times the oracle port.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

FRAMES_PER_STEP = 60
EDITS_PER_STEP = 32
METRIC = "cell-updates/s (% HBM roofline); p50/p99 batched vs plain launch, bit-exact"
UNIT = "cell-updates/s"


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=40)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", default="world16384",
                    choices=["world16384", "world8192", "world4096", "world256", "batch4096", "serve"])
    ap.add_argument("--worlds", type=int, default=4096, help="batch4096: number of worlds")
    ap.add_argument("--resident-limit", type=int, default=None,
                    help="batch4096: shared-memory bytes up to which a world stays resident (0: none)")
    ap.add_argument("--k", type=int, default=0, help="frames per launch (0 = autotuned)")
    ap.add_argument("--cpu-seconds", type=float, default=10.0, help="CPU baseline sample length")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--light", action="store_true",
                    help="world workloads: keep the light field (light pass after every frame, one-frame "
                         "launches) and composite the frame once per step")
    return ap.parse_args()


def workload(name):
    from sandengine_gb300 import workloads as wl
    if name == "world16384":
        return dict(name="world16384", ruleset="twelve_materials", size=16384,
                    grid=lambda: wl.world_16384(2), edit_mats=[0, 3], fill="seed-2 64x64 patches")
    if name == "world8192":  # the same world family at 1/4 size (ncu captures)
        return dict(name="world8192", ruleset="twelve_materials", size=8192,
                    grid=lambda: wl.world_16384(2, 8192), edit_mats=[0, 3], fill="seed-2 64x64 patches")
    if name.startswith("batch"):  # CPU arms sample one 1024^2 world of the batch family
        return dict(name=name, ruleset="twelve_materials", size=1024,
                    grid=lambda: wl.patch_fill(1024, 1024, 1000, *wl.twelve_fill_spec(), patch=16),
                    edit_mats=[0, 3], fill="per-world seeded 16x16 patches")
    if name == "world4096":
        return dict(name="world4096", ruleset="four_materials", size=4096,
                    grid=lambda: wl.world_4096(1), edit_mats=[0, 3], fill="seed-1 iid 0.6/0.2/0.15/0.05")
    return dict(name="world256", ruleset="four_materials", size=256,
                grid=lambda: wl.world_256(0), edit_mats=[0, 3], fill="seed-0 iid 0.6/0.2/0.15/0.05")


def step_mods(se, wl, size, r, mats):
    raw = wl.circle_edits(size, size, 2, r, EDITS_PER_STEP, mats)
    return [se.SimModification((m[0], m[1]), m[2], m[3], m[4]) for m in raw]


def load_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def load_traffic(cells_per_launch):
    """DRAM bytes of one tile-kernel launch: the committed ncu capture's bytes per cell (an
    8192^2 world of the same family) scaled to the launch's cells."""
    p = os.path.join(ROOT, "profiles", "tile_kernel_traffic.txt")
    if not os.path.exists(p):
        return None
    vals = {}
    for line in open(p):
        if "=" in line and not line.startswith("#"):
            a, b = line.strip().split("=", 1)
            vals[a.strip()] = b.strip()
    try:
        return float(vals["dram_bytes_per_cell"]) * cells_per_launch
    except Exception:
        return None


class ClockSampler:
    """nvidia-smi clock / throttle samples every 100 ms during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.proc = None
        self.path = None

    def __enter__(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.out = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.idx), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=self.out, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.out.close()

    def summary(self):
        if not self.path or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"], "samples": 0}
        sms, maxs, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sms.append(float(parts[1]))
                maxs.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sms) if sms else None, "sm_max_mhz": max(maxs) if maxs else None,
                "reasons": sorted(reasons), "samples": len(sms)}


def cpu_info():
    model = ""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True).stdout
        for line in out.splitlines():
            if line.startswith("Model name"):
                model = line.split(":", 1)[1].strip()
    except Exception:
        pass
    return os.cpu_count() or 1, model


def cpu_rate(W, wl_spec, seconds, prefer_reference=True):
    """Cell-updates/s of the CPU implementation on a band of the workload's world.
    Returns (rate, kind, cores, sample)."""
    from sandengine_gb300 import workloads as wl
    from oracle.build import Port, Ref
    cores, model = cpu_info()
    text = wl.ruleset_text(wl_spec["ruleset"])
    full = wl_spec["grid"]()
    kind = "port"
    ref = None
    if prefer_reference:
        try:
            ref = Ref(text)
            kind = "reference"
        except Exception:
            ref = None
    # band height giving ~0.5 s per frame, from a 16-row probe
    probe = np.ascontiguousarray(full[:16])
    port = None if ref else Port(text)

    def run_band(band, frames):
        t0 = time.perf_counter()
        if ref:
            tot = 0.0
            for f in range(frames):
                tot += ref.time_rows(band, 2 + f, 0, band.shape[0], cores)
            return tot
        g = band.copy()
        port.run(g, 1, frames, None, cores)
        return time.perf_counter() - t0

    t = run_band(probe, 1)
    rows = int(max(16, min(full.shape[0], 16 * 0.5 / max(t, 1e-6))))
    band = np.ascontiguousarray(full[:rows])
    t1 = run_band(band, 1)
    frames = max(1, int(seconds / max(t1, 1e-6)))
    secs = run_band(band, frames)
    rate = band.size * frames / secs
    sample = (f"{wl_spec['name']} rows 0-{rows - 1} ({W} x {rows} band of the seeded world), {frames} frame(s), "
              f"{secs:.1f} s on {cores} threads ({model})")
    return rate, kind, cores, sample


def run_ours(args, rep):
    import torch
    import sandengine_gb300 as se
    from sandengine_gb300 import workloads as wl

    spec = workload(args.workload)
    W = H = spec["size"]
    rs = se.parse_string(wl.ruleset_text(spec["ruleset"]))
    grid0 = spec["grid"]()
    sim = se.Simulation(rs, (W, H))
    sim.grid = grid0
    sim.params.frame = 1
    if args.k:
        sim.set_steps_per_launch(args.k)
        k = args.k
    else:
        k = sim.autotune(3)
    stream = torch.cuda.ExternalStream(sim.stream)
    mods = [step_mods(se, wl, W, r, spec["edit_mats"]) for r in range(args.warmup + args.steps)]
    if args.light:
        sim.set_light(True)

    def one_step(r):
        sim.run_frames(FRAMES_PER_STEP, mods[r])
        if args.light:
            sim.composite_device()  # colour render, its pyramid and the composite

    for r in range(args.warmup):
        one_step(r)
    sim.synchronize()

    sim.set_timing(True)
    sim.read_timing()
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    rep.barrier()
    torch.cuda.synchronize()
    with ClockSampler(torch.cuda.current_device()) as clocks:
        start.record(stream)
        for r in range(args.steps):
            one_step(args.warmup + r)
        end.record(stream)
        torch.cuda.synchronize()
    rep.barrier()
    ms = start.elapsed_time(end)
    timing = sim.read_timing()
    passes = {p: sim.read_pass_timing(p) for p in (1, 2, 3)} if args.light else {}
    sim.set_timing(False)
    ms_max = rep.max(ms)
    updates = float(W) * H * FRAMES_PER_STEP * args.steps
    value = rep.sum(updates) / (ms_max / 1e3)

    # e2e through the public API with host buffers: per step the mods go host->device
    # (kernel parameters) and the grid comes back into pinned host memory.
    e2e = None
    if not args.no_e2e:
        # two pinned buffers; each step's grid is snapshotted on the device and copied to the
        # host on a copy stream while the next step computes
        hosts = [torch.empty((H, W), dtype=torch.int32, pin_memory=True) for _ in range(2)]
        from sandengine_gb300._lib import check, lib
        rep.barrier()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for r in range(args.steps):
            one_step(args.warmup + r)
            check(lib().se_world_read_grid_overlapped(sim.handle, hosts[r & 1].data_ptr(), W * H))
        sim.synchronize()
        e2e_s = rep.max(time.perf_counter() - t0)
        e2e = {"value": rep.sum(updates) / e2e_s, "unit": UNIT,
               "h2d_bytes_per_step": EDITS_PER_STEP * 32, "d2h_bytes_per_step": W * H * 4}

    peak, peak_src = load_peak()
    launches = timing["launches"]
    kernel_ms = timing["kernel_ms"]
    alg_bytes_per_launch = 8.0 * timing["cells"] / max(launches, 1)
    avg_launch_s = kernel_ms / max(launches, 1) / 1e3
    achieved = alg_bytes_per_launch / avg_launch_s / 1e9 if launches else None
    traffic = load_traffic(W * H) if spec["ruleset"] == "twelve_materials" else None
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": rep.world_size, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic (seeded splitmix64)",
        "config": {"workload": f"{spec['name']}: {W}x{H} u32 cells, {spec['ruleset']} rule set, {spec['fill']}, "
                               f"{FRAMES_PER_STEP} frames per step, {EDITS_PER_STEP} circle edits on the first",
                   "frames_per_launch": k, "l2": "inputs larger than L2 (1 GiB per buffer)" if W >= 8192
                   else "world fits in L2; no flush", "parallelism": f"replicas{rep.world_size}"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": (achieved / peak) if achieved else None, "traffic": traffic,
                     "kernel": f"se_tile (k={k})", "peak_source": peak_src,
                     "algorithmic_bytes_per_launch": alg_bytes_per_launch,
                     "avg_launch_ms": avg_launch_s * 1e3, "kernel_share_of_step": kernel_ms / ms if ms else None,
                     # k frames per launch: 8 B per cell per launch cover k updates.  The
                     # same updates from one-frame launches would move value * 8 bytes/s.
                     "unfused_equivalent_gbs": value * 8.0 / 1e9,
                     "unfused_equivalent_frac": value * 8.0 / 1e9 / peak},
        "gpu_launches": launches + args.steps + sum(p["launches"] for p in passes.values()),
        "clocks": clocks.summary(),
    }
    # algorithmic bytes per cell: light = old id, new id, old light in, light out (4 + 4 + 16 + 16);
    # colour (inside the composite) = id, noise, RGBA out and a quarter of the level-1 alpha
    # float; composite = colour, light, RGBA out (the smaller pyramid levels are not counted)
    for p, name, bpc in ((1, "light_pass", 40.0), (2, "color_pass", 25.0), (3, "composite_pass", 48.0)):
        if p in passes and passes[p]["launches"]:
            t = passes[p]
            avg_s = t["kernel_ms"] / t["launches"] / 1e3
            ach = bpc * t["cells"] / t["launches"] / avg_s / 1e9
            out[name] = {"bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak,
                         "algorithmic_bytes_per_cell": bpc, "launches": t["launches"], "avg_launch_ms": avg_s * 1e3,
                         "share_of_step": t["kernel_ms"] / ms if ms else None}
    if args.light:
        out["config"]["workload"] += ("; light field kept (light pass after every frame), one headless composite "
                                      "(colour render, pyramid, composite) per step")
    if e2e:
        out["e2e"] = e2e
    if rep.rank == 0 and rep.world_size == 1 and not args.no_cpu_baseline:
        rate, kind, cores, sample = cpu_rate(W, spec, args.cpu_seconds)
        out["cpu_baseline"] = {"value": rate, "unit": UNIT, "cores": cores, "kind": kind, "sample": sample}
    return out


def percentile(xs, q):
    s = sorted(xs)
    if not s:
        return None
    i = min(len(s) - 1, max(0, int(round(q / 100.0 * (len(s) - 1)))))
    return s[i]


def run_batch(args, rep):
    """4096 worlds (sides log-uniform in [64, 1024], multiples of 32, per-world seeds), the
    twelve-material rule set; one step = one 100-frame launch of every world."""
    import torch
    import sandengine_gb300 as se
    from sandengine_gb300 import workloads as wl
    from sandengine_gb300.batch import Batch
    frames = 100
    sizes = wl.batch_sizes(args.worlds, 4)
    rs = se.parse_string(wl.ruleset_text("twelve_materials"))
    b = Batch(rs, sizes)
    if args.resident_limit is not None:
        b.set_resident_limit(args.resident_limit)
    spec = wl.twelve_fill_spec()
    for i, (w, h) in enumerate(sizes):
        b.set_grid(i, wl.patch_fill(w, h, 1000 + i, *spec, patch=16))
        b.set_frame(i, 1)
    k = b.autotune(2) if not args.k else (b.set_steps_per_launch(args.k) or args.k)
    info = b.info()
    cells = info["cells"]
    stream = torch.cuda.ExternalStream(b.stream)
    for _ in range(args.warmup):
        b.step(frames)
    b.synchronize()
    evs = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps + 1)]
    rep.barrier()
    torch.cuda.synchronize()
    with ClockSampler(torch.cuda.current_device()) as clocks:
        evs[0].record(stream)
        for s in range(args.steps):
            b.step(frames)
            evs[s + 1].record(stream)
        torch.cuda.synchronize()
    rep.barrier()
    lat = [evs[s].elapsed_time(evs[s + 1]) for s in range(args.steps)]
    ms = evs[0].elapsed_time(evs[-1])
    ms_max = rep.max(ms)
    updates = float(cells) * frames * args.steps
    value = rep.sum(updates) / (ms_max / 1e3)
    # the plain path: one launch per world per frame, as the reference dispatches
    plain_frames = 3
    b.step_plain(1)
    b.synchronize()
    t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    t0.record(stream)
    b.step_plain(plain_frames)
    t1.record(stream)
    torch.cuda.synchronize()
    plain_ms = t0.elapsed_time(t1)
    plain_rate = float(cells) * plain_frames / (plain_ms / 1e3)
    plain_100 = plain_ms / plain_frames * frames
    peak, peak_src = load_peak()
    return {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": rep.world_size, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u32", "data": "synthetic (seeded splitmix64)",
        "config": {"workload": f"batch{args.worlds}: {args.worlds} worlds, sides log-uniform in [64, 1024] "
                               f"(multiples of 32), {cells} cells, twelve_materials rule set, per-world seeds; "
                               f"one step = {frames} frames of every world in one CUDA-graph launch",
                   "frames_per_pass": k, "resident_worlds": info["resident_worlds"],
                   "tiled_worlds": info["tiled_worlds"], "parallelism": f"replicas{rep.world_size}",
                   "l2": "inputs larger than L2"},
        "batched": {"p50_ms": percentile(lat, 50), "p99_ms": percentile(lat, 99),
                    "plain_value": plain_rate, "plain_ms_per_100_frames": plain_100,
                    "speedup_vs_plain": value / plain_rate},
        "roofline": {"bound": "issue (compute)", "achieved": None, "peak": peak, "unit": "GB/s", "frac": None,
                     "traffic": None, "peak_source": peak_src,
                     "note": "worlds that fit in shared memory stay on chip for all 100 frames; HBM is not the bound"},
        "gpu_launches": args.steps * ((-(-frames // k) if info["tiled_worlds"] else 0) + 3 + 1),
        "clocks": clocks.summary(),
    }


def serve_workload(rate, n_requests, seed=5):
    """Poisson arrivals at `rate` req/s; each request opens a new session (p=0.5) or reuses an
    earlier one; sides log-uniform in [128, 2048] (multiples of 32); N ~ U[1, 600] frames;
    0-8 circle edits (radius 8-64, EMPTY or sand) on the first frame."""
    from sandengine_gb300 import workloads as wl
    u = wl.uniform53(seed, 9, np.arange(8 * n_requests, dtype=np.uint64)).astype(np.float64) / float(1 << 53)
    u = u.reshape(n_requests, 8)
    t = np.cumsum(-np.log1p(-u[:, 0]) / rate) * 1e3  # ms
    sessions, reqs = [], []
    for i in range(n_requests):
        if not sessions or u[i, 1] < 0.5:
            w = int(np.clip(np.round(np.exp(np.log(128) + u[i, 2] * np.log(16)) / 32) * 32, 128, 2048))
            h = int(np.clip(np.round(np.exp(np.log(128) + u[i, 3] * np.log(16)) / 32) * 32, 128, 2048))
            sessions.append((w, h))
            s = len(sessions) - 1
        else:
            s = int(u[i, 1] * 2 * len(sessions)) % len(sessions)
        n = 1 + int(u[i, 4] * 600)
        ne = int(u[i, 5] * 9)
        w, h = sessions[s]
        mods = wl.circle_edits(w, h, seed, i, ne, [0, 3]) if ne else []
        reqs.append((s, n, mods, float(t[i])))
    return sessions, reqs


def run_serve(args, rep):
    import sandengine_gb300 as se
    from sandengine_gb300 import workloads as wl
    from sandengine_gb300.serving import Server
    rs = se.parse_string(wl.ruleset_text("twelve_materials"))
    spec = wl.twelve_fill_spec()
    budget = 150 << 30
    sweep = []
    for rate in (200, 1000, 4000, 16000):
        n_req = int(min(1200, max(200, rate * 0.6)))
        sessions, reqs = serve_workload(rate, n_req)
        grids = [wl.patch_fill(w, h, 3000 + i, *spec, patch=64) for i, (w, h) in enumerate(sessions)]
        row = {"rate_req_s": rate, "requests": n_req, "sessions": len(sessions)}
        for mode in ("batched", "plain"):
            srv = Server(rs, budget)
            for (w, h), g in zip(sessions, grids):
                srv.open_session(w, h, g, 1)
            for (s, n, mods, t) in reqs:
                srv.submit(s, n, [se.SimModification((m[0], m[1]), m[2], m[3], m[4]) for m in mods], t)
            srv.run(plain=(mode == "plain"))
            st = srv.stats()
            row[mode] = {"throughput": st["cell_updates"] / (st["wall_ms"] / 1e3), "p50_ms": st["p50_ms"],
                         "p99_ms": st["p99_ms"], "wall_ms": st["wall_ms"], "iterations": st["iterations"],
                         "evictions": st["evictions"]}
            del srv
        row["speedup"] = row["batched"]["throughput"] / row["plain"]["throughput"]
        sweep.append(row)
    best = max(sweep, key=lambda r: r["batched"]["throughput"])
    return {
        "metric": METRIC, "value": best["batched"]["throughput"], "unit": UNIT, "n_gpus": rep.world_size,
        "steps": len(sweep), "warmup": 0, "ms_per_step": best["batched"]["wall_ms"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic (seeded splitmix64)",
        "config": {"workload": "serve: Poisson arrivals (200-16000 req/s), sides log-uniform in [128, 2048], "
                               "N ~ U[1, 600] frames, 0-8 circle edits, twelve_materials rule set, 150 GB budget; "
                               "continuous batching vs one request at a time",
                   "parallelism": f"replicas{rep.world_size}"},
        "serving": sweep,
    }


def run_reference(args, rep):
    if rep.rank != 0:
        return None
    spec = workload(args.workload)
    W = spec["size"]
    from sandengine_gb300 import workloads as wl
    from oracle.build import Port, Ref
    text = wl.ruleset_text(spec["ruleset"])
    full = spec["grid"]()
    cores, model = cpu_info()
    try:
        ref = Ref(text)
        kind = "reference"
    except Exception:
        ref = None
        kind = "port"
    port = None if ref else Port(text)
    rows = 64 if W >= 4096 else W
    band = np.ascontiguousarray(full[:rows])

    def one(f):
        if ref:
            return ref.time_rows(band, f, 0, rows, cores)
        g = band.copy()
        t0 = time.perf_counter()
        port.run(g, f - 1, 1, None, cores)
        return time.perf_counter() - t0

    for i in range(args.warmup):
        one(2 + i)
    times = [one(2 + args.warmup + i) for i in range(args.steps)]
    value = band.size * args.steps / sum(times)
    sample = f"{spec['name']} rows 0-{rows - 1} ({W} x {rows} band), one frame per step, {cores} threads ({model})"
    return {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": rep.world_size,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * sum(times) / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32 texels (ids)",
            "data": "synthetic (seeded splitmix64)",
            "config": {"workload": f"{spec['name']}: {spec['ruleset']} rule set, {spec['fill']}; "
                                   f"reference compute shader on the CPU, bounded band sample",
                       "parallelism": "host threads"},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": kind, "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main():
    args = parse_args()
    from sandengine_gb300.replicas import Replicas
    rep = Replicas("nccl" if args.impl == "ours" else "gloo")
    try:
        if args.impl == "reference":
            out = run_reference(args, rep)
        elif args.workload.startswith("batch"):
            out = run_batch(args, rep)
        elif args.workload == "serve":
            out = run_serve(args, rep)
        else:
            out = run_ours(args, rep)
        if rep.rank == 0 and out is not None:
            print(json.dumps(out), flush=True)
    finally:
        rep.close()


if __name__ == "__main__":
    main()
