#!/usr/bin/env python3
"""Benchmark of sandengine's Margolus grid update on GB300.

Workload (default, the 16384^2 world): 16384 x 16384 cells (u32 ids, 1 GiB per buffer),
the bundled twelve-material rule set (fire ignites wood p=1/16 and burns out p=1/32, acid
eats stone p=1/8, lava, water, steam, ...), seed-2 fill in 64x64 material patches.  One
step = 60 frames whose first frame carries 32 circle edits (radius 8-64, uniform
positions, EMPTY or sand), i.e. one edit period.  Metric: cell-updates/s (one cell
advanced one frame = one update).  Inputs are larger than L2 (129 MB), so no flush is
needed between steps.

The default line also carries, measured in the same run:
  batched   4096 worlds (sides log-uniform in [64, 1024]) advanced 100 frames per launch
            group, p50/p99 per group, against one launch per world and frame;
  serving   the live serving loop fed with Poisson arrivals at 100-20000 requests/s,
            continuous batching against one request at a time, p50/p99 per request, the
            highest throughput each mode sustains under one p99 bound, and a run under a
            small HBM budget (LRU eviction to host and restores);
  cpu_baseline / cpu_baseline_grid   the reference's compute shader compiled for the CPU
            (the whole shader: grid, colour, light) and the oracle port (the grid update
            alone), on all host cores.

    python bench.py [--steps K] [--warmup W] [--gpus N] [--impl ours|reference]
                    [--workload world16384|world8192|world4096|world256|batch4096|serve]
                    [--parallelism replicas|bands] [--k FRAMES_PER_LAUNCH] [--tile WxHxK]

--gpus N (N > 1) without a torch.distributed environment relaunches this script under
torch.distributed.run with N ranks, one GPU each.  --parallelism replicas (default): every
rank runs its own copy of the workload (weak scaling, no data-path collective); bands:
one world split into row bands over the ranks, halo rows exchanged by NCCL send/recv
before each launch group (strong scaling).

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
    ap.add_argument("--tile", default=None,
                    help="world workloads: use the compiled tile variant WxHxK (e.g. 256x128x8) instead of the "
                         "autotuner's choice")
    ap.add_argument("--cpu-seconds", type=float, default=10.0, help="CPU baseline sample length")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--parallelism", choices=["replicas", "bands"], default="replicas")
    ap.add_argument("--no-batched", action="store_true", help="world workloads: leave out the batched figures")
    ap.add_argument("--no-serving", action="store_true", help="world workloads: leave out the serving figures")
    ap.add_argument("--serve-requests", type=int, default=300, help="requests per arrival rate")
    ap.add_argument("--serve-k", type=int, default=8, help="frames per batched serving iteration")
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
    raw = wl.world_edits(size, r, mats)
    return [se.SimModification((m[0], m[1]), m[2], m[3], m[4]) for m in raw]


def load_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def load_traffic(workload_name, variant, k):
    """DRAM bytes of one tile-kernel launch from the committed ncu capture, when it was taken
    on this workload, variant and frames per launch (else None), with a note of its source."""
    p = os.path.join(ROOT, "profiles", "tile_kernel_traffic.txt")
    if not os.path.exists(p):
        return None, None
    vals = {}
    for line in open(p):
        if "=" in line and not line.startswith("#"):
            a, b = line.strip().split("=", 1)
            vals[a.strip()] = b.strip()
    try:
        if vals["workload"] != workload_name or vals["variant"] != variant or int(vals["k"]) != k:
            return None, (f"no capture of {variant} at k={k} on {workload_name} "
                          f"(the committed one is {vals['variant']} k={vals['k']} on {vals['workload']})")
        return float(vals["dram_bytes_per_launch"]), (f"ncu dram__bytes_read.sum + dram__bytes_write.sum of one "
                                                      f"{variant} launch at k={k} on {workload_name} "
                                                      f"(profiles/tile_kernel_256x128_k8_world16384.md)")
    except (KeyError, ValueError):
        return None, None


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
    """Cell-updates/s of the reference's compute shader compiled for the CPU (the whole
    shader: grid update, colour and light per invocation; the oracle port when that build is
    missing) on a band of the workload's world, one frame per sample, all host threads.
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
              f"{secs:.1f} s on {cores} threads ({model}); the whole compute shader per invocation: grid update, "
              f"colour and light")
    return rate, kind, cores, sample


def cpu_rate_grid(W, wl_spec, seconds):
    """Cell-updates/s of the grid update alone on the CPU (the oracle port, all host
    threads): a band of the workload's world advanced in the benchmark's own steps (60
    frames, the step's edit round on the first).  Returns (rate, cores, sample)."""
    import sandengine_gb300 as se  # noqa: F401  (workloads)
    from sandengine_gb300 import workloads as wl
    from oracle.build import Port
    cores, model = cpu_info()
    port = Port(wl.ruleset_text(wl_spec["ruleset"]))
    full = wl_spec["grid"]()
    # rows giving ~1 s per 60-frame step, from a one-frame probe of 64 rows
    probe = np.ascontiguousarray(full[:64]).copy()
    t0 = time.perf_counter()
    port.run(probe, 1, 1, None, cores)
    per_cell_frame = (time.perf_counter() - t0) / probe.size
    rows = int(max(64, min(full.shape[0], 1.0 / max(per_cell_frame * W * FRAMES_PER_STEP, 1e-12)))) // 2 * 2
    g = np.ascontiguousarray(full[:rows]).copy()
    frame, steps, secs = 1, 0, 0.0
    while secs < seconds or steps == 0:
        mods = wl.world_edits(W, steps, wl_spec["edit_mats"]) if W >= 4096 else None
        t0 = time.perf_counter()
        port.run(g, frame, FRAMES_PER_STEP, mods, cores)
        secs += time.perf_counter() - t0
        frame += FRAMES_PER_STEP
        steps += 1
    rate = g.size * FRAMES_PER_STEP * steps / secs
    sample = (f"{wl_spec['name']} rows 0-{rows - 1} ({W} x {rows} band of the seeded world), {steps} step(s) of "
              f"{FRAMES_PER_STEP} frames with the step's edits, {secs:.1f} s on {cores} threads ({model}); "
              f"the grid update alone")
    return rate, cores, sample


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
    if args.tile:
        tw, th, k = (int(v) for v in args.tile.lower().split("x"))
        sim.set_tile(tw, th, k)
    elif args.k:
        sim.set_steps_per_launch(args.k)
        k = args.k
    else:
        k = sim.autotune(3)
    tile = sim.tile()
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
    if not args.k and not args.tile:
        # tune again on the warmed-up world: its state (half of the chunks dynamic) is the one
        # the timed steps see, unlike the freshly filled world the first tuning saw
        k = sim.autotune(3)
        tile = sim.tile()
        one_step(0)
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
    timing_k = sim.peek_timing_frames(k)  # the launches of the full fusion depth
    timing = sim.read_timing()
    passes = {p: sim.read_pass_timing(p) for p in (1, 2, 3)} if args.light else {}
    sim.set_timing(False)
    ms_max = rep.max(ms)
    updates = float(W) * H * FRAMES_PER_STEP * args.steps
    value = rep.sum(updates) / (ms_max / 1e3)

    # e2e through the public API with host buffers: per step the mods go host->device
    # (kernel parameters) and the whole grid comes back into pinned host memory, its ids
    # packed into bytes on the device (exact: after a frame every id names a material)
    e2e = None
    if not args.no_e2e:
        # two pinned buffers; each step's grid is packed on the device and copied to the host
        # on copy streams while the next step computes
        hosts = [torch.empty((H, W), dtype=torch.uint8, pin_memory=True) for _ in range(2)]
        from sandengine_gb300._lib import check, lib
        rep.barrier()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for r in range(args.steps):
            one_step(args.warmup + r)
            check(lib().se_world_read_grid_u8_overlapped(sim.handle, hosts[r & 1].data_ptr(), W * H))
        sim.synchronize()
        e2e_s = rep.max(time.perf_counter() - t0)
        e2e = {"value": rep.sum(updates) / e2e_s, "unit": UNIT,
               "h2d_bytes_per_step": EDITS_PER_STEP * 32, "d2h_bytes_per_step": W * H,
               "d2h": "the whole grid every step, one byte per cell (se_world_read_grid_u8_overlapped)"}

    peak, peak_src = load_peak()
    launches = timing["launches"]
    kernel_ms = timing["kernel_ms"]
    # every tile launch reads and writes the whole grid once (8 B per cell), whatever its
    # frame count; the launches of the full fusion depth k are also reported alone
    alg_bytes_per_launch = 8.0 * W * H
    avg_launch_s = kernel_ms / max(launches, 1) / 1e3
    achieved = alg_bytes_per_launch / avg_launch_s / 1e9 if launches else None
    k_launch_ms = timing_k["kernel_ms"] / timing_k["launches"] if timing_k["launches"] else None
    traffic, traffic_source = load_traffic(spec["name"], f"se_tile_{tile[0]}x{tile[1]}_k{tile[2]}", k)
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": rep.world_size, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic (seeded splitmix64)",
        "config": {"workload": f"{spec['name']}: {W}x{H} u32 cells, {spec['ruleset']} rule set, {spec['fill']}, "
                               f"{FRAMES_PER_STEP} frames per step, {EDITS_PER_STEP} circle edits on the first",
                   "frames_per_launch": k, "tile": f"{tile[0]}x{tile[1]}",
                   "tuning": ("fixed by --k/--tile" if (args.k or args.tile) else
                              "autotuned on the fresh world, then again after the warm-up steps "
                              "(one more untimed step follows)"),
                   "l2": "inputs larger than L2 (1 GiB per buffer)" if W >= 8192
                   else "world fits in L2; no flush", "parallelism": f"replicas{rep.world_size}"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": (achieved / peak) if achieved else None, "traffic": traffic,
                     "traffic_source": traffic_source,
                     "kernel": f"se_tile_{tile[0]}x{tile[1]}_k{tile[2]} (up to {k} frames per launch)",
                     "peak_source": peak_src,
                     "bound_note": "issue-bound at k >= 2: the integer ALU pipe runs at 73% of its peak and DRAM "
                                   "traffic equals the algorithmic bytes (profiles/tile_kernel_256x128_k8_world16384.md); "
                                   "one_frame_launches gives the same kernel at one frame per launch, HBM-bound",
                     "algorithmic_bytes_per_launch": alg_bytes_per_launch,
                     "avg_launch_ms": avg_launch_s * 1e3, "launches": launches,
                     "k_launches": timing_k["launches"], "k_launch_avg_ms": k_launch_ms,
                     "k_launch_frac": (alg_bytes_per_launch / (k_launch_ms / 1e3) / 1e9 / peak) if k_launch_ms else None,
                     "kernel_share_of_step": kernel_ms / ms if ms else None,
                     # k frames per launch: 8 B per cell per launch cover k updates.  The
                     # same updates from one-frame launches would move value * 8 bytes/s.
                     "unfused_equivalent_gbs": value * 8.0 / 1e9,
                     "unfused_equivalent_frac": value * 8.0 / 1e9 / peak},
        # the edits of each step run inside its first tile launch
        "gpu_launches": launches + sum(p["launches"] for p in passes.values()),
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
    if spec["name"] == "world16384" and not args.light and not args.k and not args.tile:
        # the same kernel at one frame per launch, the memory-bound form: two 60-frame steps
        sim.set_steps_per_launch(1)
        sim.set_timing(True)
        sim.read_timing()
        for r in range(2):
            sim.run_frames(FRAMES_PER_STEP, mods[r % len(mods)])
        t1 = sim.read_timing()
        sim.set_timing(False)
        avg1 = t1["kernel_ms"] / max(t1["launches"], 1)
        ach1 = 8.0 * W * H / (avg1 / 1e3) / 1e9
        out["one_frame_launches"] = {"launches": t1["launches"], "avg_launch_ms": avg1, "achieved": ach1,
                                     "peak": peak, "unit": "GB/s", "frac": ach1 / peak,
                                     "cell_updates_per_s": float(W) * H / (avg1 / 1e3)}
    if rep.rank == 0 and rep.world_size == 1 and not args.no_cpu_baseline:
        rate, kind, cores, sample = cpu_rate(W, spec, args.cpu_seconds)
        out["cpu_baseline"] = {"value": rate, "unit": UNIT, "cores": cores, "kind": kind, "sample": sample,
                               "includes": "the whole compute shader per cell (grid update, colour, light), "
                                           "as the reference dispatches it"}
        rate, cores, sample = cpu_rate_grid(W, spec, args.cpu_seconds)
        out["cpu_baseline_grid"] = {"value": rate, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample,
                                    "includes": "the grid update alone, the work the GPU figure measures"}
    del sim
    if spec["name"] == "world16384" and not args.light:
        if not args.no_batched:
            out["batched"] = measure_batch(rep, 4096, steps=20, warmup=3)
        if not args.no_serving:
            out["serving"] = measure_serving(rep, args.serve_requests, args.serve_k)
    return out


def percentile(xs, q):
    s = sorted(xs)
    if not s:
        return None
    i = min(len(s) - 1, max(0, int(round(q / 100.0 * (len(s) - 1)))))
    return s[i]


def measure_batch(rep, worlds, steps, warmup, k=0, resident_limit=None):
    """`worlds` worlds (sides log-uniform in [64, 1024], multiples of 32, per-world seeds),
    the twelve-material rule set; one step = one 100-frame launch group of every world (a
    captured CUDA graph).  Against the plain path: one launch per world and frame, as the
    reference dispatches (sandengine-core/src/simulation.rs:220-234)."""
    import torch
    import sandengine_gb300 as se
    from sandengine_gb300 import workloads as wl
    from sandengine_gb300.batch import Batch
    frames = 100
    sizes = wl.batch_sizes(worlds, 4)
    rs = se.parse_string(wl.ruleset_text("twelve_materials"))
    b = Batch(rs, sizes)
    if resident_limit is not None:
        b.set_resident_limit(resident_limit)
    spec = wl.twelve_fill_spec()
    for i, (w, h) in enumerate(sizes):
        b.set_grid(i, wl.patch_fill(w, h, 1000 + i, *spec, patch=16))
        b.set_frame(i, 1)
    k = b.autotune(2) if not k else (b.set_steps_per_launch(k) or k)
    info = b.info()
    cells = info["cells"]
    stream = torch.cuda.ExternalStream(b.stream)
    for _ in range(warmup):
        b.step(frames)
    b.synchronize()
    evs = [torch.cuda.Event(enable_timing=True) for _ in range(steps + 1)]
    rep.barrier()
    torch.cuda.synchronize()
    evs[0].record(stream)
    for i in range(steps):
        b.step(frames)
        evs[i + 1].record(stream)
    torch.cuda.synchronize()
    rep.barrier()
    lat = [evs[i].elapsed_time(evs[i + 1]) for i in range(steps)]
    ms = rep.max(evs[0].elapsed_time(evs[-1]))
    value = rep.sum(float(cells) * frames * steps) / (ms / 1e3)
    # the plain path: one launch per world per frame
    plain_frames = 3
    b.step_plain(1)
    b.synchronize()
    t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    t0.record(stream)
    b.step_plain(plain_frames)
    t1.record(stream)
    torch.cuda.synchronize()
    plain_ms = t0.elapsed_time(t1)
    plain_rate = rep.sum(float(cells) * plain_frames / (plain_ms / 1e3))
    return {"workload": f"batch{worlds}: {worlds} worlds, sides log-uniform in [64, 1024] (multiples of 32), "
                        f"{cells} cells, twelve_materials rule set, per-world seeds; one step = {frames} frames of "
                        f"every world in one CUDA-graph launch",
            "value": value, "unit": UNIT, "steps": steps, "warmup": warmup, "ms_per_step": ms / steps,
            "p50_ms": percentile(lat, 50), "p99_ms": percentile(lat, 99), "frames_per_pass": k,
            "resident_worlds": info["resident_worlds"], "tiled_worlds": info["tiled_worlds"],
            "plain_value": plain_rate, "plain_ms_per_100_frames": plain_ms / plain_frames * frames,
            "speedup_vs_plain": value / plain_rate, "cells": cells,
            "gpu_launches_per_step": (-(-frames // k) if info["tiled_worlds"] else 0) + 3 + 1}


def run_batch(args, rep):
    peak, peak_src = load_peak()
    import torch
    with ClockSampler(torch.cuda.current_device()) as clocks:
        m = measure_batch(rep, args.worlds, args.steps, args.warmup, args.k, args.resident_limit)
    alg_bytes = 8.0 * m["cells"]
    achieved = alg_bytes / (m["ms_per_step"] / 1e3) / 1e9
    return {
        "metric": METRIC, "value": m["value"], "unit": UNIT, "n_gpus": rep.world_size, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": m["ms_per_step"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u32", "data": "synthetic (seeded splitmix64)",
        "config": {"workload": m["workload"], "frames_per_pass": m["frames_per_pass"],
                   "resident_worlds": m["resident_worlds"], "tiled_worlds": m["tiled_worlds"],
                   "parallelism": f"replicas{rep.world_size}", "l2": "inputs larger than L2"},
        "batched": {k: m[k] for k in ("p50_ms", "p99_ms", "plain_value", "plain_ms_per_100_frames",
                                      "speedup_vs_plain")},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak if peak else None, "traffic": None, "peak_source": peak_src,
                     "algorithmic_bytes_per_step": alg_bytes,
                     "bound_note": "8 B per cell per launch group (one u32 read and one u32 write of every world "
                                   "per 100 frames): the worlds that fit in shared memory stay on chip for all "
                                   "100 frames and the tile passes fuse 8-16 frames, so the kernels are bound "
                                   "by issue, not by HBM"},
        "gpu_launches": args.steps * m["gpu_launches_per_step"],
        "clocks": clocks.summary(),
    }


SERVE_RATES = (100, 300, 1000, 3000, 10000, 20000)
SERVE_P99_BOUND_MS = 100.0
SERVE_BUDGET = 150 << 30
SERVE_SMALL_BUDGET = 256 << 20


def measure_serving(rep, n_req, frames_per_iteration=8):
    """The live serving loop (se_server_start) fed from this thread with Poisson arrivals at
    each of SERVE_RATES, in both modes: continuous batching, and one request at a time with
    one launch per frame (the reference's dispatch).  Each rate replays the same sessions
    and requests (workloads.serve_requests), only the arrival times scale.  Per mode: the highest
    throughput whose p99 latency stays within SERVE_P99_BOUND_MS.  Then one rate under a
    256 MB budget, so that sessions are evicted to host memory and restored."""
    import sandengine_gb300 as se
    from sandengine_gb300 import workloads as wl
    from sandengine_gb300.serving import Server
    rs = se.parse_string(wl.ruleset_text("twelve_materials"))
    spec = wl.twelve_fill_spec()
    sessions, reqs = wl.serve_requests(1.0, n_req)  # arrival times at 1 req/s; scaled per rate
    grids = [wl.serve_session_grid(w, h, i) for i, (w, h) in enumerate(sessions)]
    subs = [(s, n, [se.SimModification((m[0], m[1]), m[2], m[3], m[4]) for m in mods], t)
            for (s, n, mods, t) in reqs]

    def one(rate, plain, budget):
        srv = Server(rs, budget, frames_per_iteration)
        for (w, h), g in zip(sessions, grids):
            srv.open_session(w, h, g, 1)
        srv.start(plain=plain)
        t_start = time.perf_counter()
        ids = []
        for (sid, n, mods, t) in subs:
            wait = t / rate / 1e3 - (time.perf_counter() - t_start)
            if wait > 0:
                time.sleep(wait)
            ids.append(srv.submit(sid, n, mods))
        span = time.perf_counter() - t_start
        for r in ids:
            srv.wait(r)
        srv.stop()
        st = srv.stats()
        del srv
        return {"throughput": rep.sum(st["cell_updates"] / (st["wall_ms"] / 1e3)),
                "p50_ms": rep.max(st["p50_ms"]), "p99_ms": rep.max(st["p99_ms"]),
                "offered_req_s": len(subs) / span, "wall_ms": st["wall_ms"], "iterations": st["iterations"],
                "gpu_busy": st["kernel_ms"] / st["wall_ms"] if st["wall_ms"] > 0 else None,
                "evictions": st["evictions"], "restores": st["restores"], "restore_ms": st["restore_ms"]}

    sweep = []
    for rate in SERVE_RATES:
        row = {"rate_req_s": rate, "batched": one(rate, False, SERVE_BUDGET), "plain": one(rate, True, SERVE_BUDGET)}
        row["speedup"] = row["batched"]["throughput"] / row["plain"]["throughput"]
        sweep.append(row)

    def sustained(mode):
        ok = [r[mode]["throughput"] for r in sweep if r[mode]["p99_ms"] <= SERVE_P99_BOUND_MS]
        return max(ok) if ok else None

    b, p = sustained("batched"), sustained("plain")
    evict_rate = 3000
    ev = one(evict_rate, False, SERVE_SMALL_BUDGET)
    return {"workload": f"serve: {n_req} requests per rate, Poisson arrivals at {SERVE_RATES[0]}-{SERVE_RATES[-1]} "
                        f"req/s submitted to the live loop, {len(sessions)} sessions (sides log-uniform in "
                        f"[128, 2048]), N ~ U[1, 600] frames, 0-8 circle edits, twelve_materials rule set, "
                        f"{SERVE_BUDGET >> 30} GB budget, up to {frames_per_iteration} frames per batched iteration",
            "unit": UNIT, "sweep": sweep, "p99_bound_ms": SERVE_P99_BOUND_MS,
            "sustained_under_bound": {"batched": b, "plain": p,
                                      "speedup": (b / p) if (b and p) else None},
            "small_budget": dict(ev, rate_req_s=evict_rate, budget_bytes=SERVE_SMALL_BUDGET)}


def run_serve(args, rep):
    m = measure_serving(rep, args.serve_requests, args.serve_k)
    best = max(m["sweep"], key=lambda r: r["batched"]["throughput"])
    return {
        "metric": METRIC, "value": best["batched"]["throughput"], "unit": UNIT, "n_gpus": rep.world_size,
        "steps": len(m["sweep"]), "warmup": 0, "ms_per_step": best["batched"]["wall_ms"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic (seeded splitmix64)",
        "config": {"workload": m["workload"], "parallelism": f"replicas{rep.world_size}"},
        "serving": m,
    }


def run_bands(args, rep):
    """One world in row bands over the ranks (--parallelism bands): each rank advances its
    band (se_world_create_band) and the ranks exchange halo rows with NCCL send/recv before
    every launch group of `halo` frames.  value = the whole world's cell-updates/s."""
    import torch
    import torch.distributed as dist
    import sandengine_gb300 as se
    from sandengine_gb300 import workloads as wl
    from sandengine_gb300.bands import DistributedBand
    spec = workload(args.workload)
    W = H = spec["size"]
    k = args.k or 8
    rs = se.parse_string(wl.ruleset_text(spec["ruleset"]))
    comm = dist if rep.world_size > 1 else _SingleRank()
    band = DistributedBand(rs, W, H, k, comm, device=f"cuda:{torch.cuda.current_device()}")
    band.set_world(spec["grid"]())
    band.frame = 1
    mods = [step_mods(se, wl, W, r, spec["edit_mats"]) for r in range(args.warmup + args.steps)]
    for r in range(args.warmup):
        band.step(FRAMES_PER_STEP, mods[r])
    torch.cuda.synchronize()
    rep.barrier()
    with ClockSampler(torch.cuda.current_device()) as clocks:
        t0 = time.perf_counter()
        for r in range(args.steps):
            band.step(FRAMES_PER_STEP, mods[args.warmup + r])
        torch.cuda.synchronize()
        rep.barrier()
        secs = rep.max(time.perf_counter() - t0)
    value = float(W) * H * FRAMES_PER_STEP * args.steps / secs
    return {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": rep.world_size, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * secs / args.steps, "higher_is_better": True,
        "scaling": "strong", "vs_baseline": None, "dtype": "u32", "data": "synthetic (seeded splitmix64)",
        "config": {"workload": f"{spec['name']}: {W}x{H} u32 cells, {spec['ruleset']} rule set, {spec['fill']}, "
                               f"{FRAMES_PER_STEP} frames per step, {EDITS_PER_STEP} circle edits on the first",
                   "parallelism": f"bands{rep.world_size}", "halo_rows": band.halo,
                   "band_rows": [n for _, n in band.split]},
        "gpu_launches": None, "clocks": clocks.summary(),
    }


class _SingleRank:
    """torch.distributed's surface for one rank (no neighbours, so nothing is exchanged)."""

    @staticmethod
    def get_rank():
        return 0

    @staticmethod
    def get_world_size():
        return 1


def run_reference(args, rep):
    """The reference's own compute shader compiled for the CPU (the whole shader per
    invocation, as the reference dispatches it), all host threads, on the workload's own
    steps: each step is one edit period (60 frames, the step's edit round on the first) of
    a band of the same world (rows 0..R-1 as a world of their own); only the dispatches are
    timed.  Without that build, the oracle port."""
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
    rows = 16 if W >= 4096 else W  # a few seconds per 60-frame step on 16 cores
    band = np.ascontiguousarray(full[:rows]).copy()
    frame = 1

    def one(r):
        nonlocal band, frame
        mods = [(x, y, sh, rad, m) for (x, y, sh, rad, m) in wl.world_edits(W, r, spec["edit_mats"])
                if y - rad < rows] if W >= 4096 else None
        if ref:
            band, secs = ref.run_timed(band, frame, FRAMES_PER_STEP, mods, cores)
        else:
            t0 = time.perf_counter()
            port.run(band, frame, FRAMES_PER_STEP, mods, cores)
            secs = time.perf_counter() - t0
        frame += FRAMES_PER_STEP
        return secs

    for i in range(args.warmup):
        one(i)
    times = [one(args.warmup + i) for i in range(args.steps)]
    value = band.size * FRAMES_PER_STEP * args.steps / sum(times)
    sample = (f"{spec['name']} rows 0-{rows - 1} ({W} x {rows} band of the seeded world as a world of its own), "
              f"{FRAMES_PER_STEP} frames per step with the step's edits, {cores} threads ({model}); the whole "
              f"compute shader per invocation (grid update, colour, light)")
    return {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": rep.world_size,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * sum(times) / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32 texels (ids)",
            "data": "synthetic (seeded splitmix64)",
            "config": {"workload": f"{spec['name']}: {spec['ruleset']} rule set, {spec['fill']}, "
                                   f"{FRAMES_PER_STEP} frames per step, the step's circle edits on the first; "
                                   f"reference compute shader on the CPU, {W} x {rows} band",
                       "parallelism": "host threads"},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": kind, "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def relaunch(args) -> int:
    """--gpus N > 1 outside a torch.distributed environment: run this script under
    torch.distributed.run with N ranks on this node; returns their exit status."""
    import socket
    with socket.socket() as so:
        so.bind(("127.0.0.1", 0))
        port = so.getsockname()[1]
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", f"--nproc-per-node={args.gpus}",
           "--master-addr=127.0.0.1", f"--master-port={port}", os.path.abspath(__file__)] + sys.argv[1:]
    return subprocess.run(cmd).returncode


def main():
    args = parse_args()
    if args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        sys.exit(relaunch(args))
    from sandengine_gb300.replicas import Replicas
    rep = Replicas("nccl" if args.impl == "ours" else "gloo")
    try:
        if args.impl == "reference":
            out = run_reference(args, rep)
        elif args.workload.startswith("batch"):
            out = run_batch(args, rep)
        elif args.workload == "serve":
            out = run_serve(args, rep)
        elif args.parallelism == "bands":
            out = run_bands(args, rep)
        else:
            out = run_ours(args, rep)
        if rep.rank == 0 and out is not None:
            print(json.dumps(out), flush=True)
    finally:
        rep.close()


if __name__ == "__main__":
    main()
