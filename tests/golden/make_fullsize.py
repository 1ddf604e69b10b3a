"""Golden digests of the two benchmark worlds at full size, from the oracle port.

The per-frame goldens in grids.json stop at 256^2; this script pins the worlds the
benchmark numbers are quoted on, at their full sizes, so that the GPU path can be compared
with the oracle where it is measured (tests/test_gpu_fullsize_parity.py):

* ``world16384_edits``: the 16384^2 twelve-material world (seed-2 64x64 patches), frame
  counter 1, ``ROUNDS`` rounds of 60 frames; round r carries ``workloads.world_edits(16384,
  r)`` (32 circles) on its first frame, as one benchmark step does.  Digest and material
  histogram after every round.
* ``world4096_iid``: the 4096^2 four-material world (seed-1 i.i.d. fill), frame counter 1,
  10,000 frames without edits; digest and histogram every 500 frames.
* ``batch4096``: the 4096 worlds of the batched workload, 100 and 200 frames; every
  world's digest (see run_batch).
* ``serve``: the 300 requests of the serving workload; every session's digest after its
  requests (see run_serve).

Before the port's digests are written, the port is checked against the reference's own
compute shader compiled for the CPU (oracle/_ref, built from the reference checkout named
by ``SANDENGINE_REF``): at the initial state and at every checkpoint of each world, three
64-row bands (top, middle, bottom) are cut out as W x 64 worlds of their own and advanced
``BAND_FRAMES`` frames by both, edits (moved into band coordinates) included where the
checkpoint starts an edit round; every frame must agree cell for cell.  The outcome is
recorded in the fixture.

    SANDENGINE_REF=<reference checkout> python tests/golden/make_fullsize.py [names...]

Writes fullsize.json in this folder.  Runs in about ten minutes on 8 cores (the port is
multi-threaded with OpenMP over block rows).
"""
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle.build import Port, Ref, reference_root  # noqa: E402
from sandengine_gb300 import workloads as wl  # noqa: E402
from sandengine_gb300.simulation import grid_digest  # noqa: E402

ROUNDS = 4
C2_FRAMES, C2_EVERY = 10000, 500
BATCH_WORLDS, BATCH_FRAMES, BATCH_CHECKPOINTS = 4096, 100, 2
SERVE_REQUESTS = 300
BAND_ROWS, BAND_FRAMES = 64, 4
THREADS = os.cpu_count() or 1


def world16384_spec():
    return dict(name="world16384_edits", ruleset="twelve_materials", frame0=1,
                grid=lambda: wl.world_16384(2), checkpoints=[60 * (r + 1) for r in range(ROUNDS)],
                mods_at=lambda i: wl.world_edits(16384, i // 60) if i % 60 == 0 else None)


def world4096_spec():
    return dict(name="world4096_iid", ruleset="four_materials", frame0=1, grid=lambda: wl.world_4096(1),
                checkpoints=list(range(C2_EVERY, C2_FRAMES + 1, C2_EVERY)), mods_at=lambda i: None)


def band_check(port, ref, grid, frame0, mods, y0):
    """Rows [y0, y0 + 64) of ``grid`` as a world of their own, BAND_FRAMES frames from counter
    frame0 (mods on the first, in band coordinates) by the port and by the reference
    shader: True when every frame agrees."""
    a = np.ascontiguousarray(grid[y0:y0 + BAND_ROWS]).copy()
    b = a.copy()
    local = [(x, y - y0, s, r, m) for (x, y, s, r, m) in (mods or [])]
    for i in range(BAND_FRAMES):
        f = frame0 + 1 + i
        port.step(a, f, local if i == 0 else None, THREADS)
        b = ref.step(b, f, local if i == 0 else None, nthreads=THREADS)
        if not np.array_equal(a, b):
            return False
    return True


def run(spec):
    text = wl.ruleset_text(spec["ruleset"])
    port = Port(text)
    ref = Ref(text)
    g = np.ascontiguousarray(spec["grid"](), dtype=np.uint32)
    H = g.shape[0]
    bands = [0, (H // 2) & ~1, H - BAND_ROWS]
    checks = []

    def check_here(frame, i):
        for y0 in bands:
            ok = band_check(port, ref, g, frame, spec["mods_at"](i), y0)
            checks.append({"frame": frame, "y0": y0, "frames": BAND_FRAMES, "equal": ok})
            if not ok:
                sys.exit(f"{spec['name']}: port and reference shader differ on the band at row {y0}, "
                         f"frames after {frame}")

    out = {"ruleset": spec["ruleset"], "width": g.shape[1], "height": H, "frame0": spec["frame0"],
           "initial_digest": str(grid_digest(g)), "checkpoints": []}
    frame = spec["frame0"]
    check_here(frame, 0)
    done = 0
    t0 = time.time()
    for cp in spec["checkpoints"]:
        while done < cp:
            m = spec["mods_at"](done)
            # an edit frame alone, else every frame up to the next edit frame or checkpoint
            n = 1 if m else next((j for j in range(done + 1, cp) if spec["mods_at"](j)), cp) - done
            port.run(g, frame, n, m, THREADS)
            frame += n
            done += n
        hist = np.bincount(g.ravel(), minlength=16)
        out["checkpoints"].append({"frames": cp, "frame": frame, "digest": str(grid_digest(g)),
                                   "histogram": [int(v) for v in hist]})
        print(f"{spec['name']}: {cp} frames ({time.time() - t0:.0f} s)", flush=True)
        check_here(frame, cp)
    out["band_checks"] = checks
    return out


def run_batch():
    """The 4096 worlds of bench.py's batched workload (sides from workloads.batch_sizes(4096,
    4), world i filled by patch_fill(w, h, 1000 + i, twelve materials, patch=16), frame
    counter 1), advanced BATCH_FRAMES frames at a time by the port, world by world: each
    world's digest after every checkpoint.  Three worlds (the smallest, the median and the
    largest by cells) are first advanced by the port and by the reference shader frame by
    frame over the first checkpoint; every frame must agree."""
    text = wl.ruleset_text("twelve_materials")
    port, ref = Port(text), Ref(text)
    sizes = wl.batch_sizes(BATCH_WORLDS, 4)
    spec = wl.twelve_fill_spec()
    fill = lambda i: np.ascontiguousarray(wl.patch_fill(sizes[i][0], sizes[i][1], 1000 + i, *spec, patch=16),
                                          dtype=np.uint32)
    order = sorted(range(len(sizes)), key=lambda i: sizes[i][0] * sizes[i][1])
    checks = []
    for i in (order[0], order[len(order) // 2], order[-1]):
        a = fill(i)
        b = a.copy()
        for n in range(BATCH_FRAMES):
            port.step(a, 2 + n, None, THREADS)
            b = ref.step(b, 2 + n, None, nthreads=THREADS)
            if not np.array_equal(a, b):
                sys.exit(f"batch world {i} {sizes[i]}: port and reference shader differ at frame {2 + n}")
        checks.append({"world": i, "size": list(sizes[i]), "frames": BATCH_FRAMES, "equal": True})
    digests = [[] for _ in range(BATCH_CHECKPOINTS)]
    t0 = time.time()
    for i in range(len(sizes)):
        g, frame = fill(i), 1
        for c in range(BATCH_CHECKPOINTS):
            port.run(g, frame, BATCH_FRAMES, None, THREADS)
            frame += BATCH_FRAMES
            digests[c].append("%016x" % grid_digest(g))
        if i % 512 == 511:
            print(f"batch4096: {i + 1} worlds ({time.time() - t0:.0f} s)", flush=True)
    return {"ruleset": "twelve_materials", "worlds": BATCH_WORLDS, "sizes": "workloads.batch_sizes(4096, 4)",
            "fill": "workloads.patch_fill(w, h, 1000 + i, *twelve_fill_spec(), patch=16)", "frame0": 1,
            "checkpoints": [{"frames": BATCH_FRAMES * (c + 1), "digests": digests[c]}
                            for c in range(BATCH_CHECKPOINTS)],
            "reference_checks": checks}


def run_serve():
    """The serving workload of bench.py (workloads.serve_requests(rate, 300): 149 sessions,
    300 requests; a session's grid is workloads.serve_session_grid, frame counter 1).  Its
    result does not depend on the arrival times or on how requests are batched: each session
    advances through its requests in submission order, each request's edits on its first
    frame.  The port plays the requests in order; every session's digest and frame counter
    at the end.  The two smallest sessions with two or more requests are first played by the
    port and by the reference shader frame by frame; every frame must agree."""
    text = wl.ruleset_text("twelve_materials")
    port, ref = Port(text), Ref(text)
    sessions, reqs = wl.serve_requests(1.0, SERVE_REQUESTS)
    count = [0] * len(sessions)
    for sid, _, _, _ in reqs:
        count[sid] += 1
    small = sorted((i for i in range(len(sessions)) if count[i] >= 2),
                   key=lambda i: sessions[i][0] * sessions[i][1])[:2]
    checks = []
    for sid in small:
        a = np.ascontiguousarray(wl.serve_session_grid(*sessions[sid], sid), dtype=np.uint32)
        b, frame, nf = a.copy(), 1, 0
        for s2, n, mods, _ in reqs:
            if s2 != sid:
                continue
            for q in range(n):
                port.step(a, frame + 1, mods if q == 0 else None, THREADS)
                b = ref.step(b, frame + 1, mods if q == 0 else None, nthreads=THREADS)
                frame += 1
                if not np.array_equal(a, b):
                    sys.exit(f"serving session {sid}: port and reference shader differ at frame {frame}")
            nf += n
        checks.append({"session": sid, "size": list(sessions[sid]), "requests": count[sid], "frames": nf,
                       "equal": True})
    grids = [np.ascontiguousarray(wl.serve_session_grid(w, h, i), dtype=np.uint32)
             for i, (w, h) in enumerate(sessions)]
    frames = [1] * len(sessions)
    t0 = time.time()
    for r, (sid, n, mods, _) in enumerate(reqs):
        port.run(grids[sid], frames[sid], n, mods or None, THREADS)
        frames[sid] += n
        if r % 50 == 49:
            print(f"serve: {r + 1} requests ({time.time() - t0:.0f} s)", flush=True)
    return {"ruleset": "twelve_materials", "requests": SERVE_REQUESTS, "sessions": len(sessions),
            "workload": "workloads.serve_requests(rate, 300), sessions workloads.serve_session_grid, frame 1",
            "digests": ["%016x" % grid_digest(g) for g in grids], "frames": frames, "reference_checks": checks}


def main():
    """With names on the command line (world16384_edits, world4096_iid, batch4096, serve), only
    those entries are made and merged into the existing fullsize.json."""
    if reference_root() is None:
        sys.exit("set SANDENGINE_REF to the reference checkout (the band checks need its shader)")
    path = os.path.join(HERE, "fullsize.json")
    want = set(sys.argv[1:]) or {"world16384_edits", "world4096_iid", "batch4096", "serve"}
    out = {}
    if sys.argv[1:] and os.path.exists(path):
        with open(path) as f:
            out = json.load(f)
    for spec in (world16384_spec(), world4096_spec()):
        if spec["name"] in want:
            out[spec["name"]] = run(spec)
    if "batch4096" in want:
        out["batch4096"] = run_batch()
    if "serve" in want:
        out["serve"] = run_serve()
    out["_about"] = ("digests (Simulation.digest / simulation.grid_digest) and id histograms of the oracle port, "
                     "checked against the reference compute shader (bands of the single worlds, whole worlds of "
                     "the batch); made by make_fullsize.py")
    with open(path, "w") as f:
        json.dump(out, f, indent=1)


if __name__ == "__main__":
    main()
