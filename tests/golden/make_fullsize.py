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

Before the port's digests are written, the port is checked against the reference's own
compute shader compiled for the CPU (oracle/_ref, built from the reference checkout named
by ``SANDENGINE_REF``): at the initial state and at every checkpoint of each world, three
64-row bands (top, middle, bottom) are cut out as W x 64 worlds of their own and advanced
``BAND_FRAMES`` frames by both, edits (moved into band coordinates) included where the
checkpoint starts an edit round; every frame must agree cell for cell.  The outcome is
recorded in the fixture.

    SANDENGINE_REF=<reference checkout> python tests/golden/make_fullsize.py

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


def main():
    if reference_root() is None:
        sys.exit("set SANDENGINE_REF to the reference checkout (the band checks need its shader)")
    out = {}
    for spec in (world16384_spec(), world4096_spec()):
        out[spec["name"]] = run(spec)
    out["_about"] = ("digests (Simulation.digest / simulation.grid_digest) and id histograms of the oracle port, "
                     "band-checked against the reference compute shader; made by make_fullsize.py")
    with open(os.path.join(HERE, "fullsize.json"), "w") as f:
        json.dump(out, f, indent=1)


if __name__ == "__main__":
    main()
