"""The benchmark worlds at full size against the oracle (tests/golden/fullsize.json, made by
tests/golden/make_fullsize.py from the oracle port, itself band-checked against the
reference's compute shader compiled for the CPU).

* 16384^2 twelve-material world with the benchmark's edit rounds (32 circles on the first
  of every 60 frames), through the path bench.py times: the autotuned fused launches, the
  edits inside the first launch of each round.  Also through fixed variants: the 256x128
  k=8 tiles the autotuner picks on this world, and one-frame launches.
* 4096^2 four-material world, 10,000 frames, digest every 500: autotuned, k=16 and k=1.
* The batched workload's 4096 worlds (bench.py's sizes, fills and frame counters), two
  launch groups of 100 frames, every world's digest: autotuned (whole worlds in shared
  memory beside tile passes), then 8 frames per tile pass.
* The serving workload's 300 requests over 149 sessions, submitted from this thread to the
  live loop while it runs: continuously batched with the benchmark's 150 GB budget, the
  same under a 256 MB budget (sessions evicted to host memory and restored), and one
  request at a time; every session's digest and frame counter.

Digests are compared with the device digest (Simulation.digest) and the material
histograms with the device histogram; bit-exact is the bar.
"""
import json
import os

import numpy as np
import pytest

from sandengine_gb300 import workloads as wl
from tests.conftest import GOLDEN

pytestmark = pytest.mark.gpu


def _golden(name):
    with open(os.path.join(GOLDEN, "fullsize.json")) as f:
        return json.load(f)[name]


def _check(sim, cp, what):
    h = sim.histogram(16)
    assert [int(v) for v in h] == cp["histogram"], f"{what}: histogram differs after {cp['frames']} frames"
    assert sim.digest() == int(cp["digest"]), f"{what}: grid differs after {cp['frames']} frames"
    assert sim.params.frame == cp["frame"]


@pytest.mark.parametrize("mode", ["autotuned", "256x128x8", "k1"])
def test_world16384_with_edits_matches_oracle(se, rulesets, mode):
    gold = _golden("world16384_edits")
    W, H = gold["width"], gold["height"]
    sim = se.Simulation(se.parse_string(rulesets[gold["ruleset"]]), (W, H))
    sim.grid = wl.world_16384(2)
    sim.params.frame = gold["frame0"]
    assert sim.digest() == int(gold["initial_digest"])
    if mode == "autotuned":
        sim.autotune(3)
    elif mode == "k1":
        sim.set_steps_per_launch(1)
    else:
        sim.set_tile(256, 128, 8)
    for r, cp in enumerate(gold["checkpoints"]):
        mods = [se.SimModification((m[0], m[1]), m[2], m[3], m[4]) for m in wl.world_edits(W, r)]
        sim.run_frames(60, mods)
        _check(sim, cp, f"world16384 ({mode}, tile {sim.tile()})")


@pytest.mark.parametrize("mode", ["autotuned", "k16", "k1"])
def test_world4096_10000_frames_matches_oracle(se, rulesets, mode):
    gold = _golden("world4096_iid")
    W, H = gold["width"], gold["height"]
    sim = se.Simulation(se.parse_string(rulesets[gold["ruleset"]]), (W, H))
    sim.grid = wl.world_4096(1)
    sim.params.frame = gold["frame0"]
    assert sim.digest() == int(gold["initial_digest"])
    if mode == "autotuned":
        sim.autotune(3)
    else:
        sim.set_steps_per_launch(int(mode[1:]))
    done = 0
    for cp in gold["checkpoints"]:
        sim.run_frames(cp["frames"] - done)
        done = cp["frames"]
        _check(sim, cp, f"world4096 ({mode}, tile {sim.tile()})")


def test_batch4096_matches_oracle(se, rulesets):
    from sandengine_gb300.batch import Batch
    from sandengine_gb300.simulation import grid_digest
    gold = _golden("batch4096")
    sizes = wl.batch_sizes(gold["worlds"], 4)
    rs = se.parse_string(rulesets[gold["ruleset"]])
    b = Batch(rs, sizes)
    spec = wl.twelve_fill_spec()
    for i, (w, h) in enumerate(sizes):
        b.set_grid(i, wl.patch_fill(w, h, 1000 + i, *spec, patch=16))
        b.set_frame(i, gold["frame0"])
    info = b.info()
    assert info["resident_worlds"] > 0 and info["tiled_worlds"] > 0, info
    b.autotune(2)
    done = 0
    for c, cp in enumerate(gold["checkpoints"]):
        if c == 1:
            b.set_steps_per_launch(8)
        b.step(cp["frames"] - done)
        done = cp["frames"]
        b.synchronize()
        bad = [i for i in range(len(sizes)) if "%016x" % grid_digest(b.grid(i)) != cp["digests"][i]]
        assert not bad, (f"{len(bad)} worlds differ after {cp['frames']} frames, first {bad[:5]} "
                         f"({[sizes[i] for i in bad[:5]]})")
        assert all(b.frame(i) == gold["frame0"] + cp["frames"] for i in range(len(sizes)))


@pytest.mark.parametrize("mode, budget", [("batched", 150 << 30), ("batched", 256 << 20), ("plain", 150 << 30)],
                         ids=["batched", "batched-256MB", "plain"])
def test_serve_workload_matches_oracle(se, rulesets, mode, budget):
    from sandengine_gb300.serving import Server
    from sandengine_gb300.simulation import grid_digest
    gold = _golden("serve")
    rs = se.parse_string(rulesets[gold["ruleset"]])
    sessions, reqs = wl.serve_requests(20000.0, gold["requests"])
    assert len(sessions) == gold["sessions"]
    srv = Server(rs, budget, 8)
    for i, (w, h) in enumerate(sessions):
        assert srv.open_session(w, h, wl.serve_session_grid(w, h, i), 1) == i
    srv.start(plain=(mode == "plain"))
    ids = [srv.submit(sid, n, [se.SimModification((m[0], m[1]), m[2], m[3], m[4]) for m in mods])
           for (sid, n, mods, _) in reqs]
    for r in ids:
        srv.wait(r)
    srv.stop()
    if budget < (1 << 30):
        assert srv.stats()["evictions"] > 0
    bad = [i for i in range(len(sessions)) if "%016x" % grid_digest(srv.grid(i)) != gold["digests"][i]]
    assert not bad, f"{len(bad)} sessions differ from the oracle, first {bad[:5]} ({[sessions[i] for i in bad[:5]]})"
    assert [srv.frame(i) for i in range(len(sessions))] == gold["frames"]
