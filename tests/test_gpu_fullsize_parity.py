"""The benchmark worlds at full size against the oracle (tests/golden/fullsize.json, made by
tests/golden/make_fullsize.py from the oracle port, itself band-checked against the
reference's compute shader compiled for the CPU).

* 16384^2 twelve-material world with the benchmark's edit rounds (32 circles on the first
  of every 60 frames), through the path bench.py times: the autotuned fused launches, the
  edits inside the first launch of each round.  Also through fixed variants: the 256x128
  k=8 tiles the autotuner picks on this world, and one-frame launches.
* 4096^2 four-material world, 10,000 frames, digest every 500: autotuned, k=16 and k=1.

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
