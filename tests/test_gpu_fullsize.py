"""Full-size checks on the GPU, through properties that hold at any size (the oracle is not
run at these sizes): the 16384^2 benchmark world, and a 40002 x 24001 world whose buffers
pass 2^31 bytes, whose width is not a multiple of 4 (the scalar load path) and whose
height is odd."""
import numpy as np
import pytest

from sandengine_gb300 import workloads as wl

pytestmark = pytest.mark.gpu

FOUR_IDS, FOUR_PROBS = [0, 3, 4, 5], [0.6, 0.2, 0.15, 0.05]  # empty, sand, water, stone


def _edits(se, W, H):
    return [se.SimModification((x, y), s, r, m) for x, y, s, r, m in wl.circle_edits(W, H, 3, 0, 32, [0, 3])]


def test_swaps_conserve_material_counts_16384(se, rulesets):
    """The four-material rules move cells only by (guarded) swaps, so the material counts
    of the 16384^2 world never change, whatever the frames per launch."""
    W = H = 16384
    sim = se.Simulation(se.parse_string(rulesets["four_materials"]), (W, H))
    sim.grid = wl.patch_fill(W, H, 11, FOUR_IDS, FOUR_PROBS, patch=8)
    sim.params.frame = 1
    h0 = sim.histogram()
    d0 = sim.digest()
    for k in (8, 1, 3):
        sim.set_steps_per_launch(k)
        sim.run_frames(24)
        assert np.array_equal(sim.histogram(), h0), f"k={k}"
    assert sim.digest() != d0  # the world did move
    assert sim.params.frame == 1 + 72


@pytest.mark.parametrize("shape", [(16384, 16384), (40002, 24001)])
def test_fused_launches_equal_one_frame_launches_full_size(se, rulesets, shape):
    """k frames per launch (shared-memory tiles with halos, the chunk list, the per-step row
    band) give the grid that one-frame launches give, edits on the first frame included."""
    W, H = shape
    rs = se.parse_string(rulesets["twelve_materials"])
    g = wl.patch_fill(W, H, 2, *wl.twelve_fill_spec(), patch=64)
    mods = _edits(se, W, H)
    digests, hists = [], []
    for k in (8, 1):
        sim = se.Simulation(rs, (W, H))
        sim.grid = g
        sim.params.frame = 5
        if k == 8:
            d_start = sim.digest()
        sim.set_steps_per_launch(k)
        sim.run_frames(20, mods)
        digests.append(sim.digest())
        hists.append(sim.histogram())
        del sim
    assert digests[0] == digests[1]
    assert np.array_equal(hists[0], hists[1])
    assert digests[0] != d_start
