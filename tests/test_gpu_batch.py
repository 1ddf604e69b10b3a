"""Batched worlds on the GPU against the oracle port, world by world."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _mixed_sizes():
    from sandengine_gb300 import workloads as wl
    sizes = wl.batch_sizes(20, 7, lo=32, hi=480)
    return sizes + [(1024, 640), (544, 600), (70, 1100), (33, 17), (1, 1)]


def test_batch_matches_port(se, ports, rulesets):
    from sandengine_gb300 import workloads as wl
    from sandengine_gb300.batch import Batch
    sizes = _mixed_sizes()
    rs = se.parse_string(rulesets["twelve_materials"])
    b = Batch(rs, sizes)
    info = b.info()
    assert info["resident_worlds"] > 0 and info["tiled_worlds"] >= 2, info
    grids = [wl.patch_fill(w, h, 100 + i, *wl.twelve_fill_spec(), patch=16) for i, (w, h) in enumerate(sizes)]
    for i, g in enumerate(grids):
        b.set_grid(i, g)
        b.set_frame(i, 1 + (i % 5))
    frames = [b.frame(i) for i in range(len(sizes))]
    port = ports["twelve_materials"]
    for nf, plain in ((37, False), (100, False), (3, True), (37, False)):
        if plain:
            b.step_plain(nf)
        else:
            b.step(nf)
        b.synchronize()
        for i, g in enumerate(grids):
            port.run(g, frames[i], nf, nthreads=8)
            frames[i] += nf
            got = b.grid(i)
            assert np.array_equal(got, g), f"world {i} {sizes[i]}: {np.count_nonzero(got != g)} cells differ"
            assert b.frame(i) == frames[i]


def test_batch_frame_zero_clears_all(se, rulesets):
    from sandengine_gb300.batch import Batch
    rs = se.parse_string(rulesets["four_materials"])
    b = Batch(rs, [(64, 64), (2000, 40)])
    b.set_grid(0, np.full((64, 64), 3, dtype=np.uint32))
    b.step(5)
    b.synchronize()
    assert not b.grid(0).any() and b.frame(0) == 5 and b.frame(1) == 5
    b.set_frame(0, 9)
    b.set_frame(1, 0)
    with pytest.raises(se.SandengineError):
        b.step(2)  # mixed frame-0 and running worlds


def test_batch_autotune_keeps_state(se, rulesets):
    from sandengine_gb300 import workloads as wl
    from sandengine_gb300.batch import Batch
    rs = se.parse_string(rulesets["twelve_materials"])
    sizes = [(800, 700), (96, 96)]
    b = Batch(rs, sizes)
    gs = [wl.patch_fill(w, h, 3, *wl.twelve_fill_spec(), patch=16) for w, h in sizes]
    for i, g in enumerate(gs):
        b.set_grid(i, g)
        b.set_frame(i, 2)
    k = b.autotune(1)
    assert k >= 1
    for i, g in enumerate(gs):
        assert np.array_equal(b.grid(i), g) and b.frame(i) == 2


def test_rules_that_set_wall_cells_keep_the_world_border(se, rulesets):
    """A rule that SETs a WALL neighbour (WALL's density singles it out) on worlds with WALL
    cells inside: single-world launches (k = 1 and 8) and a batch with resident and tiled
    worlds equal the oracle; the WALL outside the world is never written."""
    from oracle.build import Port
    from sandengine_gb300 import workloads as wl
    from sandengine_gb300.batch import Batch
    from tests.test_kernel_emulation import WALL_RULE
    text = rulesets["four_materials"].replace("rules:\n", "rules:\n" + WALL_RULE.lstrip("\n"), 1)
    text = text.replace("base_rules: [fall]", "base_rules: [fall, paint_wall]")
    rs, P = se.parse_string(text), Port(text)
    rng = np.random.default_rng(5)
    sizes = [(137, 61), (300, 150), (1100, 700), (33, 17)]
    grids = []
    for W, H in sizes:
        g = wl.iid_fill(W, H, 4, *wl.FOUR_FILL)
        g[rng.random((H, W)) < 0.05] = 2
        grids.append(g)
    for (W, H), g in zip(sizes, grids):
        for k in (1, 8):
            sim = se.Simulation(rs, (W, H))
            sim.set_steps_per_launch(k)
            sim.grid = g
            sim.params.frame = 4
            sim.run_frames(24)
            want = g.copy()
            P.run(want, 4, 24)
            assert np.array_equal(sim.grid, want), f"{W}x{H} k={k}"
    b = Batch(rs, sizes)
    for i, g in enumerate(grids):
        b.set_grid(i, g)
        b.set_frame(i, 4)
    b.step(30)
    b.synchronize()
    for i, g in enumerate(grids):
        want = g.copy()
        P.run(want, 4, 30)
        assert np.array_equal(b.grid(i), want), f"batch world {i} {sizes[i]}"


def test_resident_limit_reclassifies_and_stays_exact(se, ports, rulesets):
    """se_batch_set_resident_limit moves worlds between whole-world CTAs and tile passes
    between steps; every world stays equal to the oracle."""
    from sandengine_gb300 import workloads as wl
    from sandengine_gb300.batch import Batch
    sizes = [(96, 64), (300, 200), (33, 17), (700, 500)]
    rs = se.parse_string(rulesets["twelve_materials"])
    b = Batch(rs, sizes)
    grids = [wl.patch_fill(w, h, 40 + i, *wl.twelve_fill_spec(), patch=16) for i, (w, h) in enumerate(sizes)]
    for i, g in enumerate(grids):
        b.set_grid(i, g)
        b.set_frame(i, 2)
    frames = [2] * len(sizes)
    port = ports["twelve_materials"]
    resident_counts = []
    for limit, nf in ((0, 20), (1 << 30, 17), (20000, 25)):
        b.set_resident_limit(limit)
        resident_counts.append(b.info()["resident_worlds"])
        b.step(nf)
        b.synchronize()
        for i, g in enumerate(grids):
            port.run(g, frames[i], nf, nthreads=8)
            frames[i] += nf
            assert np.array_equal(b.grid(i), g), f"limit {limit}, world {i}"
    assert resident_counts[0] == 0 and resident_counts[1] >= 3 and 0 < resident_counts[2] < resident_counts[1]
