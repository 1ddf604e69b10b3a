"""CUDA path vs the oracle, frame by frame, through the C ABI.

Bit-exact is the bar (cells are integer ids).  Each case is checked against both the
per-frame digests recorded from the reference's own compute shader (tests/golden/grids.json)
and the oracle port run on the same inputs.
"""
import json
import os

import numpy as np
import pytest

from tests.conftest import GOLDEN
from tests.golden.cases import CASES

pytestmark = pytest.mark.gpu


def _golden():
    with open(os.path.join(GOLDEN, "grids.json")) as f:
        return json.load(f)


def _sim(se, text, w, h, k=1):
    rs = se.parse_string(text)
    sim = se.Simulation(rs, (w, h))
    if k:
        sim.set_steps_per_launch(k)
    return sim


def _mods(se, raw):
    return [se.SimModification((m[0], m[1]), m[2], m[3], m[4]) for m in (raw or [])]


@pytest.mark.parametrize("case", CASES, ids=[c.name for c in CASES])
def test_every_frame_matches_reference_digests(se, case):
    gold = _golden()[case.name]["digests"]
    g0 = case.initial_grid()
    sim = _sim(se, case.ruleset_text(), g0.shape[1], g0.shape[0])
    sim.grid = g0
    sim.params.frame = case.frame0
    for i in range(case.frames):
        sim.run_frames(1, _mods(se, case.mods_at(i)))
        assert sim.digest() == int(gold[i]), f"{case.name}: frame {case.frame0 + 1 + i} differs"


@pytest.mark.parametrize("case", CASES, ids=[c.name for c in CASES])
def test_every_frame_matches_port(se, ports, case):
    port = ports[case.ruleset]
    g = case.initial_grid()
    sim = _sim(se, case.ruleset_text(), g.shape[1], g.shape[0])
    sim.grid = g
    sim.params.frame = case.frame0
    n = min(case.frames, 200)
    for i in range(n):
        m = case.mods_at(i)
        sim.run_frames(1, _mods(se, m))
        port.step(g, case.frame0 + 1 + i, m, nthreads=8)
        got = sim.grid
        if not np.array_equal(got, g):
            bad = np.argwhere(got != g)
            pytest.fail(f"{case.name}: frame {case.frame0 + 1 + i}: {len(bad)} cells differ, first {bad[:4]}")


@pytest.mark.parametrize("k", [2, 3, 4, 8, 16])
@pytest.mark.parametrize("shape", [(517, 389), (256, 256), (130, 67)])
def test_fused_launches_match_port(se, ports, rulesets, k, shape):
    """k frames per launch (temporal blocking) give the same grid as the port, including
    ragged worlds (widths not a multiple of 4 or of the tile)."""
    from sandengine_gb300 import workloads as wl
    w, h = shape
    g = wl.patch_fill(w, h, 11, *wl.twelve_fill_spec(), patch=16)
    sim = _sim(se, rulesets["twelve_materials"], w, h, k=k)
    sim.grid = g
    sim.params.frame = 7
    port = ports["twelve_materials"]
    frame = 7
    for chunk in (k, 2 * k + 1, 37):
        sim.run_frames(chunk)
        port.run(g, frame, chunk, nthreads=8)
        frame += chunk
        got = sim.grid
        assert np.array_equal(got, g), f"k={k} {shape}: {np.count_nonzero(got != g)} cells differ at frame {frame}"
    assert sim.params.frame == frame


def test_edits_inside_fused_runs(se, ports, rulesets):
    """Mods apply to the first frame of a multi-frame call; the rest run fused."""
    from sandengine_gb300 import workloads as wl
    w, h = 300, 200
    g = wl.patch_fill(w, h, 3, *wl.twelve_fill_spec(), patch=16)
    sim = _sim(se, rulesets["twelve_materials"], w, h, k=8)
    sim.grid = g
    sim.params.frame = 2
    port = ports["twelve_materials"]
    frame = 2
    for r in range(6):
        raw = wl.circle_edits(w, h, 9, r, 12, [0, 3, 200, 14])
        raw.append((r * 7, 150, 1, 9, 5))
        sim.run_frames(23, _mods(se, raw))
        port.run(g, frame, 23, raw, nthreads=8)
        frame += 23
        assert np.array_equal(sim.grid, g), f"round {r}"


POS_RULE = """
  ledge:
    if: isType_EMPTY(DOWN) and pos.x + pos.y * 3 - frame % 7 > 11
    do: SWAP SELF DOWN
"""


def test_direct_path_matches_port(se, rulesets):
    """A rule that reads the block position and the frame cannot use the block transition
    table; the direct rule-evaluation path must be exact too."""
    from oracle.build import Port
    from sandengine_gb300 import workloads as wl
    text = rulesets["four_materials"].replace("rules:\n", "rules:\n" + POS_RULE.lstrip("\n"), 1)
    text = text.replace("base_rules: [fall]", "base_rules: [fall, ledge]")
    rs = se.parse_string(text)
    assert "SE_LUT" not in rs.cuda_source
    port = Port(text)
    w, h = 203, 131
    g = wl.iid_fill(w, h, 5, *wl.FOUR_FILL)
    for k in (1, 4):
        sim = se.Simulation(rs, (w, h))
        sim.set_steps_per_launch(k)
        a = g.copy()
        sim.grid = a
        sim.params.frame = 3
        sim.run_frames(40)
        port.run(a, 3, 40)
        assert np.array_equal(sim.grid, a), f"k={k}"


def test_narrow_table_keys_match_port(se):
    """A rule set with 544 hash classes keys its table with 3 bits per id (the generic key
    build); one-frame and fused launches must be exact too, and the device-built table must
    equal the one the same device code builds on the CPU."""
    import ctypes
    from oracle.build import Port
    from sandengine_gb300 import workloads as wl
    from tests.device_emu.emu import Emu
    with open(os.path.join(GOLDEN, "many_hash_classes.yaml")) as f:
        text = f.read()
    rs = se.parse_string(text)
    assert "#define SE_LUT_BITS 3" in rs.cuda_source
    table, bits = rs.table()
    E = Emu(rs, lut=True)
    E.lib.emu_lut.restype = ctypes.POINTER(ctypes.c_uint16)
    assert np.array_equal(table, np.ctypeslib.as_array(E.lib.emu_lut(), shape=(table.size,)))
    port = Port(text)
    w, h = 203, 131
    g = wl.iid_fill(w, h, 6, *wl.FOUR_FILL)
    for k in (1, 8):
        sim = se.Simulation(rs, (w, h))
        sim.set_steps_per_launch(k)
        a = g.copy()
        sim.grid = a
        sim.params.frame = 3
        sim.run_frames(45)
        port.run(a, 3, 45)
        assert np.array_equal(sim.grid, a), f"k={k}"


def test_frame_one_clears(se, rulesets):
    g = np.full((40, 40), 3, dtype=np.uint32)
    sim = _sim(se, rulesets["four_materials"], 40, 40)
    sim.grid = g
    assert sim.params.frame == 0
    sim.run_frames(1, [se.SimModification((5, 5), 0, 3, 3)])  # frame 1: clear, mods ignored
    assert sim.params.frame == 1
    assert not sim.grid.any()
    sim.run_frames(50)
    assert not sim.grid.any()


def test_digest_and_histogram_on_device(se, rulesets):
    from sandengine_gb300.simulation import grid_digest
    from sandengine_gb300 import workloads as wl
    g = wl.world_256(4)
    sim = _sim(se, rulesets["four_materials"], 256, 256)
    sim.grid = g
    assert sim.digest() == grid_digest(g)
    hist = sim.histogram(7)
    ref = np.bincount(np.minimum(g.ravel(), 6), minlength=7)
    assert np.array_equal(hist, ref)


@pytest.mark.parametrize("name", ["four_materials", "twelve_materials"])
def test_device_table_matches_emulated_rules(se, rulesets, name):
    """The block transition table and static-key bitset built on the GPU (se_build_lut,
    se_build_static) equal those the same device code builds on the CPU."""
    import ctypes
    from tests.device_emu.emu import Emu
    rs = se.parse_string(rulesets[name])
    table, bits = rs.table()
    assert table is not None
    E = Emu(rs, lut=True)
    E.lib.emu_lut.restype = ctypes.POINTER(ctypes.c_uint16)
    E.lib.emu_static.restype = ctypes.POINTER(ctypes.c_uint32)
    want_t = np.ctypeslib.as_array(E.lib.emu_lut(), shape=(table.size,))
    want_b = np.ctypeslib.as_array(E.lib.emu_static(), shape=(bits.size,))
    assert np.array_equal(table, want_t)
    assert np.array_equal(bits, want_b)
    assert 0 < int(np.unpackbits(bits.view(np.uint8)).sum()) < 32 * bits.size


def test_overlapped_read_back_returns_each_steps_grid(se, rulesets, ports):
    """se_world_read_grid_overlapped: two read-backs in flight, then a third that waits for
    the first; after synchronize each buffer holds the grid of the step it was issued after."""
    from sandengine_gb300 import workloads as wl
    P = ports["twelve_materials"]
    rs = se.parse_string(rulesets["twelve_materials"])
    W, H = 300, 220
    g = wl.patch_fill(W, H, 8, *wl.twelve_fill_spec(), patch=16)
    sim = se.Simulation(rs, (W, H))
    sim.grid = g
    sim.params.frame = 2
    outs, wants, f = [], [], 2
    for r in range(3):
        sim.run_frames(7)
        P.run(g, f, 7)
        f += 7
        o = np.empty((H, W), dtype=np.uint32)
        sim.read_grid_overlapped(o)
        outs.append(o)
        wants.append(g.copy())
    sim.synchronize()
    for o, w in zip(outs, wants):
        assert np.array_equal(o, w)


@pytest.mark.parametrize("shape", [(300, 220), (301, 7)])
def test_packed_read_back_returns_each_steps_grid(se, rulesets, ports, shape):
    """se_world_read_grid_u8_overlapped: the ids as bytes, three read-backs in flight over
    consecutive steps (the third waits for the first's staging buffer), each equal to the
    oracle's grid of its step; a cell count not a multiple of 4 takes the tail path.  Before
    any frame, ids that name no material read as NULL (1)."""
    from sandengine_gb300 import workloads as wl
    P = ports["twelve_materials"]
    rs = se.parse_string(rulesets["twelve_materials"])
    W, H = shape
    g = wl.patch_fill(W, H, 8, *wl.twelve_fill_spec(), patch=16)
    g[::5, ::3] = 300  # unknown ids
    sim = se.Simulation(rs, (W, H))
    sim.grid = g
    sim.params.frame = 2
    first = np.empty((H, W), dtype=np.uint8)
    sim.read_grid_u8_overlapped(first)
    sim.synchronize()
    assert np.array_equal(first, np.where(g < rs.num_materials, g, 1).astype(np.uint8))
    outs, wants, f = [], [], 2
    for r in range(3):
        sim.run_frames(7)
        P.run(g, f, 7)
        f += 7
        o = np.empty((H, W), dtype=np.uint8)
        sim.read_grid_u8_overlapped(o)
        outs.append(o)
        wants.append(g.copy())
    sim.synchronize()
    for o, w in zip(outs, wants):
        assert int(w.max()) < 256 and np.array_equal(o, w.astype(np.uint8))
    # a buffer of the wrong size is refused with a status, before any copy
    import ctypes
    from sandengine_gb300._lib import lib
    small = np.empty(W * H - 1, dtype=np.uint8)
    assert lib().se_world_read_grid_u8_overlapped(sim.handle, small.ctypes.data, small.size) == 1
    assert b"width * height" in lib().se_last_error()
