"""The oracle pinned: its front end against the reference's generated files, its error
kinds against the reference's tests, its port against the reference's own compute
shader (compiled on the CPU) and against the recorded per-frame digests."""
import hashlib
import json
import os

import numpy as np
import pytest

from oracle import frontend as fe
from oracle.build import Port, Ref, RefFrag, reference_root
from sandengine_gb300.simulation import grid_digest
from tests.conftest import GOLDEN
from tests.golden.cases import CASES
from tests.golden.yaml_corpus import CORPUS


def _gen_golden():
    with open(os.path.join(GOLDEN, "reference_gen.json")) as f:
        return json.load(f)


def _ref(text):
    """The reference shader compiled for the CPU: from the checkout SANDENGINE_REF names, or
    from the translated source an earlier build left in oracle/_ref (skip if neither)."""
    try:
        return Ref(text)
    except FileNotFoundError:
        pytest.skip("no reference checkout (SANDENGINE_REF) and no translated reference source")


def test_frontend_reproduces_reference_generated_glsl(rulesets):
    """data/materials.yaml -> gen/materials.glsl and gen/rules.glsl, byte for byte."""
    mat, rules = fe.create_glsl(fe.parse_string(rulesets["reference"]))
    gold = _gen_golden()
    for name, text in (("materials.glsl", mat), ("rules.glsl", rules)):
        data = text.encode()
        assert len(data) == gold[name]["bytes"]
        assert hashlib.sha256(data).hexdigest() == gold[name]["sha256"]


@pytest.mark.skipif(reference_root() is None, reason="needs the reference checkout (SANDENGINE_REF)")
def test_flattener_reproduces_reference_falling_sand():
    from oracle.build import reference_shader_text
    with open(os.path.join(GOLDEN, "reference_materials.yaml")) as f:
        text = reference_shader_text(f.read(), reference_root())
    gold = _gen_golden()["falling_sand.glsl"]
    assert hashlib.sha256(text.encode()).hexdigest() == gold["sha256"]


@pytest.mark.parametrize("name, kind", [
    # the reference's tests (tests/test_sandengine-lang.rs) and what its code returns for
    # their inputs: missing sections, a numeric rule name checked after the missing
    # `types`, a missing field, and a do-string the do-parser does not recognise.
    ("missing_rules", "MissingField"),
    ("missing_types", "MissingField"),
    ("missing_materials", "MissingField"),
    ("number_rule_name_without_types", "MissingField"),
    ("number_rule_name", "InvalidType"),
    ("missing_if", "MissingField"),
    ("missing_color", "MissingField"),
    ("unknown_type", "NotFound"),
    ("function_call_do", "NotRecognized"),
])
def test_error_kinds_follow_reference_code(name, kind):
    with pytest.raises(fe.ParseError) as e:
        fe.parse_string(CORPUS[name])
    assert e.value.kind == kind
    assert f"({kind})" in str(e.value)


def test_hash43_lanes_and_mirror_threshold(ports):
    """hash43 lanes equal RN(float(u)) * 2^-32 of the integer lanes, and the mirror test
    rand.x < 0.5 equals lane < 2^31 - 64 (the lane value the CUDA kernel compares)."""
    port = ports["four_materials"]

    def lanes(x, y, f):
        v = (x * 461 + y * 2131 + f * 4541161) & 0xFFFFFFFF
        out = []
        for m in (213, 2131, 21313, 213132):
            h = (v * m) & 0xFFFFFFFF
            h ^= h >> 16
            h = (h * 0x7FEB352D) & 0xFFFFFFFF
            h ^= h >> 15
            h = (h * 0x846CA68B) & 0xFFFFFFFF
            h ^= h >> 16
            out.append(h)
        return out

    rng = np.random.default_rng(1)
    for _ in range(500):
        x, y, f = (int(v) for v in rng.integers(-3, 5000, 3))
        got = port.hash43(x, y, f)
        ls = lanes(x, y, f)
        want = np.array([np.float32(np.float32(h) * np.float32(2.0 ** -32)) for h in ls], dtype=np.float32)
        assert np.array_equal(got, want)
        assert (got[0] < np.float32(0.5)) == (ls[0] < 0x7FFFFFC0)
    for u in (0x7FFFFFBF, 0x7FFFFFC0, 0x7FFFFFC1, 0x80000000):
        assert (np.float32(u) * np.float32(2.0 ** -32) < np.float32(0.5)) == (u < 0x7FFFFFC0)


@pytest.mark.parametrize("case", CASES, ids=[c.name for c in CASES])
def test_port_matches_reference_digests(case):
    with open(os.path.join(GOLDEN, "grids.json")) as f:
        gold = json.load(f)[case.name]["digests"]
    port = Port(case.ruleset_text())
    g = case.initial_grid()
    for i in range(case.frames):
        port.step(g, case.frame0 + 1 + i, case.mods_at(i), nthreads=4)
        assert grid_digest(g) == int(gold[i]), f"frame {case.frame0 + 1 + i}"


@pytest.mark.parametrize("name", ["reference", "four_materials", "twelve_materials"])
def test_port_matches_reference_shader(rulesets, name):
    """Random worlds with unknown ids, WALL/NULL cells and overlapping edits of every
    kind (unknown material, size 0 terminator, negative position, squares)."""
    text = rulesets[name]
    P, R = Port(text), _ref(text)
    rng = np.random.default_rng(7)
    for H, W in ((37, 50), (16, 16), (5, 9)):
        g = rng.integers(0, P.num_materials + 3, size=(H, W)).astype(np.uint32)
        g[rng.random((H, W)) < 0.4] = 0
        gp, gr = g.copy(), g.copy()
        for f in range(2, 90):
            mods = None
            if f % 5 == 0:
                mods = [(int(rng.integers(-5, W + 5)), int(rng.integers(-5, H + 5)), int(rng.integers(0, 3)),
                         int(rng.integers(-2, 8)), int(rng.integers(0, P.num_materials + 2))) for _ in range(6)]
            P.step(gp, f, mods)
            gr = R.step(gr, f, mods, nthreads=4)
            assert np.array_equal(gp, gr), f"{name} {H}x{W} frame {f}"


def test_port_edit_pass_extreme_mods(rulesets):
    """Mods far outside the grid, huge radii and positions whose difference wraps."""
    text = rulesets["four_materials"]
    P, R = Port(text), _ref(text)
    g = np.zeros((20, 24), dtype=np.uint32)
    g[5:15, 5:15] = 3
    mods = [(-2**31 + 3, 4, 1, 2**31 - 1, 4), (12, 10, 0, 2**23, 5), (2**31 - 1, -2**31, 0, 7, 3),
            (3, 3, 1, -4, 4), (10, 10, 0, 3, 1)]
    for f in (2, 3, 6):
        gp, gr = g.copy(), g.copy()
        P.step(gp, f, mods)
        gr = R.step(gr, f, mods)
        assert np.array_equal(gp, gr)


@pytest.mark.parametrize("name", ["reference", "twelve_materials"])
def test_port_color_and_light_match_reference_shader(rulesets, name):
    """The port's colour (material colour minus 3-octave noise) and light propagation equal
    the compiled reference shader's output_color and output_light bit for bit, frame after
    frame (the light field carried over), with edits, emitting materials (the twelve set
    has two), the frame-1 clear and worlds wider than the noise period."""
    text = rulesets[name]
    P, R = Port(text), _ref(text)
    rng = np.random.default_rng(11)
    for H, W, f0 in ((40, 300, 2), (17, 23, 0)):
        g = rng.integers(0, P.num_materials + 2, size=(H, W)).astype(np.uint32)
        g[rng.random((H, W)) < 0.4] = 0
        light = np.zeros((H, W, 4), dtype=np.float32)
        port_light = light.copy()
        gp = g.copy()
        for f in range(f0 + 1, f0 + 25):
            mods = None
            if f % 4 == 0:
                mods = [(int(rng.integers(0, W)), int(rng.integers(0, H)), int(rng.integers(0, 2)),
                         int(rng.integers(1, 6)), int(rng.integers(0, P.num_materials))) for _ in range(4)]
            color = np.zeros((H, W, 4), dtype=np.float32)
            new = R.step(g, f, mods, light=light, color=color)
            old = gp.copy()
            P.step(gp, f, mods)
            assert np.array_equal(gp, new)
            port_light = P.light(old, gp, port_light)
            assert np.array_equal(P.color(gp).view(np.uint32), color.view(np.uint32)), f"colour, frame {f}"
            assert np.array_equal(port_light.view(np.uint32), light.view(np.uint32)), f"light, frame {f}"
            g = new
        assert np.count_nonzero(light) > 0


def test_port_composite_known_answers(rulesets):
    """The composite restatement on fields with closed-form answers: an opaque uniform
    field shades with occlusion 0 (ambient 0.1) and sky light 0.5 * (1 - v'); transparent
    cells show the background tinted by the same light; the pyramid averages 2x2 blocks."""
    P = Port(rulesets["four_materials"])
    H, W = 32, 32
    color = np.zeros((H, W, 4), dtype=np.float32)
    color[...] = (0.8, 0.4, 0.2, 1.0)
    out = P.composite(color)
    d = np.float32(1.0) / (np.float32(W) / np.float32(2.0))
    v = (np.arange(H, dtype=np.float32) + np.float32(0.5)) / np.float32(H)
    pv = np.floor(v / d) * d
    sky = np.float32(0.5) * (np.float32(1.0) - pv)
    shade = np.float32(0.1)  # occ = 1 - 1 = 0
    want_r = np.float32(0.8) * shade * (np.float32(0.1) + sky)
    assert np.allclose(out[:, 0, 0], want_r, rtol=1e-6, atol=0)
    assert np.all(out[..., 3] == 1.0)
    bg = np.random.default_rng(0).random((H, W, 4)).astype(np.float32)
    clear = np.zeros_like(color)
    out2 = P.composite(clear, background=bg)
    # 1:1 bilinear at texel centres of a flipped v: the background's rows reversed
    assert np.allclose(out2[..., 3], bg[::-1, :, 3], rtol=1e-6, atol=1e-7)
    lv = P.mips(bg)
    assert lv[1].shape == (16, 16, 4)
    assert np.allclose(lv[1], bg.reshape(16, 2, 16, 2, 4).mean(axis=(1, 3)), rtol=1e-6, atol=1e-7)
    assert lv[-1].shape == (1, 1, 4)


def test_oracle_sin_is_sin_rounded_once(ports):
    """GLSL leaves sin's precision to the driver; the oracle (and the GPU colour pass) fix it
    to binary64 evaluation (Cody-Waite reduction, Taylor series) rounded once to binary32.
    Over magnitudes 2^-20 .. 2^30 (the colour noise's arguments stay below 2^30) it equals
    the binary64 sin rounded to binary32 on every sampled argument, and it is within 1 ulp
    of that by construction."""
    P = ports["twelve_materials"]
    rng = np.random.default_rng(1)
    mag = 2.0 ** rng.uniform(-20, 30, 400_000)
    x = (mag * rng.choice([-1, 1], mag.size)).astype(np.float32)
    ix, iy = np.meshgrid(np.arange(-300, 300, dtype=np.float32), np.arange(0, 200, dtype=np.float32))
    q = (ix * np.float32(127.1) + iy * np.float32(311.7)).ravel()  # old_hash2's arguments
    x = np.concatenate([x, q, np.float32([0.0, -0.0, 1e-30, np.pi / 2, np.pi, 1e9])])
    ours = P.sin(x)
    want = np.sin(x.astype(np.float64)).astype(np.float32)
    ulp = np.abs(ours.view(np.int32).astype(np.int64) - want.view(np.int32).astype(np.int64))
    assert ulp.max() <= 1
    assert np.count_nonzero(ulp) <= x.size // 100000
    special = P.sin(np.float32([np.inf, -np.inf, np.nan, 2.0**60]))
    assert np.isnan(special[:3]).all() and special[3] == 0.0


def _ref_frag():
    try:
        return RefFrag()
    except FileNotFoundError:
        pytest.skip("no reference checkout (SANDENGINE_REF) and no translated reference source")


@pytest.mark.parametrize("shape", [(64, 48), (333, 517), (7, 5), (1, 33), (2, 1)])
def test_port_composite_matches_reference_fragment_shader(rulesets, shape):
    """The composite's restatement (port_composite) equals the reference's own
    shaders/fragment140.glsl, compiled for the CPU from its text and run per pixel with the
    samplers the composite fixes (nearest magnification and LINEAR_MIPMAP_NEAREST for the
    colour pyramid, bilinear light and background, mirrored repeat), bit for bit: with a
    light field and a background image, with light alone, and with neither."""
    W, H = shape
    P, F = Port(rulesets["twelve_materials"]), _ref_frag()
    rng = np.random.default_rng(W * 1000 + H)
    g = rng.integers(0, P.num_materials + 2, size=(H, W)).astype(np.uint32)
    g[rng.random((H, W)) < 0.4] = 0
    col = P.color(g)
    light = (rng.random((H, W, 4)) * 1.5).astype(np.float32)
    bg = rng.random((211, 157, 4)).astype(np.float32)
    for li, b in ((light, bg), (light, None), (None, None)):
        want = P.composite(col, li, b)
        got = F.composite(P.mips(col), li, b)
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


def test_fullsize_batch_and_serve_fixtures_reproduce_on_the_port(ports):
    """The batch4096 and serve entries of tests/golden/fullsize.json hold for the workloads
    as workloads.py defines them today: their shape (4096 worlds, 149 sessions, 300
    requests), and the port's digests of the eight smallest batch worlds after 100 frames
    and of the two smallest serving sessions after all their requests."""
    import json
    from sandengine_gb300 import workloads as wl
    from sandengine_gb300.simulation import grid_digest
    with open(os.path.join(GOLDEN, "fullsize.json")) as f:
        gold = json.load(f)
    port = ports["twelve_materials"]
    b = gold["batch4096"]
    sizes = wl.batch_sizes(b["worlds"], 4)
    assert len(sizes) == 4096 and all(len(cp["digests"]) == 4096 for cp in b["checkpoints"])
    assert all(c["equal"] for c in b["reference_checks"])
    spec = wl.twelve_fill_spec()
    for i in sorted(range(len(sizes)), key=lambda i: sizes[i][0] * sizes[i][1])[:8]:
        g = np.ascontiguousarray(wl.patch_fill(sizes[i][0], sizes[i][1], 1000 + i, *spec, patch=16), dtype=np.uint32)
        port.run(g, b["frame0"], b["checkpoints"][0]["frames"], nthreads=8)
        assert "%016x" % grid_digest(g) == b["checkpoints"][0]["digests"][i], f"batch world {i} {sizes[i]}"
    s = gold["serve"]
    sessions, reqs = wl.serve_requests(1.0, s["requests"])
    assert len(sessions) == s["sessions"] == len(s["digests"]) and len(reqs) == 300
    assert all(c["equal"] for c in s["reference_checks"])
    for c in s["reference_checks"]:
        sid = c["session"]
        g = np.ascontiguousarray(wl.serve_session_grid(*sessions[sid], sid), dtype=np.uint32)
        frame = 1
        for s2, n, mods, _ in reqs:
            if s2 == sid:
                port.run(g, frame, n, mods or None, nthreads=8)
                frame += n
        assert "%016x" % grid_digest(g) == s["digests"][sid] and frame == s["frames"][sid], f"session {sid}"
