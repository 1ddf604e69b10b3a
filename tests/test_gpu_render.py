"""Colour and light outputs (the reference's setCell, operations.glsl:99-169) on the GPU
against the oracle port, which equals the compiled reference shader bit for bit on the CPU.

Light: bit-exact, frame after frame (additions, products, divisions and maxima in the
shader's order, no contraction).  Colour: the noise hashes sin(q) * 43758.5 through fract,
so a last-place difference between CUDA's sinf and the C library's moves a gradient by a
few thousandths, and in rare cells where the product sits next to an integer flips it;
the bounds below are on those statistics."""
import numpy as np
import pytest

from sandengine_gb300 import workloads as wl

pytestmark = pytest.mark.gpu


def _mods(se, W, H, r, mats):
    return [se.SimModification((x, y), s, size, m) for x, y, s, size, m in wl.circle_edits(W, H, 3, r, 5, mats)]


@pytest.mark.parametrize("name,shape,frame0", [("twelve_materials", (300, 200), 5), ("twelve_materials", (64, 48), 0),
                                               ("reference", (130, 70), 2)])
def test_light_matches_port_every_frame(se, rulesets, ports, name, shape, frame0):
    W, H = shape
    rs = se.parse_string(rulesets[name])
    P = ports[name]
    sim = se.Simulation(rs, (W, H))
    g = (wl.patch_fill(W, H, 9, *wl.twelve_fill_spec(), patch=16) if name == "twelve_materials"
         else np.random.default_rng(1).integers(0, P.num_materials, size=(H, W)).astype(np.uint32))
    sim.grid = g
    sim.params.frame = frame0
    sim.set_light(True)
    light = np.zeros((H, W, 4), dtype=np.float32)
    assert np.array_equal(sim.output_light, light)
    cur, f = g.copy(), frame0
    mats = list(range(3, P.num_materials))
    for r in range(12):
        mods = _mods(se, W, H, r, mats) if r % 3 == 0 else []
        sim.run_frames(1, mods)
        old = cur.copy()
        P.step(cur, f + 1, [(m.position[0], m.position[1], m.mod_shape, m.mod_size, m.mod_matID) for m in mods])
        f += 1
        light = P.light(old, cur, light)
        assert np.array_equal(sim.grid, cur), f"grid, frame {f}"
        assert np.array_equal(sim.output_light.view(np.uint32), light.view(np.uint32)), f"light, frame {f}"
    # several frames per call: the light pass still runs after every frame
    for n in (3, 7):
        sim.run_frames(n)
        for _ in range(n):
            old = cur.copy()
            P.step(cur, f + 1)
            f += 1
            light = P.light(old, cur, light)
    assert np.array_equal(sim.output_light.view(np.uint32), light.view(np.uint32))
    assert np.count_nonzero(light[..., 3]) > 0


def test_light_exact_max_with_nan_and_negative_zero(se, rulesets, ports):
    """A light field set by the caller may hold -0, NaN, negative or infinite values.  Tiles
    that stage any of them take GLSL max as written (a compare and a select), the others
    the hardware maximum; either way the field equals the oracle's.  NaNs are compared as
    NaNs (GPU arithmetic returns the canonical NaN, the CPU keeps the payload)."""
    W, H = 200, 90
    rs = se.parse_string(rulesets["twelve_materials"])
    P = ports["twelve_materials"]
    sim = se.Simulation(rs, (W, H))
    g = wl.patch_fill(W, H, 4, *wl.twelve_fill_spec(), patch=16)
    sim.grid = g
    sim.params.frame = 7
    sim.set_light(True)
    L = np.random.default_rng(3).random((H, W, 4)).astype(np.float32)
    # a few tiles (64 x 16 cells) get one unusual value each
    L[5, 10, 0] = -0.0
    L[20, 70, 3] = np.nan
    L[40, 130, 1] = -0.25
    L[70, 150, 2] = np.inf
    L[3, 190, 3] = -0.0
    sim.output_light = L
    cur, f, light = g.copy(), 7, L.copy()
    for _ in range(3):
        sim.run_frames(1)
        old = cur.copy()
        P.step(cur, f + 1)
        f += 1
        light = P.light(old, cur, light)
        got = sim.output_light
        nan = np.isnan(light)
        assert nan.any() and np.array_equal(np.isnan(got), nan), f"NaN cells, frame {f}"
        assert np.array_equal(got.view(np.uint32)[~nan], light.view(np.uint32)[~nan]), f"light, frame {f}"


def test_tall_world_spans_several_launches(se, rulesets, ports):
    """A world 2^20 rows tall has more row blocks than one launch's grid holds (65535), so
    the light, colour and composite passes are split over launches; grid, light and
    composite still equal the oracle bit for bit."""
    W, H = 8, 1 << 20
    P = ports["four_materials"]
    sim = se.Simulation(se.parse_string(rulesets["four_materials"]), (W, H))
    g = wl.patch_fill(W, H, 5, [0, 3, 4, 5], [0.6, 0.2, 0.15, 0.05], patch=4)
    sim.grid = g
    sim.params.frame = 3
    sim.set_light(True)
    sim.run_frames(2)
    cur, light = g.copy(), np.zeros((H, W, 4), dtype=np.float32)
    for f in (4, 5):
        old = cur.copy()
        P.step(cur, f)
        light = P.light(old, cur, light)
    assert np.array_equal(sim.grid, cur)
    assert np.array_equal(sim.output_light.view(np.uint32), light.view(np.uint32))
    col = sim.output_color
    assert np.array_equal(sim.composite().view(np.uint32), P.composite(col, light).view(np.uint32))


def test_light_field_round_trip_and_off(se, rulesets):
    rs = se.parse_string(rulesets["four_materials"])
    sim = se.Simulation(rs, (40, 30))
    with pytest.raises(se.SandengineError):
        sim.output_light  # off
    sim.set_light(True)
    L = np.random.default_rng(0).random((30, 40, 4)).astype(np.float32)
    sim.output_light = L
    assert np.array_equal(sim.output_light, L)
    sim.set_light(False)
    sim.run_frames(5)  # back to fused launches


@pytest.mark.parametrize("shape", [(1024, 768), (16384, 64), (5, 3)])
@pytest.mark.parametrize("name", ["twelve_materials", "reference"])
def test_color_matches_port_bit_for_bit(se, rulesets, ports, name, shape):
    """output_color (material colour minus the 3-octave simplex noise, clamped) equals the
    oracle's bit for bit: both evaluate the noise's sin the same way (binary64, rounded
    once).  A 16384-wide world reaches the noise's largest arguments on the benchmark's
    side length."""
    P = ports[name]
    rs = se.parse_string(rulesets[name])
    W, H = shape
    rng = np.random.default_rng(4)
    g = rng.integers(0, P.num_materials + 2, size=(H, W)).astype(np.uint32)
    g[rng.random((H, W)) < 0.3] = 0
    sim = se.Simulation(rs, (W, H))
    sim.grid = g
    got = sim.output_color
    want = P.color(g)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), \
        f"{int(np.count_nonzero((got != want).any(axis=-1)))} cells differ"
    # the same grid again reads the cached noise: identical output
    assert np.array_equal(sim.output_color, got)


def test_oracle_sin_within_cuda_sinf_bound(ports):
    """The sin that the colour pass and the oracle share is within CUDA's documented 2-ulp
    bound of CUDA's own sinf (torch.sin on float32 CUDA tensors), over the noise's argument
    range and beyond."""
    import torch
    P = ports["twelve_materials"]
    rng = np.random.default_rng(3)
    mag = 2.0 ** rng.uniform(-20, 30, 1_000_000)
    x = (mag * rng.choice([-1, 1], mag.size)).astype(np.float32)
    ours = P.sin(x)
    cuda = torch.sin(torch.from_numpy(x).cuda()).cpu().numpy()
    ulp = np.abs(ours.view(np.int32).astype(np.int64) - cuda.view(np.int32).astype(np.int64))
    print(f"sin vs CUDA sinf: {np.count_nonzero(ulp)} of {x.size} differ, max {ulp.max()} ulp")
    assert ulp.max() <= 2


@pytest.mark.parametrize("shape", [(640, 400), (333, 517), (64, 64), (7, 5), (1, 33), (35, 2), (2, 1)])
def test_composite_matches_port(se, rulesets, ports, shape):
    """The headless composite (fragment140.glsl) equals the oracle's restatement bit for bit
    when both start from the same colour and light fields (the GPU's own), with and
    without a background image, on non-square, odd-sized and one- or two-texel-wide worlds
    (where the pyramid's box filter clamps its second row or column)."""
    W, H = shape
    P = ports["twelve_materials"]
    rs = se.parse_string(rulesets["twelve_materials"])
    sim = se.Simulation(rs, (W, H))
    sim.grid = wl.patch_fill(W, H, 6, *wl.twelve_fill_spec(), patch=16)
    sim.params.frame = 3
    sim.set_light(True)
    sim.run_frames(20)
    col, light = sim.output_color, sim.output_light
    bg = np.random.default_rng(2).random((211, 157, 4)).astype(np.float32)
    got = sim.composite(bg)
    want = P.composite(col, light, bg)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
    got2 = sim.composite()
    assert np.array_equal(got2.view(np.uint32), P.composite(col, light).view(np.uint32))
    sim.set_light(False)  # no light field: zero light
    assert np.array_equal(sim.composite().view(np.uint32), P.composite(col).view(np.uint32))
    assert np.isfinite(got).all() and got.max() > 0


def test_composite_matches_reference_fragment_shader(se, rulesets, ports):
    """The GPU composite equals the reference's own fragment shader (fragment140.glsl
    compiled for the CPU, oracle/frag_driver.cpp's samplers) bit for bit, on the GPU's own
    colour and light fields."""
    from oracle.build import RefFrag
    try:
        F = RefFrag()
    except FileNotFoundError:
        pytest.skip("no translated reference fragment shader")
    W, H = 300, 211
    P = ports["twelve_materials"]
    rs = se.parse_string(rulesets["twelve_materials"])
    sim = se.Simulation(rs, (W, H))
    sim.grid = wl.patch_fill(W, H, 9, *wl.twelve_fill_spec(), patch=16)
    sim.params.frame = 3
    sim.set_light(True)
    sim.run_frames(12)
    col, light = sim.output_color, sim.output_light
    bg = np.random.default_rng(5).random((97, 131, 4)).astype(np.float32)
    got = sim.composite(bg)
    want = F.composite(P.mips(col), light, bg)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
