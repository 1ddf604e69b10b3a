"""The exact JIT device source (kernel template + generated rules), compiled for the CPU by
tests/device_emu and run one thread per CTA, against the oracle port.  Covers every
tile variant, ragged world sizes, world borders and the edit pass without a GPU."""
import numpy as np
import pytest

from sandengine_gb300 import workloads as wl
from tests.device_emu.emu import VARIANTS, Emu


@pytest.fixture(scope="module", params=[True, False], ids=["table", "direct"])
def emus(se, rulesets, request):
    """Kernels with the block transition table, and with it compiled out."""
    return {n: Emu(se.parse_string(t), lut=request.param) for n, t in rulesets.items()}


def _world(name, w, h, seed):
    if name == "twelve_materials":
        return wl.patch_fill(w, h, seed, *wl.twelve_fill_spec(), patch=16)
    if name == "four_materials":
        return wl.iid_fill(w, h, seed, *wl.FOUR_FILL)
    rng = np.random.default_rng(seed)
    g = rng.integers(0, 14, size=(h, w)).astype(np.uint32)
    g[rng.random((h, w)) < 0.4] = 0
    return g


@pytest.mark.parametrize("name", ["reference", "four_materials", "twelve_materials"])
@pytest.mark.parametrize("shape", [(256, 256), (517, 389), (130, 67), (7, 5), (812, 430)])
def test_tile_variants_match_port(emus, ports, name, shape):
    w, h = shape
    E, P = emus[name], ports[name]
    g0 = _world(name, w, h, 3)
    for v in VARIANTS:
        a, f0 = g0.copy(), 5
        for rep in range(2):
            k = max(1, v[2] - rep)
            b = E.tiles(a, f0, k, v)
            P.run(a, f0 - 1, k)
            f0 += k
            assert np.array_equal(a, b), f"variant {v} k={k}: {np.count_nonzero(a != b)} cells differ"
            a = b


@pytest.mark.parametrize("name", ["four_materials", "twelve_materials"])
def test_batch_kernels_match_port(emus, ports, name):
    """Whole-world (resident) kernel, multi-world tile passes and the finalize step."""
    E, P = emus[name], ports[name]
    sizes = [(64, 64), (96, 160), (33, 17), (128, 70), (260, 130), (7, 9)]
    grids = [_world(name, w, h, 10 + i) for i, (w, h) in enumerate(sizes)]
    frames0 = [1 + 3 * i for i in range(len(sizes))]
    for F, k, resident in ((13, 8, [0, 2, 4]), (9, 4, []), (6, 16, list(range(6)))):
        out, fr = E.batch(grids, frames0, F, k, resident, variant=(128, 64, 8) if k <= 8 else (128, 128, 16))
        for i, g in enumerate(grids):
            want = g.copy()
            P.run(want, frames0[i], F)
            assert np.array_equal(out[i], want), f"world {i} ({sizes[i]}) F={F} k={k} resident={i in resident}"
            assert fr[i] == frames0[i] + F


def test_serving_iteration_matches_port(emus, ports):
    """One launch advancing several worlds by different frame counts."""
    name = "twelve_materials"
    E, P = emus[name], ports[name]
    sizes = [(300, 200), (64, 64), (129, 65), (5, 300)]
    grids = [_world(name, w, h, 20 + i) for i, (w, h) in enumerate(sizes)]
    frames = [3, 10, 1, 7]
    ks = [8, 1, 5, 3]
    outs = E.serve_iteration(grids, frames, ks)
    for g, f, k, o in zip(grids, frames, ks, outs):
        want = g.copy()
        P.run(want, f, k)
        assert np.array_equal(o, want)


@pytest.mark.parametrize("name", ["reference", "twelve_materials"])
def test_edit_pass_matches_port(emus, ports, name):
    w, h = 300, 200
    E, P = emus[name], ports[name]
    g = _world(name, w, h, 4)
    mods = wl.circle_edits(w, h, 9, 0, 12, [0, 3, 200, 14]) + [
        (5, 150, 1, 9, 5), (10, 10, 0, 0, 3), (1, 1, 1, 5, 4)]
    for f in (10, 11, 12, 13):
        a, b = g.copy(), g.copy()
        P.step(a, f, mods)
        b = E.tiles(b, f, 1)
        E.edit(b, mods)
        assert np.array_equal(a, b)


@pytest.mark.parametrize("name", ["reference", "twelve_materials"])
@pytest.mark.parametrize("variant", [(128, 64, 1), (128, 64, 8), (256, 128, 8), (64, 64, 4), (128, 128, 16)])
def test_edits_inside_the_fused_launch_match_port(emus, ports, name, variant):
    """The edit variant of the tile kernel: k frames in one launch whose first frame carries
    the edit pass (applied in shared memory after that frame's block update, to halo cells
    too), against the port's frame-then-edits.  Mods include circles and squares reaching
    past the world, size 0 ending the list, an unknown material (NULL: no edit) over an
    earlier hit, and WALL."""
    w, h = 300, 200
    E, P = emus[name], ports[name]
    g = _world(name, w, h, 4)
    mods = wl.circle_edits(w, h, 9, 0, 12, [0, 3, 200, 14]) + [
        (5, 150, 1, 9, 5), (299, 0, 0, 30, 2), (150, 100, 1, 40, 3), (160, 100, 0, 12, 250),
        (-4, 199, 1, 7, 4), (10, 10, 0, 0, 3), (1, 1, 1, 5, 4)]
    k = variant[2]
    for f in (10, 11, 12, 13):
        want = g.copy()
        P.run(want, f - 1, k, mods)
        got = E.tiles_edit(g, f, k, mods, variant)
        assert np.array_equal(got, want), f"frame {f}: {int(np.count_nonzero(got != want))} cells differ"


def _narrow_keys_text():
    """A rule set with 544 hash classes: its table keys take 3 bits per id (4-bit keys would
    make the table larger than 2^24 entries)."""
    import os
    from tests.conftest import GOLDEN
    with open(os.path.join(GOLDEN, "many_hash_classes.yaml")) as f:
        return f.read()


def _text(rulesets, name):
    return _narrow_keys_text() if name == "many_hash_classes" else rulesets[name]


@pytest.mark.parametrize("lut", [True, False], ids=["table", "direct"])
def test_narrow_table_keys_match_port(se, lut):
    """Every tile variant with 3-bit table keys (the generic key build of the collect and
    eval phases) against the port, on ragged worlds."""
    from oracle.build import Port
    text = _narrow_keys_text()
    rs = se.parse_string(text)
    assert "#define SE_LUT_BITS 3" in rs.kernel_source
    E, P = Emu(rs, lut=lut), Port(text)
    for w, h in [(130, 67), (517, 389)]:
        g0 = wl.iid_fill(w, h, 4, *wl.FOUR_FILL)
        for v in VARIANTS:
            a, f0 = g0.copy(), 5
            for rep in range(2):
                k = max(1, v[2] - rep)
                b = E.tiles(a, f0, k, v)
                P.run(a, f0 - 1, k)
                f0 += k
                assert np.array_equal(a, b), f"{w}x{h} variant {v} k={k}: {np.count_nonzero(a != b)} cells differ"
                a = b


@pytest.mark.parametrize("name", ["reference", "four_materials", "twelve_materials", "many_hash_classes"])
def test_lut_decode_inverts_lut_index(se, rulesets, name):
    """For every table entry, the cells and the representative hash values lut_decode gives
    index back to that entry (the key layout and the class order agree between the table
    build and the lookups)."""
    import ctypes
    E = Emu(se.parse_string(_text(rulesets, name)), lut=True)
    assert E.has_lut
    E.lib.emu_lut_roundtrip_failures.restype = ctypes.c_ulonglong
    assert E.lib.emu_lut_roundtrip_failures() == 0


@pytest.mark.parametrize("name", ["four_materials", "twelve_materials", "many_hash_classes"])
def test_static_key_bitset(se, rulesets, name):
    """Bit `key` of se_build_static's bitset is set exactly when every table entry of that
    key maps the block to itself; the all-EMPTY key is always static."""
    import ctypes
    rs = se.parse_string(_text(rulesets, name))
    E = Emu(rs, lut=True)
    assert E.has_lut
    src = rs.kernel_source
    bits = int(src.split("#define SE_LUT_BITS ")[1].split()[0])
    entries = int(src.split("#define SE_LUT_ENTRIES ")[1].split("u")[0])
    keys = 1 << (4 * bits)
    E.lib.emu_lut.restype = ctypes.POINTER(ctypes.c_uint16)
    E.lib.emu_static.restype = ctypes.POINTER(ctypes.c_uint32)
    E.lib.emu_static_words.restype = ctypes.c_uint
    words = E.lib.emu_static_words()
    assert words == max(1, keys // 32)
    st = np.ctypeslib.as_array(E.lib.emu_static(), shape=(words,)).copy()
    C = entries // keys
    lut = np.ctypeslib.as_array(E.lib.emu_lut(), shape=(entries,)).reshape(keys, C).astype(np.uint32)
    m = (1 << bits) - 1
    k = np.arange(keys, dtype=np.uint32)
    a, c, b, d = k & m, (k >> bits) & m, (k >> (2 * bits)) & m, (k >> (3 * bits)) & m  # column order
    self_ = a | (c << 4) | (b << 8) | (d << 12)  # the table's entry layout
    want = np.all(lut == self_[:, None], axis=1)
    got = ((st[k >> 5] >> (k & 31)) & 1).astype(bool)
    assert np.array_equal(got, want)
    assert got[0]
    assert 0 < got.sum() < keys


@pytest.mark.parametrize("name", ["four_materials", "twelve_materials"])
def test_band_window_matches_port(emus, ports, name):
    """A band buffer (world rows [ya, yb) of a taller world) advanced by the tile kernel in
    window mode: after n frames, in one or several launches, every row at least n rows
    inside the buffer equals the whole world run by the port (world coordinates for the
    hash, the block parity and the border)."""
    E, P = emus[name], ports[name]
    W, H = 264, 230
    g0 = _world(name, W, H, 21)
    for ya, yb, launches, v in ((40, 130, (8,), (128, 64, 8)), (0, 90, (3, 5), (128, 64, 8)),
                                (150, 230, (4, 4), (64, 64, 4)), (62, 200, (1, 1, 2), (128, 32, 1)),
                                (62, 200, (16,), (128, 128, 16))):
        f0 = 6
        buf = g0[ya:yb].copy()
        want = g0.copy()
        n = 0
        for k in launches:
            vv = v if v[2] >= k else min((x for x in VARIANTS if x[2] >= k), key=lambda x: x[2])
            buf = E.tiles(buf, f0 + n, k, vv, band=(H, ya))
            n += k
        P.run(want, f0 - 1, n)
        lo = 0 if ya == 0 else n
        hi = (yb - ya) if yb == H else (yb - ya) - n
        assert np.array_equal(buf[lo:hi], want[ya + lo:ya + hi]), f"band [{ya}, {yb}) launches {launches}"


WALL_RULE = """
  paint_wall:
    if: RIGHT.mat.density > 5000.0
    do: SET RIGHT sand
    else:
      if: DOWN.mat.density > 5000.0
      do: SET DOWN water
"""


def test_rules_that_set_wall_cells_keep_the_world_border(se, rulesets, ports):
    """A rule that SETs a WALL neighbour (rule text cannot name WALL, but WALL's density of
    9999 singles it out) changes WALL cells inside the world but never the WALL outside it
    (getCell returns WALL there and no invocation writes it): the tile, whole-world and
    serving kernels on worlds whose edges and interior hold WALL cells."""
    from oracle.build import Port
    text = rulesets["four_materials"].replace("rules:\n", "rules:\n" + WALL_RULE.lstrip("\n"), 1)
    text = text.replace("base_rules: [fall]", "base_rules: [fall, paint_wall]")
    rs = se.parse_string(text)
    assert "SE_LUT 1" in rs.cuda_source
    E, P = Emu(rs, lut=True), Port(text)
    rng = np.random.default_rng(12)
    for W, H in ((137, 61), (40, 33), (300, 150)):
        g = wl.iid_fill(W, H, 4, *wl.FOUR_FILL)
        g[rng.random((H, W)) < 0.05] = 2  # WALL inside the world
        for v in ((128, 64, 1), (128, 64, 8), (64, 64, 4), (256, 128, 8)):
            want = g.copy()
            P.run(want, 4, v[2])
            assert np.array_equal(E.tiles(g, 5, v[2], v), want), f"tile {v} {W}x{H}"
        out, _ = E.batch([g], [4], 9, 4, [0])  # whole world resident in shared memory
        want = g.copy()
        P.run(want, 4, 9)
        assert np.array_equal(out[0], want), f"resident {W}x{H}"
        got = E.serve_iteration([g], [4], [8])[0]
        want = g.copy()
        P.run(want, 4, 8)
        assert np.array_equal(got, want), f"serving {W}x{H}"


@pytest.mark.parametrize("name", ["four_materials", "twelve_materials", "many_hash_classes"])
def test_lut_index_classes_at_every_boundary(se, rulesets, name):
    """lut_index_key's class per hash lane equals #{thresholds <= h} at every threshold and
    its neighbours, every multiple of 2^24 and its predecessor, 0 and 2^32 - 1."""
    import ctypes
    import re
    rs = se.parse_string(_text(rulesets, name))
    src = rs.kernel_source
    dec = src[src.index("lut_decode("):]
    dec = dec[:dec.index("\n}\n")]
    lanes = {}
    for m in re.finditer(r"const uint32_t reps\[(\d+)\] = \{([^}]*)\}; h(\d) = ", dec):
        lanes[int(m.group(3))] = [int(v.rstrip("u")) for v in m.group(2).split(",")][1:]
    assert lanes
    E = Emu(rs, lut=True)
    f = E.lib.emu_lut_index_key
    f.restype = ctypes.c_uint32
    f.argtypes = [ctypes.c_uint32] * 5
    for lane, T in lanes.items():
        probes = {0, 0xFFFFFFFF}
        for t in T:
            probes |= {max(0, t - 1), t, min(0xFFFFFFFF, t + 1)}
        for b in range(256):
            probes |= {b << 24, max(0, (b << 24) - 1)}
        others = {l: 0 for l in lanes}  # class 0 in the other lanes
        for h in sorted(probes):
            hs = [others.get(l, 0) for l in range(4)]
            hs[lane] = h
            got = f(0, *hs)
            # index = sum over lanes of class * (product of later lanes' class counts)
            want = 0
            for l in sorted(lanes):
                want = want * (len(lanes[l]) + 1) + (sum(1 for t in lanes[l] if t <= hs[l]) if l == lane else 0)
            assert got == want, f"lane {lane} h={h:#x}: {got} != {want}"


def test_checked_build_records_failed_checks(se, rulesets):
    """The emulated kernels are the CHECKED build: se_check records failures in the check
    word (read and cleared per launch by the emulator), so every emulated test above also
    ran the index checks and none failed."""
    E = Emu(se.parse_string(rulesets["four_materials"]), lut=True)
    assert E.lib.emu_check_word() == 0
    E.lib.emu_check_selftest()
    assert E.lib.emu_check_word() == 0x3F
    assert E.lib.emu_check_word() == 0  # cleared by the read
    with pytest.raises(AssertionError):
        E.lib.emu_check_selftest()
        E._checked()
