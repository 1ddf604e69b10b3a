"""The CHECKED build on the GPU (se_ruleset_set_checked): kernels compiled with index checks
on every shared-memory, global and table access run the parity workloads — every tile
variant through k = 1..16, ragged sizes, edits, row bands, a batch with resident and tiled
worlds, a serving mix — bit-exact against the oracle, with no failed check."""
import numpy as np
import pytest

from sandengine_gb300 import workloads as wl

pytestmark = pytest.mark.gpu


def _checked(se, text):
    rs = se.parse_string(text)
    rs.set_checked(True)
    rs.compile()
    assert "#define SE_CHECKED 1" in rs.kernel_source
    return rs


@pytest.mark.parametrize("name", ["four_materials", "twelve_materials"])
def test_checked_single_worlds(se, rulesets, ports, name):
    rs, P = _checked(se, rulesets[name]), ports[name]
    for W, H in ((517, 389), (300, 1000), (64, 64), (7, 5)):
        g = (wl.patch_fill(W, H, 3, *wl.twelve_fill_spec(), patch=16) if name == "twelve_materials"
             else wl.iid_fill(W, H, 3, *wl.FOUR_FILL))
        for k in (1, 2, 4, 8, 16):
            sim = se.Simulation(rs, (W, H))
            sim.set_steps_per_launch(k)
            sim.grid = g
            sim.params.frame = 3
            mods = [se.SimModification((m[0], m[1]), m[2], m[3], m[4])
                    for m in wl.circle_edits(W, H, 1, k, 4, [0, 3])]
            sim.run_frames(2 * k + 3, mods)
            want = g.copy()
            P.run(want, 3, 2 * k + 3, [(m.position[0], m.position[1], m.mod_shape, m.mod_size, m.mod_matID)
                                       for m in mods])
            assert np.array_equal(sim.grid, want), f"{W}x{H} k={k}"
    assert rs.check_word() == 0


def test_checked_bands_batch_and_serving(se, rulesets, ports):
    from sandengine_gb300 import bands as B
    from sandengine_gb300.batch import Batch
    from sandengine_gb300.serving import Server
    text = rulesets["twelve_materials"]
    rs, P = _checked(se, text), ports["twelve_materials"]
    W, H = 400, 330
    g = wl.patch_fill(W, H, 5, *wl.twelve_fill_spec(), patch=16)
    lb = B.LocalBands(rs, W, H, 3, 8, make=lambda r0, n, h: B.GpuBand(rs, W, H, r0, n, h, steps_per_launch=8))
    lb.grid = g
    lb.frame = 2
    lb.step(30)
    want = g.copy()
    P.run(want, 2, 30)
    assert np.array_equal(lb.grid, want)
    sizes = [(96, 64), (300, 200), (33, 17), (700, 500)]
    grids = [wl.patch_fill(w, h, 60 + i, *wl.twelve_fill_spec(), patch=16) for i, (w, h) in enumerate(sizes)]
    b = Batch(rs, sizes)
    for i, gi in enumerate(grids):
        b.set_grid(i, gi)
        b.set_frame(i, 2)
    b.step(21)
    b.synchronize()
    for i, gi in enumerate(grids):
        w2 = gi.copy()
        P.run(w2, 2, 21)
        assert np.array_equal(b.grid(i), w2), f"batch world {i}"
    srv = Server(rs, 1 << 30)
    sids = [srv.open_session(w, h, gi, 2) for (w, h), gi in zip(sizes, grids)]
    rids = [srv.submit(s, 11 + 3 * s) for s in sids]
    srv.run()
    for s, (w, h), gi in zip(sids, sizes, grids):
        w3 = gi.copy()
        P.run(w3, 2, 11 + 3 * s)
        assert np.array_equal(srv.grid(s), w3), f"session {s}"
    assert len(rids) == len(sids)
    assert rs.check_word() == 0
