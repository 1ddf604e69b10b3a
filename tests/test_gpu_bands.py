"""Row bands of one world on the GPU (se_world_create_band + sandengine_gb300.bands), all in
one process: the bands' own rows after every step equal the whole world advanced by one
Simulation, and both equal the oracle port."""
import numpy as np
import pytest

from sandengine_gb300 import bands as B
from sandengine_gb300 import workloads as wl

pytestmark = pytest.mark.gpu


def _mods(se, W, H, r):
    return [se.SimModification((x, y), s, size, m) for x, y, s, size, m in wl.circle_edits(W, H, 11, r, 6, [0, 3, 4])]


@pytest.mark.parametrize("nbands,per_exchange,k", [(2, 16, 16), (3, 8, 4), (4, 2, 1), (5, 12, 0)])
def test_bands_match_whole_world(se, rulesets, ports, nbands, per_exchange, k):
    text = rulesets["twelve_materials"]
    rs = se.parse_string(text)
    W, H = 520, 410
    g0 = wl.patch_fill(W, H, 4, *wl.twelve_fill_spec(), patch=32)
    whole = se.Simulation(rs, (W, H))
    whole.grid = g0
    whole.params.frame = 3
    lb = B.LocalBands(rs, W, H, nbands, per_exchange,
                      make=lambda r0, n, h: B.GpuBand(rs, W, H, r0, n, h, steps_per_launch=k))
    lb.grid = g0
    lb.frame = 3
    want = g0.copy()
    P = ports["twelve_materials"]
    f = 3
    for r, n in enumerate((1, 30, 5, 17)):
        mods = _mods(se, W, H, r) if r % 2 == 0 else []
        whole.run_frames(n, mods)
        lb.step(n, mods)
        P.run(want, f, n, [(m.position[0], m.position[1], m.mod_shape, m.mod_size, m.mod_matID) for m in mods])
        f += n
        got = lb.grid
        assert np.array_equal(got, whole.grid), f"after step {r}"
        assert np.array_equal(got, want), f"after step {r} (port)"
    assert lb.frame == f


def test_band_world_limits(se, rulesets, tmp_path):
    rs = se.parse_string(rulesets["four_materials"])
    b = B.GpuBand(rs, 64, 100, 40, 30, 6)
    assert (b.row0, b.rows) == (34, 42)
    with pytest.raises(se.SandengineError):
        b.step(7)  # more frames than the halo covers
    b.step(6)
    with pytest.raises(se.SandengineError):
        b.get_rows(20, 4)  # outside the buffer
    from sandengine_gb300._lib import lib
    with pytest.raises(se.SandengineError):
        from sandengine_gb300._lib import check
        check(lib().se_world_save(b._h, str(tmp_path / "band.sew").encode()))
