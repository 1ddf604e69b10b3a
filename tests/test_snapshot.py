"""World snapshots: the documented file layout, read without a GPU, and (GPU) a save /
load round trip that continues bit-exactly."""
import struct

import numpy as np
import pytest


def _write(path, w, h, frame, nmat=15, fp=0, cells=None, magic=b"SEW1"):
    cells = np.zeros((h, w), dtype="<u4") if cells is None else cells.astype("<u4")
    with open(path, "wb") as f:
        f.write(magic + struct.pack("<IIIiIQ", 32, w, h, frame, nmat, fp))
        f.write(cells.tobytes())


def test_snapshot_header_layout(se, tmp_path):
    from sandengine_gb300.simulation import snapshot_info
    p = tmp_path / "w.sew"
    _write(p, 37, 11, 123)
    assert snapshot_info(p) == {"width": 37, "height": 11, "frame": 123}
    bad = tmp_path / "bad.sew"
    _write(bad, 5, 5, 1, magic=b"NOPE")
    with pytest.raises(se.SandengineError):
        snapshot_info(bad)
    neg = tmp_path / "neg.sew"
    _write(neg, 5, 5, -4)
    with pytest.raises(se.SandengineError):
        snapshot_info(neg)


@pytest.mark.gpu
def test_save_load_continues_bit_exact(se, rulesets, tmp_path):
    from sandengine_gb300 import workloads as wl
    rs = se.parse_string(rulesets["twelve_materials"])
    a = se.Simulation(rs, (203, 131))
    a.grid = wl.patch_fill(203, 131, 8, *wl.twelve_fill_spec(), patch=16)
    a.params.frame = 5
    a.run_frames(17)
    p = tmp_path / "a.sew"
    a.save(p)
    b = se.Simulation(rs, (203, 131))
    b.load(p)
    assert b.params.frame == a.params.frame and np.array_equal(b.grid, a.grid)
    a.run_frames(29)
    b.run_frames(29)
    assert np.array_equal(a.grid, b.grid)
    other = se.parse_string(rulesets["four_materials"])
    c = se.Simulation(other, (203, 131))
    with pytest.raises(se.SandengineError):
        c.load(p)  # saved under another rule set
