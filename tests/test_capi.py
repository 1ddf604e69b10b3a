"""The C ABI library: it loads, exports every function include/sandengine.h declares,
and rejects bad arguments with a status instead of crashing (no GPU work here)."""
import ctypes
import os
import re

from tests.conftest import ROOT


def _declared():
    with open(os.path.join(ROOT, "include", "sandengine.h")) as f:
        text = f.read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(se_[a-z_0-9]+)\s*\(", text)))


def test_library_exports_every_declared_symbol(built_lib):
    lib = ctypes.CDLL(built_lib)
    names = _declared()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_bad_arguments_return_status(se):
    from sandengine_gb300._lib import lib
    L = lib()
    out = ctypes.c_void_p()
    assert L.se_ruleset_parse(None, ctypes.byref(out)) == 1
    assert b"null" in L.se_last_error()
    assert L.se_world_step(None, 1, None, 0) == 1
    host = ctypes.create_string_buffer(64)
    assert L.se_world_read_grid_u8_overlapped(None, host, 16) == 1  # null world
    assert L.se_world_read_grid_overlapped(None, host, 16) == 1
    assert L.se_ruleset_text(None, 0, None, 0, None) == 1
    rs = se.parse_string(open(os.path.join(ROOT, "sandengine_gb300", "rulesets", "four_materials.yaml")).read())
    assert L.se_ruleset_text(rs.handle, 9, None, 0, None) == 1
    n = ctypes.c_size_t()
    buf = ctypes.create_string_buffer(8)
    assert L.se_ruleset_text(rs.handle, 0, buf, 8, ctypes.byref(n)) == 13  # buffer too small
    assert n.value > 8
    assert L.se_world_create(rs.handle, 0, 5, ctypes.byref(out)) == 1
    # sides up to 2^20 cells, at most 2^36 cells: refused before any device work
    for w, h, msg in [((1 << 20) + 1, 4, b"sides"), (4, (1 << 20) + 1, b"sides"), (1 << 20, 1 << 17, b"too large")]:
        assert L.se_world_create(rs.handle, w, h, ctypes.byref(out)) == 1
        assert msg in L.se_last_error()
    assert L.se_version() >= 100


def test_modification_record_layout():
    from sandengine_gb300._lib import SeModification
    assert ctypes.sizeof(SeModification) == 32
    assert SeModification.mod_shape.offset == 8
    assert SeModification.mod_size.offset == 12
    assert SeModification.mod_matID.offset == 16


def test_noalloc_histogram_rejects_bad_arguments_without_a_gpu(built_lib):
    """se_grid_histogram_noalloc checks its arguments before any CUDA call: a null device
    pointer, a null host pointer, and nbins outside [1, 257] are SE_ERR_INVALID_ARGUMENT
    with a message."""
    import ctypes
    import numpy as np
    from sandengine_gb300._lib import lib
    L = lib()
    out = np.zeros(8, dtype=np.uint64)
    fake = ctypes.c_void_p(0x1000)  # never dereferenced: the call fails before any CUDA work
    for dev, host, nbins in ((None, out.ctypes.data, 4), (fake, None, 4), (fake, out.ctypes.data, 0),
                             (fake, out.ctypes.data, -3), (fake, out.ctypes.data, 258)):
        rc = L.se_grid_histogram_noalloc(dev, 16, nbins, host, None)
        assert rc == 1, (dev, host, nbins)
        assert L.se_last_error()
