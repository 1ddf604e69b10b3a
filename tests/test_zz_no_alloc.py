"""se_grid_histogram_noalloc: material counts of a device grid without allocating.

Callers such as a frame loop with all GPU memory sized up front, or a server whose HBM
budget is fully committed, cannot call cudaMalloc when they need the counts; this entry
point counts into a fixed static device array instead.  Its results must equal a count of
the grid read back to the host (and se_world_histogram's, which counts into memory the
world allocated) exactly, call after call, even though every call reuses the same array.  This file is collected last so that
a failure here does not stop the other tests of a run that stops at the first failure.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _noalloc(lib, device_ptr, count, nbins, stream=0):
    out = np.zeros(nbins, dtype=np.uint64)
    rc = lib.se_grid_histogram_noalloc(ctypes.c_void_p(device_ptr), count, nbins, out.ctypes.data,
                                       ctypes.c_void_p(stream))
    return rc, out


def test_noalloc_histogram_matches_world_histogram_twice(se, rulesets):
    from sandengine_gb300 import workloads as wl
    from sandengine_gb300._lib import lib
    L = lib()
    w, h = 300, 200
    rs = se.parse_string(rulesets["twelve_materials"])
    sim = se.Simulation(rs, (w, h))
    g = wl.patch_fill(w, h, 2, *wl.twelve_fill_spec(), patch=8)
    g[::7, ::5] = 200  # values that name no material land in the last bin
    sim.grid = g
    sim.params.frame = 1
    nbins = rs.num_materials + 1
    for call in range(2):
        grid = sim.grid  # read back to the host: the independent count
        want = np.bincount(np.minimum(grid.ravel(), nbins - 1), minlength=nbins).astype(np.uint64)
        rc, got = _noalloc(L, sim.device_grid_ptr(), w * h, nbins, sim.stream)
        assert rc == 0, L.se_last_error()
        assert np.array_equal(got, want), f"call {call}: {got} != {want}"
        assert np.array_equal(got, sim.histogram(nbins))  # and the allocating entry point agrees
        assert int(got.sum()) == w * h
        sim.run_frames(9)  # a different grid for the second call


def test_noalloc_histogram_rejects_too_many_bins(se, rulesets):
    from sandengine_gb300._lib import lib
    L = lib()
    rs = se.parse_string(rulesets["four_materials"])
    sim = se.Simulation(rs, (16, 16))
    rc, _ = _noalloc(L, sim.device_grid_ptr(), 256, 258)
    assert rc == 1
    assert b"257" in L.se_last_error()
    rc, out = _noalloc(L, sim.device_grid_ptr(), 256, 257)
    assert rc == 0 and int(out[0]) == 256
