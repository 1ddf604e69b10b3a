"""One world split into row bands with halo exchange (sandengine_gb300.bands), checked on
the CPU against the whole world run by the oracle port: in-process bands, and one band per
gloo rank (world_size 2 and 3).  The band engine here is the port on a buffer whose rows
outside the band read as WALL, as the CUDA kernel's window mode does."""
import multiprocessing as mp
import os
import socket

import numpy as np
import pytest

from sandengine_gb300 import bands as B
from sandengine_gb300 import workloads as wl
from sandengine_gb300.simulation import SimModification


class PortBand:
    """Band engine on the CPU: the oracle port over the world with only this buffer's rows
    present (the others WALL)."""

    def __init__(self, port, width, height, row0, rows, halo):
        self.port, self.W, self.H = port, width, height
        self.row0 = max(0, row0 - halo)
        self.rows = min(height, row0 + rows + halo) - self.row0
        self.buf = np.zeros((self.rows, width), dtype=np.uint32)
        self.frame = 0

    def get_rows(self, row, n):
        return self.buf[row - self.row0:row - self.row0 + n].copy()

    def set_rows(self, row, cells):
        self.buf[row - self.row0:row - self.row0 + len(cells)] = cells

    def step(self, n, mods=()):
        full = np.full((self.H, self.W), 2, dtype=np.uint32)
        full[self.row0:self.row0 + self.rows] = self.buf
        self.port.run(full, self.frame, n, [(m.position[0], m.position[1], m.mod_shape, m.mod_size, m.mod_matID)
                                            for m in mods])
        self.buf = full[self.row0:self.row0 + self.rows].copy()
        self.frame += n


def _mods(W, H, seed, r):
    return [SimModification((x, y), s, size, m) for x, y, s, size, m in wl.circle_edits(W, H, seed, r, 4, [0, 3, 4])]


SCHEDULE = [(1, True), (7, False), (8, True), (13, False), (2, True), (30, False)]


def _reference(port, g0, frame0, W, H):
    want = g0.copy()
    f = frame0
    for r, (n, edit) in enumerate(SCHEDULE):
        mods = _mods(W, H, 5, r) if edit else []
        port.run(want, f, n, [(m.position[0], m.position[1], m.mod_shape, m.mod_size, m.mod_matID) for m in mods])
        f += n
    return want


def test_band_split_and_halo():
    assert B.even_halo(1) == 2 and B.even_halo(8) == 8 and B.even_halo(9) == 10
    s = B.band_split(1000, 3, 8)
    assert s == [(0, 332), (332, 332), (664, 336)]
    assert all(r0 % 2 == 0 for r0, _ in s)
    with pytest.raises(ValueError):
        B.band_split(40, 4, 16)


@pytest.mark.parametrize("nbands,per_exchange", [(2, 8), (3, 4), (4, 1)])
def test_local_bands_match_whole_world(ports, nbands, per_exchange):
    P = ports["four_materials"]
    W, H = 96, 120
    g0 = wl.iid_fill(W, H, 3, *wl.FOUR_FILL)
    want = _reference(P, g0, 4, W, H)
    lb = B.LocalBands(None, W, H, nbands, per_exchange,
                      make=lambda r0, n, h: PortBand(P, W, H, r0, n, h))
    lb.grid = g0
    lb.frame = 4
    for r, (n, edit) in enumerate(SCHEDULE):
        lb.step(n, _mods(W, H, 5, r) if edit else [])
    assert lb.frame == 4 + sum(n for n, _ in SCHEDULE)
    assert np.array_equal(lb.grid, want)


def test_local_bands_from_frame_zero_clear(ports):
    """Frame 1 clears every band; edits then fill the world."""
    P = ports["twelve_materials"]
    W, H = 80, 64
    g0 = wl.patch_fill(W, H, 2, *wl.twelve_fill_spec(), patch=16)
    want = _reference(P, g0, 0, W, H)
    lb = B.LocalBands(None, W, H, 2, 6, make=lambda r0, n, h: PortBand(P, W, H, r0, n, h))
    lb.grid = g0
    for r, (n, edit) in enumerate(SCHEDULE):
        lb.step(n, _mods(W, H, 5, r) if edit else [])
    assert np.array_equal(lb.grid, want)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, world, port, yaml_text, q):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "MASTER_ADDR": "127.0.0.1",
                       "MASTER_PORT": str(port)})
    import torch.distributed as dist
    from oracle.build import Port
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        P = Port(yaml_text)
        W, H = 72, 90
        g0 = wl.iid_fill(W, H, 7, *wl.FOUR_FILL)
        db = B.DistributedBand(None, W, H, 6, dist, device="cpu",
                               make=lambda r0, n, h: PortBand(P, W, H, r0, n, h))
        db.set_world(g0)
        db.frame = 9
        for r, (n, edit) in enumerate(SCHEDULE):
            db.step(n, _mods(W, H, 5, r) if edit else [])
        full = db.gather()
        if rank == 0:
            q.put(("grid", np.array_equal(full, _reference(P, g0, 9, W, H))))
        q.put(("ok", rank))
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("world", [2, 3])
def test_distributed_bands_gloo(rulesets, ports, world):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, world, port, rulesets["four_materials"], q)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=240)
    assert all(p.exitcode == 0 for p in procs)
    got = [q.get(timeout=10) for _ in range(world + 1)]
    assert ("grid", True) in got
    assert sorted(r for k, r in got if k == "ok") == list(range(world))
