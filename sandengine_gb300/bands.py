"""One world split into row bands (no counterpart in the reference, which runs one world on
one GPU).

The rows of a W x H world are partitioned into bands with boundaries on even rows.  Each
band is advanced by its own engine (a band world on a GPU: se_world_create_band), which
holds the band's rows plus `halo` rows of each neighbour.  A Margolus frame moves
information at most one row, so after n <= halo frames a band's own rows are exact; before
the next n frames the halo rows are refreshed from the neighbours' own rows (one exchange
step per launch group: rows [y0 - halo, y0) from the band above, [y1, y1 + halo) from the
band below).  The halo is rounded up to an even number of rows so that band buffers start
on block-row boundaries.

    LocalBands      all bands in this process (one GPU, or tests on the CPU)
    DistributedBand one band per torch.distributed rank; halo rows travel by send/recv to
                    the neighbouring ranks (NCCL with device buffers, gloo with host ones)

An engine is any object with ``row0, rows`` (its buffer, in world rows), ``frame``,
``get_rows(row, n) -> np.ndarray``, ``set_rows(row, cells)`` and ``step(nframes, mods)``;
``GpuBand`` is the CUDA one.
"""
from __future__ import annotations

import ctypes
from typing import Callable, List, Optional, Sequence, Tuple

import numpy as np

from ._lib import check, lib
from .lang import Ruleset
from .simulation import SimModification, Simulation


def even_halo(frames: int) -> int:
    """Halo rows for launch groups of `frames` frames: rounded up to an even count."""
    return max(2, (int(frames) + 1) // 2 * 2)


def band_split(height: int, nbands: int, halo: int) -> List[Tuple[int, int]]:
    """(row0, rows) of each band: boundaries on even rows, every band at least `halo` rows
    (so that a halo comes from one neighbour)."""
    if nbands < 1:
        raise ValueError("need at least one band")
    base = (height // nbands) // 2 * 2
    out, y = [], 0
    for i in range(nbands):
        rows = height - y if i == nbands - 1 else base
        out.append((y, rows))
        y += rows
    if nbands > 1 and min(r for _, r in out) < halo:
        raise ValueError(f"bands of {min(r for _, r in out)} rows are thinner than the {halo}-row halo")
    return out


class GpuBand:
    """Band engine on the current CUDA device (se_world_create_band)."""

    def __init__(self, ruleset: Ruleset, width: int, height: int, row0: int, rows: int, halo: int,
                 steps_per_launch: int = 0):
        self.width, self.height = int(width), int(height)
        h = ctypes.c_void_p()
        check(lib().se_world_create_band(ruleset.handle, self.width, self.height, int(row0), int(rows), int(halo),
                                         ctypes.byref(h)))
        self._h = h
        a, n, wh, hl = ctypes.c_int(), ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        check(lib().se_world_band_info(h, ctypes.byref(a), ctypes.byref(n), ctypes.byref(wh), ctypes.byref(hl)))
        self.row0, self.rows = a.value, n.value
        if steps_per_launch:
            check(lib().se_world_set_steps_per_launch(h, int(steps_per_launch)))

    def __del__(self):
        h, self._h = getattr(self, "_h", None), None
        if h:
            lib().se_world_destroy(h)

    @property
    def frame(self) -> int:
        f = ctypes.c_int32()
        check(lib().se_world_get_frame(self._h, ctypes.byref(f)))
        return f.value

    @frame.setter
    def frame(self, f: int) -> None:
        check(lib().se_world_set_frame(self._h, int(f)))

    def get_rows(self, row: int, n: int) -> np.ndarray:
        out = np.empty((n, self.width), dtype=np.uint32)
        check(lib().se_world_copy_rows(self._h, int(row), int(n), out.ctypes.data, 0))
        return out

    def set_rows(self, row: int, cells: np.ndarray) -> None:
        a = np.ascontiguousarray(cells, dtype=np.uint32)
        check(lib().se_world_copy_rows(self._h, int(row), a.shape[0], a.ctypes.data, 1))

    def copy_rows_device(self, row: int, n: int, ptr: int, to_world: bool) -> None:
        """Rows to / from device memory at `ptr` (e.g. a torch CUDA tensor's data_ptr())."""
        check(lib().se_world_copy_rows(self._h, int(row), int(n), ctypes.c_void_p(ptr), 1 if to_world else 0))

    def step(self, nframes: int, mods: Sequence[SimModification] = ()) -> None:
        from .simulation import mods_to_c
        arr = mods_to_c(mods)
        check(lib().se_world_step(self._h, int(nframes), arr if len(mods) else None, len(mods)))


def _groups(nframes: int, halo: int):
    while nframes > 0:
        n = min(halo, nframes)
        yield n
        nframes -= n


class LocalBands:
    """All bands of one world in this process.  ``make(row0, rows, halo)`` builds an engine
    (default: GpuBand on the current device)."""

    def __init__(self, ruleset: Optional[Ruleset], width: int, height: int, nbands: int, frames_per_exchange: int,
                 make: Optional[Callable[[int, int, int], object]] = None):
        self.width, self.height = int(width), int(height)
        self.halo = even_halo(frames_per_exchange)
        self.split = band_split(self.height, nbands, self.halo)
        if make is None:
            make = lambda r0, n, h: GpuBand(ruleset, self.width, self.height, r0, n, h)  # noqa: E731
        self.bands = [make(r0, n, self.halo) for r0, n in self.split]

    @property
    def frame(self) -> int:
        return self.bands[0].frame

    @frame.setter
    def frame(self, f: int) -> None:
        for b in self.bands:
            b.frame = f

    @property
    def grid(self) -> np.ndarray:
        return np.concatenate([b.get_rows(r0, n) for b, (r0, n) in zip(self.bands, self.split)])

    @grid.setter
    def grid(self, cells: np.ndarray) -> None:
        cells = np.ascontiguousarray(cells, dtype=np.uint32)
        for b in self.bands:
            b.set_rows(b.row0, cells[b.row0:b.row0 + b.rows])

    def exchange(self) -> None:
        """Refresh every band's halo rows from its neighbours' own rows."""
        for i, b in enumerate(self.bands):
            r0, n = self.split[i]
            if i > 0 and b.row0 < r0:  # rows above, owned by band i - 1
                b.set_rows(b.row0, self.bands[i - 1].get_rows(b.row0, r0 - b.row0))
            end = b.row0 + b.rows
            if i + 1 < len(self.bands) and end > r0 + n:  # rows below, owned by band i + 1
                b.set_rows(r0 + n, self.bands[i + 1].get_rows(r0 + n, end - r0 - n))

    def step(self, nframes: int, mods: Sequence[SimModification] = ()) -> None:
        """Advance `nframes` frames; `mods` apply to the first one (world coordinates)."""
        first = True
        for n in _groups(int(nframes), self.halo):
            self.exchange()
            for b in self.bands:
                b.step(n, mods if first else ())
            first = False


class DistributedBand:
    """This rank's band of one world; ranks 0..world_size-1 hold the bands top to bottom.
    ``comm`` is torch.distributed (initialised); ``device`` a torch device for the halo
    buffers ("cuda:i" with NCCL, "cpu" with gloo)."""

    def __init__(self, ruleset: Optional[Ruleset], width: int, height: int, frames_per_exchange: int, comm,
                 device: str = "cpu", make: Optional[Callable[[int, int, int], object]] = None):
        self.width, self.height = int(width), int(height)
        self.comm = comm
        self.rank, self.size = comm.get_rank(), comm.get_world_size()
        self.device = device
        self.halo = even_halo(frames_per_exchange)
        self.split = band_split(self.height, self.size, self.halo)
        self.own = self.split[self.rank]
        if make is None:
            make = lambda r0, n, h: GpuBand(ruleset, self.width, self.height, r0, n, h)  # noqa: E731
        self.band = make(self.own[0], self.own[1], self.halo)

    @property
    def frame(self) -> int:
        return self.band.frame

    @frame.setter
    def frame(self, f: int) -> None:
        self.band.frame = f

    def set_world(self, cells: np.ndarray) -> None:
        """Take this band's buffer rows from the whole world's grid."""
        b = self.band
        self.band.set_rows(b.row0, np.ascontiguousarray(cells[b.row0:b.row0 + b.rows], dtype=np.uint32))

    def own_rows(self) -> np.ndarray:
        return self.band.get_rows(*self.own)

    def _send_recv(self, sends, recvs) -> None:
        ops = [self.comm.P2POp(self.comm.isend, t, peer) for t, peer in sends]
        ops += [self.comm.P2POp(self.comm.irecv, t, peer) for t, peer in recvs]
        if ops:
            for r in self.comm.batch_isend_irecv(ops):
                r.wait()

    def exchange(self) -> None:
        import torch
        b, (r0, n) = self.band, self.own
        up = r0 - b.row0                      # halo rows above (from rank - 1)
        down = b.row0 + b.rows - (r0 + n)     # halo rows below (from rank + 1)
        # what the neighbours need: our top rows for rank - 1, our bottom rows for rank + 1
        need_up = 0 if self.rank == 0 else min(self.halo, r0)
        need_down = 0 if self.rank == self.size - 1 else min(self.halo, self.height - (r0 + n))
        sends, recvs, into = [], [], []
        dev = torch.device(self.device)
        if need_up:
            sends.append((self._rows_tensor(r0, need_up, dev), self.rank - 1))
        if need_down:
            sends.append((self._rows_tensor(r0 + n - need_down, need_down, dev), self.rank + 1))
        if up:
            t = torch.empty((up, self.width), dtype=torch.int32, device=dev)
            recvs.append((t, self.rank - 1))
            into.append((b.row0, t))
        if down:
            t = torch.empty((down, self.width), dtype=torch.int32, device=dev)
            recvs.append((t, self.rank + 1))
            into.append((r0 + n, t))
        self._send_recv(sends, recvs)
        if dev.type == "cuda":
            torch.cuda.synchronize(dev)
        for row, t in into:
            if dev.type == "cuda" and hasattr(b, "copy_rows_device"):
                b.copy_rows_device(row, t.shape[0], t.data_ptr(), True)
            else:
                b.set_rows(row, t.cpu().numpy().view(np.uint32))

    def _rows_tensor(self, row: int, n: int, dev):
        import torch
        b = self.band
        if dev.type == "cuda" and hasattr(b, "copy_rows_device"):
            t = torch.empty((n, self.width), dtype=torch.int32, device=dev)
            b.copy_rows_device(row, n, t.data_ptr(), False)
            return t
        return torch.from_numpy(b.get_rows(row, n).view(np.int32).copy()).to(dev)

    def step(self, nframes: int, mods: Sequence[SimModification] = ()) -> None:
        first = True
        for n in _groups(int(nframes), self.halo):
            self.exchange()
            self.band.step(n, mods if first else ())
            first = False

    def gather(self) -> Optional[np.ndarray]:
        """The whole grid on rank 0 (None elsewhere)."""
        import torch
        own = torch.from_numpy(self.own_rows().view(np.int32).copy())
        dev = torch.device(self.device)
        if self.rank == 0:
            parts = [own.numpy().view(np.uint32)]
            for r in range(1, self.size):
                t = torch.empty((self.split[r][1], self.width), dtype=torch.int32, device=dev)
                self.comm.recv(t, src=r)
                parts.append(t.cpu().numpy().view(np.uint32))
            return np.concatenate(parts)
        self.comm.send(own.to(dev), dst=0)
        return None
