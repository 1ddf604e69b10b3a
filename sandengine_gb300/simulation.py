"""One simulated world, mirroring sandengine-core's ``Simulation``
(sandengine-core/src/simulation.rs:97-253).

    sim = Simulation(ruleset, (width, height))     # Simulation::new, all EMPTY, frame 0
    sim.modifications.append(SimModification(...))
    sim.run()                                      # Simulation::run: frame += 1, one step,
                                                   #   mods applied, list cleared
    sim.params.frame                               # Params.frame

Extensions over the reference: ``run_frames(n, mods)`` advances n frames in one call
(fused launches), ``grid`` reads/writes the cells as a numpy array, and ``digest()`` /
``histogram()`` check a world on the device.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass, field
from typing import List, Optional, Sequence, Tuple

import numpy as np

from ._lib import SeModification, check, lib
from .lang import Ruleset

MODSHAPE_CIRCLE = 0  # simulation.rs:41
MODSHAPE_SQUARE = 1  # simulation.rs:42
MAX_MODIFICATIONS = 256  # simulation.rs:43


@dataclass
class SimModification:
    """simulation.rs:45-56 (the padding is implicit)."""
    position: Tuple[int, int] = (0, 0)
    mod_shape: int = MODSHAPE_CIRCLE
    mod_size: int = 0
    mod_matID: int = 0


def mods_to_c(mods: Sequence[SimModification]):
    arr = (SeModification * max(1, len(mods)))()
    for i, m in enumerate(mods):
        arr[i].position[0], arr[i].position[1] = int(m.position[0]), int(m.position[1])
        arr[i].mod_shape, arr[i].mod_size, arr[i].mod_matID = int(m.mod_shape), int(m.mod_size), int(m.mod_matID)
    return arr


class Params:
    """The part of simulation.rs:67-79 that drives the grid: the frame counter."""

    def __init__(self, sim: "Simulation"):
        self._sim = sim

    @property
    def frame(self) -> int:
        f = ctypes.c_int32(0)
        check(lib().se_world_get_frame(self._sim._h, ctypes.byref(f)))
        return f.value

    @frame.setter
    def frame(self, value: int) -> None:
        check(lib().se_world_set_frame(self._sim._h, int(value)))


class Simulation:
    def __init__(self, ruleset: Ruleset, size: Tuple[int, int], steps_per_launch: int = 0):
        self.ruleset = ruleset
        self.size = (int(size[0]), int(size[1]))
        h = ctypes.c_void_p()
        check(lib().se_world_create(ruleset.handle, self.size[0], self.size[1], ctypes.byref(h)))
        self._h = h
        self.params = Params(self)
        self.modifications: List[SimModification] = []
        if steps_per_launch:
            self.set_steps_per_launch(steps_per_launch)

    def __del__(self):
        h, self._h = getattr(self, "_h", None), None
        if h:
            lib().se_world_destroy(h)

    @property
    def handle(self) -> ctypes.c_void_p:
        return self._h

    def set_steps_per_launch(self, k: int) -> None:
        check(lib().se_world_set_steps_per_launch(self._h, int(k)))

    @property
    def stream(self) -> int:
        s = ctypes.c_void_p()
        check(lib().se_world_get_stream(self._h, ctypes.byref(s)))
        return s.value or 0

    def set_stream(self, stream_ptr: Optional[int]) -> None:
        check(lib().se_world_set_stream(self._h, ctypes.c_void_p(stream_ptr or 0)))

    def run(self) -> None:
        """Simulation::run (simulation.rs:195-253)."""
        self.run_frames(1, self.modifications)
        self.modifications.clear()

    def run_frames(self, nframes: int, mods: Sequence[SimModification] = ()) -> None:
        """Advance ``nframes`` frames; ``mods`` apply to the first one."""
        arr = mods_to_c(mods)
        check(lib().se_world_step(self._h, int(nframes), arr if len(mods) else None, len(mods)))

    def synchronize(self) -> None:
        check(lib().se_world_synchronize(self._h))

    @property
    def grid(self) -> np.ndarray:
        w, h = self.size
        out = np.empty((h, w), dtype=np.uint32)
        check(lib().se_world_get_grid(self._h, out.ctypes.data, out.size))
        return out

    @grid.setter
    def grid(self, cells: np.ndarray) -> None:
        w, h = self.size
        a = np.ascontiguousarray(cells, dtype=np.uint32)
        if a.shape != (h, w):
            raise ValueError(f"grid must have shape {(h, w)}, got {a.shape}")
        check(lib().se_world_set_grid(self._h, a.ctypes.data, a.size))

    def read_grid_overlapped(self, out: np.ndarray) -> None:
        """Start copying the current grid into ``out`` ((H, W) uint32, ideally pinned) without
        holding back the next frames; ``out`` is filled once synchronize() returns."""
        w, h = self.size
        assert out.shape == (h, w) and out.dtype == np.uint32 and out.flags.c_contiguous
        check(lib().se_world_read_grid_overlapped(self._h, out.ctypes.data, out.size))

    def read_grid_u8_overlapped(self, out: np.ndarray) -> None:
        """read_grid_overlapped with the ids packed into bytes ((H, W) uint8); ids that name
        no material read as NULL (1)."""
        w, h = self.size
        assert out.shape == (h, w) and out.dtype == np.uint8 and out.flags.c_contiguous
        check(lib().se_world_read_grid_u8_overlapped(self._h, out.ctypes.data, out.size))

    def device_grid_ptr(self) -> int:
        p = ctypes.c_void_p()
        check(lib().se_world_device_grid(self._h, ctypes.byref(p)))
        return p.value or 0

    def save(self, path: str) -> None:
        """Write the world's grid and frame counter to a snapshot file."""
        check(lib().se_world_save(self._h, os.fspath(path).encode()))

    def load(self, path: str) -> None:
        """Replace the grid and frame counter from a snapshot of the same size and rule set."""
        check(lib().se_world_load(self._h, os.fspath(path).encode()))

    def set_tile(self, tile_w: int, tile_h: int, k: int) -> None:
        """Use the compiled tile variant tile_w x tile_h with up to k frames per launch (an
        override of the autotuner)."""
        check(lib().se_world_set_tile(self._h, int(tile_w), int(tile_h), int(k)))

    def tile(self):
        """(tile_w, tile_h, k) of the variant multi-frame launches use."""
        a, b, c = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        check(lib().se_world_get_tile(self._h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)))
        return a.value, b.value, c.value

    def autotune(self, reps: int = 3) -> int:
        """Pick the fastest tile shape / frames per launch for this world (state unchanged);
        returns the chosen frames per launch."""
        k = ctypes.c_int(0)
        check(lib().se_world_autotune(self._h, int(reps), ctypes.byref(k)))
        return k.value

    def set_timing(self, enable: bool) -> None:
        """Bracket every tile-kernel launch with CUDA events (see read_timing)."""
        check(lib().se_world_set_timing(self._h, 1 if enable else 0))

    def peek_timing_frames(self, frames: int) -> dict:
        """Kernel time and launches of the timed tile launches of exactly `frames` frames
        since the last read_timing (synchronizes; does not reset)."""
        ms, n = ctypes.c_double(), ctypes.c_longlong()
        check(lib().se_world_peek_timing_frames(self._h, int(frames), ctypes.byref(ms), ctypes.byref(n)))
        return {"kernel_ms": ms.value, "launches": n.value}

    def read_timing(self) -> dict:
        """Kernel time, launches, cell updates and cells read by tile launches since the
        last read (synchronizes)."""
        ms, n, cf, c = ctypes.c_double(), ctypes.c_longlong(), ctypes.c_longlong(), ctypes.c_longlong()
        check(lib().se_world_read_timing(self._h, ctypes.byref(ms), ctypes.byref(n), ctypes.byref(cf),
                                         ctypes.byref(c)))
        return {"kernel_ms": ms.value, "launches": n.value, "cell_frames": cf.value, "cells": c.value}

    def set_light(self, enable: bool = True) -> None:
        """Keep the light field (Simulation::output_light): each later frame is followed by
        the light pass.  Starts at zero, as the reference's texture does."""
        check(lib().se_world_set_light(self._h, 1 if enable else 0))

    @property
    def output_light(self) -> np.ndarray:
        """The current light field, (H, W, 4) float32 RGBA."""
        w, h = self.size
        out = np.empty((h, w, 4), dtype=np.float32)
        check(lib().se_world_get_light(self._h, out.ctypes.data, out.size))
        return out

    @output_light.setter
    def output_light(self, rgba: np.ndarray) -> None:
        w, h = self.size
        a = np.ascontiguousarray(rgba, dtype=np.float32)
        if a.shape != (h, w, 4):
            raise ValueError(f"light must have shape {(h, w, 4)}")
        check(lib().se_world_set_light_field(self._h, a.ctypes.data, a.size))

    @property
    def output_color(self) -> np.ndarray:
        """Simulation::output_color of the current grid, (H, W, 4) float32 RGBA."""
        w, h = self.size
        out = np.empty((h, w, 4), dtype=np.float32)
        check(lib().se_world_render_color(self._h, out.ctypes.data, out.size))
        return out

    def composite(self, background: Optional[np.ndarray] = None) -> np.ndarray:
        """Headless composite of the current grid (fragment140.glsl): (H, W, 4) float32 RGBA,
        rows top to bottom.  ``background``: optional (bh, bw, 4) float32 image."""
        w, h = self.size
        out = np.empty((h, w, 4), dtype=np.float32)
        bg, bw, bh = None, 0, 0
        if background is not None:
            bgarr = np.ascontiguousarray(background, dtype=np.float32)
            assert bgarr.ndim == 3 and bgarr.shape[2] == 4
            bg, bh, bw = bgarr.ctypes.data, bgarr.shape[0], bgarr.shape[1]
        check(lib().se_world_composite(self._h, bg, bw, bh, out.ctypes.data, out.size))
        return out

    def composite_device(self) -> int:
        """Composite into the world's device buffer (stream-ordered); returns its address."""
        p = ctypes.c_void_p()
        check(lib().se_world_composite_device(self._h, None, 0, 0, ctypes.byref(p)))
        return p.value or 0

    def render_color_device(self) -> int:
        """Render output_color into the world's device buffer (stream-ordered); returns its
        address (RGBA32F, height x width x 4)."""
        p = ctypes.c_void_p()
        check(lib().se_world_render_color_device(self._h, ctypes.byref(p)))
        return p.value or 0

    def read_pass_timing(self, pass_: int) -> dict:
        """Kernel time, launches and cells of the light (1) or colour (2) passes since the
        last read (synchronizes)."""
        ms, n, c = ctypes.c_double(), ctypes.c_longlong(), ctypes.c_longlong()
        check(lib().se_world_read_pass_timing(self._h, int(pass_), ctypes.byref(ms), ctypes.byref(n),
                                              ctypes.byref(c)))
        return {"kernel_ms": ms.value, "launches": n.value, "cells": c.value}

    def digest(self) -> int:
        d = ctypes.c_uint64(0)
        check(lib().se_world_digest(self._h, ctypes.byref(d)))
        return d.value

    def histogram(self, nbins: Optional[int] = None) -> np.ndarray:
        n = nbins or (self.ruleset.num_materials + 1)
        out = np.zeros(n, dtype=np.uint64)
        check(lib().se_world_histogram(self._h, out.ctypes.data, n))
        return out


def snapshot_info(path: str) -> dict:
    """Size and frame counter stored in a snapshot file (no GPU needed)."""
    w, h, f = ctypes.c_int(), ctypes.c_int(), ctypes.c_int32()
    check(lib().se_snapshot_info(os.fspath(path).encode(), ctypes.byref(w), ctypes.byref(h), ctypes.byref(f)))
    return {"width": w.value, "height": h.value, "frame": f.value}


def grid_digest(grid: np.ndarray) -> int:
    """Host computation of Simulation.digest() for a (H, W) uint32 grid (in slices of 2^24
    cells, so a 2^28-cell grid needs no more than a few hundred MB of temporaries)."""
    flat = np.ascontiguousarray(grid, dtype=np.uint32).ravel()
    total = np.uint64(0)
    step = 1 << 24
    for s in range(0, flat.size, step):
        g = flat[s:s + step].astype(np.uint64)
        z = (np.arange(s, s + g.size, dtype=np.uint64) << np.uint64(32)) | g
        with np.errstate(over="ignore"):
            z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
            z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
            z = z ^ (z >> np.uint64(31))
            total = total + z.sum(dtype=np.uint64)
    return int(total)
