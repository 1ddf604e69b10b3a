"""Many independent worlds advanced together (no counterpart in the reference).

    b = Batch(ruleset, [(w0, h0), (w1, h1), ...])
    b.set_grid(i, cells); b.set_frame(i, f)
    b.step(100)          # every world 100 frames: one CUDA graph launch
    b.step_plain(100)    # the same with one launch per world per frame (the reference's way)
"""
from __future__ import annotations

import ctypes
from typing import Sequence, Tuple

import numpy as np

from ._lib import check, lib
from .lang import Ruleset


class Batch:
    def __init__(self, ruleset: Ruleset, sizes: Sequence[Tuple[int, int]]):
        self.ruleset = ruleset
        self.sizes = [(int(w), int(h)) for w, h in sizes]
        n = len(self.sizes)
        ws = (ctypes.c_int * n)(*[w for w, _ in self.sizes])
        hs = (ctypes.c_int * n)(*[h for _, h in self.sizes])
        h = ctypes.c_void_p()
        check(lib().se_batch_create(ruleset.handle, n, ws, hs, ctypes.byref(h)))
        self._h = h

    def __del__(self):
        h, self._h = getattr(self, "_h", None), None
        if h:
            lib().se_batch_destroy(h)

    def __len__(self) -> int:
        return len(self.sizes)

    def set_grid(self, i: int, cells: np.ndarray) -> None:
        w, h = self.sizes[i]
        a = np.ascontiguousarray(cells, dtype=np.uint32)
        if a.shape != (h, w):
            raise ValueError(f"world {i}: grid must have shape {(h, w)}")
        check(lib().se_batch_set_grid(self._h, i, a.ctypes.data, a.size))

    def grid(self, i: int) -> np.ndarray:
        w, h = self.sizes[i]
        out = np.empty((h, w), dtype=np.uint32)
        check(lib().se_batch_get_grid(self._h, i, out.ctypes.data, out.size))
        return out

    def set_frame(self, i: int, frame: int) -> None:
        check(lib().se_batch_set_frame(self._h, i, int(frame)))

    def frame(self, i: int) -> int:
        f = ctypes.c_int32()
        check(lib().se_batch_get_frame(self._h, i, ctypes.byref(f)))
        return f.value

    def step(self, nframes: int) -> None:
        check(lib().se_batch_step(self._h, int(nframes)))

    def step_plain(self, nframes: int) -> None:
        check(lib().se_batch_step_plain(self._h, int(nframes)))

    def autotune(self, reps: int = 2) -> int:
        k = ctypes.c_int()
        check(lib().se_batch_autotune(self._h, int(reps), ctypes.byref(k)))
        return k.value

    def set_steps_per_launch(self, k: int) -> None:
        check(lib().se_batch_set_steps_per_launch(self._h, int(k)))

    def set_resident_limit(self, nbytes: int) -> None:
        """Keep worlds needing at most ``nbytes`` of shared memory resident (0: none)."""
        check(lib().se_batch_set_resident_limit(self._h, int(nbytes)))

    def synchronize(self) -> None:
        check(lib().se_batch_synchronize(self._h))

    @property
    def stream(self) -> int:
        s = ctypes.c_void_p()
        check(lib().se_batch_get_stream(self._h, ctypes.byref(s)))
        return s.value or 0

    def info(self) -> dict:
        r, t, c, k = ctypes.c_int(), ctypes.c_int(), ctypes.c_longlong(), ctypes.c_int()
        check(lib().se_batch_info(self._h, ctypes.byref(r), ctypes.byref(t), ctypes.byref(c), ctypes.byref(k)))
        return {"resident_worlds": r.value, "tiled_worlds": t.value, "cells": c.value, "steps_per_launch": k.value}
