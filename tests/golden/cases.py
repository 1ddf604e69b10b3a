"""Seeded cases whose per-frame grid digests are pinned to the reference shader
(tests/golden/grids.json, made by make_golden.py).  Shared by the CPU oracle tests and
the GPU parity tests."""
import os
from dataclasses import dataclass
from typing import Callable, List, Optional

import numpy as np

from sandengine_gb300 import workloads as wl

HERE = os.path.dirname(os.path.abspath(__file__))


def _reference_yaml() -> str:
    with open(os.path.join(HERE, "reference_materials.yaml")) as f:
        return f.read()


@dataclass
class Case:
    name: str
    ruleset: str            # "reference" or a bundled rule-set name
    frames: int
    frame0: int             # counter before the first frame
    grid: Callable[[], np.ndarray]
    mods: Callable[[int], Optional[list]] = lambda i: None

    def ruleset_text(self) -> str:
        return _reference_yaml() if self.ruleset == "reference" else wl.ruleset_text(self.ruleset)

    def initial_grid(self) -> np.ndarray:
        return np.ascontiguousarray(self.grid(), dtype=np.uint32)

    def mods_at(self, i: int):
        return self.mods(i)


def _noisy(w, h, seed, nmat):
    """i.i.d. ids including unknown ones (>= nmat read as NULL)."""
    u = wl.uniform53(seed, 7, np.arange(w * h, dtype=np.uint64))
    ids = (u % np.uint64(nmat + 3)).astype(np.uint32)
    empty = (wl.uniform53(seed, 8, np.arange(w * h, dtype=np.uint64)) % np.uint64(10)) < np.uint64(4)
    ids[empty] = 0
    return ids.reshape(h, w)


def _ref_mods(i):
    if i % 9 == 0:
        return [(10, 5, 0, 4, 3), (40, 20, 1, 3, 5), (0, 0, 0, 2, 99), (60, 40, 0, 6, 0),
                (33, 33, 1, 0, 4), (5, 5, 0, 3, 4)]  # the size-0 entry ends the list
    if i % 9 == 4:
        return [(20, 30, 0, 7, 7), (22, 31, 1, 2, 1), (-3, 10, 1, 5, 2), (70, 47, 0, 9, 10)]
    return None


def _twelve_mods(i):
    if i % 60 == 0:
        return wl.circle_edits(96, 80, 2, i // 60, 8, [0, 3], rmin=2, rmax=12)
    return None


CASES: List[Case] = [
    Case("four_256_seed0", "four_materials", 1000, 1, lambda: wl.world_256(0)),
    Case("reference_noisy_67x45", "reference", 300, 1, lambda: _noisy(67, 45, 5, 11), _ref_mods),
    Case("twelve_patches_96x80", "twelve_materials", 300, 5,
         lambda: wl.patch_fill(96, 80, 2, *wl.twelve_fill_spec(), patch=8), _twelve_mods),
]
