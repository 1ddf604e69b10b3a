"""Seeded synthetic inputs for the benchmark and test workloads.

The reference ships no benchmark inputs, so every workload here is synthetic and
defined by a fixed generator: splitmix64 over (seed, index), vectorised in numpy.

* ``iid_fill``       i.i.d. materials per cell (256^2 seed 0 and 4096^2 seed 1 worlds:
                     0.60 EMPTY / 0.20 sand / 0.15 water / 0.05 stone).
* ``patch_fill``     one material per 64x64 patch (16384^2 seed-2 world).
* ``circle_edits``   rounds of circle modifications (radius 8-64, uniform positions,
                     EMPTY or sand).
* ``batch_sizes``    world sides log-uniform in [lo, hi], rounded to multiples of 32.
"""
from __future__ import annotations

import os
from typing import List, Sequence, Tuple

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
RULESETS = os.path.join(HERE, "rulesets")


def ruleset_text(name: str) -> str:
    with open(os.path.join(RULESETS, name + ".yaml")) as f:
        return f.read()


def splitmix64(x: np.ndarray) -> np.ndarray:
    """splitmix64 (Steele, Lea, Flood 2014) of each uint64 in x."""
    z = np.asarray(x, dtype=np.uint64)
    with np.errstate(over="ignore"):
        z = z + np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        return z ^ (z >> np.uint64(31))


def uniform53(seed: int, stream: int, idx: np.ndarray) -> np.ndarray:
    """53-bit uniforms u in [0, 2^53) for (seed, stream, index)."""
    key = np.uint64(((seed & 0xFFFF) << 48) | ((stream & 0xFFFF) << 32))
    return splitmix64(np.asarray(idx, dtype=np.uint64) ^ key) >> np.uint64(11)


def pick(u53: np.ndarray, ids: Sequence[int], probs: Sequence[float]) -> np.ndarray:
    """Material ids by inverse CDF of integer thresholds round(cum_p * 2^53)."""
    cum = np.cumsum(np.asarray(probs, dtype=np.float64))
    thr = np.round(cum / cum[-1] * float(1 << 53)).astype(np.uint64)
    k = np.searchsorted(thr, u53, side="right")
    k = np.minimum(k, len(ids) - 1)
    return np.asarray(ids, dtype=np.uint32)[k]


def iid_fill(width: int, height: int, seed: int, ids: Sequence[int], probs: Sequence[float]) -> np.ndarray:
    u = uniform53(seed, 0, np.arange(width * height, dtype=np.uint64))
    return pick(u, ids, probs).reshape(height, width)


def patch_fill(width: int, height: int, seed: int, ids: Sequence[int], probs: Sequence[float],
               patch: int = 64) -> np.ndarray:
    px, py = (width + patch - 1) // patch, (height + patch - 1) // patch
    u = uniform53(seed, 1, np.arange(px * py, dtype=np.uint64))
    mats = pick(u, ids, probs).reshape(py, px)
    return np.ascontiguousarray(np.repeat(np.repeat(mats, patch, 0), patch, 1)[:height, :width])


def circle_edits(width: int, height: int, seed: int, round_idx: int, count: int, materials: Sequence[int],
                 rmin: int = 8, rmax: int = 64) -> List[Tuple[int, int, int, int, int]]:
    """``count`` circle mods (x, y, shape=0, radius, material) for one edit round."""
    base = np.uint64(round_idx * 4 * count) + np.arange(4 * count, dtype=np.uint64)
    u = uniform53(seed, 2, base).reshape(count, 4).astype(np.float64) / float(1 << 53)
    out = []
    for j in range(count):
        x = int(u[j, 0] * width)
        y = int(u[j, 1] * height)
        r = rmin + int(u[j, 2] * (rmax - rmin + 1))
        m = materials[int(u[j, 3] * len(materials))]
        out.append((x, y, 0, r, int(m)))
    return out


def batch_sizes(n: int, seed: int, lo: int = 64, hi: int = 1024, multiple: int = 32) -> List[Tuple[int, int]]:
    """``n`` (width, height) pairs, each side log-uniform in [lo, hi], rounded to ``multiple``."""
    u = uniform53(seed, 3, np.arange(2 * n, dtype=np.uint64)).astype(np.float64) / float(1 << 53)
    sides = np.exp(np.log(lo) + u * (np.log(hi) - np.log(lo)))
    sides = np.clip(np.round(sides / multiple) * multiple, lo, hi).astype(int)
    return [(int(sides[2 * i]), int(sides[2 * i + 1])) for i in range(n)]


# ---- the named workloads -----------------------------------------------------------------

FOUR = "four_materials"
TWELVE = "twelve_materials"
FOUR_FILL = ((0, 3, 4, 5), (0.60, 0.20, 0.15, 0.05))  # EMPTY, sand, water, stone


def world_256(seed: int = 0) -> np.ndarray:
    """256^2, four materials, i.i.d. fill (seed 0)."""
    return iid_fill(256, 256, seed, *FOUR_FILL)


def world_4096(seed: int = 1) -> np.ndarray:
    """4096^2, four materials, i.i.d. fill (seed 1)."""
    return iid_fill(4096, 4096, seed, *FOUR_FILL)


def twelve_fill_spec(num_materials: int = 15):
    """EMPTY with p=0.4, else uniform over the 12 user materials (ids 3..14)."""
    ids = [0] + list(range(3, num_materials))
    probs = [0.4] + [0.6 / (num_materials - 3)] * (num_materials - 3)
    return ids, probs


def world_16384(seed: int = 2, size: int = 16384) -> np.ndarray:
    """16384^2 (or ``size``^2), twelve materials, 64x64 patches (seed 2)."""
    return patch_fill(size, size, seed, *twelve_fill_spec())


WORLD_EDITS_PER_ROUND = 32
WORLD_FRAMES_PER_ROUND = 60


def world_edits(size: int, round_idx: int, materials: Sequence[int] = (0, 3)):
    """The edit round ``round_idx`` of the size^2 patch world: 32 circles (radius 8-64,
    uniform positions, EMPTY or sand), applied on the first frame of every 60."""
    return circle_edits(size, size, 2, round_idx, WORLD_EDITS_PER_ROUND, materials)


# ---- the serving workload ----------------------------------------------------------------

def serve_requests(rate: float, n_requests: int, seed: int = 5):
    """The serving workload: Poisson arrivals at ``rate`` req/s; each request opens a new
    session (p = 0.5) or reuses an earlier one; sides log-uniform in [128, 2048] (multiples of
    32); N ~ U[1, 600] frames; 0-8 circle edits (radius 8-64, EMPTY or sand) on the first
    frame.  Returns the session sizes and the requests (session, frames, edits, arrival ms)."""
    u = uniform53(seed, 9, np.arange(8 * n_requests, dtype=np.uint64)).astype(np.float64) / float(1 << 53)
    u = u.reshape(n_requests, 8)
    t = np.cumsum(-np.log1p(-u[:, 0]) / rate) * 1e3  # ms
    sessions, reqs = [], []
    for i in range(n_requests):
        if not sessions or u[i, 1] < 0.5:
            w = int(np.clip(np.round(np.exp(np.log(128) + u[i, 2] * np.log(16)) / 32) * 32, 128, 2048))
            h = int(np.clip(np.round(np.exp(np.log(128) + u[i, 3] * np.log(16)) / 32) * 32, 128, 2048))
            sessions.append((w, h))
            s = len(sessions) - 1
        else:
            s = int(u[i, 1] * 2 * len(sessions)) % len(sessions)
        n = 1 + int(u[i, 4] * 600)
        ne = int(u[i, 5] * 9)
        w, h = sessions[s]
        mods = circle_edits(w, h, seed, i, ne, [0, 3]) if ne else []
        reqs.append((s, n, mods, float(t[i])))
    return sessions, reqs


def serve_session_grid(width: int, height: int, index: int) -> np.ndarray:
    """The initial grid of serving session ``index`` (frame counter 1): twelve materials in
    64x64 patches, seed 3000 + index."""
    return patch_fill(width, height, 3000 + index, *twelve_fill_spec(), patch=64)
