"""Serving simulation sessions with continuous batching (no counterpart in the reference).

Replay (a recorded trace of requests with arrival times):

    srv = Server(ruleset, budget_bytes=150 << 30)
    s = srv.open_session(w, h, cells=None, frame=1)
    r = srv.submit(s, nframes=300, mods=[SimModification(...)], arrival_ms=12.5)
    srv.run()              # continuous batching; srv.run(plain=True): one request at a time
    srv.stats()            # p50/p99 latency, throughput, evictions

Live (requests submitted from any thread while the loop runs):

    srv.start()            # the serving loop on its own host thread
    r = srv.submit(s, 300) # arrives now; admitted at the loop's next iteration
    srv.wait(r)            # latency in ms once it has completed on the GPU
    srv.stop()
"""
from __future__ import annotations

import ctypes
from typing import Optional, Sequence

import numpy as np

from ._lib import check, lib
from .lang import Ruleset
from .simulation import SimModification, mods_to_c


class ServerStats(ctypes.Structure):
    _fields_ = [("requests", ctypes.c_longlong), ("p50_ms", ctypes.c_double), ("p99_ms", ctypes.c_double),
                ("mean_ms", ctypes.c_double), ("max_ms", ctypes.c_double), ("wall_ms", ctypes.c_double),
                ("cell_updates", ctypes.c_double), ("iterations", ctypes.c_longlong),
                ("evictions", ctypes.c_longlong), ("restores", ctypes.c_longlong),
                ("peak_resident_bytes", ctypes.c_longlong), ("restore_ms", ctypes.c_double),
                ("kernel_ms", ctypes.c_double)]


class Server:
    def __init__(self, ruleset: Ruleset, budget_bytes: int, frames_per_iteration: int = 8):
        self.ruleset = ruleset
        h = ctypes.c_void_p()
        check(lib().se_server_create(ruleset.handle, int(budget_bytes), ctypes.byref(h)))
        self._h = h
        self.sizes = []
        self.set_frames_per_iteration(frames_per_iteration)

    def __del__(self):
        h, self._h = getattr(self, "_h", None), None
        if h:
            lib().se_server_destroy(h)

    def set_frames_per_iteration(self, k: int) -> None:
        check(lib().se_server_set_frames_per_iteration(self._h, int(k)))

    def open_session(self, width: int, height: int, cells: Optional[np.ndarray] = None, frame: int = 0) -> int:
        sid = ctypes.c_int()
        ptr = None
        if cells is not None:
            cells = np.ascontiguousarray(cells, dtype=np.uint32)
            assert cells.shape == (height, width)
            ptr = cells.ctypes.data
        check(lib().se_server_open_session(self._h, int(width), int(height), ptr, int(frame), ctypes.byref(sid)))
        self.sizes.append((int(width), int(height)))
        return sid.value

    def save_session(self, session: int, path: str) -> None:
        check(lib().se_server_save_session(self._h, int(session), str(path).encode()))

    def open_session_from(self, path: str) -> int:
        from .simulation import snapshot_info
        info = snapshot_info(path)
        sid = ctypes.c_int()
        check(lib().se_server_open_session_from(self._h, str(path).encode(), ctypes.byref(sid)))
        self.sizes.append((info["width"], info["height"]))
        return sid.value

    def close_session(self, session: int) -> None:
        check(lib().se_server_close_session(self._h, int(session)))

    def submit(self, session: int, nframes: int, mods: Sequence[SimModification] = (), arrival_ms: float = 0.0) -> int:
        rid = ctypes.c_int()
        arr = mods_to_c(mods)
        check(lib().se_server_submit(self._h, int(session), int(nframes), arr if len(mods) else None, len(mods),
                                     float(arrival_ms), ctypes.byref(rid)))
        return rid.value

    def cancel(self, request: int) -> None:
        """Withdraw a request that has not been run yet."""
        check(lib().se_server_cancel(self._h, int(request)))

    def run(self, plain: bool = False) -> None:
        check(lib().se_server_run(self._h, 1 if plain else 0))

    def start(self, plain: bool = False) -> None:
        """Start the live serving loop (its own host thread)."""
        check(lib().se_server_start(self._h, 1 if plain else 0))

    def stop(self) -> None:
        """Serve what was submitted, then end the live loop."""
        check(lib().se_server_stop(self._h))

    def wait(self, request: int, timeout_ms: float = -1.0) -> float:
        """Block until the request has completed on the GPU; returns its latency in ms.
        Raises SandengineError (kind Timeout) when timeout_ms passes first."""
        v = ctypes.c_double()
        check(lib().se_server_wait(self._h, int(request), float(timeout_ms), ctypes.byref(v)))
        return v.value

    def poll(self, request: int) -> Optional[float]:
        """The request's latency in ms once it has completed, else None (does not block)."""
        d, v = ctypes.c_int(), ctypes.c_double()
        check(lib().se_server_poll(self._h, int(request), ctypes.byref(d), ctypes.byref(v)))
        return v.value if d.value else None

    def stats(self) -> dict:
        st = ServerStats()
        check(lib().se_server_stats_get(self._h, ctypes.byref(st)))
        return {name: getattr(st, name) for name, _ in ServerStats._fields_}

    def latency_ms(self, request: int) -> float:
        v = ctypes.c_double()
        check(lib().se_server_request_latency(self._h, int(request), ctypes.byref(v)))
        return v.value

    def grid(self, session: int) -> np.ndarray:
        w, h = self.sizes[session]
        out = np.empty((h, w), dtype=np.uint32)
        check(lib().se_server_get_grid(self._h, int(session), out.ctypes.data, out.size))
        return out

    def frame(self, session: int) -> int:
        f = ctypes.c_int32()
        check(lib().se_server_get_frame(self._h, int(session), ctypes.byref(f)))
        return f.value
