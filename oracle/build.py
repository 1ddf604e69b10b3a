"""Builds and loads the CPU oracle.  TEST INFRASTRUCTURE ONLY.

* ``Port(yaml_text)``: oracle/port.cpp + the GLSL the oracle front end emits for the rule
  set (rewritten by glsl2cpp) -> ``oracle/_build/port_<hash>/port.so``.  Needs only the
  files in this repository, so it builds on any machine with g++ (also the GPU machine).
* ``Ref(yaml_text)``: the reference's own shaders/compute/falling_sand.glsl, flattened
  with the reference's include rule from the reference tree, rewritten by glsl2cpp and
  driven by oracle/ref_driver.cpp -> ``oracle/_ref/<hash>/ref.so``.  The translation step
  reads the reference checkout named by the ``SANDENGINE_REF`` environment variable and
  writes the generated source into oracle/_ref/; where no checkout is named but that
  generated source exists, it is compiled from there.

Compiler flags: ``-O2 -ffp-contract=off`` (no FMA contraction, no fast-math) so binary32
arithmetic matches the fixed IEEE semantics; OpenMP for the multi-core CPU baseline.
Symbols are hidden and bound locally (``-fvisibility=hidden -Wl,-Bsymbolic``): the shader's
globals (``time``, ``frame``, ...) must not bind to libc's functions of the same name.
"""
from __future__ import annotations

import ctypes
import hashlib
import os
import subprocess
from typing import Optional

import numpy as np

from . import frontend as fe
from .glsl2cpp import fragment_to_cpp, glsl_to_cpp

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
REF_OUT = os.path.join(HERE, "_ref")
CXXFLAGS = ["-std=c++20", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-fopenmp", "-w",
            "-fvisibility=hidden", "-Wl,-Bsymbolic"]


def reference_root() -> Optional[str]:
    """The reference checkout named by SANDENGINE_REF (None when unset or not a checkout)."""
    r = os.environ.get("SANDENGINE_REF")
    return r if r and os.path.isdir(os.path.join(r, "shaders", "compute")) else None


def _digest(*parts: str) -> str:
    h = hashlib.sha256()
    for p in parts:
        h.update(p.encode())
        h.update(b"\0")
    return h.hexdigest()[:16]


def _read(p: str) -> str:
    with open(p) as f:
        return f.read()


def _write_if_changed(path: str, text: str) -> None:
    if os.path.exists(path) and _read(path) == text:
        return
    with open(path, "w") as f:
        f.write(text)


def _compile(srcs, out, incs) -> None:
    tmp = out + f".tmp{os.getpid()}"
    cmd = ["g++", *CXXFLAGS, *[f"-I{i}" for i in incs], *srcs, "-o", tmp]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed: {' '.join(cmd)}\n{r.stderr[-4000:]}")
    os.replace(tmp, out)


def build_port(yaml_text: str) -> str:
    res = fe.parse_string(yaml_text)
    mat, rules = fe.create_glsl(res)
    srcs = [_read(os.path.join(HERE, f)) for f in ("port.cpp", "glsl_shim.hpp", "glsl2cpp.py")]
    d = os.path.join(BUILD, "port_" + _digest(mat, rules, *srcs))
    so = os.path.join(d, "port.so")
    if not os.path.exists(so):
        os.makedirs(d, exist_ok=True)
        _write_if_changed(os.path.join(d, "gen_materials.inc"), glsl_to_cpp(mat))
        _write_if_changed(os.path.join(d, "gen_rules.inc"), glsl_to_cpp(rules))
        _compile([os.path.join(HERE, "port.cpp")], so, [d, HERE])
    return so


def reference_shader_text(yaml_text: str, ref: str) -> str:
    """The flattened compute shader the reference would build for this rule set."""
    res = fe.parse_string(yaml_text)
    mat, rules = fe.create_glsl(res)
    cdir = os.path.join(ref, "shaders", "compute")

    def read_include(p: str):
        if p == "gen/materials.glsl":
            return mat
        if p == "gen/rules.glsl":
            return rules
        try:
            return _read(os.path.join(cdir, p))
        except OSError:
            return None

    return fe.flatten_includes(_read(os.path.join(cdir, "falling_sand.glsl")), read_include)


def build_ref(yaml_text: str) -> str:
    srcs = [_read(os.path.join(HERE, f)) for f in ("ref_driver.cpp", "glsl_shim.hpp", "glsl2cpp.py")]
    ref = reference_root()
    key = _digest(yaml_text, *srcs)
    d = os.path.join(REF_OUT, key)
    inc = os.path.join(d, "ref_shader.inc")
    so = os.path.join(d, "ref.so")
    if os.path.exists(so):
        return so
    os.makedirs(d, exist_ok=True)
    if ref is not None:
        _write_if_changed(inc, glsl_to_cpp(reference_shader_text(yaml_text, ref)))
    elif not os.path.exists(inc):
        raise FileNotFoundError("no reference checkout and no generated reference source")
    _compile([os.path.join(HERE, "ref_driver.cpp")], so, [d, HERE])
    return so


def build_ref_frag() -> str:
    """The reference's shaders/fragment140.glsl (fragment_to_cpp) driven by
    oracle/frag_driver.cpp -> ``oracle/_ref/frag_<hash>/ref_frag.so``."""
    srcs = [_read(os.path.join(HERE, f)) for f in ("frag_driver.cpp", "glsl_shim.hpp", "glsl2cpp.py")]
    ref = reference_root()
    d = os.path.join(REF_OUT, "frag_" + _digest(*srcs))
    inc = os.path.join(d, "ref_frag.inc")
    so = os.path.join(d, "ref_frag.so")
    if os.path.exists(so):
        return so
    os.makedirs(d, exist_ok=True)
    if ref is not None:
        _write_if_changed(inc, fragment_to_cpp(_read(os.path.join(ref, "shaders", "fragment140.glsl"))))
    elif not os.path.exists(inc):
        raise FileNotFoundError("no reference checkout and no generated reference source")
    _compile([os.path.join(HERE, "frag_driver.cpp")], so, [d, HERE])
    return so


MOD_DTYPE = np.dtype([("px", "<i4"), ("py", "<i4"), ("shape", "<i4"), ("size", "<i4"),
                      ("mat", "<i4"), ("pad", "<i4", (3,))])


def mods_array(mods) -> np.ndarray:
    """(x, y, shape, size, mat) tuples -> 32-byte SimModification records."""
    a = np.zeros(len(mods), dtype=MOD_DTYPE)
    for i, m in enumerate(mods):
        a[i]["px"], a[i]["py"], a[i]["shape"], a[i]["size"], a[i]["mat"] = m
    return a


class Port:
    """The oracle port for one rule set."""

    def __init__(self, yaml_text: str):
        self.lib = ctypes.CDLL(build_port(yaml_text))
        self.lib.port_step.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                       ctypes.c_void_p, ctypes.c_int, ctypes.c_int]
        self.lib.port_run.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                      ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_int]
        self.lib.port_hash43.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p]
        self.lib.port_sin.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
        self.lib.port_color.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p]
        self.lib.port_light.argtypes = [ctypes.c_void_p] * 4 + [ctypes.c_int, ctypes.c_int]
        self.lib.port_mip_level.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p]
        self.lib.port_composite.argtypes = [ctypes.c_void_p] * 3 + [ctypes.c_int] + [ctypes.c_void_p] * 2 + \
            [ctypes.c_int, ctypes.c_int] + [ctypes.c_void_p] * 2
        self.num_materials = self.lib.port_num_materials()

    def color(self, grid: np.ndarray) -> np.ndarray:
        """output_color of a grid: (H, W, 4) float32 RGBA."""
        g = np.ascontiguousarray(grid, dtype=np.uint32)
        out = np.empty(g.shape + (4,), dtype=np.float32)
        self.lib.port_color(g.ctypes.data, g.shape[1], g.shape[0], out.ctypes.data)
        return out

    def mips(self, color: np.ndarray):
        """The box-filter pyramid of an (H, W, 4) float32 field, level 0 first."""
        levels = [np.ascontiguousarray(color, dtype=np.float32)]
        while levels[-1].shape[0] > 1 or levels[-1].shape[1] > 1:
            h, w = levels[-1].shape[:2]
            nxt = np.empty((max(1, h // 2), max(1, w // 2), 4), dtype=np.float32)
            self.lib.port_mip_level(levels[-1].ctypes.data, w, h, nxt.ctypes.data)
            levels.append(nxt)
        return levels

    # exp(-gamma) for gamma 0.5, 0.35, 0.2, rounded to binary32 (the library's constants)
    BLUR_SIDE = np.array([0.606530666, 0.704688072, 0.818730772], dtype=np.float32)

    def composite(self, color: np.ndarray, light=None, background=None) -> np.ndarray:
        """fragment140.glsl over a colour field (and its pyramid), an optional light field and
        an optional background image: (H, W, 4) float32."""
        levels = self.mips(color)
        ptrs = (ctypes.c_void_p * len(levels))(*[lv.ctypes.data for lv in levels])
        lw = (ctypes.c_int * len(levels))(*[lv.shape[1] for lv in levels])
        lh = (ctypes.c_int * len(levels))(*[lv.shape[0] for lv in levels])
        li = None if light is None else np.ascontiguousarray(light, dtype=np.float32)
        bg = None if background is None else np.ascontiguousarray(background, dtype=np.float32)
        out = np.empty(levels[0].shape, dtype=np.float32)
        self.lib.port_composite(ptrs, lw, lh, len(levels), None if li is None else li.ctypes.data,
                                None if bg is None else bg.ctypes.data, 0 if bg is None else bg.shape[1],
                                0 if bg is None else bg.shape[0], self.BLUR_SIDE.ctypes.data, out.ctypes.data)
        return out

    def light(self, old: np.ndarray, new: np.ndarray, light_in: np.ndarray) -> np.ndarray:
        """output_light of the frame that took ``old`` to ``new``, from the previous light
        field ``light_in``: (H, W, 4) float32."""
        o = np.ascontiguousarray(old, dtype=np.uint32)
        n = np.ascontiguousarray(new, dtype=np.uint32)
        li = np.ascontiguousarray(light_in, dtype=np.float32)
        out = np.empty(o.shape + (4,), dtype=np.float32)
        self.lib.port_light(o.ctypes.data, n.ctypes.data, li.ctypes.data, out.ctypes.data, o.shape[1], o.shape[0])
        return out

    def step(self, grid: np.ndarray, frame: int, mods=None, nthreads: int = 1) -> None:
        """In place: one frame with counter value ``frame``."""
        assert grid.dtype == np.uint32 and grid.flags.c_contiguous and grid.ndim == 2
        m = mods_array(mods or [])
        self.lib.port_step(grid.ctypes.data, grid.shape[1], grid.shape[0], frame,
                           m.ctypes.data if len(m) else None, len(m), nthreads)

    def run(self, grid: np.ndarray, frame0: int, nframes: int, mods=None, nthreads: int = 1) -> None:
        assert grid.dtype == np.uint32 and grid.flags.c_contiguous and grid.ndim == 2
        m = mods_array(mods or [])
        self.lib.port_run(grid.ctypes.data, grid.shape[1], grid.shape[0], frame0, nframes,
                          m.ctypes.data if len(m) else None, len(m), nthreads)

    def sin(self, x: np.ndarray) -> np.ndarray:
        """sin of binary32 arguments as the oracle (and the GPU colour pass) evaluates it."""
        a = np.ascontiguousarray(x, dtype=np.float32)
        out = np.empty_like(a)
        self.lib.port_sin(a.ctypes.data, out.ctypes.data, a.size)
        return out

    def hash43(self, x: int, y: int, frame: int) -> np.ndarray:
        out = np.zeros(4, dtype=np.float32)
        self.lib.port_hash43(x, y, frame, out.ctypes.data)
        return out


class Ref:
    """The reference's compute shader, run on the CPU, for one rule set."""

    def __init__(self, yaml_text: str):
        self.lib = ctypes.CDLL(build_ref(yaml_text))
        self.lib.ref_dispatch.argtypes = [ctypes.c_void_p] * 5 + [ctypes.c_int] * 3 + \
            [ctypes.c_void_p, ctypes.c_int, ctypes.c_int]
        self.lib.ref_dispatch_rows.argtypes = [ctypes.c_void_p] * 5 + [ctypes.c_int] * 3 + \
            [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int]

    def time_rows(self, grid: np.ndarray, frame: int, y0: int, y1: int, nthreads: int) -> float:
        """Seconds for the invocations of rows [y0, y1) of one dispatch over ``grid``."""
        import time
        H, W = grid.shape
        tex_in = np.zeros((H, W, 4), dtype=np.float32)
        tex_in[..., 0] = np.minimum(grid, (1 << 24) - 1).astype(np.float32)
        out = np.zeros_like(tex_in)
        light_in = np.zeros_like(tex_in)
        light_out = np.zeros_like(tex_in)
        color = np.zeros_like(tex_in)
        t = time.perf_counter()
        self.lib.ref_dispatch_rows(tex_in.ctypes.data, out.ctypes.data, color.ctypes.data,
                                   light_in.ctypes.data, light_out.ctypes.data, W, H, frame, None, 0,
                                   nthreads, y0, y1)
        return time.perf_counter() - t

    def run_timed(self, grid: np.ndarray, frame0: int, nframes: int, mods=None, nthreads: int = 1):
        """``nframes`` dispatches with counters frame0 + 1 .. (mods on the first), the data and
        light textures ping-ponged as the reference's Simulation::run does; returns the new
        grid and the seconds spent in the dispatches alone."""
        import time
        H, W = grid.shape
        g = grid.astype(np.int64)
        tex = [np.zeros((H, W, 4), dtype=np.float32) for _ in range(2)]
        tex[0][..., 0] = np.where(g < (1 << 24), g, (1 << 24) - 1).astype(np.float32)
        light = [np.zeros((H, W, 4), dtype=np.float32) for _ in range(2)]
        color = np.zeros((H, W, 4), dtype=np.float32)
        m = mods_array(mods or [])
        secs = 0.0
        for i in range(nframes):
            a, b = i & 1, (i + 1) & 1
            t = time.perf_counter()
            self.lib.ref_dispatch(tex[a].ctypes.data, tex[b].ctypes.data, color.ctypes.data, light[a].ctypes.data,
                                  light[b].ctypes.data, W, H, frame0 + 1 + i,
                                  m.ctypes.data if (i == 0 and len(m)) else None, len(m) if i == 0 else 0, nthreads)
            secs += time.perf_counter() - t
        return tex[nframes & 1][..., 0].astype(np.int64).astype(np.uint32), secs

    def step(self, grid: np.ndarray, frame: int, mods=None, nthreads: int = 1,
             light: Optional[np.ndarray] = None, color: Optional[np.ndarray] = None) -> np.ndarray:
        """One dispatch with counter value ``frame``; returns the new grid (ids as uint32).
        ``light`` (H, W, 4) float32 is advanced in place when given; ``color`` receives the
        colour output."""
        H, W = grid.shape
        tex_in = np.zeros((H, W, 4), dtype=np.float32)
        g = grid.astype(np.int64)
        tex_in[..., 0] = np.where(g < (1 << 24), g, (1 << 24) - 1).astype(np.float32)
        tex_out = np.zeros_like(tex_in)
        lin = light if light is not None else np.zeros_like(tex_in)
        lout = np.zeros_like(tex_in)
        col = color if color is not None else np.zeros_like(tex_in)
        m = mods_array(mods or [])
        self.lib.ref_dispatch(tex_in.ctypes.data, tex_out.ctypes.data, col.ctypes.data,
                              lin.ctypes.data, lout.ctypes.data, W, H, frame,
                              m.ctypes.data if len(m) else None, len(m), nthreads)
        if light is not None:
            light[...] = lout
        return tex_out[..., 0].astype(np.int64).astype(np.uint32)


class RefFrag:
    """The reference's fragment shader (the composite of colour, light and background), run
    on the CPU one pixel at a time with the samplers oracle/frag_driver.cpp fixes."""

    def __init__(self):
        self.lib = ctypes.CDLL(build_ref_frag())
        self.lib.ref_frag_composite.argtypes = [ctypes.c_void_p] * 3 + [ctypes.c_int] + [ctypes.c_void_p] * 2 + \
            [ctypes.c_int, ctypes.c_int, ctypes.c_void_p]

    def composite(self, levels, light=None, background=None) -> np.ndarray:
        """levels: the colour field's pyramid, level 0 first (Port.mips); light: (H, W, 4)
        float32 or None; background: (bh, bw, 4) float32 or None.  Returns (H, W, 4)."""
        levels = [np.ascontiguousarray(lv, dtype=np.float32) for lv in levels]
        ptrs = (ctypes.c_void_p * len(levels))(*[lv.ctypes.data for lv in levels])
        lw = (ctypes.c_int * len(levels))(*[lv.shape[1] for lv in levels])
        lh = (ctypes.c_int * len(levels))(*[lv.shape[0] for lv in levels])
        li = None if light is None else np.ascontiguousarray(light, dtype=np.float32)
        bg = None if background is None else np.ascontiguousarray(background, dtype=np.float32)
        out = np.empty(levels[0].shape, dtype=np.float32)
        self.lib.ref_frag_composite(ptrs, lw, lh, len(levels), None if li is None else li.ctypes.data,
                                    None if bg is None else bg.ctypes.data, 0 if bg is None else bg.shape[1],
                                    0 if bg is None else bg.shape[0], out.ctypes.data)
        return out
