"""The rule language, mirroring sandengine-lang's public API.

    parse_string(text)              sandengine-lang/src/parser.rs:93-152
    parse_path(path)                sandengine-lang/src/lib.rs:10-13
    create_glsl_from_parser(rs)     sandengine-lang/src/lib.rs:17-147

All work happens in the C++ front end of libsandengine_gb300 (YAML -> IR -> the same GLSL
text the reference writes -> CUDA device code).  Errors raise ``ParseError`` whose
``kind`` is the reference's ParsingErr kind and whose message carries its text.
"""
from __future__ import annotations

import ctypes
import os
from typing import Optional

from ._lib import ParseError, check, lib  # noqa: F401  (ParseError re-exported)


class Ruleset:
    """A parsed rule set (the reference's ParsingResult) plus its CUDA kernels."""

    def __init__(self, handle: ctypes.c_void_p):
        self._h = handle

    def __del__(self):
        h, self._h = getattr(self, "_h", None), None
        if h:
            lib().se_ruleset_free(h)

    @property
    def handle(self) -> ctypes.c_void_p:
        return self._h

    def _text(self, which: int) -> str:
        n = ctypes.c_size_t(0)
        check(lib().se_ruleset_text(self._h, which, None, 0, ctypes.byref(n)))
        buf = ctypes.create_string_buffer(n.value + 1)
        check(lib().se_ruleset_text(self._h, which, buf, n.value + 1, ctypes.byref(n)))
        return buf.raw[:n.value].decode()

    @property
    def materials_glsl(self) -> str:
        """Text of gen/materials.glsl."""
        return self._text(0)

    @property
    def rules_glsl(self) -> str:
        """Text of gen/rules.glsl."""
        return self._text(1)

    @property
    def cuda_source(self) -> str:
        """The generated CUDA rule code."""
        return self._text(2)

    @property
    def kernel_source(self) -> str:
        """The complete device source handed to NVRTC."""
        return self._text(3)

    @property
    def num_materials(self) -> int:
        n = ctypes.c_int(0)
        check(lib().se_ruleset_num_materials(self._h, ctypes.byref(n)))
        return n.value

    def material_id(self, name: str) -> int:
        i = ctypes.c_int(0)
        check(lib().se_ruleset_material_id(self._h, name.encode(), ctypes.byref(i)))
        return i.value

    def set_checked(self, enable: bool = True) -> None:
        """CHECKED build: compile this rule set's kernels with index checks (before first use)."""
        check(lib().se_ruleset_set_checked(self._h, 1 if enable else 0))

    def check_word(self, reset: bool = True) -> int:
        """Bits of the failed index checks of a CHECKED build since the last reset (0: none)."""
        w = ctypes.c_uint(0)
        check(lib().se_ruleset_check_word(self._h, ctypes.byref(w), 1 if reset else 0))
        return w.value

    def table(self):
        """(table, static_bits) as built on the current CUDA device: the block transition
        table (u16 entries) and the bitset of static keys (u32 words), or (None, None) when
        the rules take the direct path.  Needs a GPU."""
        import numpy as np
        e, w = ctypes.c_ulonglong(), ctypes.c_ulonglong()
        check(lib().se_ruleset_table(self._h, None, 0, None, 0, ctypes.byref(e), ctypes.byref(w)))
        if not e.value:
            return None, None
        t = np.empty(e.value, dtype=np.uint16)
        b = np.empty(w.value, dtype=np.uint32)
        check(lib().se_ruleset_table(self._h, t.ctypes.data, t.size, b.ctypes.data, b.size, ctypes.byref(e),
                                     ctypes.byref(w)))
        return t, b

    def compile(self) -> None:
        """NVRTC-compile the kernels for sm_103a (needs no GPU; cached on disk)."""
        check(lib().se_ruleset_compile(self._h))


def parse_string(text: str) -> Ruleset:
    h = ctypes.c_void_p()
    check(lib().se_ruleset_parse(text.encode(), ctypes.byref(h)), parse=True)
    return Ruleset(h)


def parse_path(path: str) -> Ruleset:
    h = ctypes.c_void_p()
    check(lib().se_ruleset_parse_path(os.fspath(path).encode(), ctypes.byref(h)), parse=True)
    return Ruleset(h)


def create_glsl_from_parser(result: Ruleset, root: Optional[str] = None) -> None:
    """Writes shaders/compute/gen/{materials,rules}.glsl under ``root`` (default: the
    working directory), as the reference does."""
    gen = os.path.join(root or os.getcwd(), "shaders", "compute", "gen")
    os.makedirs(gen, exist_ok=True)
    with open(os.path.join(gen, "materials.glsl"), "w") as f:
        f.write(result.materials_glsl)
    with open(os.path.join(gen, "rules.glsl"), "w") as f:
        f.write(result.rules_glsl)
