"""Mechanical GLSL -> C++20 rewrites so shader text compiles against oracle/glsl_shim.hpp.

TEST INFRASTRUCTURE ONLY (oracle).  Each rewrite is syntax-only; none changes what the
shader computes:

* drop ``#version`` and ``layout(...) in;`` lines, and the ``layout(...)``, ``uniform``,
  ``writeonly``/``readonly``/``volatile``/``coherent`` qualifiers;
* unwrap uniform interface blocks (``uniform Name { decls };`` -> ``decls``);
* ``inout T x`` -> ``T& x`` and ``in T x`` -> ``T x``;
* array types ``T[N] f(`` / ``T[N] x`` and declarators ``T x[N]`` -> ``garr<T,N>``;
* float literals get an ``f`` suffix so C++ parses them straight to binary32, as GLSL does
  (without it ``rand.y <= 0.1`` would compare against the double 0.1);
* the read-only swizzles ``.rgb``/``.xy`` become calls;
* a ``case`` label that jumps over ``float v = e;`` becomes ``float v; v = e;``;
* ``void main()`` is renamed ``glsl_main()``;
* struct ``Material``/``Cell``/``SimModification`` get a defaulted ``operator==`` (GLSL
  compares structs member-wise).

``fragment_to_cpp`` applies, before those, the rewrites a fragment shader needs: the
global ``in``/``out`` storage qualifiers are dropped (the driver sets the inputs and reads
the outputs as globals), and assignments to the ``.rgb`` swizzle (``v.rgb = e;``,
``v.rgb *= e;``) become ``v.set_rgb(e);`` / ``v.set_rgb(v.rgb * (e));``.
"""
from __future__ import annotations

import re

_TYPES = r"(?:float|int|uint|bool|vec[234]|ivec[234]|uvec[234]|Cell|Material|SimModification)"


def glsl_to_cpp(src: str) -> str:
    s = src
    s = re.sub(r"^\s*#version[^\n]*\n", "", s, flags=re.M)
    s = re.sub(r"^\s*layout\s*\([^)]*\)\s*in\s*;[^\n]*\n", "", s, flags=re.M)
    s = re.sub(r"\buniform\s+(\w+)\s*\{([^}]*)\}\s*;", r"\2", s)
    s = re.sub(r"layout\s*\([^)]*\)\s*", "", s)
    s = re.sub(r"\b(uniform|writeonly|readonly|volatile|coherent)\s+", "", s)
    s = re.sub(r"\binout\s+(\w+)\s+", r"\1& ", s)
    s = re.sub(r"([(,]\s*)in\s+(\w+\s+\w+)", r"\1\2", s)
    # array return types / array-typed declarations:  T[N] name
    s = re.sub(r"\b(" + _TYPES + r")\[(\d+)\]\s+(\w+)", r"garr<\1,\2> \3", s)
    # array declarators:  T name[N]
    s = re.sub(r"\b(" + _TYPES + r")\s+(\w+)\[(\d+)\]", r"garr<\1,\3> \2", s)
    # float literals -> binary32 literals
    s = re.sub(r"(?<![\w.])((?:\d+\.\d*|\.\d+)(?:[eE][-+]?\d+)?|\d+[eE][-+]?\d+)(?![\w.])",
               r"\1f", s)
    s = re.sub(r"\.(rgb|xy)\b(?!\s*\()", r".\1()", s)
    s = re.sub(r"(case\s+\w+\s*:\s*\n\s*)float\s+(\w+)\s*=", r"\1float \2; \2 =", s)
    s = re.sub(r"\bvoid\s+main\s*\(\s*\)", "void glsl_main()", s)
    for name in ("Material", "Cell", "SimModification"):
        s = re.sub(r"(struct\s+" + name + r"\s*\{)",
                   r"\1 bool operator==(const " + name + r"&) const = default;", s)
    return s


def fragment_to_cpp(src: str) -> str:
    s = re.sub(r"^(\s*)(?:in|out)\s+(?=\w+\s+\w+\s*;)", r"\1", src, flags=re.M)
    s = re.sub(r"\b(\w+)\.rgb\s*\*=\s*([^;]+);", r"\1.set_rgb(\1.rgb * (\2));", s)
    s = re.sub(r"\b(\w+)\.rgb\s*=(?!=)\s*([^;]+);", r"\1.set_rgb(\2);", s)
    return glsl_to_cpp(s)
