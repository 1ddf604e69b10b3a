"""The product's C++ rule compiler (through the C ABI) against the oracle front end:
byte-identical GLSL, the same error kinds, and CUDA back-end behaviour."""
import re

import numpy as np
import pytest

from oracle import frontend as fe
from tests.golden.yaml_corpus import CORPUS


def _oracle(text):
    try:
        m, r = fe.create_glsl(fe.parse_string(text))
        return ("ok", m, r)
    except fe.ParseError as e:
        return ("err", e.kind, str(e))


@pytest.mark.parametrize("name", sorted(CORPUS))
def test_corpus_matches_oracle(se, name):
    text = CORPUS[name]
    want = _oracle(text)
    try:
        rs = se.parse_string(text)
        got = ("ok", rs.materials_glsl, rs.rules_glsl)
    except se.ParseError as e:
        got = ("err", e.kind, str(e))
    assert got[0] == want[0], (got, want)
    if want[0] == "ok":
        assert got[1] == want[1]
        assert got[2] == want[2]
    else:
        assert got[1] == want[1]
        if want[1] != "Yaml":  # YAML syntax errors carry the YAML reader's own wording
            assert want[2] in got[2]  # same message text (the product prefixes its status)


@pytest.mark.parametrize("name", ["reference", "four_materials", "twelve_materials"])
def test_bundled_rulesets_match_oracle_and_compile(se, rulesets, name):
    rs = se.parse_string(rulesets[name])
    m, r = fe.create_glsl(fe.parse_string(rulesets[name]))
    assert rs.materials_glsl == m and rs.rules_glsl == r
    rs.compile()  # NVRTC, sm_103a; needs no GPU
    assert "se_gen" in rs.cuda_source


@pytest.mark.parametrize("name, kind", [
    ("double_material_capture", "Glsl"),      # `sand` replaced twice -> MAT_MAT_sand
    ("do_number", "Glsl"),                    # condition `x` is undeclared
    ("type_named_empty", "Glsl"),             # TYPE_EMPTY defined twice
])
def test_shader_build_failures_surface_at_compile(se, name, kind):
    rs = se.parse_string(CORPUS[name])  # parses, as in the reference
    with pytest.raises(se.ParseError) as e:
        rs.compile()
    assert e.value.kind == kind


@pytest.mark.parametrize("cond, kind", [
    ("SELF.pos.x > 3", "Unsupported"),
    ("getCell(pos).mat == sand", "Unsupported"),
    ("moveRight", "Unsupported"),
    ("SELF.mat.density > 1 and UP.y < 0", "Unsupported"),  # the shader's UP macro
    ("SELF.mat.density > 1 and UPLEFT.y < 0", "Glsl"),     # LEFT -> left: 'UPleft' is undeclared
    ("left.mat == sand", "Glsl"),
    ("SELF.mat.density", "Glsl"),
    ("SELF.mat.densty < 1.0", "Glsl"),
])
def test_codegen_rejects(se, cond, kind):
    text = CORPUS["precondition_false_and_right"].replace("DOWN.mat.density < SELF.mat.density", cond)
    rs = se.parse_string(text)
    with pytest.raises(se.ParseError) as e:
        rs.compile()
    assert e.value.kind == kind


def test_rand_thresholds_are_exact(se):
    """`rand.y <= p` becomes `h1 < T`; check T against binary32 rounding for several p."""
    text = CORPUS["precondition_false_and_right"]
    for p in ("0.1", "0.004", "0.3", "0.0000001", "0.999", "1e-9"):
        rs = se.parse_string(text.replace("    mirrored: false", f"    probability: {p}\n    mirrored: false"))
        src = rs.cuda_source
        m = re.search(r"\(h1 < (0x[0-9a-f]+)u\)", src)
        pf = np.float32(float(p))
        if m is None:
            assert "false" in src or "true" in src
            continue
        T = int(m.group(1), 16)

        def g(u):
            return np.float32(np.float32(u) * np.float32(2.0 ** -32))
        assert g(T - 1) <= pf and not (g(T) <= pf)


def test_parse_path_and_create_glsl(se, tmp_path, rulesets):
    p = tmp_path / "materials.yaml"
    p.write_text(rulesets["reference"])
    rs = se.parse_path(str(p))
    se.create_glsl_from_parser(rs, str(tmp_path))
    m, r = fe.create_glsl(fe.parse_string(rulesets["reference"]))
    assert (tmp_path / "shaders" / "compute" / "gen" / "materials.glsl").read_text() == m
    assert (tmp_path / "shaders" / "compute" / "gen" / "rules.glsl").read_text() == r
