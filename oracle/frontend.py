"""Oracle front end: a CPU restatement of sandengine-lang (YAML rule language -> GLSL).

TEST INFRASTRUCTURE ONLY.  This module is the checker for the product's C++ rule
compiler (``sandengine_gb300/csrc/lang``).  Only ``tests/``, ``__graft_entry__.smoke()``
and ``bench.py``'s CPU-baseline leg may import it; the product path never does.

It restates, step by step, what the reference does in
  sandengine-lang/src/parser.rs        (parse_string, key checks, error kinds)
  sandengine-lang/src/parser/rules.rs  (parse_rules, parse_conditionals, parse_do,
                                        parse_global_scope, get_func_logic, get_glsl_code)
  sandengine-lang/src/parser/types.rs  (parse_types, add_child_to_type, get_parents_rules)
  sandengine-lang/src/parser/materials.rs (parse_materials)
  sandengine-lang/src/lib.rs           (create_glsl_from_parser: gen/materials.glsl, gen/rules.glsl)
  src/lib.rs:31-76                     (build_compute_shaders: the #include flattener)

The YAML reader below covers the subset of YAML 1.2 that the rule language uses
(block mappings kept in insertion order as serde_yaml 0.9.34 + indexmap do, block and
flow sequences, plain/quoted scalars with core-schema typing, comments).  serde_yaml and
the regex crate are not vendored in the reference, so their behaviour is restated from
their published semantics: Python's ``re`` gives the same leftmost-first matches as the
regex crate for the four patterns used here.

Pinned by: the reference's checked-in generated files ``shaders/compute/gen/materials.glsl``,
``gen/rules.glsl`` and ``gen/falling_sand.glsl`` for ``data/materials.yaml`` (byte-exact;
``tests/golden/make_golden.py`` records their SHA-256), and by the error kinds of the
reference's ``tests/test_sandengine-lang.rs``.
"""
from __future__ import annotations

import math
import re
from dataclasses import dataclass, field
from typing import Any, Dict, List, Optional, Tuple

import numpy as np

# --------------------------------------------------------------------------------------
# Errors (sandengine-lang/src/parser.rs:42-73).  Messages follow the thiserror formats
# with colours off (the `colored` crate emits none when stdout is not a terminal).
# --------------------------------------------------------------------------------------


class ParseError(Exception):
    """A parse failure. ``kind`` is one of MissingField, InvalidType, NotFound,
    NotRecognized, Yaml, Panic (the reference would panic / stack-overflow)."""

    def __init__(self, kind: str, message: str):
        super().__init__(message)
        self.kind = kind


def _missing_field(field_name: str, missing_in: str) -> ParseError:
    return ParseError("MissingField",
                      f"(MissingField) Mandatory field '{field_name}' is missing in '{missing_in}'")


def _invalid_type(wrong: str, missing_in: str, expected: str) -> ParseError:
    return ParseError("InvalidType",
                      f"(InvalidType) The type of the field '{wrong}' inside of '{missing_in}' "
                      f"is invalid. Expected: '{expected}'")


def _not_found(missing: str, missing_in: str) -> ParseError:
    return ParseError("NotFound",
                      f"(NotFound) The name '{missing}' (in '{missing_in}') was not found. "
                      f"Make sure it was defined before referencing it.")


def _not_recognized(unrecog: str, missing_in: str) -> ParseError:
    return ParseError("NotRecognized",
                      f"(NotRecognized) The expression '{unrecog}' (in '{missing_in}') was not "
                      f"recognized as valid syntax. Please check it is valid.")


def _wrap(prefix: str, err: ParseError) -> ParseError:
    return ParseError(err.kind, f"Error while parsing {prefix}: '{err}'")


TYPE_HINT_STRING = "string"
TYPE_HINT_BOOL = "bool (true/false)"
TYPE_HINT_FLOAT = "float (0.0 to 1.0)"
TYPE_HINT_SEQUENCE = "sequence (array, '[...]')"
TYPE_HINT_COLOR = ("sequence (array, '[...]') of 3-4 floats (range 0.0-1.0) OR integers "
                   "(range 0-255). (With 3 elements, the alpha channel defaults to 1.0)")
TYPE_HINT_MAPPING = "mapping (dictionary-like)"

GLOBAL_CELLNAMES = ["SELF", "LEFT", "RIGHT", "DOWN", "DOWNRIGHT", "DOWNLEFT"]  # parser.rs:26-33
DEFAULT_VAL_MIRRORED = True       # parser.rs:37
DEFAULT_VAL_PRECONDITION = True   # parser.rs:38
DEFAULT_VAL_PROBABILITY = np.float32(1.0)  # parser.rs:39

# --------------------------------------------------------------------------------------
# YAML subset reader
# --------------------------------------------------------------------------------------


class YamlError(Exception):
    pass


_INT_RE = re.compile(r"^[-+]?[0-9]+$")
_HEX_RE = re.compile(r"^0x[0-9a-fA-F]+$")
_OCT_RE = re.compile(r"^0o[0-7]+$")
_FLOAT_RE = re.compile(r"^[-+]?(\.[0-9]+|[0-9]+(\.[0-9]*)?)([eE][-+]?[0-9]+)?$")


def _resolve_plain(s: str) -> Any:
    """YAML 1.2 core-schema resolution of a plain scalar, as serde_yaml 0.9 does it."""
    if s in ("", "~", "null", "Null", "NULL"):
        return None
    if s in ("true", "True", "TRUE"):
        return True
    if s in ("false", "False", "FALSE"):
        return False
    if _INT_RE.match(s):
        v = int(s, 10)
        if -(1 << 63) <= v < (1 << 64):
            return v
        return float(s)
    if _HEX_RE.match(s):
        return int(s[2:], 16)
    if _OCT_RE.match(s):
        return int(s[2:], 8)
    if _FLOAT_RE.match(s):
        return float(s)
    low = s.lower()
    if low in (".inf", "+.inf"):
        return math.inf
    if low == "-.inf":
        return -math.inf
    if low == ".nan":
        return math.nan
    return s


class _Str(str):
    """A string that came from a quoted scalar (never re-typed)."""


def _strip_comment(line: str) -> str:
    out = []
    q = None
    prev = " "
    for ch in line:
        if q:
            out.append(ch)
            if ch == q:
                q = None
        else:
            if ch in ("'", '"') and (prev in " \t[{,:" or not out):
                q = ch
            elif ch == "#" and prev in " \t":
                break
            out.append(ch)
        prev = ch
    return "".join(out).rstrip()


def _unquote(tok: str) -> str:
    if tok.startswith("'"):
        if not tok.endswith("'") or len(tok) < 2:
            raise YamlError(f"unterminated quoted scalar: {tok}")
        return _Str(tok[1:-1].replace("''", "'"))
    if tok.startswith('"'):
        if not tok.endswith('"') or len(tok) < 2:
            raise YamlError(f"unterminated quoted scalar: {tok}")
        body = tok[1:-1]
        return _Str(bytes(body, "utf-8").decode("unicode_escape") if "\\" in body else body)
    raise AssertionError


def _scalar(tok: str) -> Any:
    tok = tok.strip()
    if tok[:1] in ("'", '"'):
        return _unquote(tok)
    return _resolve_plain(tok)


def _parse_flow(text: str) -> Any:
    pos = 0

    def ws():
        nonlocal pos
        while pos < len(text) and text[pos] in " \t\n":
            pos += 1

    def node():
        nonlocal pos
        ws()
        if pos >= len(text):
            raise YamlError("unexpected end of flow collection")
        c = text[pos]
        if c == "[":
            pos += 1
            items = []
            ws()
            if pos < len(text) and text[pos] == "]":
                pos += 1
                return items
            while True:
                items.append(node())
                ws()
                if pos < len(text) and text[pos] == ",":
                    pos += 1
                    ws()
                    if pos < len(text) and text[pos] == "]":
                        pos += 1
                        return items
                    continue
                if pos < len(text) and text[pos] == "]":
                    pos += 1
                    return items
                raise YamlError(f"bad flow sequence: {text!r}")
        if c == "{":
            pos += 1
            m: Dict[Any, Any] = {}
            ws()
            if pos < len(text) and text[pos] == "}":
                pos += 1
                return m
            while True:
                k = node()
                ws()
                if pos < len(text) and text[pos] == ":":
                    pos += 1
                    v = node()
                else:
                    v = None
                if k in m:
                    raise YamlError(f"duplicate entry with key {k!r}")
                m[k] = v
                ws()
                if pos < len(text) and text[pos] == ",":
                    pos += 1
                    continue
                if pos < len(text) and text[pos] == "}":
                    pos += 1
                    return m
                raise YamlError(f"bad flow mapping: {text!r}")
        if c in ("'", '"'):
            end = pos + 1
            while end < len(text):
                if text[end] == c:
                    if c == "'" and end + 1 < len(text) and text[end + 1] == "'":
                        end += 2
                        continue
                    break
                end += 1
            tok = text[pos:end + 1]
            pos = end + 1
            return _unquote(tok)
        start = pos
        while pos < len(text) and text[pos] not in ",]}":
            if text[pos] == ":" and (pos + 1 >= len(text) or text[pos + 1] in " ,]}"):
                break
            pos += 1
        return _resolve_plain(text[start:pos].strip())

    v = node()
    ws()
    if pos != len(text):
        raise YamlError(f"trailing characters after flow collection: {text!r}")
    return v


def _find_colon(s: str) -> int:
    """Index of the ':' that ends a mapping key, or -1."""
    q = None
    depth = 0
    for i, ch in enumerate(s):
        if q:
            if ch == q:
                q = None
            continue
        if ch in ("'", '"') and (i == 0 or s[i - 1] in " \t[{,"):
            q = ch
        elif ch in "[{":
            depth += 1
        elif ch in "]}":
            depth -= 1
        elif ch == ":" and depth == 0 and (i + 1 == len(s) or s[i + 1] in " \t"):
            return i
    return -1


def load_yaml(text: str) -> Any:
    raw = text.replace("\r\n", "\n").replace("\t", "    ").split("\n")
    lines: List[Tuple[int, str]] = []
    for ln in raw:
        s = _strip_comment(ln)
        if s.strip() in ("", "---"):
            lines.append((-1, ""))
            continue
        if s.strip() == "...":
            break
        ind = len(s) - len(s.lstrip(" "))
        lines.append((ind, s.strip()))
    pos = 0

    def skip_blank():
        nonlocal pos
        while pos < len(lines) and lines[pos][0] < 0:
            pos += 1

    def gather_flow(first: str) -> str:
        nonlocal pos
        buf = first
        depth = 0

        def balance(t):
            d = 0
            q = None
            for ch in t:
                if q:
                    if ch == q:
                        q = None
                elif ch in "'\"":
                    q = ch
                elif ch in "[{":
                    d += 1
                elif ch in "]}":
                    d -= 1
            return d

        depth = balance(buf)
        while depth > 0:
            if pos >= len(lines):
                raise YamlError("unterminated flow collection")
            ind, t = lines[pos]
            pos += 1
            if ind < 0:
                continue
            buf += " " + t
            depth = balance(buf)
        return buf

    def parse_value_text(t: str, parent_indent: int) -> Any:
        nonlocal pos
        if t[:1] in ("[", "{"):
            return _parse_flow(gather_flow(t))
        if t[:1] in ("|", ">"):
            raise YamlError("block scalars are not supported by this reader")
        if t[:1] in ("'", '"'):
            return _scalar(t)
        # plain scalar, possibly folded over more-indented continuation lines
        parts = [t]
        while True:
            save = pos
            skip_blank()
            if pos < len(lines) and lines[pos][0] > parent_indent and _find_colon(lines[pos][1]) < 0 \
                    and not lines[pos][1].startswith("- "):
                parts.append(lines[pos][1])
                pos += 1
                continue
            pos = save
            break
        return _resolve_plain(" ".join(parts))

    def parse_block(indent: int) -> Any:
        nonlocal pos
        skip_blank()
        if pos >= len(lines):
            return None
        ind, t = lines[pos]
        if t == "-" or t.startswith("- "):
            return parse_seq(ind)
        if _find_colon(t) >= 0:
            return parse_map(ind)
        pos += 1
        return parse_value_text(t, indent - 1)

    def parse_seq(indent: int) -> list:
        nonlocal pos
        items = []
        while True:
            skip_blank()
            if pos >= len(lines):
                break
            ind, t = lines[pos]
            if ind != indent or not (t == "-" or t.startswith("- ")):
                if ind > indent:
                    raise YamlError(f"bad indentation in sequence: {t!r}")
                break
            rest = t[1:].strip()
            pos += 1
            if rest == "":
                skip_blank()
                if pos < len(lines) and lines[pos][0] > indent:
                    items.append(parse_block(lines[pos][0]))
                else:
                    items.append(None)
            elif _find_colon(rest) >= 0 and rest[:1] not in "[{'\"":
                # "- key: value" starts a compact mapping
                sub_indent = indent + 2
                lines.insert(pos, (sub_indent, rest))
                items.append(parse_map(sub_indent))
            else:
                items.append(parse_value_text(rest, indent))
        return items

    def parse_map(indent: int) -> dict:
        nonlocal pos
        m: Dict[Any, Any] = {}
        while True:
            skip_blank()
            if pos >= len(lines):
                break
            ind, t = lines[pos]
            if ind < indent:
                break
            if ind > indent:
                raise YamlError(f"bad indentation: {t!r}")
            c = _find_colon(t)
            if c < 0:
                raise YamlError(f"could not find expected ':' in {t!r}")
            key = _scalar(t[:c]) if t[:c].strip() else None
            rest = t[c + 1:].strip()
            pos += 1
            if rest == "":
                skip_blank()
                if pos < len(lines) and lines[pos][0] > indent:
                    val = parse_block(lines[pos][0])
                elif pos < len(lines) and lines[pos][0] == indent and \
                        (lines[pos][1] == "-" or lines[pos][1].startswith("- ")):
                    val = parse_seq(indent)
                else:
                    val = None
            else:
                val = parse_value_text(rest, indent)
            if key in m:
                raise YamlError(f"duplicate entry with key {key!r}")
            m[key] = val
        return m

    skip_blank()
    if pos >= len(lines):
        return None
    doc = parse_block(lines[pos][0])
    skip_blank()
    if pos < len(lines):
        raise YamlError(f"unexpected content: {lines[pos][1]!r}")
    return doc


# serde_yaml::Value accessors -----------------------------------------------------------

def y_get(v: Any, key: str) -> Any:
    """Value::get(&str): only mappings with a string key; None (absent) otherwise."""
    if isinstance(v, dict):
        for k, val in v.items():
            if isinstance(k, str) and k == key:
                return _Present(val)
    return None


class _Present:
    __slots__ = ("v",)

    def __init__(self, v):
        self.v = v


def as_str(v: Any) -> Optional[str]:
    return str(v) if isinstance(v, str) else None


def as_bool(v: Any) -> Optional[bool]:
    return v if isinstance(v, bool) else None


def as_f64(v: Any) -> Optional[float]:
    if isinstance(v, bool) or not isinstance(v, (int, float)):
        return None
    return float(v)


def as_u64(v: Any) -> Optional[int]:
    if isinstance(v, bool) or not isinstance(v, int) or v < 0:
        return None
    return v


def as_seq(v: Any) -> Optional[list]:
    return v if isinstance(v, list) else None


def as_map(v: Any) -> Optional[dict]:
    return v if isinstance(v, dict) else None


def _debug_value(v: Any) -> str:
    """Debug rendering of a serde_yaml Value (only used inside error messages)."""
    if v is None:
        return "Null"
    if isinstance(v, bool):
        return f"Bool({str(v).lower()})"
    if isinstance(v, (int, float)):
        return f"Number({v})"
    if isinstance(v, str):
        return f"String({v!r})"
    if isinstance(v, list):
        return "Sequence"
    return "Mapping"


# --------------------------------------------------------------------------------------
# Rust f32 formatting: Display prints the shortest round-trip decimal, never exponent form.
# --------------------------------------------------------------------------------------

def f32_display(x) -> str:
    f = np.float32(x)
    if np.isnan(f):
        return "NaN"
    if np.isinf(f):
        return "inf" if f > 0 else "-inf"
    s = np.format_float_positional(f, unique=True, trim="-")
    if s in ("-0",):
        return "-0"
    return s


# --------------------------------------------------------------------------------------
# IR (rules.rs:25-44, types.rs:12-26, materials.rs:11-29)
# --------------------------------------------------------------------------------------

@dataclass
class SandRule:
    name: str
    ruletype: str  # "Mirrored" | "Left" | "Right"
    if_conds: List[str]
    do_actions: List[str]
    probabilities: List[np.float32]
    mirror: bool
    precondition: Optional[str]
    used: bool = False


@dataclass
class SandType:
    id: int
    name: str
    inherits: str = ""
    children: List[str] = field(default_factory=list)
    base_rules: List[str] = field(default_factory=list)


@dataclass
class SandMaterial:
    id: int
    name: str
    mattype: str
    color: List[np.float32]
    emission: List[np.float32]
    selectable: bool
    density: np.float32
    extra_rules: List[str] = field(default_factory=list)


@dataclass
class ParsingResult:
    rules: List[SandRule]
    types: List[SandType]
    materials: List[SandMaterial]


# --------------------------------------------------------------------------------------
# parse_string (parser.rs:93-152)
# --------------------------------------------------------------------------------------

def _check_and_convert_key_to_mapping(data: Any, keyname: str) -> dict:  # parser.rs:174-187
    p = y_get(data, keyname)
    if p is None:
        raise _missing_field(keyname, "Root/ Base level of YAML file")
    m = as_map(p.v)
    if m is None:
        raise _invalid_type(_debug_value(p.v), "Root/ Base level of YAML file", TYPE_HINT_MAPPING)
    return m


def _preparse_keys(m: dict, err_name: str) -> List[str]:  # parser.rs:156-168
    names = []
    for k in m:
        s = as_str(k)
        if s is None:
            raise _invalid_type(_debug_value(k), err_name, TYPE_HINT_STRING)
        names.append(s)
    return names


def parse_string(text: str) -> ParsingResult:
    try:
        data = load_yaml(text)
    except YamlError as e:
        raise ParseError("Yaml", str(e))
    raw_rules = _check_and_convert_key_to_mapping(data, "rules")
    raw_types = _check_and_convert_key_to_mapping(data, "types")
    raw_materials = _check_and_convert_key_to_mapping(data, "materials")
    rule_names = _preparse_keys(raw_rules, "rules")
    type_names = _preparse_keys(raw_types, "types") + ["EMPTY"]
    material_names = _preparse_keys(raw_materials, "materials") + ["EMPTY"]
    try:
        rules = parse_rules(raw_rules, type_names, material_names)
    except ParseError as e:
        raise _wrap("rules", e)
    try:
        types = parse_types(raw_types, rules, rule_names, type_names)
    except ParseError as e:
        raise _wrap("types", e)
    try:
        materials = parse_materials(raw_materials, rules, type_names)
    except ParseError as e:
        raise _wrap("materials", e)
    return ParsingResult(rules, types, materials)


# --------------------------------------------------------------------------------------
# rules.rs
# --------------------------------------------------------------------------------------

def parse_global_scope(s: str) -> str:  # rules.rs:338-351
    s = s.replace(" or ", " || ")
    s = s.replace(" and ", " && ")
    s = s.replace("not ", " !")
    s = s.replace("empty", "MAT_EMPTY")
    s = s.replace("SELF", "self")
    s = s.replace("RIGHT", "right")
    s = s.replace("LEFT", "left")
    s = s.replace("DOWN", "down")
    s = s.replace("DOWNRIGHT", "downright")
    s = s.replace("DOWNLEFT", "downleft")
    return s


_SWAP_RE = re.compile(r"SWAP (\w+) (\w+)")
_SET_RE = re.compile(r"SET (\w+) (\w+)")
_MAT_RE = re.compile(r"\w*.mat\s*(==|!=)\s*(\w*)")
_TYPE_RE = re.compile(r"isType_(\w*)\(\w*\)")


def parse_do(parent: str, do_str: str) -> str:  # rules.rs:355-420
    out = ""
    found = False
    m = _SWAP_RE.search(do_str)
    if m:
        found = True
        a, b = m.group(1), m.group(2)
        if a not in GLOBAL_CELLNAMES:
            raise _not_found(a, parent)
        if b not in GLOBAL_CELLNAMES:
            raise _not_found(b, parent)
        out += f"swap({a}, {b});\n"
    m = _SET_RE.search(do_str)
    if m:
        found = True
        a, b = m.group(1), m.group(2)
        if a not in GLOBAL_CELLNAMES:
            raise _not_found(a, parent)
        out += f"{a} = newCell(MAT_{b}, pos);\n"
    if not found:
        raise _not_recognized(do_str, parent)
    return out


def parse_conditionals(parent: Any, parent_is_else: bool, parent_path: str,
                       if_conds: List[str], do_actions: List[str], probabilities: list,
                       type_names: List[str], material_names: List[str]) -> None:  # rules.rs:207-334
    p_if = y_get(parent, "if")
    if p_if is None and not parent_is_else:
        raise _missing_field("if", parent_path)
    elif p_if is not None:
        if_path = f"{parent_path}/if"
        cond = as_str(p_if.v)
        if cond is None:
            raise _invalid_type('"if"', if_path, TYPE_HINT_STRING)
        cond = parse_global_scope(cond)
        original = cond
        for mm in _MAT_RE.finditer(original):
            cap = mm.group(2)
            for mname in material_names:
                if mname == cap:
                    cond = cond.replace(mname, f"MAT_{mname}")
                    break
            else:
                raise _not_found(cap, if_path)
        for mm in _TYPE_RE.finditer(cond):
            cap = mm.group(1)
            if cap not in type_names:
                raise _not_found(cap, f"{if_path} -> isType_")
        if_conds.append(cond)
    p_do = y_get(parent, "do")
    if p_do is None:
        raise _missing_field("do", parent_path)
    do_path = f"{parent_path}/do"
    do_string = ""
    s = as_str(p_do.v)
    if s is not None:
        do_string = parse_global_scope(parse_do(do_path, s))
    seq = as_seq(p_do.v)
    if seq is not None:
        for item in seq:
            si = as_str(item)
            if si is not None:
                do_string += parse_global_scope(parse_do(do_path, si))
    do_actions.append(do_string.rstrip())
    p_prob = y_get(parent, "probability")
    if p_prob is not None:
        f = as_f64(p_prob.v)
        if f is None:
            raise _invalid_type('"probability"', parent_path, TYPE_HINT_FLOAT)
        probabilities.append(np.float32(f))
    else:
        probabilities.append(DEFAULT_VAL_PROBABILITY)
    p_else = y_get(parent, "else")
    if p_else is not None:
        parse_conditionals(p_else.v, True, f"{parent_path}/else", if_conds, do_actions,
                           probabilities, type_names, material_names)


def parse_rules(rules: dict, type_names: List[str], material_names: List[str]) -> List[SandRule]:
    out = []
    for k, v in rules.items():  # rules.rs:109-200
        name = as_str(k)
        if_conds: List[str] = []
        do_actions: List[str] = []
        probs: list = []
        parse_conditionals(v, False, f"rules/{name}", if_conds, do_actions, probs,
                           type_names, material_names)
        p_m = y_get(v, "mirrored")
        if p_m is not None:
            mirror = as_bool(p_m.v)
            if mirror is None:
                raise _invalid_type('"mirrored"', f"rules/{name}", TYPE_HINT_BOOL)
        else:
            mirror = DEFAULT_VAL_MIRRORED
        if mirror:
            ruletype = "Mirrored"
        else:
            ruletype = "Left" if "LEFT" in do_actions[0] else "Right"
        p_pre = y_get(v, "precondition")
        if p_pre is not None:
            pre = as_bool(p_pre.v)
            if pre is None:
                raise _invalid_type('"precondition"', f"rules/{name}", TYPE_HINT_BOOL)
        else:
            pre = DEFAULT_VAL_PRECONDITION
        out.append(SandRule(name, ruletype, if_conds, do_actions, probs, mirror,
                            "" if pre else None))
    return out


def _get_func_logic(if_conds: List[str], do_actions: List[str], probs: list, lvl: int) -> str:
    # rules.rs:47-73
    if not if_conds and not do_actions:
        return ""
    if not if_conds and do_actions:
        return do_actions.pop(0)
    if if_conds and do_actions:
        ind1 = " " * (lvl * 4)
        ind2 = " " * ((lvl + 1) * 4)
        p = probs.pop(0)
        prob = "" if p == DEFAULT_VAL_PROBABILITY else f"rand.y <= {f32_display(p)} && "
        c = if_conds.pop(0)
        d = do_actions.pop(0)
        inner = _get_func_logic(if_conds, do_actions, probs, lvl + 1)
        return f"{ind1}if ({prob}{c}) {{\n{ind2}{d}\n{ind1}}} else {{\n{inner}\n{ind1}}}"
    return ""


def rule_glsl(r: SandRule) -> str:  # rules.rs:75-98
    celldir = "left" if r.ruletype == "Left" else "right"
    pre = "" if r.precondition is None else \
        f"    if (!({r.precondition})) {{\n        return;\n    }}\n"
    text = _get_func_logic(list(r.if_conds), list(r.do_actions), list(r.probabilities), 1)
    return (f"void rule_{r.name} (inout Cell self, inout Cell {celldir}, inout Cell down, "
            f"inout Cell downright, vec4 rand, ivec2 pos) {{\n{pre}{text}\n}}")


# --------------------------------------------------------------------------------------
# types.rs
# --------------------------------------------------------------------------------------

def _update_precondition(rule: SandRule, typename: str) -> None:  # types.rs:78-88
    if rule.precondition is not None:
        if rule.precondition == "":
            rule.precondition = f"isType_{typename}(self)"
        else:
            rule.precondition = f"{rule.precondition} || isType_{typename}(self)"


def _add_child_to_type(parent: str, child: str, types: List[SandType], depth: int = 0) -> None:
    # types.rs:186-200
    if depth > 10000:
        raise ParseError("Panic", "type inheritance cycle (the reference overflows its stack)")
    pp = ""
    for t in types:
        if t.name == parent:
            t.children.append(child)
            pp = t.inherits
            break
    if pp:
        _add_child_to_type(pp, child, types, depth + 1)


def _get_parents_rules(all_types: List[SandType], cur: SandType, depth: int = 0) -> List[str]:
    # types.rs:202-210
    if not cur.inherits:
        return []
    if depth > len(all_types):
        raise ParseError("Panic", "type inheritance cycle (the reference overflows its stack)")
    parent = next((t for t in all_types if t.name == cur.inherits), None)
    if parent is None:
        raise ParseError("Panic", f"type '{cur.name}' inherits unknown type '{cur.inherits}' "
                                  f"(the reference panics on unwrap)")
    return list(parent.base_rules) + _get_parents_rules(all_types, parent, depth + 1)


def parse_types(types: dict, rules: List[SandRule], rule_names: List[str],
                type_names: List[str]) -> List[SandType]:  # types.rs:51-182
    structs = [SandType(0, "EMPTY"), SandType(1, "NULL"), SandType(2, "WALL")]
    idx = 3
    for k, v in types.items():
        name = as_str(k)
        parent = ""
        p_inh = y_get(v, "inherits")
        if p_inh is not None:
            parent = as_str(p_inh.v)
            if parent is None:
                raise _invalid_type('"inherits"', f"types/{name}", TYPE_HINT_STRING)
            for tn in type_names:
                if tn == parent:
                    _add_child_to_type(parent, name, structs)
        base_rules = []
        p_br = y_get(v, "base_rules")
        if p_br is not None:
            seq = as_seq(p_br.v)
            if seq is None:
                raise _invalid_type('"base_rules"', f"types/{name}", TYPE_HINT_SEQUENCE)
            for item in seq:
                rn = as_str(item)
                if rn is None:
                    raise _invalid_type('"base_rules"', f"types/{name}", TYPE_HINT_STRING)
                if rn not in rule_names:
                    raise _not_found(rn, f"types/{name}/base_rules")
                rule = next(r for r in rules if r.name == rn)
                rule.used = True
                _update_precondition(rule, name)
                base_rules.append(rn)
        structs.append(SandType(idx, name, parent, [], base_rules))
        idx += 1
    for t in [SandType(s.id, s.name, s.inherits, list(s.children), list(s.base_rules))
              for s in structs]:
        if not t.inherits:
            continue
        for rn in _get_parents_rules(structs, t):
            rule = next(r for r in rules if r.name == rn)
            _update_precondition(rule, t.name)
    return structs


def type_checker_glsl(t: SandType) -> str:  # types.rs:30-39
    tc = f"return cell.mat.type == TYPE_{t.name}"
    for c in t.children:
        tc += f" || cell.mat.type == TYPE_{c}"
    return f"bool isType_{t.name}(Cell cell) {{\n    {tc};\n}}\n\n"


def type_define_glsl(t: SandType) -> str:  # types.rs:41-45
    return f"#define TYPE_{t.name} {t.id}\n\n"


# --------------------------------------------------------------------------------------
# materials.rs + parser.rs:191-250 (extract_vec4)
# --------------------------------------------------------------------------------------

def _extract_vec4(yaml_data: Any, parent_name: str, field_name: str, default, mandatory: bool):
    missing_in = f"materials/{parent_name}/{field_name}"
    p = y_get(yaml_data, field_name)
    if p is None:
        if mandatory:
            raise _missing_field(field_name, missing_in)
        return [np.float32(x) for x in default]
    vec = [np.float32(x) for x in default]
    seq = as_seq(p.v)
    if seq is None or len(seq) == 0 or len(seq) > 4 or len(seq) < 3:
        raise _invalid_type(f'"{field_name}"', missing_in, TYPE_HINT_COLOR)
    for i, comp in enumerate(seq):
        u = as_u64(comp)
        if u is not None and 0 < u <= 255:
            vec[i] = np.float32(np.float32(u) / np.float32(255.0))
            continue
        f = as_f64(comp)
        if f is not None:
            if 1.0 < f <= 255.0:
                vec[i] = np.float32(np.float32(f) / np.float32(255.0))
                continue
            if 0.0 <= f <= 1.0:
                vec[i] = np.float32(f)
                continue
        raise _invalid_type(f'"{field_name}"', missing_in, TYPE_HINT_COLOR)
    return vec


def parse_materials(materials: dict, rules: List[SandRule],
                    type_names: List[str]) -> List[SandMaterial]:  # materials.rs:51-201
    f32 = np.float32
    structs = [
        SandMaterial(0, "EMPTY", "EMPTY", [f32(0)] * 4, [f32(0)] * 4, True, f32(1.0)),
        SandMaterial(1, "NULL", "NULL", [f32(1), f32(0), f32(1), f32(1)], [f32(0)] * 4, False, f32(0.0)),
        SandMaterial(2, "WALL", "WALL", [f32(0.1), f32(0.2), f32(0.3), f32(1.0)], [f32(0)] * 4,
                     False, f32(9999.0)),
    ]
    idx = 3
    for k, v in materials.items():
        name = as_str(k)
        p_t = y_get(v, "type")
        if p_t is None:
            raise _missing_field("type", f"materials/{name}")
        mattype = as_str(p_t.v)
        if mattype is None:
            raise _invalid_type('"type"', f"materials/{name}", TYPE_HINT_STRING)
        if mattype not in type_names:
            raise _not_found(mattype, f"materials/{name}/type")
        color = _extract_vec4(v, name, "color", [1.0, 0.0, 1.0, 1.0], True)
        emission = _extract_vec4(v, name, "emission", [0.0, 0.0, 0.0, 0.0], False)
        p_sel = y_get(v, "selectable")
        if p_sel is not None:
            b = as_bool(p_sel.v)
            selectable = b if b is not None else False
        else:
            selectable = True
        p_d = y_get(v, "density")
        if p_d is None:
            raise _missing_field("density", f"materials/{name}")
        d = as_f64(p_d.v)
        if d is None:
            raise _invalid_type('"density"', f"materials/{name}/density", TYPE_HINT_FLOAT)
        density = f32(d)
        extra = []
        p_x = y_get(v, "extra_rules")
        if p_x is not None:
            seq = as_seq(p_x.v)
            if seq is None:
                raise _invalid_type('"extra_rules"', f"materials/{name}", TYPE_HINT_SEQUENCE)
            for item in seq:
                rn = as_str(item)
                if rn is None:
                    raise _invalid_type('"extra_rules"', f"materials/{name}", TYPE_HINT_STRING)
                for r in rules:
                    if r.name == rn:
                        r.used = True
                        if r.precondition is not None:
                            if r.precondition == "":
                                r.precondition = f"self.mat == MAT_{name}"
                            else:
                                r.precondition = f"{r.precondition} || self.mat == MAT_{name}"
                        extra.append(rn)
        structs.append(SandMaterial(idx, name, mattype, color, emission, selectable, density, extra))
        idx += 1
    return structs


def material_define_glsl(m: SandMaterial) -> str:  # materials.rs:30-47
    c = [f32_display(x) for x in m.color]
    e = [f32_display(x) for x in m.emission]
    return (f"#define MAT_{m.name} Material({m.id}, vec4({c[0]}, {c[1]}, {c[2]}, {c[3]}), "
            f"{f32_display(m.density)}, vec4({e[0]}, {e[1]}, {e[2]}, {e[3]}), TYPE_{m.mattype})\n")


# --------------------------------------------------------------------------------------
# create_glsl_from_parser (sandengine-lang/src/lib.rs:17-147)
# --------------------------------------------------------------------------------------

def materials_glsl(res: ParsingResult) -> str:
    out = "".join(type_define_glsl(t) for t in res.types)
    out += "".join(type_checker_glsl(t) for t in res.types)
    out += "\n"
    n = len(res.materials)
    lst = ""
    for i, m in enumerate(res.materials):
        out += material_define_glsl(m)
        lst += f"        MAT_{m.name}" + ("" if i == n - 1 else ",\n")
    out += (f"\nMaterial[{n}] materials() {{\n    Material allMaterials[{n}] = {{\n{lst}\n    }};\n"
            f"    return allMaterials;\n}}\n\nMaterial getMaterialFromID(int id) {{\n"
            f"    for (int i = 0; i < materials().length(); i++) {{\n"
            f"        if (id == materials()[i].id) {{\n            return materials()[i];\n"
            f"        }};\n    }};\n    return MAT_NULL;\n}}\n\n")
    return out


_CALLER_HEAD = ("    inout Cell self,\n    inout Cell right,\n    inout Cell down,\n"
                "    inout Cell downright,\n    vec4 rand,\n    ivec2 pos) {\n")


def rules_glsl(res: ParsingResult) -> str:
    funcs = ""
    mirrored = left = right = ""
    for r in res.rules:
        if not r.used:
            continue
        funcs += f"{rule_glsl(r)}\n\n"
        if r.ruletype == "Mirrored":
            mirrored += f"rule_{r.name}(self, right, down, downright, rand, pos);\n"
        elif r.ruletype == "Left":
            left += f"rule_{r.name}(self, left, down, downright, rand, pos);\n"
        else:
            right += f"rule_{r.name}(self, right, down, downright, rand, pos);\n"
    return ("\n// =============== RULES ===============\n" + funcs +
            "\n\n\n// =============== CALLERS ===============\nvoid applyMirroredRules(\n" +
            _CALLER_HEAD + "    " + mirrored.rstrip() + "\n}\n\n\nvoid applyLeftRules(\n" +
            _CALLER_HEAD + "    " + left.rstrip() + "\n}\n\nvoid applyRightRules(\n" +
            _CALLER_HEAD + "    " + right.rstrip() + "\n}")


def create_glsl(res: ParsingResult) -> Tuple[str, str]:
    return materials_glsl(res), rules_glsl(res)


# --------------------------------------------------------------------------------------
# The #include flattener (src/lib.rs:31-76), for one shader file
# --------------------------------------------------------------------------------------

def flatten_includes(contents: str, read_include) -> str:
    """Inline ``\\n#include "x"`` the way build_compute_shaders does: an include whose
    preceding character is ' ' or '/' (e.g. a commented-out include) is deleted instead."""
    search = '\n#include "'
    start = contents.find(search)
    start = 0 if start < 0 else start
    while start != 0:
        incl_path = contents[start + len(search):].split('"')[0]
        src = read_include(incl_path)
        if src is not None:
            src = src + "\n\n\n"
            s = contents.find(search)
            e = s + len(search) + len(incl_path) + 1
            # src/lib.rs:60 indexes chars() with a BYTE offset; with multi-byte text
            # earlier in the file this looks at a later character.  Reproduced as is.
            byte_s = len(contents[:s].encode("utf-8"))
            before = contents[byte_s - 1]
            if before in (" ", "/"):
                contents = contents[:s] + contents[e:]
            else:
                contents = contents[:s] + src + contents[e:]
        nxt = contents.find(search)
        start = 0 if nxt < 0 else nxt
        if src is None and nxt == start and nxt != 0:
            # the reference loops forever on an unreadable include; stop instead
            raise ParseError("Panic", f"unreadable include {incl_path!r}")
    return contents
