"""Rule-language inputs for front-end parity tests: each is run through the product's
C++ front end and the oracle's Python restatement; both must emit byte-identical GLSL or
fail with the same error kind.  The first group mirrors what the reference's own tests
(tests/test_sandengine-lang.rs) exercise: missing sections, a non-string rule name, a
missing field, an unknown name; the rest cover the other branches of parser.rs,
rules.rs, types.rs and materials.rs."""

BASE_TYPES = """
types:
  solid:
  powder:
    base_rules: [fall]
"""
BASE_MATS = """
materials:
  sand:
    type: powder
    color: [1.0, 1.0, 0.0]
    density: 1.5
"""
FALL = """
rules:
  fall:
    if: DOWN.mat.density < SELF.mat.density
    do: SWAP SELF DOWN
"""


def doc(rules=FALL, types=BASE_TYPES, mats=BASE_MATS):
    return rules + types + mats


CORPUS = {
    # --- what the reference's tests probe (test_sandengine-lang.rs:3-165) ---
    "missing_rules": BASE_TYPES + BASE_MATS,
    "missing_types": FALL + BASE_MATS,
    "missing_materials": FALL + BASE_TYPES,
    "number_rule_name_without_types": "\n    rules:\n        2.5:\n            if: SELF.mat.density > 1\n"
                                      "            do: SWAP SELF DOWN\n",
    "number_rule_name": "rules:\n  2.5:\n    if: x\n    do: SWAP SELF DOWN\n" + BASE_TYPES + BASE_MATS,
    "missing_if": doc(rules="rules:\n  fall:\n    do: SWAP SELF DOWN\n"),
    "missing_color": doc(mats="materials:\n  sand:\n    type: powder\n    density: 1.5\n"),
    "unknown_type": doc(mats="materials:\n  sand:\n    type: liquid\n    color: [1, 1, 1]\n    density: 1\n"),
    "function_call_do": doc(rules="rules:\n  fall:\n    if: SELF.mat.density > 1\n    do: swap(SELF, DOWN)\n"),
    "indented_document": "\n    rules:\n        fall:\n            if: DOWN.mat.density < SELF.mat.density\n"
                         "            do: SWAP SELF DOWN\n    types:\n        powder:\n"
                         "            base_rules: [\n                fall\n            ]\n    materials:\n"
                         "        sand:\n            color: [1.0, 1.0, 0.0, 1.0]\n            type: powder\n"
                         "            density: 1.5\n            selectable: true\n",
    # --- sections and keys ---
    "root_is_sequence": "- rules\n- types\n",
    "rules_not_mapping": "rules: [a, b]\n" + BASE_TYPES + BASE_MATS,
    "yaml_syntax_error": "rules:\n  fall: [unclosed\n",
    "duplicate_key": FALL + "  fall:\n    if: x\n    do: SWAP SELF DOWN\n" + BASE_TYPES + BASE_MATS,
    # --- rules.rs ---
    "if_not_string": doc(rules="rules:\n  fall:\n    if: 3\n    do: SWAP SELF DOWN\n"),
    "missing_do": doc(rules="rules:\n  fall:\n    if: SELF.mat.density > 1\n"),
    "swap_unknown_cell": doc(rules="rules:\n  fall:\n    if: x\n    do: SWAP SELF UP\n"),
    "set_unknown_cell": doc(rules="rules:\n  fall:\n    if: x\n    do: SET UP sand\n"),
    "cond_unknown_material": doc(rules="rules:\n  fall:\n    if: DOWN.mat == lava\n    do: SWAP SELF DOWN\n"),
    "cond_unknown_type": doc(rules="rules:\n  fall:\n    if: isType_gas(DOWN)\n    do: SWAP SELF DOWN\n"),
    "probability_not_number": doc(rules="rules:\n  fall:\n    if: x\n    probability: often\n    do: SWAP SELF DOWN\n"),
    "mirrored_not_bool": doc(rules=FALL + "    mirrored: 3\n"),
    "precondition_not_bool": doc(rules=FALL + "    precondition: maybe\n"),
    "else_without_if": doc(rules="rules:\n  fall:\n    if: DOWN.mat == EMPTY\n    do: SWAP SELF DOWN\n"
                                 "    probability: 0.5\n    else:\n      do: SWAP SELF DOWNRIGHT\n"
                                 "      probability: 0.25\n      else:\n        if: RIGHT.mat == EMPTY\n"
                                 "        do: SWAP SELF RIGHT\n"),
    "do_list": doc(rules="rules:\n  fall:\n    if: DOWN.mat == sand\n    do:\n      - SWAP SELF DOWN\n"
                         "      - SET RIGHT sand\n      - 7\n"),
    "do_number": doc(rules="rules:\n  fall:\n    if: x\n    do: 5\n"),
    "swap_and_set_in_one_string": doc(rules="rules:\n  fall:\n    if: x\n    do: SWAP SELF DOWN then SET DOWN sand\n"),
    "not_and_or_empty": doc(rules="rules:\n  fall:\n    if: not isType_EMPTY(DOWN) or DOWN.mat == EMPTY and RIGHT.mat != sand\n"
                                  "    do: SWAP SELF DOWN\n"),
    "precondition_false_and_right": doc(rules=FALL + "    precondition: false\n    mirrored: false\n"),
    "probability_int": doc(rules=FALL + "    probability: 1\n"),
    "probability_tiny": doc(rules=FALL + "    probability: 0.0000001\n"),
    "unused_rule": doc(rules=FALL + "  other:\n    if: SELF.mat == sand\n    do: SET SELF EMPTY\n"),
    "double_material_capture": doc(rules="rules:\n  fall:\n    if: DOWN.mat == sand and RIGHT.mat == sand\n"
                                         "    do: SWAP SELF DOWN\n"),
    "lowercase_empty_everywhere": doc(rules="rules:\n  fall:\n    if: isType_empty(DOWN)\n    do: SWAP SELF DOWN\n"),
    # --- types.rs ---
    "inherits_chain": doc(types="types:\n  solid:\n    base_rules: [fall]\n  powder:\n    inherits: solid\n"
                                "  fine:\n    inherits: powder\n",
                          mats="materials:\n  sand:\n    type: fine\n    color: [1, 1, 1]\n    density: 1.5\n"),
    "inherits_later_parent": doc(types="types:\n  powder:\n    inherits: solid\n  solid:\n    base_rules: [fall]\n"),
    "inherits_unknown": doc(types="types:\n  powder:\n    inherits: nope\n    base_rules: [fall]\n"),
    "inherits_cycle": doc(types="types:\n  a:\n    inherits: b\n  b:\n    inherits: a\n    base_rules: [fall]\n",
                          mats="materials:\n  sand:\n    type: a\n    color: [1, 1, 1]\n    density: 1\n"),
    "inherits_not_string": doc(types="types:\n  powder:\n    inherits: [solid]\n"),
    "base_rules_unknown": doc(types="types:\n  powder:\n    base_rules: [fly]\n"),
    "base_rules_not_sequence": doc(types="types:\n  powder:\n    base_rules: fall\n"),
    "base_rules_item_not_string": doc(types="types:\n  powder:\n    base_rules: [fall, 3]\n"),
    "type_named_empty": doc(types="types:\n  EMPTY:\n  powder:\n    base_rules: [fall]\n"),
    "inherit_from_empty": doc(types="types:\n  powder:\n    inherits: EMPTY\n    base_rules: [fall]\n"),
    # --- materials.rs / extract_vec4 ---
    "colors_mixed": doc(mats="materials:\n  sand:\n    type: powder\n    color: [255, 0.5, 1, 128]\n"
                             "    emission: [0, 0, 17]\n    density: 2\n    selectable: false\n"
                             "  rock:\n    type: solid\n    color: [1.5, 0, 0]\n    density: -3.25\n"
                             "    selectable: 7\n"),
    "color_too_many": doc(mats="materials:\n  sand:\n    type: powder\n    color: [1, 1, 1, 1, 1]\n    density: 1\n"),
    "color_too_large": doc(mats="materials:\n  sand:\n    type: powder\n    color: [256, 1, 1]\n    density: 1\n"),
    "color_negative": doc(mats="materials:\n  sand:\n    type: powder\n    color: [-1, 1, 1]\n    density: 1\n"),
    "color_not_sequence": doc(mats="materials:\n  sand:\n    type: powder\n    color: red\n    density: 1\n"),
    "missing_density": doc(mats="materials:\n  sand:\n    type: powder\n    color: [1, 1, 1]\n"),
    "density_string": doc(mats="materials:\n  sand:\n    type: powder\n    color: [1, 1, 1]\n    density: heavy\n"),
    "density_nan": doc(mats="materials:\n  sand:\n    type: powder\n    color: [1, 1, 1]\n    density: .nan\n"
                            "    extra_rules: [fall]\n"),
    "missing_type_field": doc(mats="materials:\n  sand:\n    color: [1, 1, 1]\n    density: 1\n"),
    "type_null": doc(mats="materials:\n  sand:\n    type: NULL\n    color: [1, 1, 1]\n    density: 1\n"),
    "extra_rules_unknown_ignored": doc(mats=BASE_MATS + "    extra_rules: [nope]\n"),
    "extra_rules_not_sequence": doc(mats=BASE_MATS + "    extra_rules: fall\n"),
    "extra_rules_item_not_string": doc(mats=BASE_MATS + "    extra_rules: [1]\n"),
    "material_type_empty": doc(mats="materials:\n  air:\n    type: EMPTY\n    color: [0, 0, 0, 0]\n    density: 0.5\n"),
    "comments_quotes_flow": "# rules first\nrules:\n  'fall':   # quoted key\n    if: \"DOWN.mat.density < SELF.mat.density\"\n"
                            "    do: 'SWAP SELF DOWN'\ntypes: {solid: , powder: {base_rules: [fall]}}\n"
                            "materials:\n  sand: {type: powder, color: [1, 1, 0], density: 1.5}\n",
}
