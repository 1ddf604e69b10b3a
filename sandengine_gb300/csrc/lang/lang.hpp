// The sandengine rule language front end: YAML -> rule/type/material IR -> GLSL text.
//
// Follows sandengine-lang (parser.rs, parser/rules.rs, parser/types.rs,
// parser/materials.rs, lib.rs) step for step, including its string-level rewrites, so the
// GLSL it emits is byte-identical to what the reference writes into
// shaders/compute/gen/{materials,rules}.glsl.  The CUDA back end (codegen.hpp) then
// compiles that GLSL rule text.
#pragma once

#include <cstddef>
#include <string>
#include <vector>

namespace se::lang {

// Error kinds of parser.rs:42-73, plus: Yaml (serde_yaml rejected the text), Panic (the
// reference panics or overflows its stack on this input), Glsl (the generated GLSL would
// not compile, so the reference panics at shader build, simulation.rs:133-137) and
// Unsupported (valid GLSL the CUDA back end does not translate).
struct ParseError {
  std::string kind;
  std::string message;
};

struct Rule {  // rules.rs:25-44
  enum Kind { Mirrored, Left, Right };
  std::string name;
  Kind ruletype = Mirrored;
  std::vector<std::string> if_conds;
  std::vector<std::string> do_actions;
  std::vector<float> probabilities;
  bool mirror = true;
  bool has_precondition = true;
  std::string precondition;
  bool used = false;
};

struct Type {  // types.rs:12-26
  size_t id = 0;
  std::string name;
  std::string inherits;
  std::vector<std::string> children;
  std::vector<std::string> base_rules;
};

struct Material {  // materials.rs:11-29
  size_t id = 0;
  std::string name;
  std::string mattype;
  float color[4] = {0, 0, 0, 0};
  float emission[4] = {0, 0, 0, 0};
  bool selectable = true;
  float density = 0;
  std::vector<std::string> extra_rules;
};

struct ParsingResult {
  std::vector<Rule> rules;
  std::vector<Type> types;
  std::vector<Material> materials;
};

// parser.rs:93-152.  Returns false and fills *err on failure.
bool parse_string(const std::string& text, ParsingResult* out, ParseError* err);

// sandengine-lang/src/lib.rs:17-147
std::string materials_glsl(const ParsingResult& r);
std::string rules_glsl(const ParsingResult& r);
std::string rule_glsl(const Rule& r);  // rules.rs:75-98

// Rust's `{}` for f32: shortest round-trip decimal, positional notation.
std::string f32_display(float f);

}  // namespace se::lang
