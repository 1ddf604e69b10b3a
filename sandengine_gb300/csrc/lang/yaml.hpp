// A reader for the subset of YAML 1.2 the sandengine rule language uses.
//
// serde_yaml 0.9.34 (Cargo.lock:1803-1805) parses the reference's rule files into a
// serde_yaml::Value whose mappings keep insertion order (indexmap 2.2.6).  This reader
// produces the same value tree for block mappings, block and flow sequences, plain and
// quoted scalars (core-schema typing: null, bool, int, float, string) and comments.
// Block scalars (| and >), anchors, aliases and tags are rejected with an error.
#pragma once

#include <cstdint>
#include <memory>
#include <string>
#include <utility>
#include <vector>

namespace se::yaml {

struct Value;
using ValuePtr = std::shared_ptr<Value>;

struct Value {
  enum Kind { Null, Bool, Int, Float, String, Seq, Map } kind = Null;
  bool b = false;
  bool int_negative = false;  // Int: value = neg ? -(int64)u : u
  uint64_t u = 0;             // Int magnitude
  double f = 0.0;             // Float
  std::string s;              // String
  std::vector<ValuePtr> seq;  // Seq
  std::vector<std::pair<ValuePtr, ValuePtr>> map;  // Map, insertion order

  // serde_yaml::Value accessors.
  const std::string* as_str() const { return kind == String ? &s : nullptr; }
  bool as_bool(bool* out) const {
    if (kind != Bool) return false;
    *out = b;
    return true;
  }
  bool as_f64(double* out) const;  // Int or Float
  bool as_u64(uint64_t* out) const;  // non-negative Int
  const std::vector<ValuePtr>* as_seq() const { return kind == Seq ? &seq : nullptr; }
  bool is_map() const { return kind == Map; }
  // Value::get(&str): the value for a string key of a mapping, or null if absent / not a map.
  const Value* get(const std::string& key) const;
  std::string debug() const;  // rendering used inside error messages
};

// Parses `text`; on failure returns null and sets *err.
ValuePtr parse(const std::string& text, std::string* err);

}  // namespace se::yaml
