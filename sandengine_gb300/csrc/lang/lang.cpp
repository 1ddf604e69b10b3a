#include "lang.hpp"

#include <algorithm>
#include <charconv>
#include <cmath>
#include <functional>
#include <map>
#include <set>

#include "yaml.hpp"

namespace se::lang {
namespace {

using yaml::Value;

// ---- error constructors (parser.rs:42-73; thiserror formats, colours off) -------------
ParseError missing_field(const std::string& field, const std::string& in) {
  return {"MissingField", "(MissingField) Mandatory field '" + field + "' is missing in '" + in + "'"};
}
ParseError invalid_type(const std::string& wrong, const std::string& in, const std::string& expected) {
  return {"InvalidType", "(InvalidType) The type of the field '" + wrong + "' inside of '" + in +
                             "' is invalid. Expected: '" + expected + "'"};
}
ParseError not_found(const std::string& missing, const std::string& in) {
  return {"NotFound", "(NotFound) The name '" + missing + "' (in '" + in +
                          "') was not found. Make sure it was defined before referencing it."};
}
ParseError not_recognized(const std::string& what, const std::string& in) {
  return {"NotRecognized", "(NotRecognized) The expression '" + what + "' (in '" + in +
                               "') was not recognized as valid syntax. Please check it is valid."};
}
ParseError wrap(const std::string& section, const ParseError& e) {
  return {e.kind, "Error while parsing " + section + ": '" + e.message + "'"};
}

const char* TYPE_HINT_STRING = "string";
const char* TYPE_HINT_BOOL = "bool (true/false)";
const char* TYPE_HINT_FLOAT = "float (0.0 to 1.0)";
const char* TYPE_HINT_SEQUENCE = "sequence (array, '[...]')";
const char* TYPE_HINT_COLOR =
    "sequence (array, '[...]') of 3-4 floats (range 0.0-1.0) OR integers (range 0-255). (With 3 "
    "elements, the alpha channel defaults to 1.0)";
const char* TYPE_HINT_MAPPING = "mapping (dictionary-like)";

const std::vector<std::string> GLOBAL_CELLNAMES = {"SELF", "LEFT", "RIGHT", "DOWN", "DOWNRIGHT", "DOWNLEFT"};

struct Fail {
  ParseError e;
};

// ---- string helpers --------------------------------------------------------------------
std::string replace_all(std::string s, const std::string& from, const std::string& to) {
  if (from.empty()) return s;
  std::string out;
  size_t p = 0;
  for (;;) {
    size_t q = s.find(from, p);
    if (q == std::string::npos) break;
    out.append(s, p, q - p);
    out += to;
    p = q + from.size();
  }
  out.append(s, p, std::string::npos);
  return out;
}

// Regex `\w`: ASCII word characters; bytes of multi-byte UTF-8 sequences count as word
// characters (the regex crate's Unicode \w accepts letters there).
bool is_word(unsigned char c) {
  return (c >= 'a' && c <= 'z') || (c >= 'A' && c <= 'Z') || (c >= '0' && c <= '9') || c == '_' || c >= 0x80;
}
bool is_space(char c) { return c == ' ' || c == '\t' || c == '\n' || c == '\r' || c == '\f' || c == '\v'; }
size_t word_end(const std::string& s, size_t i) {
  while (i < s.size() && is_word((unsigned char)s[i])) ++i;
  return i;
}

// All group-2 captures of `\w*.mat\s*(==|!=)\s*(\w*)` (rules.rs:246), leftmost-first,
// non-overlapping, as the regex crate's captures_iter yields them.
std::vector<std::string> material_captures(const std::string& s) {
  std::vector<std::string> caps;
  size_t i = 0;
  while (i <= s.size()) {
    bool matched = false;
    size_t we = word_end(s, i);
    for (size_t j = we + 1; j-- > i;) {
      if (j >= s.size() || s[j] == '\n') continue;
      if (s.compare(j + 1, 3, "mat") != 0) continue;
      size_t k = j + 4;
      while (k < s.size() && is_space(s[k])) ++k;
      if (s.compare(k, 2, "==") != 0 && s.compare(k, 2, "!=") != 0) continue;
      k += 2;
      while (k < s.size() && is_space(s[k])) ++k;
      size_t e = word_end(s, k);
      caps.push_back(s.substr(k, e - k));
      i = e;
      matched = true;
      break;
    }
    if (!matched) ++i;
  }
  return caps;
}

// All captures of `isType_(\w*)\(\w*\)` (rules.rs:262).
std::vector<std::string> type_captures(const std::string& s) {
  std::vector<std::string> caps;
  size_t p = 0;
  for (;;) {
    size_t i = s.find("isType_", p);
    if (i == std::string::npos) break;
    size_t k = i + 7, e1 = word_end(s, k);
    if (e1 < s.size() && s[e1] == '(') {
      size_t e2 = word_end(s, e1 + 1);
      if (e2 < s.size() && s[e2] == ')') {
        caps.push_back(s.substr(k, e1 - k));
        p = e2 + 1;
        continue;
      }
    }
    p = i + 1;
  }
  return caps;
}

// First match of `<VERB> (\w+) (\w+)` (rules.rs:364, :393).
bool verb_match(const std::string& s, const std::string& verb, std::string* a, std::string* b) {
  std::string lit = verb + " ";
  size_t p = 0;
  for (;;) {
    size_t i = s.find(lit, p);
    if (i == std::string::npos) return false;
    size_t k = i + lit.size(), e1 = word_end(s, k);
    if (e1 > k && e1 < s.size() && s[e1] == ' ') {
      size_t e2 = word_end(s, e1 + 1);
      if (e2 > e1 + 1) {
        *a = s.substr(k, e1 - k);
        *b = s.substr(e1 + 1, e2 - e1 - 1);
        return true;
      }
    }
    p = i + 1;
  }
}

bool contains(const std::vector<std::string>& v, const std::string& x) {
  return std::find(v.begin(), v.end(), x) != v.end();
}

// ---- rules.rs ---------------------------------------------------------------------------
std::string parse_global_scope(std::string s) {  // rules.rs:338-351
  s = replace_all(s, " or ", " || ");
  s = replace_all(s, " and ", " && ");
  s = replace_all(s, "not ", " !");
  s = replace_all(s, "empty", "MAT_EMPTY");
  s = replace_all(s, "SELF", "self");
  s = replace_all(s, "RIGHT", "right");
  s = replace_all(s, "LEFT", "left");
  s = replace_all(s, "DOWN", "down");
  s = replace_all(s, "DOWNRIGHT", "downright");
  s = replace_all(s, "DOWNLEFT", "downleft");
  return s;
}

std::string parse_do(const std::string& parent, const std::string& do_str) {  // rules.rs:355-420
  std::string out, a, b;
  bool found = false;
  if (verb_match(do_str, "SWAP", &a, &b)) {
    found = true;
    if (!contains(GLOBAL_CELLNAMES, a)) throw Fail{not_found(a, parent)};
    if (!contains(GLOBAL_CELLNAMES, b)) throw Fail{not_found(b, parent)};
    out += "swap(" + a + ", " + b + ");\n";
  }
  if (verb_match(do_str, "SET", &a, &b)) {
    found = true;
    if (!contains(GLOBAL_CELLNAMES, a)) throw Fail{not_found(a, parent)};
    out += a + " = newCell(MAT_" + b + ", pos);\n";
  }
  if (!found) throw Fail{not_recognized(do_str, parent)};
  return out;
}

std::string rtrim(std::string s) {
  while (!s.empty() && is_space(s.back())) s.pop_back();
  return s;
}

void parse_conditionals(const Value* parent, bool parent_is_else, const std::string& parent_path, Rule& r,
                        const std::vector<std::string>& type_names,
                        const std::vector<std::string>& material_names) {  // rules.rs:207-334
  const Value* vif = parent->get("if");
  if (!vif && !parent_is_else) throw Fail{missing_field("if", parent_path)};
  if (vif) {
    std::string if_path = parent_path + "/if";
    const std::string* s = vif->as_str();
    if (!s) throw Fail{invalid_type("\"if\"", if_path, TYPE_HINT_STRING)};
    std::string cond = parse_global_scope(*s);
    const std::string original = cond;
    for (const std::string& cap : material_captures(original)) {
      bool hit = false;
      for (const std::string& m : material_names)
        if (m == cap) {
          cond = replace_all(cond, m, "MAT_" + m);
          hit = true;
          break;
        }
      if (!hit) throw Fail{not_found(cap, if_path)};
    }
    for (const std::string& cap : type_captures(cond))
      if (!contains(type_names, cap)) throw Fail{not_found(cap, if_path + " -> isType_")};
    r.if_conds.push_back(cond);
  }
  const Value* vdo = parent->get("do");
  if (!vdo) throw Fail{missing_field("do", parent_path)};
  std::string do_path = parent_path + "/do";
  std::string do_string;
  if (const std::string* s = vdo->as_str()) do_string = parse_global_scope(parse_do(do_path, *s));
  if (auto* seq = vdo->as_seq())
    for (auto& item : *seq)
      if (const std::string* s = item->as_str()) do_string += parse_global_scope(parse_do(do_path, *s));
  r.do_actions.push_back(rtrim(do_string));
  const Value* vp = parent->get("probability");
  if (vp) {
    double f;
    if (!vp->as_f64(&f)) throw Fail{invalid_type("\"probability\"", parent_path, TYPE_HINT_FLOAT)};
    r.probabilities.push_back((float)f);
  } else {
    r.probabilities.push_back(1.0f);
  }
  if (const Value* ve = parent->get("else"))
    parse_conditionals(ve, true, parent_path + "/else", r, type_names, material_names);
}

std::vector<Rule> parse_rules(const Value& rules, const std::vector<std::string>& type_names,
                              const std::vector<std::string>& material_names) {  // rules.rs:105-203
  std::vector<Rule> out;
  for (auto& kv : rules.map) {
    Rule r;
    r.name = *kv.first->as_str();
    parse_conditionals(kv.second.get(), false, "rules/" + r.name, r, type_names, material_names);
    if (const Value* vm = kv.second->get("mirrored")) {
      if (!vm->as_bool(&r.mirror)) throw Fail{invalid_type("\"mirrored\"", "rules/" + r.name, TYPE_HINT_BOOL)};
    } else {
      r.mirror = true;
    }
    if (r.mirror)
      r.ruletype = Rule::Mirrored;
    else
      r.ruletype = r.do_actions[0].find("LEFT") != std::string::npos ? Rule::Left : Rule::Right;
    bool pre = true;
    if (const Value* vpre = kv.second->get("precondition")) {
      if (!vpre->as_bool(&pre)) throw Fail{invalid_type("\"precondition\"", "rules/" + r.name, TYPE_HINT_BOOL)};
    }
    r.has_precondition = pre;
    r.precondition.clear();
    out.push_back(std::move(r));
  }
  return out;
}

// ---- types.rs ---------------------------------------------------------------------------
void update_precondition(Rule& rule, const std::string& cond) {  // types.rs:78-88
  if (!rule.has_precondition) return;
  rule.precondition = rule.precondition.empty() ? cond : rule.precondition + " || " + cond;
}

void add_child_to_type(const std::string& parent, const std::string& child, std::vector<Type>& types,
                       int depth) {  // types.rs:186-200
  if (depth > 100000) throw Fail{{"Panic", "type inheritance cycle (the reference overflows its stack)"}};
  std::string pp;
  for (auto& t : types)
    if (t.name == parent) {
      t.children.push_back(child);
      pp = t.inherits;
      break;
    }
  if (!pp.empty()) add_child_to_type(pp, child, types, depth + 1);
}

std::vector<std::string> get_parents_rules(const std::vector<Type>& all, const Type& cur,
                                           size_t depth) {  // types.rs:202-210
  if (cur.inherits.empty()) return {};
  if (depth > all.size())
    throw Fail{{"Panic", "type inheritance cycle (the reference overflows its stack)"}};
  const Type* parent = nullptr;
  for (auto& t : all)
    if (t.name == cur.inherits) {
      parent = &t;
      break;
    }
  if (!parent)
    throw Fail{{"Panic", "type '" + cur.name + "' inherits unknown type '" + cur.inherits +
                             "' (the reference panics on unwrap)"}};
  std::vector<std::string> r = parent->base_rules;
  auto more = get_parents_rules(all, *parent, depth + 1);
  r.insert(r.end(), more.begin(), more.end());
  return r;
}

std::vector<Type> parse_types(const Value& types, std::vector<Rule>& rules,
                              const std::vector<std::string>& rule_names,
                              const std::vector<std::string>& type_names) {  // types.rs:51-182
  std::vector<Type> out(3);
  out[0].id = 0, out[0].name = "EMPTY";
  out[1].id = 1, out[1].name = "NULL";
  out[2].id = 2, out[2].name = "WALL";
  size_t idx = 3;
  for (auto& kv : types.map) {
    std::string name = *kv.first->as_str();
    std::string parent;
    if (const Value* vi = kv.second->get("inherits")) {
      const std::string* s = vi->as_str();
      if (!s) throw Fail{invalid_type("\"inherits\"", "types/" + name, TYPE_HINT_STRING)};
      parent = *s;
      for (auto& tn : type_names)
        if (tn == parent) add_child_to_type(parent, name, out, 0);
    }
    std::vector<std::string> base_rules;
    if (const Value* vb = kv.second->get("base_rules")) {
      auto* seq = vb->as_seq();
      if (!seq) throw Fail{invalid_type("\"base_rules\"", "types/" + name, TYPE_HINT_SEQUENCE)};
      for (auto& item : *seq) {
        const std::string* rn = item->as_str();
        if (!rn) throw Fail{invalid_type("\"base_rules\"", "types/" + name, TYPE_HINT_STRING)};
        if (!contains(rule_names, *rn)) throw Fail{not_found(*rn, "types/" + name + "/base_rules")};
        for (auto& r : rules)
          if (r.name == *rn) {
            r.used = true;
            update_precondition(r, "isType_" + name + "(self)");
            break;
          }
        base_rules.push_back(*rn);
      }
    }
    Type t;
    t.id = idx++;
    t.name = name;
    t.inherits = parent;
    t.base_rules = base_rules;
    out.push_back(t);
  }
  const std::vector<Type> snapshot = out;
  for (const Type& t : snapshot) {
    if (t.inherits.empty()) continue;
    for (const std::string& rn : get_parents_rules(snapshot, t, 0))
      for (auto& r : rules)
        if (r.name == rn) {
          update_precondition(r, "isType_" + t.name + "(self)");
          break;
        }
  }
  return out;
}

// ---- materials.rs + parser.rs:191-250 --------------------------------------------------
void extract_vec4(const Value* data, const std::string& parent, const std::string& field,
                  const float def[4], bool mandatory, float out[4]) {
  std::string in = "materials/" + parent + "/" + field;
  for (int i = 0; i < 4; ++i) out[i] = def[i];
  const Value* v = data->get(field);
  if (!v) {
    if (mandatory) throw Fail{missing_field(field, in)};
    return;
  }
  auto* seq = v->as_seq();
  if (!seq || seq->size() < 3 || seq->size() > 4) throw Fail{invalid_type("\"" + field + "\"", in, TYPE_HINT_COLOR)};
  for (size_t i = 0; i < seq->size(); ++i) {
    const Value& c = *(*seq)[i];
    uint64_t u;
    if (c.as_u64(&u) && u > 0 && u <= 255) {
      out[i] = (float)u / 255.0f;
      continue;
    }
    double f;
    if (c.as_f64(&f)) {
      if (f > 1.0 && f <= 255.0) {
        out[i] = (float)f / 255.0f;
        continue;
      }
      if (f >= 0.0 && f <= 1.0) {
        out[i] = (float)f;
        continue;
      }
    }
    throw Fail{invalid_type("\"" + field + "\"", in, TYPE_HINT_COLOR)};
  }
}

std::vector<Material> parse_materials(const Value& mats, std::vector<Rule>& rules,
                                      const std::vector<std::string>& type_names) {  // materials.rs:51-201
  std::vector<Material> out(3);
  out[0] = Material{0, "EMPTY", "EMPTY", {0, 0, 0, 0}, {0, 0, 0, 0}, true, 1.0f, {}};
  out[1] = Material{1, "NULL", "NULL", {1, 0, 1, 1}, {0, 0, 0, 0}, false, 0.0f, {}};
  out[2] = Material{2, "WALL", "WALL", {0.1f, 0.2f, 0.3f, 1.0f}, {0, 0, 0, 0}, false, 9999.0f, {}};
  size_t idx = 3;
  for (auto& kv : mats.map) {
    Material m;
    m.name = *kv.first->as_str();
    const Value* d = kv.second.get();
    const Value* vt = d->get("type");
    if (!vt) throw Fail{missing_field("type", "materials/" + m.name)};
    const std::string* ts = vt->as_str();
    if (!ts) throw Fail{invalid_type("\"type\"", "materials/" + m.name, TYPE_HINT_STRING)};
    m.mattype = *ts;
    if (!contains(type_names, m.mattype)) throw Fail{not_found(m.mattype, "materials/" + m.name + "/type")};
    const float cdef[4] = {1, 0, 1, 1}, edef[4] = {0, 0, 0, 0};
    extract_vec4(d, m.name, "color", cdef, true, m.color);
    extract_vec4(d, m.name, "emission", edef, false, m.emission);
    if (const Value* vs = d->get("selectable")) {
      bool b;
      m.selectable = vs->as_bool(&b) ? b : false;
    } else {
      m.selectable = true;
    }
    const Value* vd = d->get("density");
    if (!vd) throw Fail{missing_field("density", "materials/" + m.name)};
    double dens;
    if (!vd->as_f64(&dens)) throw Fail{invalid_type("\"density\"", "materials/" + m.name + "/density", TYPE_HINT_FLOAT)};
    m.density = (float)dens;
    if (const Value* vx = d->get("extra_rules")) {
      auto* seq = vx->as_seq();
      if (!seq) throw Fail{invalid_type("\"extra_rules\"", "materials/" + m.name, TYPE_HINT_SEQUENCE)};
      for (auto& item : *seq) {
        const std::string* rn = item->as_str();
        if (!rn) throw Fail{invalid_type("\"extra_rules\"", "materials/" + m.name, TYPE_HINT_STRING)};
        for (auto& r : rules)
          if (r.name == *rn) {
            r.used = true;
            update_precondition(r, "self.mat == MAT_" + m.name);
            m.extra_rules.push_back(*rn);
          }
      }
    }
    m.id = idx++;
    out.push_back(m);
  }
  return out;
}

const Value* check_mapping(const Value* data, const std::string& key) {  // parser.rs:174-187
  const Value* v = data ? data->get(key) : nullptr;
  if (!v) throw Fail{missing_field(key, "Root/ Base level of YAML file")};
  if (!v->is_map()) throw Fail{invalid_type(v->debug(), "Root/ Base level of YAML file", TYPE_HINT_MAPPING)};
  return v;
}

std::vector<std::string> preparse_keys(const Value& m, const std::string& err_name) {  // parser.rs:156-168
  std::vector<std::string> names;
  for (auto& kv : m.map) {
    const std::string* s = kv.first->as_str();
    if (!s) throw Fail{invalid_type(kv.first->debug(), err_name, TYPE_HINT_STRING)};
    names.push_back(*s);
  }
  return names;
}

// rules.rs:47-73
std::string func_logic(std::vector<std::string>& conds, std::vector<std::string>& dos, std::vector<float>& probs,
                       size_t lvl) {
  if (conds.empty() && dos.empty()) return "";
  if (conds.empty()) {
    std::string d = dos.front();
    dos.erase(dos.begin());
    return d;
  }
  if (dos.empty()) return "";
  std::string ind1(lvl * 4, ' '), ind2((lvl + 1) * 4, ' ');
  float p = probs.front();
  probs.erase(probs.begin());
  std::string prob = p == 1.0f ? "" : "rand.y <= " + f32_display(p) + " && ";
  std::string c = conds.front();
  conds.erase(conds.begin());
  std::string d = dos.front();
  dos.erase(dos.begin());
  std::string inner = func_logic(conds, dos, probs, lvl + 1);
  return ind1 + "if (" + prob + c + ") {\n" + ind2 + d + "\n" + ind1 + "} else {\n" + inner + "\n" + ind1 + "}";
}

const char* CALLER_HEAD =
    "    inout Cell self,\n    inout Cell right,\n    inout Cell down,\n    inout Cell downright,\n"
    "    vec4 rand,\n    ivec2 pos) {\n";

}  // namespace

std::string f32_display(float f) {
  if (std::isnan(f)) return "NaN";
  if (std::isinf(f)) return f > 0 ? "inf" : "-inf";
  char buf[128];
  auto r = std::to_chars(buf, buf + sizeof buf, f, std::chars_format::fixed);
  return std::string(buf, r.ptr);
}

bool parse_string(const std::string& text, ParsingResult* out, ParseError* err) {
  try {
    std::string yerr;
    auto data = yaml::parse(text, &yerr);
    if (!data) throw Fail{{"Yaml", yerr}};
    const Value* raw_rules = check_mapping(data.get(), "rules");
    const Value* raw_types = check_mapping(data.get(), "types");
    const Value* raw_mats = check_mapping(data.get(), "materials");
    auto rule_names = preparse_keys(*raw_rules, "rules");
    auto type_names = preparse_keys(*raw_types, "types");
    type_names.push_back("EMPTY");
    auto material_names = preparse_keys(*raw_mats, "materials");
    material_names.push_back("EMPTY");
    ParsingResult r;
    try {
      r.rules = parse_rules(*raw_rules, type_names, material_names);
    } catch (Fail& f) {
      throw Fail{wrap("rules", f.e)};
    }
    try {
      r.types = parse_types(*raw_types, r.rules, rule_names, type_names);
    } catch (Fail& f) {
      throw Fail{wrap("types", f.e)};
    }
    try {
      r.materials = parse_materials(*raw_mats, r.rules, type_names);
    } catch (Fail& f) {
      throw Fail{wrap("materials", f.e)};
    }
    *out = std::move(r);
    return true;
  } catch (Fail& f) {
    if (err) *err = f.e;
    return false;
  }
}

std::string rule_glsl(const Rule& r) {
  std::string celldir = r.ruletype == Rule::Left ? "left" : "right";
  std::string pre = r.has_precondition ? "    if (!(" + r.precondition + ")) {\n        return;\n    }\n" : "";
  auto conds = r.if_conds;
  auto dos = r.do_actions;
  auto probs = r.probabilities;
  return "void rule_" + r.name + " (inout Cell self, inout Cell " + celldir +
         ", inout Cell down, inout Cell downright, vec4 rand, ivec2 pos) {\n" + pre +
         func_logic(conds, dos, probs, 1) + "\n}";
}

std::string materials_glsl(const ParsingResult& r) {
  std::string out;
  for (auto& t : r.types) out += "#define TYPE_" + t.name + " " + std::to_string(t.id) + "\n\n";
  for (auto& t : r.types) {
    std::string tc = "return cell.mat.type == TYPE_" + t.name;
    for (auto& c : t.children) tc += " || cell.mat.type == TYPE_" + c;
    out += "bool isType_" + t.name + "(Cell cell) {\n    " + tc + ";\n}\n\n";
  }
  out += "\n";
  std::string lst;
  size_t n = r.materials.size();
  for (size_t i = 0; i < n; ++i) {
    const Material& m = r.materials[i];
    out += "#define MAT_" + m.name + " Material(" + std::to_string(m.id) + ", vec4(" + f32_display(m.color[0]) +
           ", " + f32_display(m.color[1]) + ", " + f32_display(m.color[2]) + ", " + f32_display(m.color[3]) +
           "), " + f32_display(m.density) + ", vec4(" + f32_display(m.emission[0]) + ", " +
           f32_display(m.emission[1]) + ", " + f32_display(m.emission[2]) + ", " + f32_display(m.emission[3]) +
           "), TYPE_" + m.mattype + ")\n";
    lst += "        MAT_" + m.name + (i == n - 1 ? "" : ",\n");
  }
  std::string ns = std::to_string(n);
  out += "\nMaterial[" + ns + "] materials() {\n    Material allMaterials[" + ns + "] = {\n" + lst +
         "\n    };\n    return allMaterials;\n}\n\nMaterial getMaterialFromID(int id) {\n"
         "    for (int i = 0; i < materials().length(); i++) {\n        if (id == materials()[i].id) {\n"
         "            return materials()[i];\n        };\n    };\n    return MAT_NULL;\n}\n\n";
  return out;
}

std::string rules_glsl(const ParsingResult& r) {
  std::string funcs, mirrored, left, right;
  for (auto& rule : r.rules) {
    if (!rule.used) continue;
    funcs += rule_glsl(rule) + "\n\n";
    switch (rule.ruletype) {
      case Rule::Mirrored: mirrored += "rule_" + rule.name + "(self, right, down, downright, rand, pos);\n"; break;
      case Rule::Left: left += "rule_" + rule.name + "(self, left, down, downright, rand, pos);\n"; break;
      case Rule::Right: right += "rule_" + rule.name + "(self, right, down, downright, rand, pos);\n"; break;
    }
  }
  return "\n// =============== RULES ===============\n" + funcs +
         "\n\n\n// =============== CALLERS ===============\nvoid applyMirroredRules(\n" + CALLER_HEAD + "    " +
         rtrim(mirrored) + "\n}\n\n\nvoid applyLeftRules(\n" + CALLER_HEAD + "    " + rtrim(left) +
         "\n}\n\nvoid applyRightRules(\n" + CALLER_HEAD + "    " + rtrim(right) + "\n}";
}

}  // namespace se::lang
