#include "yaml.hpp"

#include <cmath>
#include <cstdlib>
#include <cstring>
#include <stdexcept>

namespace se::yaml {

bool Value::as_f64(double* out) const {
  if (kind == Float) {
    *out = f;
    return true;
  }
  if (kind == Int) {
    *out = int_negative ? -(double)u : (double)u;
    return true;
  }
  return false;
}

bool Value::as_u64(uint64_t* out) const {
  if (kind != Int || int_negative) return false;
  *out = u;
  return true;
}

const Value* Value::get(const std::string& key) const {
  if (kind != Map) return nullptr;
  for (auto& kv : map)
    if (kv.first->kind == String && kv.first->s == key) return kv.second.get();
  return nullptr;
}

std::string Value::debug() const {
  switch (kind) {
    case Null: return "Null";
    case Bool: return b ? "Bool(true)" : "Bool(false)";
    case Int: return std::string("Number(") + (int_negative ? "-" : "") + std::to_string(u) + ")";
    case Float: {
      char buf[64];
      snprintf(buf, sizeof buf, "Number(%g)", f);
      return buf;
    }
    case String: return "String(\"" + s + "\")";
    case Seq: return "Sequence";
    case Map: return "Mapping";
  }
  return "?";
}

namespace {

struct Err : std::runtime_error {
  using std::runtime_error::runtime_error;
};

ValuePtr mk(Value::Kind k) {
  auto v = std::make_shared<Value>();
  v->kind = k;
  return v;
}

bool all_of(const std::string& s, size_t i, bool (*pred)(char)) {
  if (i >= s.size()) return false;
  for (; i < s.size(); ++i)
    if (!pred(s[i])) return false;
  return true;
}
bool isdig(char c) { return c >= '0' && c <= '9'; }
bool ishex(char c) { return isdig(c) || (c >= 'a' && c <= 'f') || (c >= 'A' && c <= 'F'); }
bool isoct(char c) { return c >= '0' && c <= '7'; }

bool is_float_literal(const std::string& s) {
  // [-+]?(\.[0-9]+|[0-9]+(\.[0-9]*)?)([eE][-+]?[0-9]+)?
  size_t i = 0, n = s.size();
  if (i < n && (s[i] == '+' || s[i] == '-')) ++i;
  size_t digits = 0;
  if (i < n && s[i] == '.') {
    ++i;
    while (i < n && isdig(s[i])) ++i, ++digits;
    if (!digits) return false;
  } else {
    while (i < n && isdig(s[i])) ++i, ++digits;
    if (!digits) return false;
    if (i < n && s[i] == '.') {
      ++i;
      while (i < n && isdig(s[i])) ++i;
    }
  }
  if (i < n && (s[i] == 'e' || s[i] == 'E')) {
    ++i;
    if (i < n && (s[i] == '+' || s[i] == '-')) ++i;
    size_t e = 0;
    while (i < n && isdig(s[i])) ++i, ++e;
    if (!e) return false;
  }
  return i == n;
}

// Core-schema resolution of a plain scalar.
ValuePtr resolve_plain(const std::string& s) {
  if (s.empty() || s == "~" || s == "null" || s == "Null" || s == "NULL") return mk(Value::Null);
  if (s == "true" || s == "True" || s == "TRUE" || s == "false" || s == "False" || s == "FALSE") {
    auto v = mk(Value::Bool);
    v->b = s[0] == 't' || s[0] == 'T';
    return v;
  }
  {
    size_t i = 0;
    bool neg = false;
    if (s[0] == '+' || s[0] == '-') {
      neg = s[0] == '-';
      i = 1;
    }
    if (all_of(s, i, isdig)) {
      errno = 0;
      unsigned long long u = strtoull(s.c_str() + i, nullptr, 10);
      bool fits = errno != ERANGE && (!neg || u <= (1ull << 63));
      if (fits) {
        auto v = mk(Value::Int);
        v->u = u;
        v->int_negative = neg && u != 0;
        return v;
      }
      auto v = mk(Value::Float);
      v->f = strtod(s.c_str(), nullptr);
      return v;
    }
  }
  if (s.size() > 2 && s[0] == '0' && s[1] == 'x' && all_of(s, 2, ishex)) {
    auto v = mk(Value::Int);
    v->u = strtoull(s.c_str() + 2, nullptr, 16);
    return v;
  }
  if (s.size() > 2 && s[0] == '0' && s[1] == 'o' && all_of(s, 2, isoct)) {
    auto v = mk(Value::Int);
    v->u = strtoull(s.c_str() + 2, nullptr, 8);
    return v;
  }
  if (is_float_literal(s)) {
    auto v = mk(Value::Float);
    v->f = strtod(s.c_str(), nullptr);
    return v;
  }
  std::string low;
  for (char c : s) low += (char)tolower((unsigned char)c);
  if (low == ".inf" || low == "+.inf" || low == "-.inf" || low == ".nan") {
    auto v = mk(Value::Float);
    v->f = low == ".nan" ? NAN : (low[0] == '-' ? -INFINITY : INFINITY);
    return v;
  }
  auto v = mk(Value::String);
  v->s = s;
  return v;
}

std::string rstrip(const std::string& s) {
  size_t e = s.size();
  while (e && (s[e - 1] == ' ' || s[e - 1] == '\t' || s[e - 1] == '\r')) --e;
  return s.substr(0, e);
}
std::string strip(const std::string& s) {
  size_t b = 0;
  while (b < s.size() && (s[b] == ' ' || s[b] == '\t')) ++b;
  return rstrip(s.substr(b));
}

std::string strip_comment(const std::string& line) {
  std::string out;
  char q = 0, prev = ' ';
  for (char ch : line) {
    if (q) {
      out += ch;
      if (ch == q) q = 0;
    } else {
      if ((ch == '\'' || ch == '"') && (out.empty() || strchr(" \t[{,:", prev))) q = ch;
      else if (ch == '#' && (prev == ' ' || prev == '\t')) break;
      out += ch;
    }
    prev = ch;
  }
  return rstrip(out);
}

ValuePtr unquote(const std::string& tok) {
  if (tok.size() < 2 || tok.back() != tok.front()) throw Err("unterminated quoted scalar: " + tok);
  auto v = mk(Value::String);
  std::string body = tok.substr(1, tok.size() - 2);
  if (tok[0] == '\'') {
    for (size_t i = 0; i < body.size(); ++i) {
      v->s += body[i];
      if (body[i] == '\'' && i + 1 < body.size() && body[i + 1] == '\'') ++i;
    }
  } else {
    for (size_t i = 0; i < body.size(); ++i) {
      char c = body[i];
      if (c == '\\' && i + 1 < body.size()) {
        char e = body[++i];
        switch (e) {
          case 'n': v->s += '\n'; break;
          case 't': v->s += '\t'; break;
          case '\\': v->s += '\\'; break;
          case '"': v->s += '"'; break;
          case '0': v->s += '\0'; break;
          default: v->s += '\\'; v->s += e;
        }
      } else {
        v->s += c;
      }
    }
  }
  return v;
}

ValuePtr scalar(const std::string& tok0) {
  std::string tok = strip(tok0);
  if (!tok.empty() && (tok[0] == '\'' || tok[0] == '"')) return unquote(tok);
  return resolve_plain(tok);
}

bool key_equal(const Value& a, const Value& b) {
  if (a.kind != b.kind) return false;
  switch (a.kind) {
    case Value::Null: return true;
    case Value::Bool: return a.b == b.b;
    case Value::Int: return a.u == b.u && a.int_negative == b.int_negative;
    case Value::Float: return a.f == b.f;
    case Value::String: return a.s == b.s;
    default: return false;
  }
}

struct FlowParser {
  const std::string& t;
  size_t p = 0;
  explicit FlowParser(const std::string& s) : t(s) {}
  void ws() {
    while (p < t.size() && (t[p] == ' ' || t[p] == '\t' || t[p] == '\n')) ++p;
  }
  ValuePtr node() {
    ws();
    if (p >= t.size()) throw Err("unexpected end of flow collection");
    char c = t[p];
    if (c == '[') {
      ++p;
      auto v = mk(Value::Seq);
      ws();
      if (p < t.size() && t[p] == ']') {
        ++p;
        return v;
      }
      for (;;) {
        v->seq.push_back(node());
        ws();
        if (p < t.size() && t[p] == ',') {
          ++p;
          ws();
          if (p < t.size() && t[p] == ']') {
            ++p;
            return v;
          }
          continue;
        }
        if (p < t.size() && t[p] == ']') {
          ++p;
          return v;
        }
        throw Err("bad flow sequence: " + t);
      }
    }
    if (c == '{') {
      ++p;
      auto v = mk(Value::Map);
      ws();
      if (p < t.size() && t[p] == '}') {
        ++p;
        return v;
      }
      for (;;) {
        auto k = node();
        ws();
        ValuePtr val = mk(Value::Null);
        if (p < t.size() && t[p] == ':') {
          ++p;
          val = node();
        }
        for (auto& kv : v->map)
          if (key_equal(*kv.first, *k)) throw Err("duplicate entry with key " + k->debug());
        v->map.emplace_back(k, val);
        ws();
        if (p < t.size() && t[p] == ',') {
          ++p;
          continue;
        }
        if (p < t.size() && t[p] == '}') {
          ++p;
          return v;
        }
        throw Err("bad flow mapping: " + t);
      }
    }
    if (c == '\'' || c == '"') {
      size_t e = p + 1;
      while (e < t.size()) {
        if (t[e] == c) {
          if (c == '\'' && e + 1 < t.size() && t[e + 1] == '\'') {
            e += 2;
            continue;
          }
          break;
        }
        if (c == '"' && t[e] == '\\') ++e;
        ++e;
      }
      std::string tok = t.substr(p, e + 1 - p);
      p = e + 1;
      return unquote(tok);
    }
    size_t s = p;
    while (p < t.size() && t[p] != ',' && t[p] != ']' && t[p] != '}') {
      if (t[p] == ':' && (p + 1 >= t.size() || strchr(" ,]}", t[p + 1]))) break;
      ++p;
    }
    return resolve_plain(strip(t.substr(s, p - s)));
  }
};

ValuePtr parse_flow(const std::string& text) {
  FlowParser fp(text);
  auto v = fp.node();
  fp.ws();
  if (fp.p != text.size()) throw Err("trailing characters after flow collection: " + text);
  return v;
}

long find_colon(const std::string& s) {
  char q = 0;
  int depth = 0;
  for (size_t i = 0; i < s.size(); ++i) {
    char ch = s[i];
    if (q) {
      if (ch == q) q = 0;
      continue;
    }
    if ((ch == '\'' || ch == '"') && (i == 0 || strchr(" \t[{,", s[i - 1]))) q = ch;
    else if (ch == '[' || ch == '{') ++depth;
    else if (ch == ']' || ch == '}') --depth;
    else if (ch == ':' && depth == 0 && (i + 1 == s.size() || s[i + 1] == ' ' || s[i + 1] == '\t'))
      return (long)i;
  }
  return -1;
}

bool starts_seq(const std::string& t) { return t == "-" || (t.size() > 1 && t[0] == '-' && t[1] == ' '); }

struct Line {
  int indent;  // -1 for blank
  std::string text;
};

struct BlockParser {
  std::vector<Line> lines;
  size_t pos = 0;

  void skip_blank() {
    while (pos < lines.size() && lines[pos].indent < 0) ++pos;
  }

  static int balance(const std::string& t) {
    int d = 0;
    char q = 0;
    for (char ch : t) {
      if (q) {
        if (ch == q) q = 0;
      } else if (ch == '\'' || ch == '"') {
        q = ch;
      } else if (ch == '[' || ch == '{') {
        ++d;
      } else if (ch == ']' || ch == '}') {
        --d;
      }
    }
    return d;
  }

  std::string gather_flow(const std::string& first) {
    std::string buf = first;
    while (balance(buf) > 0) {
      if (pos >= lines.size()) throw Err("unterminated flow collection");
      const Line& l = lines[pos++];
      if (l.indent < 0) continue;
      buf += " " + l.text;
    }
    return buf;
  }

  ValuePtr value_text(const std::string& t, int parent_indent) {
    if (!t.empty() && (t[0] == '[' || t[0] == '{')) return parse_flow(gather_flow(t));
    if (!t.empty() && (t[0] == '|' || t[0] == '>')) throw Err("block scalars are not supported");
    if (!t.empty() && (t[0] == '&' || t[0] == '*' || t[0] == '!'))
      throw Err("anchors, aliases and tags are not supported");
    if (!t.empty() && (t[0] == '\'' || t[0] == '"')) return scalar(t);
    std::string joined = t;
    for (;;) {
      size_t save = pos;
      skip_blank();
      if (pos < lines.size() && lines[pos].indent > parent_indent && find_colon(lines[pos].text) < 0 &&
          !starts_seq(lines[pos].text)) {
        joined += " " + lines[pos].text;
        ++pos;
        continue;
      }
      pos = save;
      break;
    }
    return resolve_plain(joined);
  }

  ValuePtr block(int indent) {
    skip_blank();
    if (pos >= lines.size()) return mk(Value::Null);
    const Line& l = lines[pos];
    if (starts_seq(l.text)) return seq(l.indent);
    if (find_colon(l.text) >= 0) return map(l.indent);
    ++pos;
    return value_text(l.text, indent - 1);
  }

  ValuePtr seq(int indent) {
    auto v = mk(Value::Seq);
    for (;;) {
      skip_blank();
      if (pos >= lines.size()) break;
      Line l = lines[pos];
      if (l.indent != indent || !starts_seq(l.text)) {
        if (l.indent > indent) throw Err("bad indentation in sequence: " + l.text);
        break;
      }
      std::string rest = strip(l.text.substr(1));
      ++pos;
      if (rest.empty()) {
        skip_blank();
        if (pos < lines.size() && lines[pos].indent > indent)
          v->seq.push_back(block(lines[pos].indent));
        else
          v->seq.push_back(mk(Value::Null));
      } else if (find_colon(rest) >= 0 && !strchr("[{'\"", rest[0])) {
        int sub = indent + 2;
        lines.insert(lines.begin() + (long)pos, Line{sub, rest});
        v->seq.push_back(map(sub));
      } else {
        v->seq.push_back(value_text(rest, indent));
      }
    }
    return v;
  }

  ValuePtr map(int indent) {
    auto v = mk(Value::Map);
    for (;;) {
      skip_blank();
      if (pos >= lines.size()) break;
      Line l = lines[pos];
      if (l.indent < indent) break;
      if (l.indent > indent) throw Err("bad indentation: " + l.text);
      long c = find_colon(l.text);
      if (c < 0) throw Err("could not find expected ':' in " + l.text);
      std::string ktext = l.text.substr(0, (size_t)c);
      ValuePtr key = strip(ktext).empty() ? mk(Value::Null) : scalar(ktext);
      std::string rest = strip(l.text.substr((size_t)c + 1));
      ++pos;
      ValuePtr val;
      if (rest.empty()) {
        skip_blank();
        if (pos < lines.size() && lines[pos].indent > indent)
          val = block(lines[pos].indent);
        else if (pos < lines.size() && lines[pos].indent == indent && starts_seq(lines[pos].text))
          val = seq(indent);
        else
          val = mk(Value::Null);
      } else {
        val = value_text(rest, indent);
      }
      for (auto& kv : v->map)
        if (key_equal(*kv.first, *key)) throw Err("duplicate entry with key " + key->debug());
      v->map.emplace_back(key, val);
    }
    return v;
  }
};

}  // namespace

ValuePtr parse(const std::string& text, std::string* err) {
  try {
    BlockParser bp;
    std::string cur;
    std::vector<std::string> raw;
    for (size_t i = 0; i <= text.size(); ++i) {
      if (i == text.size() || text[i] == '\n') {
        raw.push_back(cur);
        cur.clear();
      } else {
        cur += text[i];
      }
    }
    for (auto& r0 : raw) {
      std::string r;
      for (char c : r0) {
        if (c == '\t') r += "    ";
        else r += c;
      }
      std::string s = strip_comment(r);
      std::string st = strip(s);
      if (st.empty() || st == "---") {
        bp.lines.push_back(Line{-1, ""});
        continue;
      }
      if (st == "...") break;
      int ind = 0;
      while (ind < (int)s.size() && s[(size_t)ind] == ' ') ++ind;
      bp.lines.push_back(Line{ind, st});
    }
    bp.skip_blank();
    if (bp.pos >= bp.lines.size()) return mk(Value::Null);
    auto doc = bp.block(bp.lines[bp.pos].indent);
    bp.skip_blank();
    if (bp.pos < bp.lines.size()) throw Err("unexpected content: " + bp.lines[bp.pos].text);
    return doc;
  } catch (const std::exception& e) {
    if (err) *err = e.what();
    return nullptr;
  }
}

}  // namespace se::yaml
