#include "codegen.hpp"

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <set>
#include <sstream>
#include <vector>

namespace se::lang {
namespace {

struct Fail {
  ParseError e;
};
[[noreturn]] void glsl_error(const std::string& rule, const std::string& msg) {
  throw Fail{{"Glsl", "(Glsl) rule_" + rule + ": " + msg + " (the reference's shader would not compile)"}};
}
[[noreturn]] void unsupported(const std::string& rule, const std::string& msg) {
  throw Fail{{"Unsupported", "(Unsupported) rule_" + rule + ": " + msg +
                                 " is valid shader code but outside the CUDA back end's rule subset"}};
}

// ---- lexer -----------------------------------------------------------------------------
enum class T { Ident, Int, UInt, Float, Punct, End };
struct Tok {
  T t;
  std::string s;
  double f = 0;    // Float: the binary32 value
  uint64_t u = 0;  // Int/UInt
};

std::vector<Tok> lex(const std::string& src, const std::string& rule) {
  std::vector<Tok> out;
  size_t i = 0, n = src.size();
  auto isid0 = [](char c) { return isalpha((unsigned char)c) || c == '_'; };
  auto isid = [](char c) { return isalnum((unsigned char)c) || c == '_'; };
  static const char* puncts[] = {"&&", "||", "^^", "==", "!=", "<=", ">=", "++", "--", "+=", "-=", "*=",
                                 "/=", "<<", ">>", "%=", "&=", "|=", "^="};
  while (i < n) {
    char c = src[i];
    if (isspace((unsigned char)c)) {
      ++i;
      continue;
    }
    if (c == '/' && i + 1 < n && src[i + 1] == '/') {
      while (i < n && src[i] != '\n') ++i;
      continue;
    }
    if (c == '/' && i + 1 < n && src[i + 1] == '*') {
      size_t e = src.find("*/", i + 2);
      if (e == std::string::npos) glsl_error(rule, "unterminated comment");
      i = e + 2;
      continue;
    }
    if (isid0(c)) {
      size_t s = i;
      while (i < n && isid(src[i])) ++i;
      out.push_back({T::Ident, src.substr(s, i - s)});
      continue;
    }
    if (isdigit((unsigned char)c) || (c == '.' && i + 1 < n && isdigit((unsigned char)src[i + 1]))) {
      size_t s = i;
      bool is_float = false;
      if (c == '0' && i + 1 < n && (src[i + 1] == 'x' || src[i + 1] == 'X')) {
        i += 2;
        while (i < n && isxdigit((unsigned char)src[i])) ++i;
      } else {
        while (i < n && isdigit((unsigned char)src[i])) ++i;
        if (i < n && src[i] == '.') {
          is_float = true;
          ++i;
          while (i < n && isdigit((unsigned char)src[i])) ++i;
        }
        if (i < n && (src[i] == 'e' || src[i] == 'E')) {
          size_t save = i++;
          if (i < n && (src[i] == '+' || src[i] == '-')) ++i;
          if (i < n && isdigit((unsigned char)src[i])) {
            is_float = true;
            while (i < n && isdigit((unsigned char)src[i])) ++i;
          } else {
            i = save;
          }
        }
      }
      std::string lit = src.substr(s, i - s);
      Tok t;
      if (is_float) {
        if (i < n && (src[i] == 'f' || src[i] == 'F')) ++i;
        else if (i + 1 < n && (src[i] == 'l' || src[i] == 'L') && (src[i + 1] == 'f' || src[i + 1] == 'F'))
          unsupported(rule, "double literal '" + lit + "'");
        t.t = T::Float;
        t.f = (double)strtof(lit.c_str(), nullptr);
      } else {
        bool uns = false;
        if (i < n && (src[i] == 'u' || src[i] == 'U')) {
          uns = true;
          ++i;
        }
        errno = 0;
        unsigned long long v;
        if (lit.size() > 2 && (lit[1] == 'x' || lit[1] == 'X'))
          v = strtoull(lit.c_str() + 2, nullptr, 16);
        else if (lit.size() > 1 && lit[0] == '0')
          v = strtoull(lit.c_str(), nullptr, 8);
        else
          v = strtoull(lit.c_str(), nullptr, 10);
        if (errno == ERANGE || v > 0xffffffffull) glsl_error(rule, "integer literal '" + lit + "' is too large");
        t.t = uns ? T::UInt : T::Int;
        t.u = v;
      }
      t.s = lit;
      if (i < n && isid(src[i])) glsl_error(rule, "bad numeric literal near '" + lit + "'");
      out.push_back(t);
      continue;
    }
    std::string p(1, c);
    for (const char* q : puncts)
      if (src.compare(i, strlen(q), q) == 0) {
        p = q;
        break;
      }
    i += p.size();
    out.push_back({T::Punct, p});
  }
  out.push_back({T::End, ""});
  return out;
}

// ---- AST -------------------------------------------------------------------------------
struct Expr;
using EP = std::unique_ptr<Expr>;
struct Expr {
  enum K { Lit, Id, Member, Call, Unary, Binary, Ternary, Assign } k;
  Tok lit;            // Lit
  std::string name;   // Id / Member field / Call callee / operator
  std::vector<EP> a;  // operands / args
};
struct Stmt;
using SP = std::unique_ptr<Stmt>;
struct Stmt {
  enum K { Block, If, Return, ExprS, Empty } k;
  std::vector<SP> body;  // Block
  EP e;                  // If cond / ExprS
  SP then_s, else_s;
};

struct Parser {
  std::vector<Tok> t;
  size_t p = 0;
  std::string rule;
  const Tok& peek(size_t o = 0) const { return t[std::min(p + o, t.size() - 1)]; }
  bool is(const char* s) const { return peek().t == T::Punct && peek().s == s; }
  bool is_ident(const char* s) const { return peek().t == T::Ident && peek().s == s; }
  void expect(const char* s) {
    if (!is(s)) glsl_error(rule, std::string("expected '") + s + "' near '" + peek().s + "'");
    ++p;
  }

  static int binprec(const std::string& op) {
    static const std::map<std::string, int> m = {
        {"||", 1}, {"^^", 2}, {"&&", 3}, {"|", 4},  {"^", 5},  {"&", 6},  {"==", 7}, {"!=", 7},
        {"<", 8},  {">", 8},  {"<=", 8}, {">=", 8}, {"<<", 9}, {">>", 9}, {"+", 10}, {"-", 10},
        {"*", 11}, {"/", 11}, {"%", 11}};
    auto it = m.find(op);
    return it == m.end() ? -1 : it->second;
  }

  EP primary() {
    const Tok& tk = peek();
    if (tk.t == T::Int || tk.t == T::UInt || tk.t == T::Float) {
      auto e = std::make_unique<Expr>();
      e->k = Expr::Lit;
      e->lit = tk;
      ++p;
      return e;
    }
    if (tk.t == T::Ident) {
      auto e = std::make_unique<Expr>();
      e->name = tk.s;
      ++p;
      if (is("(")) {
        ++p;
        e->k = Expr::Call;
        if (!is(")")) {
          for (;;) {
            e->a.push_back(assignment());
            if (is(",")) {
              ++p;
              continue;
            }
            break;
          }
        }
        expect(")");
      } else {
        e->k = Expr::Id;
      }
      return e;
    }
    if (is("(")) {
      ++p;
      EP e = expression();
      expect(")");
      return e;
    }
    glsl_error(rule, "unexpected '" + tk.s + "'");
  }
  EP postfix() {
    EP e = primary();
    for (;;) {
      if (is(".")) {
        ++p;
        if (peek().t != T::Ident) glsl_error(rule, "expected a field name after '.'");
        auto m = std::make_unique<Expr>();
        m->k = Expr::Member;
        m->name = peek().s;
        ++p;
        m->a.push_back(std::move(e));
        e = std::move(m);
      } else if (is("[")) {
        unsupported(rule, "indexing");
      } else if (is("++") || is("--")) {
        unsupported(rule, "increment/decrement");
      } else {
        return e;
      }
    }
  }
  EP unary() {
    if (is("!") || is("-") || is("+") || is("~")) {
      std::string op = peek().s;
      ++p;
      auto e = std::make_unique<Expr>();
      e->k = Expr::Unary;
      e->name = op;
      e->a.push_back(unary());
      return e;
    }
    if (is("++") || is("--")) unsupported(rule, "increment/decrement");
    return postfix();
  }
  EP binary(int minp) {
    EP lhs = unary();
    for (;;) {
      if (peek().t != T::Punct) return lhs;
      int pr = binprec(peek().s);
      if (pr < minp || pr < 0) return lhs;
      std::string op = peek().s;
      ++p;
      EP rhs = binary(pr + 1);
      auto e = std::make_unique<Expr>();
      e->k = Expr::Binary;
      e->name = op;
      e->a.push_back(std::move(lhs));
      e->a.push_back(std::move(rhs));
      lhs = std::move(e);
    }
  }
  EP conditional() {
    EP c = binary(1);
    if (is("?")) {
      ++p;
      EP x = assignment();
      expect(":");
      EP y = assignment();
      auto e = std::make_unique<Expr>();
      e->k = Expr::Ternary;
      e->a.push_back(std::move(c));
      e->a.push_back(std::move(x));
      e->a.push_back(std::move(y));
      return e;
    }
    return c;
  }
  EP assignment() {
    EP lhs = conditional();
    if (is("=")) {
      ++p;
      EP rhs = assignment();
      auto e = std::make_unique<Expr>();
      e->k = Expr::Assign;
      e->a.push_back(std::move(lhs));
      e->a.push_back(std::move(rhs));
      return e;
    }
    for (const char* op : {"+=", "-=", "*=", "/=", "%=", "&=", "|=", "^="})
      if (is(op)) unsupported(rule, "compound assignment");
    return lhs;
  }
  EP expression() {
    EP e = assignment();
    if (is(",")) unsupported(rule, "comma expressions");
    return e;
  }
  SP statement() {
    auto s = std::make_unique<Stmt>();
    if (is("{")) {
      ++p;
      s->k = Stmt::Block;
      while (!is("}")) {
        if (peek().t == T::End) glsl_error(rule, "missing '}'");
        s->body.push_back(statement());
      }
      ++p;
      return s;
    }
    if (is(";")) {
      ++p;
      s->k = Stmt::Empty;
      return s;
    }
    if (is_ident("if")) {
      ++p;
      expect("(");
      s->k = Stmt::If;
      s->e = expression();
      expect(")");
      s->then_s = statement();
      if (is_ident("else")) {
        ++p;
        s->else_s = statement();
      }
      return s;
    }
    if (is_ident("return")) {
      ++p;
      if (!is(";")) glsl_error(rule, "void function returns a value");
      ++p;
      s->k = Stmt::Return;
      return s;
    }
    for (const char* kw : {"for", "while", "do", "switch", "break", "continue", "discard"})
      if (is_ident(kw)) unsupported(rule, std::string("'") + kw + "' statements");
    for (const char* ty : {"float", "int", "uint", "bool", "vec2", "vec3", "vec4", "ivec2", "ivec3",
                           "ivec4", "uvec2", "uvec3", "uvec4", "Cell", "Material", "const"})
      if (is_ident(ty) && peek(1).t == T::Ident) unsupported(rule, "local variable declarations");
    s->k = Stmt::ExprS;
    s->e = expression();
    expect(";");
    return s;
  }
};

// ---- typing and emission ---------------------------------------------------------------
enum class Ty { Bool, Int, UInt, Float, Cell, Material, Vec4, IVec2, Void };
const char* ty_name(Ty t) {
  switch (t) {
    case Ty::Bool: return "bool";
    case Ty::Int: return "int";
    case Ty::UInt: return "uint";
    case Ty::Float: return "float";
    case Ty::Cell: return "Cell";
    case Ty::Material: return "Material";
    case Ty::Vec4: return "vec4";
    case Ty::IVec2: return "ivec2";
    case Ty::Void: return "void";
  }
  return "?";
}

struct Val {
  Ty ty = Ty::Void;
  std::string code;
  bool is_const = false;
  double cval = 0;      // numeric constant value (Float: the binary32 value)
  int cell_slot = -1;   // Cell lvalue: parameter slot
  int rand_lane = -1;   // Float: rand.<lane>
  int const_mat = -1;   // Material constant id
  enum VecKind { VNone, VRand, VColor, VEmission, VPos, VSimSize } vk = VNone;
  std::string vbase;    // Vec4 material code
};

std::string hexf(float f) {
  char buf[64];
  if (!std::isfinite(f)) {  // no literal spelling; build from the bit pattern
    uint32_t u;
    memcpy(&u, &f, 4);
    snprintf(buf, sizeof buf, "__uint_as_float(0x%08xu)", u);
  } else {
    snprintf(buf, sizeof buf, "%af", (double)f);
  }
  return buf;
}

// Names declared by the reference shader before gen/rules.glsl is included, and GLSL
// built-in functions: referencing one is valid GLSL the back end does not translate.
const std::set<std::string>& shader_names() {
  static const std::set<std::string> s = {
      "getMoveDirs", "PHI", "gold_noise", "hashi", "hash4i", "old_hash2", "hash", "hash2", "hash3",
      "hash4", "hash42", "hash43", "_noise", "noise", "rotatePoint", "getNeighbours",
      "getOnlyDiagonalNeighbours", "getDiagonalNeighbours", "NEIGH_IDX_UP", "NEIGH_IDX_UPLEFT",
      "NEIGH_IDX_UPRIGHT", "NEIGH_IDX_LEFT", "NEIGH_IDX_RIGHT", "NEIGH_IDX_DOWN", "NEIGH_IDX_DOWNLEFT",
      "NEIGH_IDX_DOWNRIGHT", "materials", "getMaterialFromID", "input_data", "output_data", "output_color",
      "moveRight", "time", "collision_data", "input_light", "output_light", "output_effects", "image_lock",
      "MODSHAPE_CIRCLE", "MODSHAPE_SQUARE", "sim_modifications", "outOfBounds", "getMargolusOffset",
      "cellToID", "IDToCell", "getCell", "isCollider", "isLightObstacle", "CalculateNewLight", "gt",
      "setCell", "UP", "DOWN", "LEFT", "RIGHT", "UPLEFT", "UPRIGHT", "DOWNLEFT", "DOWNRIGHT",
      "EMPTY_MAX_DISPERSION_CHECK", "Material", "Cell", "SimModification", "gl_GlobalInvocationID",
      "gl_LocalInvocationID", "gl_WorkGroupID", "gl_NumWorkGroups", "gl_LocalInvocationIndex",
      // GLSL built-ins
      "radians", "degrees", "sin", "cos", "tan", "asin", "acos", "atan", "sinh", "cosh", "tanh", "pow",
      "exp", "log", "exp2", "log2", "sqrt", "inversesqrt", "sign", "floor", "trunc", "round", "roundEven",
      "ceil", "fract", "mod", "modf", "clamp", "mix", "step", "smoothstep", "isnan", "isinf", "length",
      "distance", "dot", "cross", "normalize", "texelFetch", "texture", "imageLoad", "imageStore", "vec2",
      "vec3", "vec4", "ivec2", "ivec3", "ivec4", "uvec2", "uvec3", "uvec4", "bool", "uint",
      "floatBitsToInt", "intBitsToFloat", "any", "all", "not", "lessThan", "greaterThan", "equal",
      "notEqual", "atomicAdd", "barrier", "memoryBarrier", "fma", "frexp", "ldexp", "bitfieldExtract",
      "bitCount", "findLSB", "findMSB", "packUnorm4x8", "unpackUnorm4x8"};
  return s;
}

struct Gen {
  const ParsingResult& R;
  std::string rule;                      // rule name being compiled
  std::vector<std::string> cell_names;   // parameter names, slot order
  std::map<std::string, int> type_ids;   // TYPE_<name> -> id
  int nmat = 0;
  std::vector<int> mat_type;             // material -> type id
  std::vector<bool> mat_nan;
  bool any_nan = false;
  bool used_density = false, used_type = false, used_color = false, used_emission = false;
  bool uses_lane[4] = {false, false, false, false};
  std::set<uint64_t> bounds[4];  // threshold boundaries of rand.<lane> comparisons
  std::string all_bodies;        // generated rule bodies (scanned for table eligibility)
  std::vector<std::vector<bool>> sets;   // material bit sets
  std::map<std::vector<bool>, int> set_index;

  explicit Gen(const ParsingResult& r) : R(r) {}

  int add_set(const std::vector<bool>& s) {
    auto it = set_index.find(s);
    if (it != set_index.end()) return it->second;
    int k = (int)sets.size();
    sets.push_back(s);
    set_index[s] = k;
    return k;
  }

  const Material* find_mat(const std::string& name) const {
    for (auto& m : R.materials)
      if (m.name == name) return &m;
    return nullptr;
  }

  static std::string to_float(const Val& v) {
    if (v.ty == Ty::Float) return v.code;
    if (v.ty == Ty::Int) return "__int2float_rn(" + v.code + ")";
    return "__uint2float_rn(" + v.code + ")";
  }
  static std::string to_uint(const Val& v) { return v.ty == Ty::UInt ? v.code : "(unsigned)(" + v.code + ")"; }
  static bool numeric(Ty t) { return t == Ty::Int || t == Ty::UInt || t == Ty::Float; }

  Val make(Ty t, std::string code) {
    Val v;
    v.ty = t;
    v.code = std::move(code);
    return v;
  }

  // Integer-threshold form of `rand.<lane> OP c` (c a float constant); see header.
  std::string rand_compare(int lane, const std::string& op, float c, bool lane_on_left) {
    std::string o = op;
    if (!lane_on_left) {  // c OP lane  ->  lane OP' c
      if (o == "<") o = ">";
      else if (o == ">") o = "<";
      else if (o == "<=") o = ">=";
      else if (o == ">=") o = "<=";
    }
    uses_lane[lane] = true;
    std::string h = "h" + std::to_string(lane);
    if (std::isnan(c)) return o == "!=" ? "true" : "false";
    auto g = [](uint64_t u) -> float { return (float)(uint32_t)u * 0x1p-32f; };
    // first u in [0, 2^32] with pred(u) true (pred monotone false->true), 2^32 if none
    auto first = [&](auto pred) -> uint64_t {
      uint64_t lo = 0, hi = 1ull << 32;
      while (lo < hi) {
        uint64_t mid = (lo + hi) / 2;
        if (pred(g(mid))) hi = mid;
        else lo = mid + 1;
      }
      return lo;
    };
    uint64_t ge = first([&](float x) { return x >= c; });
    uint64_t gt = first([&](float x) { return x > c; });
    // The comparison is constant between consecutive boundaries: remember them for the
    // block transition table (see generate_cuda).
    auto bound = [&](uint64_t T) {
      if (T > 0 && T < (1ull << 32)) bounds[lane].insert(T);
    };
    if (o == "<" || o == ">=" || o == "==" || o == "!=") bound(ge);
    if (o == "<=" || o == ">" || o == "==" || o == "!=") bound(gt);
    auto lit = [](uint64_t v) {
      char b[32];
      snprintf(b, sizeof b, "0x%08llxu", (unsigned long long)v);
      return std::string(b);
    };
    auto below = [&](uint64_t T) -> std::string {  // u < T
      if (T == 0) return "false";
      if (T >= (1ull << 32)) return "true";
      return "(" + h + " < " + lit(T) + ")";
    };
    auto atleast = [&](uint64_t T) -> std::string {  // u >= T
      if (T == 0) return "true";
      if (T >= (1ull << 32)) return "false";
      return "(" + h + " >= " + lit(T) + ")";
    };
    if (o == "<") return below(ge);
    if (o == "<=") return below(gt);
    if (o == ">") return atleast(gt);
    if (o == ">=") return atleast(ge);
    std::string in_range = ge >= gt ? "false"
                           : (ge == 0 && gt >= (1ull << 32))
                               ? "true"
                               : "((" + h + " - " + lit(ge) + ") < " + lit(gt - ge) + ")";
    return o == "==" ? in_range : "(!" + in_range + ")";
  }

  Val id(const Expr& e) {
    const std::string& n = e.name;
    for (size_t i = 0; i < cell_names.size(); ++i)
      if (n == cell_names[i]) {
        Val v = make(Ty::Cell, n);
        v.cell_slot = (int)i;
        return v;
      }
    if (n == "rand") {
      Val v = make(Ty::Vec4, "");
      v.vk = Val::VRand;
      return v;
    }
    if (n == "pos") {
      Val v = make(Ty::IVec2, "");
      v.vk = Val::VPos;
      return v;
    }
    if (n == "simSize") {
      Val v = make(Ty::IVec2, "");
      v.vk = Val::VSimSize;
      return v;
    }
    if (n == "frame") return make(Ty::Int, "frame");
    if (n == "true" || n == "false") {
      Val v = make(Ty::Bool, n);
      v.is_const = true;
      v.cval = n == "true";
      return v;
    }
    if (n == "SCREEN_IS_BORDER") glsl_error(rule, "SCREEN_IS_BORDER is an empty macro");
    if (n.rfind("MAT_", 0) == 0) {
      const Material* m = find_mat(n.substr(4));
      if (!m) glsl_error(rule, "undeclared identifier '" + n + "'");
      Val v = make(Ty::Material, std::to_string(m->id) + "u");
      v.const_mat = (int)m->id;
      return v;
    }
    if (n.rfind("TYPE_", 0) == 0) {
      auto it = type_ids.find(n.substr(5));
      if (it == type_ids.end()) glsl_error(rule, "undeclared identifier '" + n + "'");
      Val v = make(Ty::Int, std::to_string(it->second));
      v.is_const = true;
      v.cval = it->second;
      return v;
    }
    if (n == "EMPTY_MAX_DISPERSION_CHECK") {
      Val v = make(Ty::Int, "8");
      v.is_const = true;
      v.cval = 8;
      return v;
    }
    if (n == "MODSHAPE_CIRCLE" || n == "MODSHAPE_SQUARE") {
      int c = n == "MODSHAPE_SQUARE";
      Val v = make(Ty::Int, std::to_string(c));
      v.is_const = true;
      v.cval = c;
      return v;
    }
    if (shader_names().count(n)) unsupported(rule, "use of '" + n + "'");
    glsl_error(rule, "undeclared identifier '" + n + "'");
  }

  Val member(const Expr& e) {
    Val b = expr(*e.a[0]);
    const std::string& f = e.name;
    auto comp = [&](const std::string& s) -> int {
      if (s == "x" || s == "r" || s == "s") return 0;
      if (s == "y" || s == "g" || s == "t") return 1;
      if (s == "z" || s == "b" || s == "p") return 2;
      if (s == "w" || s == "a" || s == "q") return 3;
      return -1;
    };
    switch (b.ty) {
      case Ty::Cell:
        if (f == "mat") {
          Val v = make(Ty::Material, b.code);
          return v;
        }
        if (f == "pos") unsupported(rule, "cell positions ('.pos')");
        glsl_error(rule, "Cell has no field '" + f + "'");
      case Ty::Material:
        if (f == "id") return make(Ty::Int, "(int)(" + b.code + ")");
        if (f == "density") {
          used_density = true;
          return make(Ty::Float, "se_gen::density(" + b.code + ")");
        }
        if (f == "type") {
          used_type = true;
          return make(Ty::Int, "se_gen::mtype(" + b.code + ")");
        }
        if (f == "color" || f == "emission") {
          Val v = make(Ty::Vec4, "");
          v.vk = f == "color" ? Val::VColor : Val::VEmission;
          v.vbase = b.code;
          return v;
        }
        glsl_error(rule, "Material has no field '" + f + "'");
      case Ty::Vec4: {
        int c = comp(f);
        if (c < 0) {
          bool swz = f.size() > 1 && f.size() <= 4;
          for (char ch : f) swz = swz && comp(std::string(1, ch)) >= 0;
          if (swz) unsupported(rule, "multi-component swizzles");
          glsl_error(rule, "vec4 has no field '" + f + "'");
        }
        if (b.vk == Val::VRand) {
          Val v = make(Ty::Float, "se_randf(h" + std::to_string(c) + ")");
          v.rand_lane = c;
          uses_lane[c] = true;
          return v;
        }
        if (b.vk == Val::VColor) {
          used_color = true;
          return make(Ty::Float, "se_gen::color(" + b.vbase + ", " + std::to_string(c) + ")");
        }
        used_emission = true;
        return make(Ty::Float, "se_gen::emission(" + b.vbase + ", " + std::to_string(c) + ")");
      }
      case Ty::IVec2: {
        int c = comp(f);
        if (c < 0 || c > 1) glsl_error(rule, "ivec2 has no field '" + f + "'");
        if (b.vk == Val::VPos) return make(Ty::Int, c ? "pos_y" : "pos_x");
        return make(Ty::Int, c ? "sim_h" : "sim_w");
      }
      default:
        glsl_error(rule, std::string("'") + ty_name(b.ty) + "' has no field '" + f + "'");
    }
  }

  Val call(const Expr& e) {
    const std::string& n = e.name;
    if (n.rfind("isType_", 0) == 0) {
      std::string tn = n.substr(7);
      const Type* ty = nullptr;
      for (auto& t : R.types)
        if (t.name == tn) ty = &t;
      if (!ty) glsl_error(rule, "undeclared function '" + n + "'");
      if (e.a.size() != 1) glsl_error(rule, n + " takes one argument");
      Val c = expr(*e.a[0]);
      if (c.ty != Ty::Cell) glsl_error(rule, n + " expects a Cell");
      // types.rs:30-39: cell.mat.type == TYPE_<t> || cell.mat.type == TYPE_<child> ...
      std::set<int> tids = {type_ids.at(ty->name)};
      for (auto& ch : ty->children) tids.insert(type_ids.at(ch));
      std::vector<bool> s((size_t)nmat);
      for (int m = 0; m < nmat; ++m) s[(size_t)m] = tids.count(mat_type[(size_t)m]) > 0;
      int k = add_set(s);
      return make(Ty::Bool, "se_gen::in_set" + std::to_string(k) + "(" + c.code + ")");
    }
    if (n == "newCell") {
      if (e.a.size() != 2) glsl_error(rule, "newCell takes two arguments");
      Val m = expr(*e.a[0]);
      Val p = expr(*e.a[1]);
      if (m.ty != Ty::Material || p.ty != Ty::IVec2) glsl_error(rule, "newCell(Material, ivec2) argument types");
      return make(Ty::Cell, m.code);
    }
    if (n == "swap") {
      if (e.a.size() != 2) glsl_error(rule, "swap takes two arguments");
      Val a = expr(*e.a[0]);
      Val b = expr(*e.a[1]);
      if (a.ty == Ty::Vec4 || b.ty == Ty::Vec4) unsupported(rule, "swap(vec4, vec4)");
      if (a.ty != Ty::Cell || b.ty != Ty::Cell) glsl_error(rule, "no swap overload for these arguments");
      if (a.cell_slot < 0 || b.cell_slot < 0) glsl_error(rule, "swap arguments must be l-values");
      return make(Ty::Void, "se_swap(" + a.code + ", " + b.code + ")");
    }
    if (n == "abs" || n == "min" || n == "max") {
      size_t want = n == "abs" ? 1 : 2;
      if (e.a.size() != want) glsl_error(rule, n + ": wrong number of arguments");
      std::vector<Val> v;
      for (auto& x : e.a) v.push_back(expr(*x));
      bool fl = false;
      for (auto& x : v) {
        if (!numeric(x.ty)) glsl_error(rule, n + ": numeric arguments expected");
        fl = fl || x.ty == Ty::Float;
      }
      if (n == "abs") {
        if (fl) return make(Ty::Float, "fabsf(" + v[0].code + ")");
        if (v[0].ty == Ty::UInt) glsl_error(rule, "abs(uint) is not defined");
        return make(Ty::Int, "se_iabs(" + v[0].code + ")");
      }
      if (fl) return make(Ty::Float, "se_f" + n + "(" + to_float(v[0]) + ", " + to_float(v[1]) + ")");
      if (v[0].ty != v[1].ty) glsl_error(rule, n + ": mismatched argument types");
      return make(v[0].ty, "se_" + n + "(" + v[0].code + ", " + v[1].code + ")");
    }
    if (n == "float" || n == "int") {
      if (e.a.size() != 1) glsl_error(rule, n + "() takes one argument here");
      Val v = expr(*e.a[0]);
      if (n == "float") {
        if (v.ty == Ty::Bool) return make(Ty::Float, "((" + v.code + ") ? 1.0f : 0.0f)");
        if (!numeric(v.ty)) glsl_error(rule, "float(): bad argument");
        Val r = make(Ty::Float, to_float(v));
        if (v.is_const) {
          r.is_const = true;
          r.cval = (double)(float)v.cval;
        }
        return r;
      }
      if (v.ty == Ty::Bool) return make(Ty::Int, "((" + v.code + ") ? 1 : 0)");
      if (v.ty == Ty::Float) return make(Ty::Int, "__float2int_rz(" + v.code + ")");
      if (!numeric(v.ty)) glsl_error(rule, "int(): bad argument");
      return make(Ty::Int, "(int)(" + v.code + ")");
    }
    if (n.rfind("rule_", 0) == 0 || n.rfind("apply", 0) == 0) unsupported(rule, "calls to other rules");
    if (n.rfind("isType_", 0) != 0 && shader_names().count(n)) unsupported(rule, "calls to '" + n + "'");
    glsl_error(rule, "undeclared function '" + n + "'");
  }

  Val unary(const Expr& e) {
    Val v = expr(*e.a[0]);
    if (e.name == "!") {
      if (v.ty != Ty::Bool) glsl_error(rule, "'!' needs a bool operand");
      Val r = make(Ty::Bool, "(!" + v.code + ")");
      return r;
    }
    if (e.name == "~") {
      if (v.ty != Ty::Int && v.ty != Ty::UInt) glsl_error(rule, "'~' needs an integer operand");
      return make(v.ty, "(~" + v.code + ")");
    }
    if (!numeric(v.ty)) glsl_error(rule, "unary '" + e.name + "' needs a numeric operand");
    if (e.name == "+") return v;
    Val r;
    if (v.ty == Ty::Float) r = make(Ty::Float, "(-" + v.code + ")");
    else if (v.ty == Ty::Int) r = make(Ty::Int, "(int)(0u - (unsigned)(" + v.code + "))");
    else r = make(Ty::UInt, "(0u - " + v.code + ")");
    if (v.is_const) {
      r.is_const = true;
      r.cval = v.ty == Ty::Float ? -v.cval : (double)(int64_t)(-(int64_t)v.cval);
      if (v.ty == Ty::Float) r.code = "(" + hexf((float)r.cval) + ")";
    }
    return r;
  }

  Val binary(const Expr& e) {
    const std::string& op = e.name;
    Val a = expr(*e.a[0]);
    Val b = expr(*e.a[1]);
    if (op == "&&" || op == "||" || op == "^^") {
      if (a.ty != Ty::Bool || b.ty != Ty::Bool) glsl_error(rule, "'" + op + "' needs bool operands");
      if (op == "^^") return make(Ty::Bool, "(" + a.code + " != " + b.code + ")");
      return make(Ty::Bool, "(" + a.code + " " + op + " " + b.code + ")");
    }
    bool cmp = op == "<" || op == ">" || op == "<=" || op == ">=";
    bool eq = op == "==" || op == "!=";
    if (eq && (a.ty == Ty::Material || b.ty == Ty::Material)) {
      if (a.ty != b.ty) glsl_error(rule, "'" + op + "' between Material and " + ty_name(a.ty == Ty::Material ? b.ty : a.ty));
      std::string c;
      // GLSL compares structs member-wise, so a material whose density is NaN never
      // equals anything; ids are unique, so otherwise equality is id equality.
      int k = a.const_mat >= 0 ? a.const_mat : b.const_mat;
      const Val& var = a.const_mat >= 0 ? b : a;
      if (a.const_mat >= 0 && b.const_mat >= 0)
        c = (a.const_mat == b.const_mat && !mat_nan[(size_t)a.const_mat]) ? "true" : "false";
      else if (k >= 0)
        c = mat_nan[(size_t)k] ? "false" : "(" + var.code + " == " + std::to_string(k) + "u)";
      else
        c = any_nan ? "se_gen::mat_eq(" + a.code + ", " + b.code + ")" : "(" + a.code + " == " + b.code + ")";
      return make(Ty::Bool, op == "==" ? c : "(!" + c + ")");
    }
    if (eq && (a.ty == Ty::Cell || b.ty == Ty::Cell)) unsupported(rule, "comparing whole cells (their positions)");
    if (eq && (a.ty == Ty::Vec4 || b.ty == Ty::Vec4 || a.ty == Ty::IVec2 || b.ty == Ty::IVec2))
      unsupported(rule, "vector comparisons");
    if (eq && a.ty == Ty::Bool && b.ty == Ty::Bool) return make(Ty::Bool, "(" + a.code + " " + op + " " + b.code + ")");
    if (!numeric(a.ty) || !numeric(b.ty))
      glsl_error(rule, std::string("'") + op + "' on " + ty_name(a.ty) + " and " + ty_name(b.ty));
    bool fl = a.ty == Ty::Float || b.ty == Ty::Float;
    if (cmp || eq) {
      if (fl) {
        // exact integer form for rand.<lane> compared with a constant
        if (a.rand_lane >= 0 && b.is_const) return make(Ty::Bool, rand_compare(a.rand_lane, op, (float)b.cval, true));
        if (b.rand_lane >= 0 && a.is_const) return make(Ty::Bool, rand_compare(b.rand_lane, op, (float)a.cval, false));
        return make(Ty::Bool, "(" + to_float(a) + " " + op + " " + to_float(b) + ")");
      }
      if (a.ty == Ty::UInt || b.ty == Ty::UInt)
        return make(Ty::Bool, "(" + to_uint(a) + " " + op + " " + to_uint(b) + ")");
      return make(Ty::Bool, "(" + a.code + " " + op + " " + b.code + ")");
    }
    if (op == "+" || op == "-" || op == "*" || op == "/") {
      if (fl) {
        const char* fn = op == "+" ? "__fadd_rn" : op == "-" ? "__fsub_rn" : op == "*" ? "__fmul_rn" : "__fdiv_rn";
        return make(Ty::Float, std::string(fn) + "(" + to_float(a) + ", " + to_float(b) + ")");
      }
      bool un = a.ty == Ty::UInt || b.ty == Ty::UInt;
      if (op == "/") {
        if (un) return make(Ty::UInt, "se_udiv(" + to_uint(a) + ", " + to_uint(b) + ")");
        return make(Ty::Int, "se_idiv(" + a.code + ", " + b.code + ")");
      }
      std::string u = "(" + to_uint(a) + " " + op + " " + to_uint(b) + ")";
      return un ? make(Ty::UInt, u) : make(Ty::Int, "(int)" + u);
    }
    if (fl) glsl_error(rule, "'" + op + "' needs integer operands");
    bool un = a.ty == Ty::UInt || b.ty == Ty::UInt;
    if (op == "%") {
      if (un) return make(Ty::UInt, "se_umod(" + to_uint(a) + ", " + to_uint(b) + ")");
      return make(Ty::Int, "se_imod(" + a.code + ", " + b.code + ")");
    }
    if (op == "<<" || op == ">>") return make(a.ty, "(" + a.code + " " + op + " (" + b.code + " & 31))");
    std::string u = "(" + to_uint(a) + " " + op + " " + to_uint(b) + ")";
    return un ? make(Ty::UInt, u) : make(Ty::Int, "(int)" + u);
  }

  Val expr(const Expr& e) {
    switch (e.k) {
      case Expr::Lit: {
        Val v;
        v.is_const = true;
        if (e.lit.t == T::Float) {
          v.ty = Ty::Float;
          v.cval = e.lit.f;
          v.code = hexf((float)e.lit.f);
        } else if (e.lit.t == T::UInt) {
          v.ty = Ty::UInt;
          v.cval = (double)e.lit.u;
          v.code = std::to_string(e.lit.u) + "u";
        } else {
          v.ty = Ty::Int;
          v.cval = (double)(int32_t)(uint32_t)e.lit.u;
          v.code = "(int)" + std::to_string(e.lit.u) + "u";
        }
        return v;
      }
      case Expr::Id: return id(e);
      case Expr::Member: return member(e);
      case Expr::Call: return call(e);
      case Expr::Unary: return unary(e);
      case Expr::Binary: return binary(e);
      case Expr::Ternary: {
        Val c = expr(*e.a[0]);
        Val x = expr(*e.a[1]);
        Val y = expr(*e.a[2]);
        if (c.ty != Ty::Bool) glsl_error(rule, "'?:' condition must be bool");
        if (x.ty != y.ty || (x.ty != Ty::Bool && !numeric(x.ty) && x.ty != Ty::Material))
          unsupported(rule, "this conditional expression");
        return make(x.ty, "(" + c.code + " ? " + x.code + " : " + y.code + ")");
      }
      case Expr::Assign: {
        Val l = expr(*e.a[0]);
        Val r = expr(*e.a[1]);
        if (l.ty != Ty::Cell || l.cell_slot < 0) unsupported(rule, "assignments other than to a block cell");
        if (r.ty != Ty::Cell) glsl_error(rule, "assigning a non-Cell value to a Cell");
        return make(Ty::Void, l.code + " = " + r.code);
      }
    }
    glsl_error(rule, "bad expression");
  }

  void stmt(const Stmt& s, std::string& out, int ind) {
    std::string pad((size_t)ind * 2, ' ');
    switch (s.k) {
      case Stmt::Block:
        out += pad + "{\n";
        for (auto& b : s.body) stmt(*b, out, ind + 1);
        out += pad + "}\n";
        break;
      case Stmt::Empty: break;
      case Stmt::Return: out += pad + "return;\n"; break;
      case Stmt::If: {
        Val c = expr(*s.e);
        if (c.ty != Ty::Bool) glsl_error(rule, "if condition must be bool, not " + std::string(ty_name(c.ty)));
        out += pad + "if (" + c.code + ")\n";
        stmt(*s.then_s, out, ind + 1);
        if (s.then_s->k == Stmt::Empty) out += pad + "  ;\n";
        if (s.else_s) {
          out += pad + "else\n";
          stmt(*s.else_s, out, ind + 1);
          if (s.else_s->k == Stmt::Empty) out += pad + "  ;\n";
        }
        break;
      }
      case Stmt::ExprS: {
        Val v = expr(*s.e);
        if (v.ty == Ty::Void) out += pad + v.code + ";\n";
        else out += pad + "(void)(" + v.code + ");\n";
        break;
      }
    }
  }

  std::string rule_function(const Rule& r) {
    rule = r.name;
    Parser P;
    P.rule = r.name;
    P.t = lex(rule_glsl(r), r.name);
    // void rule_<name> (inout Cell self, inout Cell <dir>, inout Cell down, inout Cell downright,
    //                   vec4 rand, ivec2 pos) { ... }
    if (!P.is_ident("void")) glsl_error(rule, "bad function header");
    ++P.p;
    ++P.p;  // name
    P.expect("(");
    cell_names.clear();
    while (!P.is(")")) {
      std::vector<std::string> words;
      while (P.peek().t == T::Ident) words.push_back(P.peek().s), ++P.p;
      if (words.size() >= 2 && words[words.size() - 2] == "Cell") cell_names.push_back(words.back());
      if (P.is(",")) ++P.p;
      else if (!P.is(")")) glsl_error(rule, "bad parameter list");
    }
    ++P.p;
    SP body = P.statement();
    if (P.peek().t != T::End) glsl_error(rule, "trailing text after function body");
    std::string code;
    stmt(*body, code, 1);
    all_bodies += code;
    std::string sig = "__device__ __forceinline__ void rule_" + r.name + "(uint32_t& " + cell_names[0] +
                      ", uint32_t& " + cell_names[1] + ", uint32_t& " + cell_names[2] + ", uint32_t& " +
                      cell_names[3] + SE_RULE_TAIL_PARAMS + ")\n";
    return sig + code;
  }
  static constexpr const char* SE_RULE_TAIL_PARAMS =
      ", uint32_t h0, uint32_t h1, uint32_t h2, uint32_t h3, int pos_x, int pos_y, int frame, int sim_w, "
      "int sim_h";
};

// Tables are stored as binary32 bit patterns (NaN and infinity have no literal form).
std::string float_table(const char* name, const std::vector<float>& v) {
  std::string s = "static __device__ const unsigned c_" + std::string(name) + "[] = {";
  for (size_t i = 0; i < v.size(); ++i) {
    uint32_t u;
    memcpy(&u, &v[i], 4);
    char b[16];
    snprintf(b, sizeof b, "0x%08xu", u);
    s += (i ? ", " : "") + std::string(b);
  }
  return s + "};\n__shared__ float s_" + name + "[" + std::to_string(v.size()) + "];\n";
}

}  // namespace

bool generate_cuda(const ParsingResult& r, CudaRules* out, ParseError* err) {
  try {
    Gen g(r);
    g.nmat = (int)r.materials.size();
    if (g.nmat > 256) throw Fail{{"Unsupported", "(Unsupported) at most 256 materials fit the 8-bit cell ids"}};
    // Duplicate names make the generated GLSL redefine TYPE_/MAT_ macros and functions.
    std::set<std::string> seen;
    for (auto& t : r.types) {
      if (!seen.insert(t.name).second)
        throw Fail{{"Glsl", "(Glsl) type '" + t.name + "' is defined twice in the generated shader"}};
      g.type_ids[t.name] = (int)t.id;
    }
    seen.clear();
    for (auto& m : r.materials)
      if (!seen.insert(m.name).second)
        throw Fail{{"Glsl", "(Glsl) material '" + m.name + "' is defined twice in the generated shader"}};
    for (auto& m : r.materials) {
      g.mat_type.push_back(g.type_ids.at(m.mattype));
      bool nan = std::isnan(m.density);
      g.mat_nan.push_back(nan);
      g.any_nan = g.any_nan || nan;
    }
    for (auto& rule : r.rules)
      if (rule.used && rule.ruletype == Rule::Left)
        throw Fail{{"Glsl", "(Glsl) applyLeftRules passes the undeclared 'left' to rule_" + rule.name}};
    if (!r.rules.empty())
      for (auto& rule : r.rules)
        if (rule.used && rule.has_precondition && rule.precondition.empty())
          throw Fail{{"Glsl", "(Glsl) rule_" + rule.name + " has an empty precondition '()'"}};

    std::string funcs;
    std::string mirrored, right;
    for (auto& rule : r.rules) {
      if (!rule.used) continue;
      funcs += g.rule_function(rule) + "\n";
      std::string call = "  rule_" + rule.name + "(self, right, down, downright, h0, h1, h2, h3, pos_x, pos_y, "
                                                  "frame, sim_w, sim_h);\n";
      if (rule.ruletype == Rule::Mirrored) mirrored += call;
      else right += call;
    }

    std::ostringstream o;
    o << "// Generated by the sandengine_gb300 rule compiler from the rule set's GLSL.\n";
    o << "#define SE_NMAT " << g.nmat << "\n";
    o << "namespace se_gen {\n";
    // material tables
    std::vector<float> dens, col, emi;
    std::vector<int> mtype;
    for (auto& m : r.materials) {
      dens.push_back(m.density);
      for (int i = 0; i < 4; ++i) col.push_back(m.color[i]), emi.push_back(m.emission[i]);
      mtype.push_back(g.type_ids.at(m.mattype));
    }
    if (g.used_density) o << float_table("density", dens);
    if (g.used_color) o << float_table("color", col);
    if (g.used_emission) o << float_table("emission", emi);
    if (g.used_type) {
      o << "static __device__ const int c_mtype[] = {";
      for (size_t i = 0; i < mtype.size(); ++i) o << (i ? ", " : "") << mtype[i];
      o << "};\n__shared__ int s_mtype[" << mtype.size() << "];\n";
    }
    // material sets
    for (size_t k = 0; k < g.sets.size(); ++k) {
      const auto& s = g.sets[k];
      if (g.nmat <= 64) {
        uint64_t mask = 0;
        for (int m = 0; m < g.nmat; ++m)
          if (s[(size_t)m]) mask |= 1ull << m;
        char b[64];
        snprintf(b, sizeof b, "0x%016llxull", (unsigned long long)mask);
        o << "__device__ __forceinline__ bool in_set" << k << "(uint32_t m) { return (" << b
          << " >> m) & 1ull; }\n";
      } else {
        uint32_t words[8] = {0};
        for (int m = 0; m < g.nmat; ++m)
          if (s[(size_t)m]) words[m >> 5] |= 1u << (m & 31);
        o << "static __device__ const uint32_t c_set" << k << "[8] = {";
        for (int i = 0; i < 8; ++i) o << (i ? ", " : "") << words[i] << "u";
        o << "};\n__shared__ uint32_t s_set" << k << "[8];\n";
        o << "__device__ __forceinline__ bool in_set" << k << "(uint32_t m) { return (s_set" << k
          << "[m >> 5] >> (m & 31)) & 1u; }\n";
      }
    }
    if (g.used_density) o << "__device__ __forceinline__ float density(uint32_t m) { return s_density[m]; }\n";
    if (g.used_color) o << "__device__ __forceinline__ float color(uint32_t m, int c) { return s_color[4 * m + c]; }\n";
    if (g.used_emission)
      o << "__device__ __forceinline__ float emission(uint32_t m, int c) { return s_emission[4 * m + c]; }\n";
    if (g.used_type) o << "__device__ __forceinline__ int mtype(uint32_t m) { return s_mtype[m]; }\n";
    if (g.any_nan) {
      uint64_t nanmask[4] = {0, 0, 0, 0};
      for (int m = 0; m < g.nmat; ++m)
        if (g.mat_nan[(size_t)m]) nanmask[m >> 6] |= 1ull << (m & 63);
      o << "__device__ __forceinline__ bool mat_eq(uint32_t a, uint32_t b) {\n"
        << "  const unsigned long long nan[4] = {" << nanmask[0] << "ull, " << nanmask[1] << "ull, " << nanmask[2]
        << "ull, " << nanmask[3] << "ull};\n"
        << "  return a == b && !((nan[a >> 6] >> (a & 63)) & 1ull);\n}\n";
    }
    // shared-table initialisation (all threads of the CTA, then a barrier by the caller)
    o << "__device__ __forceinline__ void init_tables(int tid, int nthr) {\n";
    if (g.used_density)
      o << "  for (int i = tid; i < SE_NMAT; i += nthr) s_density[i] = __uint_as_float(c_density[i]);\n";
    if (g.used_color)
      o << "  for (int i = tid; i < 4 * SE_NMAT; i += nthr) s_color[i] = __uint_as_float(c_color[i]);\n";
    if (g.used_emission)
      o << "  for (int i = tid; i < 4 * SE_NMAT; i += nthr) s_emission[i] = __uint_as_float(c_emission[i]);\n";
    if (g.used_type) o << "  for (int i = tid; i < SE_NMAT; i += nthr) s_mtype[i] = c_mtype[i];\n";
    if (g.nmat > 64)
      for (size_t k = 0; k < g.sets.size(); ++k)
        o << "  for (int i = tid; i < 8; i += nthr) s_set" << k << "[i] = c_set" << k << "[i];\n";
    o << "}\n";
    o << funcs;
    const char* params =
        "(uint32_t& self, uint32_t& right, uint32_t& down, uint32_t& downright, uint32_t h0, uint32_t h1, "
        "uint32_t h2, uint32_t h3, int pos_x, int pos_y, int frame, int sim_w, int sim_h)";
    o << "__device__ __forceinline__ void apply_mirrored" << params << " {\n" << mirrored << "}\n";
    o << "__device__ __forceinline__ void apply_right" << params << " {\n" << right << "}\n";
    o << "__device__ __forceinline__ void apply_left" << params << " {}\n";

    // Block transition table.  When the rules read nothing but the four cells and rand
    // lanes compared with constants, a block's update is a function of the four material
    // ids and, per lane, the interval between consecutive comparison boundaries that the
    // lane falls in (lane 0 also carries the mirror test, rand.x < 0.5 <=> h0 < 0x7fffffc0).
    // The runtime fills the table once by running the rules above on one representative
    // hash value per interval (se_build_lut); the tile kernel then replaces the rule
    // evaluation by one lookup.
    auto has_tok = [&](const std::string& tok) {
      size_t p = 0;
      while ((p = g.all_bodies.find(tok, p)) != std::string::npos) {
        bool l = p == 0 || !(isalnum((unsigned char)g.all_bodies[p - 1]) || g.all_bodies[p - 1] == '_');
        size_t e = p + tok.size();
        bool r = e >= g.all_bodies.size() || !(isalnum((unsigned char)g.all_bodies[e]) || g.all_bodies[e] == '_');
        if (l && r) return true;
        p = e;
      }
      return false;
    };
    bool lut = g.nmat <= 16;
    for (const char* t : {"pos_x", "pos_y", "frame", "sim_w", "sim_h", "se_randf"}) lut = lut && !has_tok(t);
    g.bounds[0].insert(0x7fffffc0ull);
    uint64_t classes = 1;
    for (int l = 0; l < 4; ++l) classes *= g.bounds[l].size() + 1;
    // Ids take 4 bits of the key whenever that table fits: the tile kernel then builds two
    // blocks' keys from a row pair with one permute, and no table is copied into shared
    // memory (a small table's copy costs CTAs per SM and its lookups conflict in the banks).
    // Otherwise the fewest bits that hold every id.
    const int min_bits = g.nmat <= 2 ? 1 : g.nmat <= 4 ? 2 : g.nmat <= 8 ? 3 : 4;
    const int bits = (classes << 16) <= (1ull << 24) ? 4 : min_bits;
    const uint64_t entries = (1ull << (4 * bits)) * classes;
    if (entries > (1ull << 24)) lut = false;
    const uint64_t keys = 1ull << (4 * bits);
    if (lut) {
      o << "#define SE_LUT 1\n#define SE_LUT_BITS " << bits << "\n#define SE_LUT_ENTRIES " << entries << "u\n"
        << "#define SE_LUT_KEYS " << keys << "u\n#define SE_LUT_STATIC_WORDS " << std::max<uint64_t>(1, keys / 32)
        << "u\n";
      // The key of the block [a b / c d] (top-left, top-right, bottom-left, bottom-right) in
      // column order, a | c << bits | b << 2 bits | d << 3 bits: with 4 bits, a row pair's
      // two keys are its top row word plus its bottom row word << 4 (se_chunk_eval).
      o << "__device__ __forceinline__ uint32_t lut_key(uint32_t a, uint32_t b, uint32_t c, uint32_t d) {\n"
        << "  return a | (c << " << bits << ") | (b << " << 2 * bits << ") | (d << " << 3 * bits << ");\n}\n";
      o << "__device__ __forceinline__ uint32_t lut_index_key(uint32_t i, uint32_t h0, uint32_t h1, uint32_t h2, "
           "uint32_t h3) {\n";
      for (int l = 0; l < 4; ++l) {
        if (g.bounds[l].empty()) continue;
        o << "  i = i * " << g.bounds[l].size() + 1 << "u";
        for (uint64_t T : g.bounds[l]) o << " + (h" << l << " >= " << T << "u)";
        o << ";\n";
      }
      o << "  return i;\n}\n";
      o << "__device__ __forceinline__ uint32_t lut_index(uint32_t a, uint32_t b, uint32_t c, uint32_t d, "
           "uint32_t h0, uint32_t h1, uint32_t h2, uint32_t h3) {\n"
        << "  return lut_index_key(lut_key(a, b, c, d), h0, h1, h2, h3);\n}\n";
      // decode: idx -> cells and one representative hash value per lane
      o << "__device__ __forceinline__ void lut_decode(uint32_t i, uint32_t& a, uint32_t& b, uint32_t& c, "
           "uint32_t& d, uint32_t& h0, uint32_t& h1, uint32_t& h2, uint32_t& h3) {\n"
        << "  h0 = h1 = h2 = h3 = 0u;\n";
      for (int l = 3; l >= 0; --l) {
        if (g.bounds[l].empty()) continue;
        const size_t n = g.bounds[l].size() + 1;
        o << "  { const uint32_t reps[" << n << "] = {0u";
        for (uint64_t T : g.bounds[l]) o << ", " << T << "u";
        o << "}; h" << l << " = reps[i % " << n << "u]; i /= " << n << "u; }\n";
      }
      const uint32_t mask = (1u << bits) - 1;
      o << "  a = i & " << mask << "u; c = (i >> " << bits << ") & " << mask << "u; b = (i >> " << 2 * bits
        << ") & " << mask << "u; d = (i >> " << 3 * bits << ") & " << mask << "u;\n}\n";
    }
    o << "}  // namespace se_gen\n";
    out->source = o.str();
    out->lut_entries = lut ? entries : 0;
    out->lut_static_words = lut ? std::max<uint64_t>(1, keys / 32) : 0;
    out->num_materials = g.nmat;
    for (int i = 0; i < 4; ++i) out->uses_rand_lane[i] = g.uses_lane[i];
    return true;
  } catch (Fail& f) {
    if (err) *err = f.e;
    return false;
  }
}

}  // namespace se::lang
