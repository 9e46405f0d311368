// frontend.cpp -- WGSL / GLSL SDF sources -> typed AST -> CUDA C.
//
// Covers the subset of both languages that SDF code uses: functions,
// module / function scope `const`, `let`, `var`, scalar / vector / matrix
// arithmetic with swizzles (read, write, compound), `if`, `for`, `while`,
// `loop` / `continuing`, `break`, `continue`, `return`, GLSL `out` / `inout`
// parameters, `#define` object macros, and the shader builtins.  WGSL
// abstract numerics follow the WGSL rules (abstract expressions are folded in
// binary64 and rounded once when they meet an f32), which is how the
// reference's toolchain (naga) evaluates `.sdf3d` constants such as
// `KEY_SIZE * 0.15`.
//
// The lowered code calls only s2m_prelude.cuh, so the same text compiles for
// the device (NVRTC) and for the host (frontend tests).
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <map>
#include <memory>
#include <set>
#include <sstream>
#include <stdexcept>

#include "frontend.h"
#include "prune.h"
#include "../../include/sdf2mesh.h"

namespace s2m {
namespace {

// ---------------------------------------------------------------------------
// Errors

struct CompileError : std::runtime_error {
  int line;
  CompileError(int l, const std::string &m) : std::runtime_error(m), line(l) {}
};
[[noreturn]] void fail(int line, const std::string &msg) { throw CompileError(line, msg); }

// ---------------------------------------------------------------------------
// Lexer

enum class TK { End, Ident, Int, Float, Punct };
struct Tok {
  TK k = TK::End;
  std::string s;
  int line = 0;
  double num = 0;     // value (ints and abstract floats)
  float fnum = 0;     // value for f32-typed float literals
  char suffix = 0;    // 'i', 'u', 'f', 'h' or 0
};

bool is_id0(char c) { return std::isalpha((unsigned char)c) || c == '_'; }
bool is_id(char c) { return std::isalnum((unsigned char)c) || c == '_'; }

std::vector<Tok> lex(const std::string &src, Lang lang) {
  std::vector<Tok> out;
  std::map<std::string, std::vector<Tok>> macros;
  size_t i = 0, n = src.size();
  int line = 1;
  bool line_start = true;
  static const char *puncts[] = {"<<=", ">>=", "->", "&&", "||", "==", "!=", "<=", ">=", "+=", "-=",
                                 "*=",  "/=",  "%=", "&=", "|=", "^=", "++", "--", "<<", ">>", "::"};
  auto emit_tok = [&](Tok t) {
    if (t.k == TK::Ident) {
      auto m = macros.find(t.s);
      if (m != macros.end()) {
        for (Tok mt : m->second) {
          mt.line = t.line;
          out.push_back(mt);
        }
        return;
      }
    }
    out.push_back(t);
  };
  while (i < n) {
    char c = src[i];
    if (c == '\n') { ++line; ++i; line_start = true; continue; }
    if (c == ' ' || c == '\t' || c == '\r' || c == '\f' || c == '\v') { ++i; continue; }
    if (c == '/' && i + 1 < n && src[i + 1] == '/') {
      while (i < n && src[i] != '\n') ++i;
      continue;
    }
    if (c == '/' && i + 1 < n && src[i + 1] == '*') {
      int depth = 1;
      i += 2;
      while (i < n && depth > 0) {
        if (src[i] == '\n') ++line;
        if (lang == Lang::WGSL && src[i] == '/' && i + 1 < n && src[i + 1] == '*') { ++depth; i += 2; continue; }
        if (src[i] == '*' && i + 1 < n && src[i + 1] == '/') { --depth; i += 2; continue; }
        ++i;
      }
      continue;
    }
    if (c == '#' && lang == Lang::GLSL && line_start) {
      // Preprocessor line (with backslash continuation).
      std::string dir;
      while (i < n && src[i] != '\n') {
        if (src[i] == '\\' && i + 1 < n && src[i + 1] == '\n') { i += 2; ++line; continue; }
        dir.push_back(src[i++]);
      }
      std::string body = dir.substr(1);
      size_t a = body.find_first_not_of(" \t");
      body = a == std::string::npos ? "" : body.substr(a);
      std::string word;
      size_t k = 0;
      while (k < body.size() && is_id(body[k])) word.push_back(body[k++]);
      if (word == "define") {
        while (k < body.size() && (body[k] == ' ' || body[k] == '\t')) ++k;
        std::string name;
        while (k < body.size() && is_id(body[k])) name.push_back(body[k++]);
        if (name.empty()) fail(line, "malformed #define");
        if (k < body.size() && body[k] == '(') fail(line, "function-like macros are not supported");
        std::vector<Tok> toks = lex(body.substr(k), Lang::GLSL);
        if (!toks.empty() && toks.back().k == TK::End) toks.pop_back();
        macros[name] = toks;
      } else if (word == "undef") {
        std::string rest = body.substr(k);
        size_t s0 = rest.find_first_not_of(" \t");
        if (s0 != std::string::npos) {
          std::string nm;
          for (size_t q = s0; q < rest.size() && is_id(rest[q]); ++q) nm.push_back(rest[q]);
          macros.erase(nm);
        }
      } else if (word == "version" || word == "extension" || word == "pragma" || word == "line" || word.empty()) {
        // ignored
      } else {
        fail(line, "unsupported preprocessor directive #" + word);
      }
      continue;
    }
    line_start = false;
    if (std::isdigit((unsigned char)c) || (c == '.' && i + 1 < n && std::isdigit((unsigned char)src[i + 1]))) {
      Tok t;
      t.line = line;
      size_t st = i;
      bool is_float = false;
      if (c == '0' && i + 1 < n && (src[i + 1] == 'x' || src[i + 1] == 'X')) {
        i += 2;
        while (i < n && std::isxdigit((unsigned char)src[i])) ++i;
        t.num = double(std::strtoull(src.substr(st + 2, i - st - 2).c_str(), nullptr, 16));
      } else {
        while (i < n && std::isdigit((unsigned char)src[i])) ++i;
        if (i < n && src[i] == '.') { is_float = true; ++i; while (i < n && std::isdigit((unsigned char)src[i])) ++i; }
        if (i < n && (src[i] == 'e' || src[i] == 'E')) {
          size_t save = i;
          ++i;
          if (i < n && (src[i] == '+' || src[i] == '-')) ++i;
          if (i < n && std::isdigit((unsigned char)src[i])) {
            is_float = true;
            while (i < n && std::isdigit((unsigned char)src[i])) ++i;
          } else {
            i = save;
          }
        }
      }
      std::string text = src.substr(st, i - st);
      char suf = 0;
      if (i < n && (src[i] == 'f' || src[i] == 'F' || src[i] == 'h')) { suf = 'f'; is_float = true; ++i; }
      else if (i < n && (src[i] == 'u' || src[i] == 'U')) { suf = 'u'; ++i; }
      else if (i < n && src[i] == 'i' && lang == Lang::WGSL) { suf = 'i'; ++i; }
      else if (i + 1 < n && (src[i] == 'l' || src[i] == 'L') && (src[i + 1] == 'f' || src[i + 1] == 'F')) { suf = 'f'; is_float = true; i += 2; }
      if (i < n && is_id(src[i])) fail(line, "malformed number '" + src.substr(st, i - st + 1) + "'");
      if (is_float) {
        t.k = TK::Float;
        t.num = std::strtod(text.c_str(), nullptr);
        t.fnum = std::strtof(text.c_str(), nullptr);
      } else {
        t.k = TK::Int;
        if (!(text.size() > 1 && (text[1] == 'x' || text[1] == 'X'))) t.num = double(std::strtoull(text.c_str(), nullptr, 10));
      }
      t.suffix = suf;
      t.s = src.substr(st, i - st);
      emit_tok(t);
      continue;
    }
    if (is_id0(c)) {
      Tok t;
      t.k = TK::Ident;
      t.line = line;
      while (i < n && is_id(src[i])) t.s.push_back(src[i++]);
      emit_tok(t);
      continue;
    }
    Tok t;
    t.k = TK::Punct;
    t.line = line;
    bool matched = false;
    for (const char *p : puncts) {
      size_t L = std::strlen(p);
      if (src.compare(i, L, p) == 0) { t.s = p; i += L; matched = true; break; }
    }
    if (!matched) {
      if (std::strchr("{}()[];,.:=<>+-*/%!&|^~?@", c) == nullptr) fail(line, std::string("unexpected character '") + c + "'");
      t.s = std::string(1, c);
      ++i;
    }
    out.push_back(t);
  }
  Tok e;
  e.k = TK::End;
  e.line = line;
  out.push_back(e);
  return out;
}

// ---------------------------------------------------------------------------
// Types

enum class B : uint8_t { Void, Bool, AInt, AFloat, I32, U32, F32 };
struct Ty {
  B b = B::Void;
  int n = 1;  // vector size (rows)
  int m = 1;  // matrix columns (> 1 for matrices)
  bool operator==(const Ty &o) const { return b == o.b && n == o.n && m == o.m; }
  bool operator!=(const Ty &o) const { return !(*this == o); }
};
Ty scalar(B b) { Ty t; t.b = b; return t; }
Ty vec(B b, int n) { Ty t; t.b = b; t.n = n; return t; }
Ty mat(int c, int r) { Ty t; t.b = B::F32; t.n = r; t.m = c; return t; }
bool is_abstract(B b) { return b == B::AInt || b == B::AFloat; }
bool is_abstract(const Ty &t) { return is_abstract(t.b); }
bool is_float_b(B b) { return b == B::F32 || b == B::AFloat; }
bool is_int_b(B b) { return b == B::I32 || b == B::U32 || b == B::AInt; }
bool is_num(B b) { return b != B::Void && b != B::Bool; }
bool is_scalar(const Ty &t) { return t.n == 1 && t.m == 1 && t.b != B::Void; }
bool is_vec(const Ty &t) { return t.n > 1 && t.m == 1; }
bool is_mat(const Ty &t) { return t.m > 1; }
int ncomp(const Ty &t) { return t.n * t.m; }
Ty with_b(Ty t, B b) { t.b = b; return t; }
B concrete_of(B b) { return b == B::AInt ? B::I32 : (b == B::AFloat ? B::F32 : b); }
Ty concrete(Ty t) { t.b = concrete_of(t.b); return t; }

std::string bname(B b) {
  switch (b) {
    case B::Void: return "void"; case B::Bool: return "bool"; case B::AInt: return "abstract-int";
    case B::AFloat: return "abstract-float"; case B::I32: return "i32"; case B::U32: return "u32";
    case B::F32: return "f32";
  }
  return "?";
}
std::string tname(const Ty &t) {
  if (is_mat(t)) return "mat" + std::to_string(t.m) + "x" + std::to_string(t.n) + "<f32>";
  if (is_vec(t)) return "vec" + std::to_string(t.n) + "<" + bname(t.b) + ">";
  return bname(t.b);
}
std::string c_scalar(B b) {
  switch (concrete_of(b)) {
    case B::Bool: return "bool"; case B::I32: return "int"; case B::U32: return "unsigned";
    case B::F32: return "float"; case B::Void: return "void"; default: return "float";
  }
}
std::string c_type(const Ty &t) {
  if (is_mat(t)) return "s2mat<" + std::to_string(t.m) + "," + std::to_string(t.n) + ">";
  if (is_vec(t)) return "s2vec<" + c_scalar(t.b) + "," + std::to_string(t.n) + ">";
  return c_scalar(t.b);
}

// Can a value of type `f` be used where `t` is wanted (abstract conversion,
// or GLSL implicit int -> float)?
int conv_rank(B f, B t, Lang lang) {
  if (f == t) return 0;
  if (f == B::AInt && (t == B::I32 || t == B::U32 || t == B::AFloat || t == B::F32)) return 1;
  if (f == B::AFloat && t == B::F32) return 1;
  if (lang == Lang::GLSL) {
    if ((f == B::I32 || f == B::U32) && t == B::F32) return 2;
    if (f == B::I32 && t == B::U32) return 2;
  }
  return -1;
}
int conv_rank(const Ty &f, const Ty &t, Lang lang) {
  if (f.n != t.n || f.m != t.m) return -1;
  return conv_rank(f.b, t.b, lang);
}

// ---------------------------------------------------------------------------
// AST

struct Sym;
struct Func;

struct Expr {
  enum K { Lit, Ref, Unary, Binary, Call, Swz, Index, Ternary } k;
  int line = 0;
  std::string s;               // Ref name, operator, or callee
  std::vector<Expr *> a;
  bool is_ctor = false;        // Call is a type constructor
  Ty ctor_t;                   // constructor target (b == Void: element type inferred)
  std::vector<int> swz;
  B lit_b = B::AFloat;         // literal type
  double lit = 0;
  float flit = 0;
  // sema
  Ty t;                        // natural type (may be abstract)
  Ty want;                     // concrete type the parent consumes (b == Void: use t)
  bool cst = false;            // folded value available in cv
  std::vector<double> cv;
  Sym *sym = nullptr;
  Func *fn = nullptr;
};

struct Stmt {
  enum K { Block, Decl, Assign, IncDec, ExprS, If, For, While, DoWhile, Loop, Break, Continue, Return, BreakIf, Empty } k;
  int line = 0;
  std::vector<Stmt *> body;    // Block / loop bodies (as blocks)
  int decl_kind = 0;           // 0 let, 1 var, 2 const
  std::string name;
  bool has_type = false;
  Ty decl_t;
  Expr *init = nullptr;
  Sym *sym = nullptr;
  Expr *lhs = nullptr, *rhs = nullptr;
  std::string op;
  bool prefix = false;
  Expr *cond = nullptr;
  Stmt *then_s = nullptr, *else_s = nullptr;
  Stmt *init_s = nullptr, *update_s = nullptr, *loop_body = nullptr, *continuing = nullptr;
  Expr *val = nullptr;
};

struct Sym {
  enum K { Const, Let, Var, Param, Global } k;
  std::string name, cname;
  Ty t;
  bool cst = false;
  std::vector<double> cv;
  bool is_ref = false;          // GLSL out / inout parameter
  bool assigned = false;
};

struct Param {
  std::string name;
  Ty t;
  bool out = false;
  Sym *sym = nullptr;
};

struct Func {
  std::string name, cname;
  std::vector<Param> params;
  Ty ret;
  Stmt *body = nullptr;
  int line = 0;
  Lang lang = Lang::WGSL;
  bool checked = false, checking = false;
  bool costed = false, costing = false;
  double fp = 0, sfu = 0;
  bool exact = true;
  bool emitted = false;
};

struct Global {
  std::string name;
  bool is_const = true;
  bool has_type = false;
  Ty t;
  Expr *init = nullptr;
  Sym *sym = nullptr;
  int line = 0;
  Lang lang = Lang::WGSL;
  bool resolving = false, resolved = false;
};

struct Module {
  std::vector<std::unique_ptr<Expr>> exprs;
  std::vector<std::unique_ptr<Stmt>> stmts;
  std::vector<std::unique_ptr<Sym>> syms;
  std::vector<std::unique_ptr<Func>> funcs_own;
  std::vector<std::unique_ptr<Global>> globals_own;
  std::vector<Func *> funcs;
  std::map<std::string, std::vector<Func *>> fn_by_name;
  std::vector<Global *> globals;
  std::map<std::string, Global *> glob_by_name;
  std::map<std::string, Ty> aliases;
  std::vector<std::string> warnings;

  Expr *ex(Expr::K k, int line) {
    exprs.emplace_back(new Expr());
    exprs.back()->k = k;
    exprs.back()->line = line;
    return exprs.back().get();
  }
  Stmt *st(Stmt::K k, int line) {
    stmts.emplace_back(new Stmt());
    stmts.back()->k = k;
    stmts.back()->line = line;
    return stmts.back().get();
  }
  Sym *sym(Sym::K k, const std::string &name, Ty t) {
    syms.emplace_back(new Sym());
    Sym *s = syms.back().get();
    s->k = k;
    s->name = name;
    s->t = t;
    return s;
  }
  void add_func(Func *f) {
    auto &v = fn_by_name[f->name];
    for (Func *g : v) {
      bool same = g->params.size() == f->params.size();
      for (size_t i = 0; same && i < f->params.size(); ++i) same = g->params[i].t == f->params[i].t;
      if (same) {
        // An identical module inserted twice by `use` redefines the same
        // function; keep the first definition.
        if (f->lang == Lang::WGSL && g->lang == Lang::WGSL && f->params.size() == g->params.size()) return;
        fail(f->line, "function '" + f->name + "' is defined twice");
      }
    }
    if (!v.empty() && f->lang == Lang::WGSL) {
      // WGSL has no overloading: a second `use` of the same module is the
      // only legitimate case, handled above.
      fail(f->line, "function '" + f->name + "' is defined twice");
    }
    v.push_back(f);
    funcs.push_back(f);
  }
};

// ---------------------------------------------------------------------------
// Type names

bool parse_glsl_type_name(const std::string &s, Ty &t) {
  static const std::map<std::string, Ty> m = {
      {"void", scalar(B::Void)}, {"float", scalar(B::F32)}, {"int", scalar(B::I32)},
      {"uint", scalar(B::U32)}, {"bool", scalar(B::Bool)},
      {"vec2", vec(B::F32, 2)}, {"vec3", vec(B::F32, 3)}, {"vec4", vec(B::F32, 4)},
      {"ivec2", vec(B::I32, 2)}, {"ivec3", vec(B::I32, 3)}, {"ivec4", vec(B::I32, 4)},
      {"uvec2", vec(B::U32, 2)}, {"uvec3", vec(B::U32, 3)}, {"uvec4", vec(B::U32, 4)},
      {"bvec2", vec(B::Bool, 2)}, {"bvec3", vec(B::Bool, 3)}, {"bvec4", vec(B::Bool, 4)},
      {"mat2", mat(2, 2)}, {"mat3", mat(3, 3)}, {"mat4", mat(4, 4)},
      {"mat2x2", mat(2, 2)}, {"mat2x3", mat(2, 3)}, {"mat2x4", mat(2, 4)},
      {"mat3x2", mat(3, 2)}, {"mat3x3", mat(3, 3)}, {"mat3x4", mat(3, 4)},
      {"mat4x2", mat(4, 2)}, {"mat4x3", mat(4, 3)}, {"mat4x4", mat(4, 4)}};
  auto it = m.find(s);
  if (it == m.end()) return false;
  t = it->second;
  return true;
}

// WGSL type words without template arguments (f32, vec3f, mat2x2f ...).
bool parse_wgsl_simple_type(const std::string &s, Ty &t) {
  if (s == "f32") { t = scalar(B::F32); return true; }
  if (s == "i32") { t = scalar(B::I32); return true; }
  if (s == "u32") { t = scalar(B::U32); return true; }
  if (s == "bool") { t = scalar(B::Bool); return true; }
  if (s.size() == 5 && s.compare(0, 3, "vec") == 0 && s[3] >= '2' && s[3] <= '4') {
    int n = s[3] - '0';
    char c = s[4];
    if (c == 'f' || c == 'h') { t = vec(B::F32, n); return true; }
    if (c == 'i') { t = vec(B::I32, n); return true; }
    if (c == 'u') { t = vec(B::U32, n); return true; }
  }
  if (s.size() == 7 && s.compare(0, 3, "mat") == 0 && s[4] == 'x' && (s[6] == 'f' || s[6] == 'h')) {
    int c = s[3] - '0', r = s[5] - '0';
    if (c >= 2 && c <= 4 && r >= 2 && r <= 4) { t = mat(c, r); return true; }
  }
  return false;
}
// Generators that take <T>: vecN, matCxR.
bool wgsl_generator(const std::string &s, int &n, int &m) {
  if (s.size() == 4 && s.compare(0, 3, "vec") == 0 && s[3] >= '2' && s[3] <= '4') { n = s[3] - '0'; m = 1; return true; }
  if (s.size() == 6 && s.compare(0, 3, "mat") == 0 && s[4] == 'x') {
    int c = s[3] - '0', r = s[5] - '0';
    if (c >= 2 && c <= 4 && r >= 2 && r <= 4) { n = r; m = c; return true; }
  }
  return false;
}

int swz_index(char c) {
  switch (c) {
    case 'x': case 'r': case 's': return 0;
    case 'y': case 'g': case 't': return 1;
    case 'z': case 'b': case 'p': return 2;
    case 'w': case 'a': case 'q': return 3;
  }
  return -1;
}

// ---------------------------------------------------------------------------
// Parser (both languages share the expression grammar)

class Parser {
 public:
  Parser(Module &m, const std::vector<Tok> &toks, Lang lang) : M(m), T(toks), L(lang) {}

  void parse_module() {
    while (!at_end()) {
      if (L == Lang::WGSL) wgsl_global();
      else glsl_global();
    }
  }

 private:
  Module &M;
  const std::vector<Tok> &T;
  Lang L;
  size_t p = 0;

  const Tok &cur() const { return T[p]; }
  const Tok &peek(int k = 1) const { return T[std::min(p + size_t(k), T.size() - 1)]; }
  bool at_end() const { return T[p].k == TK::End; }
  bool is(const char *s) const { return T[p].k == TK::Punct && T[p].s == s; }
  bool is_kw(const char *s) const { return T[p].k == TK::Ident && T[p].s == s; }
  bool accept(const char *s) { if (is(s)) { ++p; return true; } return false; }
  bool accept_kw(const char *s) { if (is_kw(s)) { ++p; return true; } return false; }
  void expect(const char *s) {
    if (!accept(s)) fail(cur().line, std::string("expected '") + s + "' but found '" + (at_end() ? "end of input" : cur().s) + "'");
  }
  std::string ident() {
    if (cur().k != TK::Ident) fail(cur().line, "expected an identifier but found '" + cur().s + "'");
    return T[p++].s;
  }

  // ---- WGSL -------------------------------------------------------------
  void skip_attributes() {
    while (accept("@")) {
      ident();
      if (accept("(")) {
        int depth = 1;
        while (!at_end() && depth > 0) {
          if (is("(")) ++depth;
          else if (is(")")) --depth;
          ++p;
        }
      }
    }
  }

  Ty wgsl_type() {
    int line = cur().line;
    std::string s = ident();
    Ty t;
    if (parse_wgsl_simple_type(s, t)) return t;
    auto al = M.aliases.find(s);
    if (al != M.aliases.end()) return al->second;
    int n, m;
    if (wgsl_generator(s, n, m)) {
      expect("<");
      Ty e = wgsl_type();
      expect(">");
      if (!is_scalar(e)) fail(line, "vector element must be a scalar");
      if (m > 1) {
        if (e.b != B::F32) fail(line, "only f32 matrices are supported");
        return mat(m, n);
      }
      return vec(e.b, n);
    }
    fail(line, "unknown or unsupported type '" + s + "'");
  }

  void wgsl_global() {
    skip_attributes();
    if (accept(";")) return;
    int line = cur().line;
    if (accept_kw("fn")) { wgsl_function(line); return; }
    if (accept_kw("const") || is_kw("override")) {
      if (is_kw("override")) fail(line, "'override' declarations are not supported");
      Global *g = new_global(line, true);
      g->name = ident();
      if (accept(":")) { g->has_type = true; g->t = wgsl_type(); }
      expect("=");
      g->init = expr();
      expect(";");
      add_global(g);
      return;
    }
    if (accept_kw("var")) {
      if (accept("<")) {
        std::string space = ident();
        if (space != "private") fail(line, "only var<private> is supported at module scope");
        expect(">");
      }
      Global *g = new_global(line, false);
      g->name = ident();
      if (accept(":")) { g->has_type = true; g->t = wgsl_type(); }
      if (accept("=")) g->init = expr();
      expect(";");
      add_global(g);
      return;
    }
    if (accept_kw("alias")) {
      std::string name = ident();
      expect("=");
      M.aliases[name] = wgsl_type();
      expect(";");
      return;
    }
    if (accept_kw("enable") || accept_kw("requires") || accept_kw("diagnostic")) {
      while (!at_end() && !is(";")) ++p;
      expect(";");
      return;
    }
    if (is_kw("struct")) fail(line, "struct declarations are not supported");
    if (is_kw("use") || is_kw("include")) fail(line, "'" + cur().s + "' must be a line of its own ending in ';'");
    fail(line, "unexpected '" + cur().s + "' at module scope");
  }

  Global *new_global(int line, bool is_const) {
    M.globals_own.emplace_back(new Global());
    Global *g = M.globals_own.back().get();
    g->line = line;
    g->is_const = is_const;
    g->lang = L;
    return g;
  }
  void add_global(Global *g) {
    if (M.glob_by_name.count(g->name)) {
      // the same module text inserted twice by `use`
      fail(g->line, "'" + g->name + "' is declared twice at module scope");
    }
    M.glob_by_name[g->name] = g;
    M.globals.push_back(g);
  }

  void wgsl_function(int line) {
    M.funcs_own.emplace_back(new Func());
    Func *f = M.funcs_own.back().get();
    f->line = line;
    f->lang = L;
    f->name = ident();
    expect("(");
    while (!is(")")) {
      skip_attributes();
      Param prm;
      prm.name = ident();
      expect(":");
      prm.t = wgsl_type();
      f->params.push_back(prm);
      if (!accept(",")) break;
    }
    expect(")");
    f->ret = scalar(B::Void);
    if (accept("->")) {
      skip_attributes();
      f->ret = wgsl_type();
    }
    f->body = block();
    M.add_func(f);
  }

  // ---- GLSL -------------------------------------------------------------
  bool glsl_is_type_start() const {
    if (cur().k != TK::Ident) return false;
    Ty t;
    return parse_glsl_type_name(cur().s, t);
  }
  Ty glsl_type() {
    int line = cur().line;
    std::string s = ident();
    Ty t;
    if (!parse_glsl_type_name(s, t)) fail(line, "unknown or unsupported type '" + s + "'");
    return t;
  }
  void glsl_qualifiers(bool &is_const, bool &is_uniform, bool &is_out) {
    for (;;) {
      if (accept_kw("const")) { is_const = true; continue; }
      if (accept_kw("uniform")) { is_uniform = true; continue; }
      if (accept_kw("in")) continue;
      if (accept_kw("out") || accept_kw("inout")) { is_out = true; continue; }
      if (accept_kw("highp") || accept_kw("mediump") || accept_kw("lowp") || accept_kw("flat") ||
          accept_kw("smooth") || accept_kw("noperspective") || accept_kw("centroid") || accept_kw("invariant") ||
          accept_kw("precise"))
        continue;
      if (accept_kw("layout")) {
        expect("(");
        int depth = 1;
        while (!at_end() && depth > 0) {
          if (is("(")) ++depth;
          else if (is(")")) --depth;
          ++p;
        }
        continue;
      }
      break;
    }
  }

  void glsl_global() {
    int line = cur().line;
    if (accept(";")) return;
    if (accept_kw("precision")) {
      while (!at_end() && !is(";")) ++p;
      expect(";");
      return;
    }
    if (is_kw("struct")) fail(line, "struct declarations are not supported");
    bool is_const = false, is_uniform = false, is_out = false;
    glsl_qualifiers(is_const, is_uniform, is_out);
    if (is_out && !glsl_is_type_start()) fail(line, "unexpected declaration");
    Ty t = glsl_type();
    std::string name = ident();
    if (is("(")) {
      glsl_function(line, t, name);
      return;
    }
    // variable list
    for (;;) {
      if (accept("[")) fail(line, "arrays are not supported");
      Global *g = new_global(line, is_const || is_uniform);
      g->name = name;
      g->has_type = true;
      g->t = t;
      if (is_uniform) {
        M.warnings.push_back("line " + std::to_string(line) + ": uniform '" + name + "' is bound to zero");
      }
      if (accept("=")) g->init = assign_free_expr();
      if (is_out) fail(line, "'out' variables at module scope are not supported");
      add_global(g);
      if (!accept(",")) break;
      name = ident();
    }
    expect(";");
  }

  void glsl_function(int line, Ty ret, const std::string &name) {
    M.funcs_own.emplace_back(new Func());
    Func *f = M.funcs_own.back().get();
    f->line = line;
    f->lang = L;
    f->name = name;
    f->ret = ret;
    expect("(");
    if (is_kw("void") && peek().k == TK::Punct && peek().s == ")") ++p;
    while (!is(")")) {
      bool c = false, u = false, o = false;
      glsl_qualifiers(c, u, o);
      Param prm;
      prm.t = glsl_type();
      prm.out = o;
      if (cur().k == TK::Ident) prm.name = ident();
      if (accept("[")) fail(line, "array parameters are not supported");
      f->params.push_back(prm);
      if (!accept(",")) break;
    }
    expect(")");
    if (accept(";")) { M.funcs_own.pop_back(); return; }  // prototype
    f->body = block();
    M.add_func(f);
  }

  // ---- statements ---------------------------------------------------------
  Stmt *block() {
    int line = cur().line;
    expect("{");
    Stmt *b = M.st(Stmt::Block, line);
    while (!is("}")) {
      if (at_end()) fail(line, "unterminated block");
      b->body.push_back(statement());
    }
    expect("}");
    return b;
  }

  Stmt *as_block(Stmt *s) {
    if (s->k == Stmt::Block) return s;
    Stmt *b = M.st(Stmt::Block, s->line);
    b->body.push_back(s);
    return b;
  }

  Stmt *statement() {
    int line = cur().line;
    if (is("{")) return block();
    if (accept(";")) return M.st(Stmt::Empty, line);
    if (L == Lang::WGSL) skip_attributes();
    if (accept_kw("return")) {
      Stmt *s = M.st(Stmt::Return, line);
      if (!is(";")) s->val = expr();
      expect(";");
      return s;
    }
    if (accept_kw("if")) {
      Stmt *s = M.st(Stmt::If, line);
      if (L == Lang::GLSL) { expect("("); s->cond = expr(); expect(")"); s->then_s = as_block(statement()); }
      else { s->cond = expr(); s->then_s = block(); }
      if (accept_kw("else")) {
        if (L == Lang::WGSL && !is_kw("if")) s->else_s = block();
        else s->else_s = as_block(statement());
      }
      return s;
    }
    if (accept_kw("for")) {
      Stmt *s = M.st(Stmt::For, line);
      expect("(");
      if (!is(";")) s->init_s = simple_statement(true);
      expect(";");
      if (!is(";")) s->cond = expr();
      expect(";");
      if (!is(")")) s->update_s = simple_statement(false);
      expect(")");
      s->loop_body = L == Lang::GLSL ? as_block(statement()) : block();
      return s;
    }
    if (accept_kw("while")) {
      Stmt *s = M.st(Stmt::While, line);
      if (L == Lang::GLSL) { expect("("); s->cond = expr(); expect(")"); s->loop_body = as_block(statement()); }
      else { s->cond = expr(); s->loop_body = block(); }
      return s;
    }
    if (L == Lang::GLSL && accept_kw("do")) {
      Stmt *s = M.st(Stmt::DoWhile, line);
      s->loop_body = as_block(statement());
      if (!accept_kw("while")) fail(cur().line, "expected 'while'");
      expect("(");
      s->cond = expr();
      expect(")");
      expect(";");
      return s;
    }
    if (L == Lang::WGSL && accept_kw("loop")) {
      Stmt *s = M.st(Stmt::Loop, line);
      expect("{");
      Stmt *b = M.st(Stmt::Block, line);
      while (!is("}")) {
        if (at_end()) fail(line, "unterminated loop");
        if (is_kw("continuing")) {
          ++p;
          s->continuing = block();
          continue;
        }
        b->body.push_back(statement());
      }
      expect("}");
      s->loop_body = b;
      return s;
    }
    if (accept_kw("break")) {
      if (L == Lang::WGSL && accept_kw("if")) {
        Stmt *s = M.st(Stmt::BreakIf, line);
        s->cond = expr();
        expect(";");
        return s;
      }
      expect(";");
      return M.st(Stmt::Break, line);
    }
    if (accept_kw("continue")) { expect(";"); return M.st(Stmt::Continue, line); }
    if (is_kw("discard")) fail(line, "'discard' is not supported in an SDF");
    if (is_kw("switch")) fail(line, "'switch' is not supported");
    Stmt *s = simple_statement(true);
    expect(";");
    return s;
  }

  // Declarations, assignments, increments and call statements (also the
  // init / update clauses of `for`).
  Stmt *simple_statement(bool allow_decl) {
    int line = cur().line;
    if (allow_decl && L == Lang::WGSL && (is_kw("let") || is_kw("var") || is_kw("const"))) {
      Stmt *s = M.st(Stmt::Decl, line);
      std::string kw = ident();
      s->decl_kind = kw == "let" ? 0 : (kw == "var" ? 1 : 2);
      if (s->decl_kind == 1 && accept("<")) { ident(); expect(">"); }
      s->name = ident();
      if (accept(":")) { s->has_type = true; s->decl_t = wgsl_type(); }
      if (accept("=")) s->init = expr();
      else if (s->decl_kind != 1) fail(line, "'" + kw + "' needs an initializer");
      if (s->decl_kind == 1 && !s->has_type && !s->init) fail(line, "'var' needs a type or an initializer");
      return s;
    }
    if (allow_decl && L == Lang::GLSL && (glsl_is_type_start() || is_kw("const") || is_kw("highp") || is_kw("mediump") || is_kw("lowp"))) {
      // `T a = x, b;` -> a block of declarations (emitted without braces)
      bool c = false, u = false, o = false;
      glsl_qualifiers(c, u, o);
      Ty t = glsl_type();
      if (is("(")) {  // constructor call used as a statement
        p -= 1;
      } else {
        Stmt *grp = M.st(Stmt::Block, line);
        grp->decl_kind = -1;  // marks a declaration group (no new scope)
        for (;;) {
          Stmt *s = M.st(Stmt::Decl, line);
          s->decl_kind = c ? 2 : 1;
          s->name = ident();
          if (accept("[")) fail(line, "arrays are not supported");
          s->has_type = true;
          s->decl_t = t;
          if (accept("=")) s->init = assign_free_expr();
          grp->body.push_back(s);
          if (!accept(",")) break;
        }
        return grp->body.size() == 1 ? grp->body[0] : grp;
      }
    }
    if (L == Lang::WGSL && is_kw("_") && peek().k == TK::Punct && peek().s == "=") {
      p += 2;
      Stmt *s = M.st(Stmt::ExprS, line);
      s->val = expr();
      return s;
    }
    if (is("++") || is("--")) {
      Stmt *s = M.st(Stmt::IncDec, line);
      s->op = cur().s;
      s->prefix = true;
      ++p;
      s->lhs = unary();
      return s;
    }
    Expr *lhs = unary();
    if (is("++") || is("--")) {
      Stmt *s = M.st(Stmt::IncDec, line);
      s->op = cur().s;
      ++p;
      s->lhs = lhs;
      return s;
    }
    static const char *aops[] = {"=", "+=", "-=", "*=", "/=", "%=", "&=", "|=", "^=", "<<=", ">>="};
    for (const char *op : aops) {
      if (is(op)) {
        ++p;
        Stmt *s = M.st(Stmt::Assign, line);
        s->op = op;
        s->lhs = lhs;
        s->rhs = expr();
        return s;
      }
    }
    // any other expression statement: must be a call (or a full expression in GLSL)
    Expr *full = binary_rest(lhs, 0);
    if (L == Lang::GLSL && is("?")) full = ternary_rest(full);
    Stmt *s = M.st(Stmt::ExprS, line);
    s->val = full;
    return s;
  }

  // ---- expressions ----------------------------------------------------------
  Expr *expr() {
    Expr *e = binary_rest(unary(), 0);
    if (L == Lang::GLSL && is("?")) e = ternary_rest(e);
    return e;
  }
  Expr *assign_free_expr() { return expr(); }
  Expr *ternary_rest(Expr *c) {
    int line = cur().line;
    expect("?");
    Expr *a = expr();
    expect(":");
    Expr *b = expr();
    Expr *e = M.ex(Expr::Ternary, line);
    e->a = {c, a, b};
    return e;
  }

  static int prec(const std::string &op) {
    if (op == "||") return 1;
    if (op == "&&") return 2;
    if (op == "|") return 3;
    if (op == "^") return 4;
    if (op == "&") return 5;
    if (op == "==" || op == "!=") return 6;
    if (op == "<" || op == ">" || op == "<=" || op == ">=") return 7;
    if (op == "<<" || op == ">>") return 8;
    if (op == "+" || op == "-") return 9;
    if (op == "*" || op == "/" || op == "%") return 10;
    return -1;
  }

  Expr *binary_rest(Expr *lhs, int min_prec) {
    for (;;) {
      if (cur().k != TK::Punct) return lhs;
      std::string op = cur().s;
      int pr = prec(op);
      if (pr < 0 || pr < min_prec) return lhs;
      int line = cur().line;
      ++p;
      Expr *rhs = unary();
      for (;;) {
        if (cur().k != TK::Punct) break;
        int p2 = prec(cur().s);
        if (p2 <= pr) break;
        rhs = binary_rest(rhs, p2);
      }
      Expr *e = M.ex(Expr::Binary, line);
      e->s = op;
      e->a = {lhs, rhs};
      lhs = e;
    }
  }

  Expr *unary() {
    int line = cur().line;
    if (is("-") || is("!") || is("~") || is("+")) {
      std::string op = cur().s;
      ++p;
      Expr *x = unary();
      if (op == "+") return x;
      Expr *e = M.ex(Expr::Unary, line);
      e->s = op;
      e->a = {x};
      return e;
    }
    if (is("&") || is("*")) fail(line, "pointers are not supported");
    if (L == Lang::GLSL && (is("++") || is("--"))) fail(line, "increment inside an expression is not supported");
    return postfix(primary());
  }

  Expr *postfix(Expr *e) {
    for (;;) {
      int line = cur().line;
      if (accept(".")) {
        std::string s = ident();
        Expr *w = M.ex(Expr::Swz, line);
        w->a = {e};
        w->s = s;
        for (char c : s) {
          int k = swz_index(c);
          if (k < 0 || s.size() > 4) fail(line, "unsupported member '." + s + "' (structs are not supported)");
          w->swz.push_back(k);
        }
        e = w;
        continue;
      }
      if (accept("[")) {
        Expr *ix = M.ex(Expr::Index, line);
        ix->a = {e, expr()};
        expect("]");
        e = ix;
        continue;
      }
      return e;
    }
  }

  std::vector<Expr *> call_args() {
    std::vector<Expr *> args;
    expect("(");
    while (!is(")")) {
      args.push_back(expr());
      if (!accept(",")) break;
    }
    expect(")");
    return args;
  }

  Expr *primary() {
    const Tok &t = cur();
    int line = t.line;
    if (t.k == TK::Int || t.k == TK::Float) {
      ++p;
      Expr *e = M.ex(Expr::Lit, line);
      e->lit = t.num;
      e->flit = t.fnum;
      if (t.k == TK::Float) e->lit_b = (L == Lang::GLSL || t.suffix == 'f') ? B::F32 : B::AFloat;
      else if (t.suffix == 'u') e->lit_b = B::U32;
      else if (t.suffix == 'i' || L == Lang::GLSL) e->lit_b = B::I32;
      else e->lit_b = B::AInt;
      if (e->lit_b == B::F32) e->lit = double(t.fnum);
      return e;
    }
    if (accept("(")) {
      Expr *e = expr();
      expect(")");
      return e;
    }
    if (t.k == TK::Ident) {
      if (t.s == "true" || t.s == "false") {
        ++p;
        Expr *e = M.ex(Expr::Lit, line);
        e->lit_b = B::Bool;
        e->lit = t.s == "true" ? 1 : 0;
        return e;
      }
      // type constructors
      if (L == Lang::WGSL) {
        int n, m;
        Ty ty;
        if (wgsl_generator(t.s, n, m)) {
          ++p;
          Expr *e = M.ex(Expr::Call, line);
          e->is_ctor = true;
          if (accept("<")) {
            Ty el = wgsl_type();
            expect(">");
            e->ctor_t = m > 1 ? mat(m, n) : vec(el.b, n);
          } else {
            e->ctor_t = m > 1 ? mat(m, n) : vec(B::Void, n);  // element type inferred
            if (m > 1) e->ctor_t.b = B::F32;
          }
          e->s = t.s;
          e->a = call_args();
          return e;
        }
        if (parse_wgsl_simple_type(t.s, ty) || M.aliases.count(t.s)) {
          if (peek().k == TK::Punct && peek().s == "(") {
            ++p;
            if (M.aliases.count(t.s)) ty = M.aliases[t.s];
            Expr *e = M.ex(Expr::Call, line);
            e->is_ctor = true;
            e->ctor_t = ty;
            e->s = t.s;
            e->a = call_args();
            return e;
          }
        }
        if (t.s == "array" || t.s == "ptr") fail(line, "'" + t.s + "' is not supported");
      } else {
        Ty ty;
        if (parse_glsl_type_name(t.s, ty)) {
          ++p;
          Expr *e = M.ex(Expr::Call, line);
          e->is_ctor = true;
          e->ctor_t = ty;
          e->s = t.s;
          e->a = call_args();
          return e;
        }
      }
      ++p;
      if (is("(")) {
        Expr *e = M.ex(Expr::Call, line);
        e->s = t.s;
        e->a = call_args();
        return e;
      }
      Expr *e = M.ex(Expr::Ref, line);
      e->s = t.s;
      return e;
    }
    fail(line, "unexpected '" + (t.k == TK::End ? std::string("end of input") : t.s) + "'");
  }
};

// ---------------------------------------------------------------------------
// Constant folding helpers

double round_as(B b, double v) {
  switch (b) {
    case B::F32: return double(float(v));
    case B::I32: return double(int32_t(int64_t(v)));
    case B::U32: return double(uint32_t(int64_t(v)));
    case B::Bool: return v != 0 ? 1 : 0;
    default: return v;
  }
}

// ---------------------------------------------------------------------------
// Semantic analysis

struct Builtin {
  const char *name;
  int id;
};

enum BI {
  B_ABS, B_SIGN, B_FLOOR, B_CEIL, B_TRUNC, B_ROUND, B_FRACT, B_SQRT, B_INVSQRT, B_EXP, B_EXP2, B_LOG,
  B_LOG2, B_POW, B_SIN, B_COS, B_TAN, B_ASIN, B_ACOS, B_ATAN, B_ATAN2, B_SINH, B_COSH, B_TANH, B_MIN,
  B_MAX, B_CLAMP, B_SATURATE, B_MIX, B_STEP, B_SMOOTHSTEP, B_MOD, B_FMA, B_RADIANS, B_DEGREES,
  B_LENGTH, B_DISTANCE, B_DOT, B_CROSS, B_NORMALIZE, B_REFLECT, B_SELECT, B_ALL, B_ANY, B_TRANSPOSE,
  B_LT, B_LE, B_GT, B_GE, B_EQ, B_NE, B_NOT
};

const std::map<std::string, int> &builtin_table(Lang lang) {
  static const std::map<std::string, int> common = {
      {"abs", B_ABS}, {"sign", B_SIGN}, {"floor", B_FLOOR}, {"ceil", B_CEIL}, {"trunc", B_TRUNC},
      {"round", B_ROUND}, {"fract", B_FRACT}, {"sqrt", B_SQRT}, {"exp", B_EXP}, {"exp2", B_EXP2},
      {"log", B_LOG}, {"log2", B_LOG2}, {"pow", B_POW}, {"sin", B_SIN}, {"cos", B_COS}, {"tan", B_TAN},
      {"asin", B_ASIN}, {"acos", B_ACOS}, {"atan", B_ATAN}, {"sinh", B_SINH}, {"cosh", B_COSH},
      {"tanh", B_TANH}, {"min", B_MIN}, {"max", B_MAX}, {"clamp", B_CLAMP}, {"mix", B_MIX},
      {"step", B_STEP}, {"smoothstep", B_SMOOTHSTEP}, {"fma", B_FMA}, {"radians", B_RADIANS},
      {"degrees", B_DEGREES}, {"length", B_LENGTH}, {"distance", B_DISTANCE}, {"dot", B_DOT},
      {"cross", B_CROSS}, {"normalize", B_NORMALIZE}, {"reflect", B_REFLECT}, {"all", B_ALL},
      {"any", B_ANY}, {"transpose", B_TRANSPOSE}};
  static std::map<std::string, int> wgsl, glsl;
  if (wgsl.empty()) {
    wgsl = common;
    wgsl["inverseSqrt"] = B_INVSQRT;
    wgsl["atan2"] = B_ATAN2;
    wgsl["saturate"] = B_SATURATE;
    wgsl["select"] = B_SELECT;
    glsl = common;
    glsl["inversesqrt"] = B_INVSQRT;
    glsl["mod"] = B_MOD;
    glsl["roundEven"] = B_ROUND;
    glsl["lessThan"] = B_LT;
    glsl["lessThanEqual"] = B_LE;
    glsl["greaterThan"] = B_GT;
    glsl["greaterThanEqual"] = B_GE;
    glsl["equal"] = B_EQ;
    glsl["notEqual"] = B_NE;
    glsl["not"] = B_NOT;
  }
  return lang == Lang::WGSL ? wgsl : glsl;
}

class Sema {
 public:
  Sema(Module &m) : M(m) {}
  Module &M;
  std::vector<std::map<std::string, Sym *>> scopes;
  Func *cur_fn = nullptr;
  Lang L = Lang::WGSL;
  int loop_depth = 0;

  // ---- globals --------------------------------------------------------
  void resolve_global(Global *g) {
    if (g->resolved) return;
    if (g->resolving) fail(g->line, "'" + g->name + "' is defined in terms of itself");
    g->resolving = true;
    Lang saved = L;
    L = g->lang;
    auto saved_scopes = scopes;
    scopes.clear();
    Sym *s = M.sym(g->is_const ? Sym::Const : Sym::Global, g->name, g->t);
    s->cname = "g_" + g->name;
    if (g->init) {
      check(g->init);
      Ty t = g->has_type ? g->t : (g->is_const ? g->init->t : concrete(g->init->t));
      coerce(g->init, t, "initializer of '" + g->name + "'");
      s->t = t;
      if (g->init->cst) {
        s->cst = true;
        s->cv = fold_to(g->init, t);
      } else if (g->is_const && g->lang == Lang::WGSL) {
        fail(g->line, "initializer of const '" + g->name + "' is not a constant expression");
      }
    } else {
      s->t = g->t;
      s->cst = true;  // zero-initialised private / uniform
      s->cv.assign(size_t(ncomp(g->t)), 0.0);
    }
    if (!s->cst) {
      fail(g->line, "module-scope variable '" + g->name + "' needs a constant initializer");
    }
    g->sym = s;
    g->resolved = true;
    g->resolving = false;
    scopes = saved_scopes;
    L = saved;
  }

  Sym *lookup(const std::string &name) {
    for (auto it = scopes.rbegin(); it != scopes.rend(); ++it) {
      auto f = it->find(name);
      if (f != it->end()) return f->second;
    }
    auto g = M.glob_by_name.find(name);
    if (g != M.glob_by_name.end()) {
      resolve_global(g->second);
      return g->second->sym;
    }
    return nullptr;
  }

  // ---- functions -------------------------------------------------------
  void check_function(Func *f) {
    if (f->checked) return;
    if (f->checking) return;  // recursion is rejected by the emitter's call graph
    f->checking = true;
    Func *saved_fn = cur_fn;
    Lang saved_l = L;
    auto saved_scopes = scopes;
    cur_fn = f;
    L = f->lang;
    scopes.clear();
    scopes.emplace_back();
    for (Param &prm : f->params) {
      if (prm.name.empty()) continue;
      Sym *s = M.sym(Sym::Param, prm.name, prm.t);
      s->cname = "a_" + prm.name;
      s->is_ref = prm.out;
      prm.sym = s;
      scopes.back()[prm.name] = s;
    }
    check_block(f->body, false);
    scopes = saved_scopes;
    L = saved_l;
    cur_fn = saved_fn;
    f->checking = false;
    f->checked = true;
  }

  void check_block(Stmt *b, bool new_scope) {
    if (new_scope) scopes.emplace_back();
    for (Stmt *s : b->body) check_stmt(s);
    if (new_scope) scopes.pop_back();
  }

  void declare(Stmt *s) {
    auto &top = scopes.back();
    if (top.count(s->name)) fail(s->line, "'" + s->name + "' is already declared in this scope");
    top[s->name] = s->sym;
  }

  void check_stmt(Stmt *s) {
    switch (s->k) {
      case Stmt::Block:
        check_block(s, s->decl_kind != -1);
        break;
      case Stmt::Empty: break;
      case Stmt::Decl: {
        Ty t;
        if (s->init) check(s->init);
        if (s->has_type) t = s->decl_t;
        else if (s->decl_kind == 2) t = s->init->t;  // const keeps abstract types
        else t = concrete(s->init->t);
        if (t.b == B::Void) fail(s->line, "cannot declare '" + s->name + "' of type void");
        if (s->init) coerce(s->init, t, "initializer of '" + s->name + "'");
        Sym *sym = M.sym(s->decl_kind == 0 ? Sym::Let : (s->decl_kind == 1 ? Sym::Var : Sym::Const), s->name, t);
        // unique per declaration: `let x = x + 1.0;` in an inner scope must
        // still read the outer x in C++
        sym->cname = "v_" + s->name + "_" + std::to_string(M.syms.size());
        if (s->decl_kind == 2) {
          if (s->init && s->init->cst) {
            sym->cst = true;
            sym->cv = fold_to(s->init, t);
          } else if (L == Lang::WGSL) {
            fail(s->line, "initializer of const '" + s->name + "' is not a constant expression");
          } else {
            sym->k = Sym::Let;  // GLSL const with a runtime initializer
          }
        }
        s->sym = sym;
        s->decl_t = t;
        declare(s);
        break;
      }
      case Stmt::Assign: {
        check(s->lhs);
        check(s->rhs);
        check_lvalue(s->lhs);
        if (s->op == "=") {
          coerce(s->rhs, s->lhs->t, "assignment");
        } else {
          std::string bop = s->op.substr(0, s->op.size() - 1);
          Ty rt = binary_type(bop, s->lhs, s->rhs, s->line);
          if (rt != s->lhs->t) fail(s->line, "compound assignment changes the type of the target");
        }
        break;
      }
      case Stmt::IncDec:
        check(s->lhs);
        check_lvalue(s->lhs);
        if (!is_scalar(s->lhs->t) || !is_num(s->lhs->t.b)) fail(s->line, "++/-- needs a numeric scalar");
        break;
      case Stmt::ExprS:
        check(s->val);
        if (s->val->k != Expr::Call && L == Lang::WGSL) fail(s->line, "expression statement must be a call");
        if (is_abstract(s->val->t)) coerce(s->val, concrete(s->val->t), "statement");
        break;
      case Stmt::If:
        check(s->cond);
        coerce(s->cond, scalar(B::Bool), "if condition");
        check_block(s->then_s, true);
        if (s->else_s) check_block(s->else_s, true);
        break;
      case Stmt::For:
        scopes.emplace_back();
        if (s->init_s) check_stmt(s->init_s);
        if (s->cond) { check(s->cond); coerce(s->cond, scalar(B::Bool), "loop condition"); }
        if (s->update_s) check_stmt(s->update_s);
        ++loop_depth;
        check_block(s->loop_body, true);
        --loop_depth;
        scopes.pop_back();
        break;
      case Stmt::While:
      case Stmt::DoWhile:
        check(s->cond);
        coerce(s->cond, scalar(B::Bool), "loop condition");
        ++loop_depth;
        check_block(s->loop_body, true);
        --loop_depth;
        break;
      case Stmt::Loop:
        ++loop_depth;
        scopes.emplace_back();
        check_block(s->loop_body, false);
        if (s->continuing) check_block(s->continuing, true);
        scopes.pop_back();
        --loop_depth;
        break;
      case Stmt::BreakIf:
        check(s->cond);
        coerce(s->cond, scalar(B::Bool), "break-if condition");
        break;
      case Stmt::Break:
      case Stmt::Continue:
        if (loop_depth == 0) fail(s->line, "break/continue outside a loop");
        break;
      case Stmt::Return:
        if (s->val) {
          check(s->val);
          if (cur_fn->ret.b == B::Void) fail(s->line, "return with a value in a void function");
          coerce(s->val, cur_fn->ret, "return value");
        } else if (cur_fn->ret.b != B::Void) {
          fail(s->line, "missing return value");
        }
        break;
    }
  }

  void check_lvalue(Expr *e) {
    Expr *base = e;
    while (base->k == Expr::Swz || base->k == Expr::Index) base = base->a[0];
    if (base->k != Expr::Ref || !base->sym) fail(e->line, "left side of assignment is not a variable");
    Sym *s = base->sym;
    if (s->k == Sym::Const || s->k == Sym::Let || s->k == Sym::Global) fail(e->line, "cannot assign to '" + s->name + "'");
    if (s->k == Sym::Param && L == Lang::WGSL) fail(e->line, "cannot assign to parameter '" + s->name + "'");
    if (e->k == Expr::Swz) {
      std::set<int> seen;
      for (int k : e->swz)
        if (!seen.insert(k).second) fail(e->line, "swizzle assignment repeats a component");
    }
    s->assigned = true;
  }

  // ---- expressions ------------------------------------------------------
  // Set the concrete type the consumer wants; abstract or (GLSL) convertible.
  void coerce(Expr *e, const Ty &want, const std::string &what) {
    if (e->t == want && !is_abstract(want)) { e->want = want; return; }
    if (is_abstract(want)) {  // abstract target (const decl): keep folded value
      if (conv_rank(e->t, want, L) < 0) fail(e->line, what + ": cannot convert " + tname(e->t) + " to " + tname(want));
      e->want = Ty();
      return;
    }
    int r = conv_rank(e->t, want, L);
    if (r < 0) fail(e->line, what + ": cannot convert " + tname(e->t) + " to " + tname(want));
    e->want = want;
  }
  Ty out_t(const Expr *e) const { return e->want.b != B::Void ? e->want : e->t; }

  std::vector<double> fold_to(const Expr *e, const Ty &t) {
    std::vector<double> v = e->cv;
    if (int(v.size()) == 1 && ncomp(t) > 1) v.assign(size_t(ncomp(t)), v[0]);
    for (double &x : v) x = round_as(t.b, x);
    return v;
  }

  // Unify two element types for a binary operation.
  B unify(B a, B b, int line, const std::string &op) {
    if (a == b) return a;
    if (is_abstract(a) && is_abstract(b)) return B::AFloat;
    if (is_abstract(a) && conv_rank(a, b, L) >= 0) return b;
    if (is_abstract(b) && conv_rank(b, a, L) >= 0) return a;
    if (L == Lang::GLSL) {
      if (conv_rank(a, b, L) >= 0) return b;
      if (conv_rank(b, a, L) >= 0) return a;
    }
    fail(line, "operator '" + op + "': mismatched types " + bname(a) + " and " + bname(b));
  }

  Ty binary_type(const std::string &op, Expr *a, Expr *b, int line) {
    Ty ta = a->t, tb = b->t;
    bool arith = op == "+" || op == "-" || op == "*" || op == "/" || op == "%";
    bool cmp = op == "<" || op == ">" || op == "<=" || op == ">=" || op == "==" || op == "!=";
    bool logic = op == "&&" || op == "||";
    bool bits = op == "&" || op == "|" || op == "^" || op == "<<" || op == ">>";
    if (logic) {
      coerce(a, scalar(B::Bool), "operand of " + op);
      coerce(b, scalar(B::Bool), "operand of " + op);
      return scalar(B::Bool);
    }
    if (ta.b == B::Void || tb.b == B::Void) fail(line, "void value in expression");
    if (bits) {
      if ((ta.b == B::Bool && tb.b == B::Bool) && (op == "&" || op == "|" || op == "^")) {
        coerce(a, ta, op); coerce(b, tb, op);
        return ta;
      }
      if (!is_int_b(ta.b) || !is_int_b(tb.b)) fail(line, "operator '" + op + "' needs integer operands");
    }
    if (is_mat(ta) || is_mat(tb)) {
      if (op != "*" && op != "+" && op != "-") fail(line, "operator '" + op + "' is not defined for matrices");
      auto fl = [&](Expr *e) { Ty t = e->t; if (is_abstract(t.b)) t.b = B::F32; coerce(e, with_b(t, B::F32), op); return with_b(t, B::F32); };
      Ty fa = fl(a), fb = fl(b);
      if (op == "*") {
        if (is_mat(fa) && is_mat(fb)) { if (fa.m != fb.n) fail(line, "matrix sizes do not match"); return mat(fb.m, fa.n); }
        if (is_mat(fa) && is_vec(fb)) { if (fa.m != fb.n) fail(line, "matrix * vector sizes do not match"); return vec(B::F32, fa.n); }
        if (is_vec(fa) && is_mat(fb)) { if (fa.n != fb.n) fail(line, "vector * matrix sizes do not match"); return vec(B::F32, fb.m); }
        if (is_mat(fa) && is_scalar(fb)) return fa;
        if (is_scalar(fa) && is_mat(fb)) return fb;
      } else if (fa == fb) {
        return fa;
      }
      fail(line, "invalid matrix operation");
    }
    if (!cmp && (!is_num(ta.b) || !is_num(tb.b))) fail(line, "operator '" + op + "' needs numeric operands");
    if (cmp && (ta.b == B::Bool || tb.b == B::Bool) && !(op == "==" || op == "!=")) fail(line, "ordering of booleans");
    if (is_vec(ta) && is_vec(tb) && ta.n != tb.n) fail(line, "operator '" + op + "': vector sizes differ");
    if ((is_vec(ta) || is_vec(tb)) && !(arith || cmp || bits)) fail(line, "invalid vector operation");
    if (cmp && L == Lang::GLSL && (is_vec(ta) || is_vec(tb))) fail(line, "GLSL compares vectors with lessThan() / equal()");
    if (cmp && (is_vec(ta) != is_vec(tb))) fail(line, "comparison of a vector with a scalar");
    B e = ta.b == B::Bool && tb.b == B::Bool ? B::Bool : unify(ta.b, tb.b, line, op);
    int n = std::max(ta.n, tb.n);
    coerce(a, with_b(ta, e), "operand of " + op);
    coerce(b, with_b(tb, e), "operand of " + op);
    if (cmp) return n > 1 ? vec(B::Bool, n) : scalar(B::Bool);
    return n > 1 ? vec(e, n) : scalar(e);
  }

  void check(Expr *e) {
    switch (e->k) {
      case Expr::Lit:
        e->t = scalar(e->lit_b);
        e->cst = true;
        e->cv = {e->lit};
        return;
      case Expr::Ref: {
        Sym *s = lookup(e->s);
        if (!s) {
          if (M.fn_by_name.count(e->s)) fail(e->line, "function '" + e->s + "' used as a value");
          fail(e->line, "unknown identifier '" + e->s + "'");
        }
        e->sym = s;
        e->t = s->t;
        if (s->cst && (s->k == Sym::Const || s->k == Sym::Global)) {
          e->cst = true;
          e->cv = s->cv;
        }
        return;
      }
      case Expr::Unary: {
        Expr *x = e->a[0];
        check(x);
        if (e->s == "!") {
          if (x->t.b != B::Bool) fail(e->line, "'!' needs a bool");
          coerce(x, x->t, "!");
          e->t = x->t;
        } else if (e->s == "-") {
          if (!is_num(x->t.b)) fail(e->line, "unary '-' needs a number");
          coerce(x, x->t, "-");
          e->t = x->t;
          if (x->t.b == B::U32 && L == Lang::WGSL) fail(e->line, "negation of u32");
        } else {
          if (!is_int_b(x->t.b)) fail(e->line, "'~' needs an integer");
          coerce(x, x->t, "~");
          e->t = x->t;
        }
        if (x->cst) {
          e->cst = true;
          e->cv = x->cv;
          for (double &v : e->cv) {
            if (e->s == "-") v = -v;
            else if (e->s == "!") v = v != 0 ? 0 : 1;
            else v = double(~int64_t(v));
            v = round_as(e->t.b, v);
          }
        }
        return;
      }
      case Expr::Binary: {
        check(e->a[0]);
        check(e->a[1]);
        e->t = binary_type(e->s, e->a[0], e->a[1], e->line);
        fold_binary(e);
        return;
      }
      case Expr::Ternary: {
        for (Expr *x : e->a) check(x);
        coerce(e->a[0], scalar(B::Bool), "?: condition");
        Ty ta = e->a[1]->t, tb = e->a[2]->t;
        if (ta.n != tb.n || ta.m != tb.m) fail(e->line, "?: branches differ in shape");
        B u = unify(ta.b, tb.b, e->line, "?:");
        e->t = with_b(ta, concrete_of(u));
        coerce(e->a[1], e->t, "?: branch");
        coerce(e->a[2], e->t, "?: branch");
        return;
      }
      case Expr::Swz: {
        Expr *x = e->a[0];
        check(x);
        if (!is_vec(x->t)) fail(e->line, "swizzle '." + e->s + "' of a non-vector (" + tname(x->t) + ")");
        for (int k : e->swz)
          if (k >= x->t.n) fail(e->line, "swizzle '." + e->s + "' out of range for " + tname(x->t));
        coerce(x, x->t, ".");
        e->t = e->swz.size() == 1 ? scalar(x->t.b) : vec(x->t.b, int(e->swz.size()));
        if (x->cst) {
          e->cst = true;
          e->cv.clear();
          for (int k : e->swz) e->cv.push_back(x->cv[size_t(k)]);
        }
        return;
      }
      case Expr::Index: {
        Expr *x = e->a[0], *i = e->a[1];
        check(x);
        check(i);
        if (!is_int_b(i->t.b) || !is_scalar(i->t)) fail(e->line, "index must be an integer");
        coerce(i, concrete(i->t), "index");
        if (is_mat(x->t)) e->t = vec(B::F32, x->t.n);
        else if (is_vec(x->t)) e->t = scalar(x->t.b);
        else fail(e->line, "indexing a non-vector");
        coerce(x, x->t, "[]");
        if (x->cst && i->cst) {
          int k = int(i->cv[0]);
          int w = is_mat(x->t) ? x->t.n : 1;
          if (k < 0 || k >= (is_mat(x->t) ? x->t.m : x->t.n)) fail(e->line, "constant index out of range");
          e->cst = true;
          e->cv.assign(x->cv.begin() + k * w, x->cv.begin() + (k + 1) * w);
        }
        return;
      }
      case Expr::Call:
        if (e->is_ctor) check_ctor(e);
        else check_call(e);
        return;
    }
  }

  void check_ctor(Expr *e) {
    for (Expr *x : e->a) check(x);
    Ty t = e->ctor_t;
    if (is_scalar(t)) {
      if (e->a.size() != 1) fail(e->line, "scalar conversion takes one argument");
      Expr *x = e->a[0];
      if (!is_scalar(x->t)) fail(e->line, "scalar conversion of a non-scalar");
      coerce(x, concrete(x->t), "conversion");
      e->t = t;
      if (x->cst) { e->cst = true; e->cv = {round_as(t.b, x->cv[0])}; }
      return;
    }
    if (is_mat(t)) {
      int total = 0;
      for (Expr *x : e->a) {
        Ty xt = x->t;
        if (is_abstract(xt.b)) xt.b = B::F32;
        if (xt.b != B::F32 && !(L == Lang::GLSL && is_num(xt.b))) fail(e->line, "matrix arguments must be float");
        coerce(x, with_b(x->t, B::F32), "matrix constructor");
        total += ncomp(x->t);
      }
      bool diag = e->a.size() == 1 && is_scalar(e->a[0]->t);
      bool cols = true;
      for (Expr *x : e->a) cols = cols && is_vec(x->t) && x->t.n == t.n;
      if (!diag && total != ncomp(t) && !(cols && int(e->a.size()) == t.m))
        fail(e->line, "matrix constructor needs " + std::to_string(ncomp(t)) + " components");
      e->t = t;
      return;
    }
    // vectors
    int n = t.n;
    B el = t.b;
    if (el == B::Void) {  // WGSL vec3(...) infers the element type
      if (e->a.empty()) { el = B::AFloat; e->t = vec(B::AFloat, n); e->cst = true; e->cv.assign(size_t(n), 0); return; }
      el = e->a[0]->t.b;
      for (Expr *x : e->a) el = unify(el, x->t.b, e->line, e->s);
    }
    int total = 0;
    for (Expr *x : e->a) {
      if (is_mat(x->t)) fail(e->line, "vector constructor from a matrix");
      total += ncomp(x->t);
    }
    bool splat = e->a.size() == 1 && is_scalar(e->a[0]->t);
    bool convert = e->a.size() == 1 && is_vec(e->a[0]->t) && e->a[0]->t.n == n;
    if (!e->a.empty() && !splat && total != n) {
      if (!(L == Lang::GLSL && total > n && e->a.size() == 1))
        fail(e->line, "vector constructor needs " + std::to_string(n) + " components, got " + std::to_string(total));
    }
    for (Expr *x : e->a) {
      Ty want = with_b(x->t, el);
      if (convert && !is_abstract(x->t.b) && x->t.b != el) {
        coerce(x, x->t, "conversion");  // explicit element conversion
      } else {
        if (!is_abstract(el) && conv_rank(x->t.b, el, L) < 0 && !(L == Lang::GLSL || (is_num(x->t.b) && is_num(el))))
          fail(e->line, "cannot convert " + tname(x->t) + " to " + bname(el));
        if (is_abstract(el)) coerce(x, want, "constructor");
        else if (conv_rank(x->t.b, el, L) >= 0) coerce(x, want, "constructor");
        else coerce(x, x->t, "constructor");  // explicit conversion (e.g. vec3<f32>(ivec))
      }
    }
    e->t = vec(el, n);
    bool all_c = true;
    for (Expr *x : e->a) all_c = all_c && x->cst;
    if (all_c) {
      e->cst = true;
      e->cv.clear();
      if (e->a.empty()) e->cv.assign(size_t(n), 0);
      else if (splat) e->cv.assign(size_t(n), e->a[0]->cv[0]);
      else for (Expr *x : e->a) for (double v : x->cv) if (int(e->cv.size()) < n) e->cv.push_back(v);
      for (double &v : e->cv) v = round_as(el, v);
    }
  }

  // Apply the builtin's signature: which args must share the float type.
  void check_call(Expr *e) {
    for (Expr *x : e->a) check(x);
    auto fit = M.fn_by_name.find(e->s);
    if (fit != M.fn_by_name.end()) {
      // user function: pick the best overload
      Func *best = nullptr;
      int best_cost = 1 << 30;
      bool ambiguous = false;
      for (Func *f : fit->second) {
        if (f->params.size() != e->a.size()) continue;
        int cost = 0;
        bool ok = true;
        for (size_t i = 0; i < e->a.size() && ok; ++i) {
          int r = conv_rank(e->a[i]->t, f->params[i].t, L);
          if (r < 0) ok = false;
          else cost += r;
        }
        if (!ok) continue;
        if (cost < best_cost) { best = f; best_cost = cost; ambiguous = false; }
        else if (cost == best_cost) ambiguous = true;
      }
      if (!best) {
        std::string sig;
        for (Expr *x : e->a) sig += (sig.empty() ? "" : ", ") + tname(x->t);
        fail(e->line, "no matching function for call to '" + e->s + "(" + sig + ")'");
      }
      if (ambiguous) fail(e->line, "ambiguous call to '" + e->s + "'");
      e->fn = best;
      for (size_t i = 0; i < e->a.size(); ++i) {
        coerce(e->a[i], best->params[i].t, "argument " + std::to_string(i + 1) + " of '" + e->s + "'");
        if (best->params[i].out) check_lvalue(e->a[i]);
      }
      e->t = best->ret;
      check_function(best);
      return;
    }
    const auto &tab = builtin_table(L);
    auto bit = tab.find(e->s);
    if (bit == tab.end()) fail(e->line, "unknown function '" + e->s + "'");
    int id = bit->second;
    if (id == B_ATAN && e->a.size() == 2) id = B_ATAN2;  // GLSL atan(y, x)
    e->cv.clear();
    e->sym = nullptr;
    e->lit = id;  // builtin id (reuses the literal slot)
    size_t na = e->a.size();
    auto need = [&](size_t k) { if (na != k) fail(e->line, "'" + e->s + "' takes " + std::to_string(k) + " arguments"); };
    // element type shared by all float arguments
    auto float_args = [&](std::initializer_list<int> idx) -> B {
      B el = B::Void;
      for (int i : idx) {
        Ty t = e->a[size_t(i)]->t;
        if (!is_num(t.b)) fail(e->line, "'" + e->s + "' needs numeric arguments");
        el = el == B::Void ? t.b : unify(el, t.b, e->line, e->s);
      }
      return el;
    };
    switch (id) {
      case B_ABS: case B_SIGN: {
        need(1);
        B el = float_args({0});
        e->t = with_b(e->a[0]->t, el);
        if (is_abstract(el)) e->t.b = el;
        coerce(e->a[0], e->t, e->s);
        fold_builtin(e, id);
        return;
      }
      case B_FLOOR: case B_CEIL: case B_TRUNC: case B_ROUND: case B_FRACT: case B_SQRT: case B_INVSQRT:
      case B_EXP: case B_EXP2: case B_LOG: case B_LOG2: case B_SIN: case B_COS: case B_TAN: case B_ASIN:
      case B_ACOS: case B_ATAN: case B_SINH: case B_COSH: case B_TANH: case B_SATURATE: case B_RADIANS:
      case B_DEGREES: {
        need(1);
        B el = float_args({0});
        el = is_abstract(el) ? B::AFloat : B::F32;
        if (e->a[0]->t.b != B::AInt && e->a[0]->t.b != B::AFloat && e->a[0]->t.b != B::F32 && L == Lang::WGSL)
          fail(e->line, "'" + e->s + "' needs a float argument");
        e->t = with_b(e->a[0]->t, el);
        coerce(e->a[0], e->t, e->s);
        fold_builtin(e, id);
        return;
      }
      case B_POW: case B_ATAN2: case B_MOD: case B_MIN: case B_MAX: case B_STEP: {
        need(2);
        B el = float_args({0, 1});
        if (id != B_MIN && id != B_MAX && id != B_MOD) el = is_abstract(el) ? B::AFloat : B::F32;
        if (id == B_MOD && !is_float_b(el) && L == Lang::GLSL) el = B::F32;
        Ty t0 = e->a[0]->t, t1 = e->a[1]->t;
        int n = std::max(t0.n, t1.n);
        if (t0.n != t1.n && !(L == Lang::GLSL || id == B_STEP) ) fail(e->line, "'" + e->s + "': argument sizes differ");
        if (t0.n != t1.n && id == B_STEP && !is_scalar(t0)) fail(e->line, "step(vec, scalar) is not defined");
        if (t0.n != t1.n && id != B_STEP && !is_scalar(t1)) fail(e->line, "'" + e->s + "': second argument must be a scalar or match");
        coerce(e->a[0], with_b(t0, el), e->s);
        coerce(e->a[1], with_b(t1, el), e->s);
        e->t = n > 1 ? vec(el, n) : scalar(el);
        fold_builtin(e, id);
        return;
      }
      case B_CLAMP: case B_MIX: case B_SMOOTHSTEP: case B_FMA: {
        need(3);
        B el = float_args({0, 1, 2});
        if (id != B_CLAMP) el = is_abstract(el) ? B::AFloat : B::F32;
        Ty t0 = e->a[0]->t, t1 = e->a[1]->t, t2 = e->a[2]->t;
        int n = std::max(t0.n, std::max(t1.n, t2.n));
        Ty rt = n > 1 ? vec(el, n) : scalar(el);
        if (id == B_CLAMP) {
          if (t0.n != n) fail(e->line, "clamp: first argument sets the size");
          coerce(e->a[0], rt, e->s);
          coerce(e->a[1], with_b(t1, el), e->s);
          coerce(e->a[2], with_b(t2, el), e->s);
          if ((t1.n != n && t1.n != 1) || (t2.n != n && t2.n != 1) || (t1.n != t2.n)) fail(e->line, "clamp argument sizes");
          if (t1.n != n && L == Lang::WGSL) fail(e->line, "clamp: bounds must match the value's size");
        } else if (id == B_MIX) {
          coerce(e->a[0], rt, e->s);
          coerce(e->a[1], rt, e->s);
          if (t0.n != n || t1.n != n) fail(e->line, "mix: first two arguments must match");
          coerce(e->a[2], with_b(t2, el), e->s);
          if (t2.n != n && t2.n != 1) fail(e->line, "mix argument sizes");
        } else if (id == B_SMOOTHSTEP) {
          if (t2.n != n) fail(e->line, "smoothstep: the value sets the size");
          coerce(e->a[0], with_b(t0, el), e->s);
          coerce(e->a[1], with_b(t1, el), e->s);
          coerce(e->a[2], rt, e->s);
          if (t0.n != t1.n || (t0.n != n && t0.n != 1)) fail(e->line, "smoothstep argument sizes");
        } else {
          for (int i = 0; i < 3; ++i) coerce(e->a[size_t(i)], rt, e->s);
          if (t0.n != n || t1.n != n || t2.n != n) fail(e->line, "fma argument sizes");
        }
        e->t = rt;
        fold_builtin(e, id);
        return;
      }
      case B_LENGTH: case B_NORMALIZE: {
        need(1);
        B el = float_args({0});
        el = is_abstract(el) ? B::AFloat : B::F32;
        coerce(e->a[0], with_b(e->a[0]->t, el), e->s);
        e->t = id == B_LENGTH ? scalar(el) : with_b(e->a[0]->t, el);
        fold_builtin(e, id);
        return;
      }
      case B_DISTANCE: case B_DOT: case B_REFLECT: case B_CROSS: {
        need(2);
        B el = float_args({0, 1});
        if (id != B_DOT) el = is_abstract(el) ? B::AFloat : B::F32;
        Ty t0 = e->a[0]->t, t1 = e->a[1]->t;
        if (t0.n != t1.n) fail(e->line, "'" + e->s + "': argument sizes differ");
        if (id == B_CROSS && t0.n != 3) fail(e->line, "cross needs vec3 arguments");
        if ((id == B_DOT || id == B_REFLECT) && !is_vec(t0)) fail(e->line, "'" + e->s + "' needs vectors");
        coerce(e->a[0], with_b(t0, el), e->s);
        coerce(e->a[1], with_b(t1, el), e->s);
        e->t = (id == B_DOT || id == B_DISTANCE) ? scalar(el) : with_b(t0, el);
        fold_builtin(e, id);
        return;
      }
      case B_SELECT: {
        need(3);
        Ty t0 = e->a[0]->t, t1 = e->a[1]->t;
        B el = unify(t0.b, t1.b, e->line, "select");
        el = concrete_of(el);
        if (t0.n != t1.n) fail(e->line, "select: value sizes differ");
        coerce(e->a[0], with_b(t0, el), "select");
        coerce(e->a[1], with_b(t1, el), "select");
        Ty ct = e->a[2]->t;
        if (ct.b != B::Bool || (ct.n != 1 && ct.n != t0.n)) fail(e->line, "select condition must be bool or vecN<bool>");
        coerce(e->a[2], ct, "select");
        e->t = with_b(t0, el);
        return;
      }
      case B_ALL: case B_ANY: case B_NOT: {
        need(1);
        if (e->a[0]->t.b != B::Bool) fail(e->line, "'" + e->s + "' needs booleans");
        coerce(e->a[0], e->a[0]->t, e->s);
        e->t = id == B_NOT ? e->a[0]->t : scalar(B::Bool);
        return;
      }
      case B_LT: case B_LE: case B_GT: case B_GE: case B_EQ: case B_NE: {
        need(2);
        B el = float_args({0, 1});
        el = concrete_of(el);
        Ty t0 = e->a[0]->t;
        if (!is_vec(t0) || t0.n != e->a[1]->t.n) fail(e->line, "'" + e->s + "' needs two vectors of one size");
        coerce(e->a[0], with_b(t0, el), e->s);
        coerce(e->a[1], with_b(e->a[1]->t, el), e->s);
        e->t = vec(B::Bool, t0.n);
        return;
      }
      case B_TRANSPOSE: {
        need(1);
        if (!is_mat(e->a[0]->t)) fail(e->line, "transpose needs a matrix");
        coerce(e->a[0], e->a[0]->t, "transpose");
        e->t = mat(e->a[0]->t.n, e->a[0]->t.m);
        return;
      }
    }
    fail(e->line, "unsupported builtin '" + e->s + "'");
  }

  // Fold binary expressions whose operands are both constant.  Abstract
  // results are kept in binary64; concrete ones round after the operation.
  void fold_binary(Expr *e) {
    Expr *a = e->a[0], *b = e->a[1];
    if (!a->cst || !b->cst) return;
    if (is_mat(a->t) || is_mat(b->t)) return;
    const std::string &op = e->s;
    Ty at = out_t(a), bt = out_t(b);
    if (at.b == B::Void) at = a->t;
    if (bt.b == B::Void) bt = b->t;
    // Concrete floating-point folding is left to the CUDA compiler (same
    // IEEE rounding); only abstract and integer / bool results fold here.
    B rb = e->t.b;
    bool cmp = rb == B::Bool && !(a->t.b == B::Bool && b->t.b == B::Bool && (op == "&&" || op == "||"));
    B opb = cmp ? (is_abstract(a->t.b) && is_abstract(b->t.b) ? B::AFloat : at.b) : rb;
    if (opb == B::F32) return;
    int n = std::max(int(a->cv.size()), int(b->cv.size()));
    e->cv.assign(size_t(n), 0);
    for (int i = 0; i < n; ++i) {
      double x = a->cv.size() == 1 ? a->cv[0] : a->cv[size_t(i)];
      double y = b->cv.size() == 1 ? b->cv[0] : b->cv[size_t(i)];
      x = round_as(opb, x);
      y = round_as(opb, y);
      double r = 0;
      bool is_int = opb == B::I32 || opb == B::U32 || opb == B::AInt;
      if (op == "+") r = x + y;
      else if (op == "-") r = x - y;
      else if (op == "*") r = x * y;
      else if (op == "/") {
        if (is_int) { if (y == 0) fail(e->line, "integer division by zero in a constant"); r = std::trunc(x / y); }
        else r = x / y;
      } else if (op == "%") {
        if (is_int) { if (y == 0) fail(e->line, "integer remainder by zero in a constant"); r = double(int64_t(x) % int64_t(y)); }
        else r = x - y * std::trunc(x / y);
      } else if (op == "<") r = x < y;
      else if (op == ">") r = x > y;
      else if (op == "<=") r = x <= y;
      else if (op == ">=") r = x >= y;
      else if (op == "==") r = x == y;
      else if (op == "!=") r = x != y;
      else if (op == "&&") r = (x != 0) && (y != 0);
      else if (op == "||") r = (x != 0) || (y != 0);
      else if (op == "&") r = double(int64_t(x) & int64_t(y));
      else if (op == "|") r = double(int64_t(x) | int64_t(y));
      else if (op == "^") r = double(int64_t(x) ^ int64_t(y));
      else if (op == "<<") r = double(int64_t(x) << int64_t(y));
      else if (op == ">>") r = double(int64_t(x) >> int64_t(y));
      e->cv[size_t(i)] = round_as(rb, r);
    }
    e->cst = true;
  }

  // Fold builtins over abstract arguments (binary64, as WGSL const-eval).
  void fold_builtin(Expr *e, int id) {
    if (!is_abstract(e->t.b)) return;
    for (Expr *x : e->a)
      if (!x->cst) fail(e->line, "abstract argument of '" + e->s + "' is not constant");
    auto arg = [&](size_t k, int i) {
      const auto &v = e->a[k]->cv;
      return v.size() == 1 ? v[0] : v[size_t(i)];
    };
    int n = ncomp(e->t);
    int an = ncomp(e->a[0]->t);
    e->cv.assign(size_t(n), 0);
    switch (id) {
      case B_LENGTH: case B_DISTANCE: case B_DOT: {
        double s = 0;
        for (int i = 0; i < an; ++i) {
          double d = id == B_DISTANCE ? arg(0, i) - arg(1, i) : arg(0, i);
          double w = id == B_DOT ? arg(1, i) : d;
          s += d * w;
        }
        e->cv[0] = id == B_DOT ? s : std::sqrt(s);
        break;
      }
      case B_NORMALIZE: {
        double s = 0;
        for (int i = 0; i < an; ++i) s += arg(0, i) * arg(0, i);
        s = std::sqrt(s);
        for (int i = 0; i < n; ++i) e->cv[size_t(i)] = arg(0, i) / s;
        break;
      }
      case B_CROSS: {
        double a0 = arg(0, 0), a1 = arg(0, 1), a2 = arg(0, 2), b0 = arg(1, 0), b1 = arg(1, 1), b2 = arg(1, 2);
        e->cv = {a1 * b2 - a2 * b1, a2 * b0 - a0 * b2, a0 * b1 - a1 * b0};
        break;
      }
      default:
        for (int i = 0; i < n; ++i) {
          double x = arg(0, i);
          double y = e->a.size() > 1 ? arg(1, i) : 0;
          double z = e->a.size() > 2 ? arg(2, i) : 0;
          double r = 0;
          switch (id) {
            case B_ABS: r = std::fabs(x); break;
            case B_SIGN: r = x > 0 ? 1 : (x < 0 ? -1 : 0); break;
            case B_FLOOR: r = std::floor(x); break;
            case B_CEIL: r = std::ceil(x); break;
            case B_TRUNC: r = std::trunc(x); break;
            case B_ROUND: r = std::nearbyint(x); break;
            case B_FRACT: r = x - std::floor(x); break;
            case B_SQRT: r = std::sqrt(x); break;
            case B_INVSQRT: r = 1.0 / std::sqrt(x); break;
            case B_EXP: r = std::exp(x); break;
            case B_EXP2: r = std::exp2(x); break;
            case B_LOG: r = std::log(x); break;
            case B_LOG2: r = std::log2(x); break;
            case B_POW: r = std::pow(x, y); break;
            case B_SIN: r = std::sin(x); break;
            case B_COS: r = std::cos(x); break;
            case B_TAN: r = std::tan(x); break;
            case B_ASIN: r = std::asin(x); break;
            case B_ACOS: r = std::acos(x); break;
            case B_ATAN: r = std::atan(x); break;
            case B_ATAN2: r = std::atan2(x, y); break;
            case B_SINH: r = std::sinh(x); break;
            case B_COSH: r = std::cosh(x); break;
            case B_TANH: r = std::tanh(x); break;
            case B_MIN: r = std::fmin(x, y); break;
            case B_MAX: r = std::fmax(x, y); break;
            case B_CLAMP: r = std::fmin(std::fmax(x, y), z); break;
            case B_SATURATE: r = std::fmin(std::fmax(x, 0.0), 1.0); break;
            case B_MIX: r = x * (1 - z) + y * z; break;
            case B_STEP: r = x <= y ? 1 : 0; break;
            case B_SMOOTHSTEP: { double t = std::fmin(std::fmax((z - x) / (y - x), 0.0), 1.0); r = t * t * (3 - 2 * t); break; }
            case B_MOD: r = x - y * std::floor(x / y); break;
            case B_FMA: r = x * y + z; break;
            case B_RADIANS: r = x * (M_PI / 180.0); break;
            case B_DEGREES: r = x * (180.0 / M_PI); break;
            case B_REFLECT: fail(e->line, "reflect of abstract vectors is not supported");
            default: fail(e->line, "cannot fold '" + e->s + "'");
          }
          e->cv[size_t(i)] = r;
        }
    }
    e->cst = true;
  }
};

// ---------------------------------------------------------------------------
// Cost model: algorithmic FP32 ops (add/sub/mul/min/max/abs/cmp/select = 1,
// fma = 2) and SFU-class ops (sqrt, div, transcendentals = 1) per call.

struct Cost {
  double fp = 0, sfu = 0;
  bool exact = true;
  Cost &operator+=(const Cost &o) { fp += o.fp; sfu += o.sfu; exact = exact && o.exact; return *this; }
};
Cost operator*(Cost c, double k) { c.fp *= k; c.sfu *= k; return c; }

class Coster {
 public:
  Cost expr(const Expr *e) {
    Cost c;
    if (e->cst && (is_abstract(e->t) || e->k == Expr::Lit)) return c;
    Ty t = e->want.b != B::Void ? e->want : e->t;
    int n = ncomp(t);
    for (const Expr *x : e->a) c += expr(x);
    bool flt = t.b == B::F32 || t.b == B::AFloat;
    switch (e->k) {
      case Expr::Binary: {
        const std::string &op = e->s;
        Ty at = e->a[0]->t;
        if (op == "*" && (is_mat(e->a[0]->t) || is_mat(e->a[1]->t))) {
          int k = is_mat(e->a[0]->t) ? e->a[0]->t.m : e->a[1]->t.n;
          c.fp += double(ncomp(t)) * (2 * k - 1);
        } else if (op == "/" && flt) c.sfu += n;
        else if (op == "%" && flt) { c.sfu += n; c.fp += 3.0 * n; }
        else if (op == "<" || op == ">" || op == "<=" || op == ">=" || op == "==" || op == "!=") c.fp += ncomp(at);
        else if (flt) c.fp += n;
        break;
      }
      case Expr::Ternary: c.fp += n; break;
      case Expr::Call:
        if (e->fn) c += func(e->fn);
        else if (!e->is_ctor) c += builtin(int(e->lit), e, n);
        break;
      default: break;
    }
    return c;
  }
  Cost builtin(int id, const Expr *e, int n) {
    Cost c;
    int an = e->a.empty() ? 1 : ncomp(e->a[0]->t);
    switch (id) {
      case B_ABS: case B_FLOOR: case B_CEIL: case B_TRUNC: case B_ROUND: case B_MIN: case B_MAX: c.fp = n; break;
      case B_SIGN: case B_STEP: c.fp = 2.0 * n; break;
      case B_FRACT: c.fp = 2.0 * n; break;
      case B_CLAMP: case B_SATURATE: c.fp = 2.0 * n; break;
      case B_MIX: c.fp = 4.0 * n; break;
      case B_SMOOTHSTEP: c.fp = 8.0 * n; c.sfu = n; break;
      case B_MOD: c.fp = 3.0 * n; c.sfu = n; break;
      case B_FMA: c.fp = 2.0 * n; break;
      case B_RADIANS: case B_DEGREES: c.fp = n; break;
      case B_SQRT: case B_EXP: case B_EXP2: case B_LOG: case B_LOG2: case B_POW: case B_SIN: case B_COS:
      case B_TAN: case B_ASIN: case B_ACOS: case B_ATAN: case B_ATAN2: case B_SINH: case B_COSH: case B_TANH:
        c.sfu = n; break;
      case B_INVSQRT: c.sfu = 2.0 * n; break;
      case B_LENGTH: c.fp = 2.0 * an - 1; c.sfu = 1; break;
      case B_DISTANCE: c.fp = 3.0 * an - 1; c.sfu = 1; break;
      case B_DOT: c.fp = 2.0 * an - 1; break;
      case B_NORMALIZE: c.fp = 2.0 * an - 1; c.sfu = 1.0 + an; break;
      case B_CROSS: c.fp = 9; break;
      case B_REFLECT: c.fp = 2.0 * an - 1 + 1 + 2.0 * an; break;
      case B_SELECT: c.fp = n; break;
      default: break;
    }
    return c;
  }
  Cost stmt(const Stmt *s) {
    Cost c;
    if (!s) return c;
    switch (s->k) {
      case Stmt::Block: for (const Stmt *x : s->body) c += stmt(x); break;
      case Stmt::Decl: if (s->init && !(s->sym && s->sym->cst)) c += expr(s->init); break;
      case Stmt::Assign: {
        c += expr(s->rhs);
        c += expr(s->lhs);
        if (s->op != "=") {
          Ty t = s->lhs->t;
          bool flt = t.b == B::F32;
          if (s->op == "/=" && flt) c.sfu += ncomp(t);
          else if (flt) c.fp += ncomp(t);
        }
        break;
      }
      case Stmt::IncDec: break;
      case Stmt::ExprS: c += expr(s->val); break;
      case Stmt::If: {
        c += expr(s->cond);
        Cost a = stmt(s->then_s), b = stmt(s->else_s);
        c += (a.fp + a.sfu >= b.fp + b.sfu) ? a : b;
        break;
      }
      case Stmt::For: {
        c += stmt(s->init_s);
        double trips = static_trips(s);
        Cost body = stmt(s->loop_body);
        body += stmt(s->update_s);
        if (s->cond) body += expr(s->cond);
        if (trips < 0) { trips = 1; c.exact = false; }
        c += body * trips;
        break;
      }
      case Stmt::While: case Stmt::DoWhile: case Stmt::Loop:
        c += stmt(s->loop_body);
        if (s->cond) c += expr(s->cond);
        c += stmt(s->continuing);
        c.exact = false;
        break;
      case Stmt::Return: if (s->val) c += expr(s->val); break;
      case Stmt::BreakIf: c += expr(s->cond); break;
      default: break;
    }
    return c;
  }
  // `for (i = a; i < b; i++)` with constant a, b.
  double static_trips(const Stmt *s) {
    if (!s->init_s || !s->cond || !s->update_s) return -1;
    const Stmt *in = s->init_s;
    if (in->k != Stmt::Decl || !in->init || !in->init->cst) return -1;
    const Expr *c = s->cond;
    if (c->k != Expr::Binary || c->a[0]->k != Expr::Ref || c->a[0]->sym != in->sym || !c->a[1]->cst) return -1;
    const Stmt *u = s->update_s;
    if (u->k != Stmt::IncDec || u->op != "++" || u->lhs->k != Expr::Ref || u->lhs->sym != in->sym) return -1;
    double a = in->init->cv[0], b = c->a[1]->cv[0];
    if (c->s == "<") return std::max(0.0, b - a);
    if (c->s == "<=") return std::max(0.0, b - a + 1);
    return -1;
  }
  Cost func(Func *f) {
    if (f->costed) { Cost c; c.fp = f->fp; c.sfu = f->sfu; c.exact = f->exact; return c; }
    if (f->costing) { Cost c; c.exact = false; return c; }
    f->costing = true;
    Cost c = stmt(f->body);
    f->costing = false;
    f->costed = true;
    f->fp = c.fp;
    f->sfu = c.sfu;
    f->exact = c.exact;
    return c;
  }
};

// ---------------------------------------------------------------------------
// Emitter

std::string flit(float v) {
  if (std::isnan(v)) return "__int_as_float(0x7fc00000)";
  if (std::isinf(v)) return v > 0 ? "__int_as_float(0x7f800000)" : "__int_as_float(0xff800000)";
  char b[64];
  std::snprintf(b, sizeof b, "%af", double(v));
  return std::string("(") + b + ")";
}

class Emitter {
 public:
  std::ostringstream out;
  int tmp = 0;
  int label = 0;
  std::vector<int> loop_labels;  // continuing labels of enclosing `loop`s (-1 = plain loop)

  std::string literal(const Ty &t, const std::vector<double> &cv) {
    auto one = [&](B b, double v) -> std::string {
      switch (concrete_of(b)) {
        case B::F32: return flit(float(v));
        case B::I32: return "(" + std::to_string(int32_t(int64_t(v))) + ")";
        case B::U32: return std::to_string(uint32_t(int64_t(v))) + "u";
        case B::Bool: return v != 0 ? "true" : "false";
        default: return "0";
      }
    };
    if (is_scalar(t)) return one(t.b, cv.empty() ? 0 : cv[0]);
    if (is_vec(t)) {
      std::string s = "s2mk(";
      for (int i = 0; i < t.n; ++i) s += (i ? ", " : "") + one(t.b, cv.size() == 1 ? cv[0] : cv[size_t(i)]);
      return s + ")";
    }
    std::string s = c_type(t) + "{{";
    for (int c = 0; c < t.m; ++c) {
      s += (c ? ", " : "") + std::string("s2mk(");
      for (int r = 0; r < t.n; ++r) s += (r ? ", " : "") + one(B::F32, cv[size_t(c * t.n + r)]);
      s += ")";
    }
    return s + "}}";
  }

  static Ty out_t(const Expr *e) { return e->want.b != B::Void ? e->want : concrete(e->t); }

  std::string convert(const std::string &code, const Ty &from, const Ty &to) {
    if (concrete(from) == to) return code;
    if (is_scalar(to)) return "((" + c_scalar(to.b) + ")(" + code + "))";
    if (is_vec(to)) return "s2cvt<" + c_scalar(to.b) + ">(" + code + ")";
    return code;
  }

  // Emit e as its consumed type.
  std::string ex(const Expr *e) {
    Ty t = out_t(e);
    if (e->cst && (is_abstract(e->t) || e->k == Expr::Lit || (e->k == Expr::Ref && e->sym &&
                                                               (e->sym->k == Sym::Const || e->sym->k == Sym::Global))))
      return literal(t, e->cv);
    std::string code = raw(e);
    return convert(code, e->t, t);
  }

  std::string raw(const Expr *e) {
    switch (e->k) {
      case Expr::Lit: return literal(concrete(e->t), e->cv);
      case Expr::Ref:
        if (e->sym->cst && (e->sym->k == Sym::Const || e->sym->k == Sym::Global)) return literal(concrete(e->t), e->sym->cv);
        return e->sym->cname;
      case Expr::Unary: return "(" + e->s + ex(e->a[0]) + ")";
      case Expr::Binary: {
        const std::string &op = e->s;
        const Expr *a = e->a[0], *b = e->a[1];
        Ty at = out_t(a);
        std::string A = ex(a), Bx = ex(b);
        if (op == "<" || op == ">" || op == "<=" || op == ">=" || op == "==" || op == "!=") {
          if (is_vec(at)) {
            static const std::map<std::string, std::string> fn = {{"<", "s2_lt"}, {">", "s2_gt"}, {"<=", "s2_le"}, {">=", "s2_ge"}, {"==", "s2_eq"}, {"!=", "s2_ne"}};
            return fn.at(op) + "(" + A + ", " + Bx + ")";
          }
          return "(" + A + " " + op + " " + Bx + ")";
        }
        if (op == "%" && (at.b == B::F32)) return "s2_fmod_wgsl(" + A + ", " + Bx + ")";
        if (op == "%") return "s2_imod(" + A + ", " + Bx + ")";
        return "(" + A + " " + op + " " + Bx + ")";
      }
      case Expr::Ternary: return "(" + ex(e->a[0]) + " ? " + ex(e->a[1]) + " : " + ex(e->a[2]) + ")";
      case Expr::Swz: {
        std::string x = ex(e->a[0]);
        if (e->swz.size() == 1) {
          static const char *nm[] = {"x", "y", "z", "w"};
          return "(" + x + ")." + nm[e->swz[0]];
        }
        std::string s = "s2sw<";
        for (size_t i = 0; i < e->swz.size(); ++i) s += (i ? "," : "") + std::to_string(e->swz[i]);
        return s + ">(" + x + ")";
      }
      case Expr::Index: return "(" + ex(e->a[0]) + ")[" + ex(e->a[1]) + "]";
      case Expr::Call:
        if (e->is_ctor) return ctor(e);
        if (e->fn) {
          std::string s = e->fn->cname + "(";
          for (size_t i = 0; i < e->a.size(); ++i) s += (i ? ", " : "") + (e->fn->params[i].out ? lvalue(e->a[i]) : ex(e->a[i]));
          return s + ")";
        }
        return builtin(e);
    }
    return "0";
  }

  std::string lvalue(const Expr *e) {
    if (e->k == Expr::Ref) return e->sym->cname;
    if (e->k == Expr::Swz && e->swz.size() == 1) {
      static const char *nm[] = {"x", "y", "z", "w"};
      return lvalue(e->a[0]) + "." + nm[e->swz[0]];
    }
    if (e->k == Expr::Index) return lvalue(e->a[0]) + "[" + ex(e->a[1]) + "]";
    fail(e->line, "unsupported assignment target");
  }

  std::string ctor(const Expr *e) {
    Ty t = concrete(e->t);
    if (is_scalar(t)) return "((" + c_scalar(t.b) + ")(" + ex(e->a[0]) + "))";
    if (is_mat(t)) {
      if (e->a.size() == 1 && is_scalar(e->a[0]->t)) return "s2mat_diag<" + std::to_string(t.m) + "," + std::to_string(t.n) + ">(" + ex(e->a[0]) + ")";
      std::string fn = t.m == 2 && t.n == 2 ? "s2mat22" : (t.m == 3 && t.n == 3 ? "s2mat33" : "");
      if (fn.empty()) fail(e->line, "only 2x2 and 3x3 matrix constructors are supported");
      std::string s = fn + "(";
      bool cols = is_vec(e->a[0]->t);
      for (size_t i = 0; i < e->a.size(); ++i) {
        if (cols != is_vec(e->a[i]->t)) fail(e->line, "mixed matrix constructor arguments are not supported");
        s += (i ? ", " : "") + ex(e->a[i]);
      }
      return s + ")";
    }
    std::string el = c_scalar(t.b);
    if (e->a.empty()) return "s2splat<" + el + "," + std::to_string(t.n) + ">(" + literal(scalar(t.b), {0}) + ")";
    if (e->a.size() == 1 && is_scalar(e->a[0]->t)) return "s2splat<" + el + "," + std::to_string(t.n) + ">(" + ex(e->a[0]) + ")";
    if (e->a.size() == 1 && is_vec(e->a[0]->t) && e->a[0]->t.n == t.n) {
      Ty at = out_t(e->a[0]);
      if (at.b == t.b) return ex(e->a[0]);
      return "s2cvt<" + el + ">(" + ex(e->a[0]) + ")";
    }
    // general: components from scalars and vectors, each vector evaluated once
    std::string pre, comps;
    int count = 0;
    std::string lam = "([&]() { ";
    for (const Expr *x : e->a) {
      Ty xt = out_t(x);
      if (is_scalar(xt)) {
        if (count < t.n) comps += (count ? ", " : "") + std::string("(") + el + ")(" + ex(x) + ")";
        ++count;
      } else {
        std::string v = "t" + std::to_string(tmp++);
        pre += "const " + c_type(xt) + " " + v + " = " + ex(x) + "; ";
        static const char *nm[] = {"x", "y", "z", "w"};
        for (int i = 0; i < xt.n; ++i) {
          if (count < t.n) comps += (count ? ", " : "") + std::string("(") + el + ")(" + v + "." + nm[i] + ")";
          ++count;
        }
      }
    }
    if (pre.empty()) return "s2mk(" + comps + ")";
    return lam + pre + "return s2mk(" + comps + "); }())";
  }

  std::string builtin(const Expr *e) {
    int id = int(e->lit);
    std::vector<std::string> a;
    for (const Expr *x : e->a) a.push_back(ex(x));
    auto call = [&](const std::string &fn) {
      std::string s = fn + "(";
      for (size_t i = 0; i < a.size(); ++i) s += (i ? ", " : "") + a[i];
      return s + ")";
    };
    switch (id) {
      case B_ABS: return call("s2_abs");
      case B_SIGN: return call("s2_sign");
      case B_FLOOR: return call("s2_floor");
      case B_CEIL: return call("s2_ceil");
      case B_TRUNC: return call("s2_trunc");
      case B_ROUND: return call("s2_round");
      case B_FRACT: return call("s2_fract");
      case B_SQRT: return call("s2_sqrt");
      case B_INVSQRT: return call("s2_inversesqrt");
      case B_EXP: return call("s2_exp");
      case B_EXP2: return call("s2_exp2");
      case B_LOG: return call("s2_log");
      case B_LOG2: return call("s2_log2");
      case B_POW: return call("s2_pow");
      case B_SIN: return call("s2_sin");
      case B_COS: return call("s2_cos");
      case B_TAN: return call("s2_tan");
      case B_ASIN: return call("s2_asin");
      case B_ACOS: return call("s2_acos");
      case B_ATAN: return call("s2_atan");
      case B_ATAN2: return call("s2_atan2");
      case B_SINH: return call("s2_sinh");
      case B_COSH: return call("s2_cosh");
      case B_TANH: return call("s2_tanh");
      case B_MIN: return call("s2_min");
      case B_MAX: return call("s2_max");
      case B_CLAMP: return call("s2_clamp");
      case B_SATURATE: return call("s2_saturate");
      case B_MIX: return call("s2_mix");
      case B_STEP: return call("s2_step");
      case B_SMOOTHSTEP: return call("s2_smoothstep");
      case B_MOD: return call("s2_fmod_glsl");
      case B_FMA: return call("s2_fma");
      case B_RADIANS: return call("s2_radians");
      case B_DEGREES: return call("s2_degrees");
      case B_LENGTH: return call("s2_length");
      case B_DISTANCE: return call("s2_distance");
      case B_DOT: return call("s2_dot");
      case B_CROSS: return call("s2_cross");
      case B_NORMALIZE: return call("s2_normalize");
      case B_REFLECT: return call("s2_reflect");
      case B_SELECT: return call("s2_select");
      case B_ALL: return call("s2_all");
      case B_ANY: return call("s2_any");
      case B_NOT: return "(!" + a[0] + ")";
      case B_TRANSPOSE: return call("s2_transpose");
      case B_LT: return call("s2_lt");
      case B_LE: return call("s2_le");
      case B_GT: return call("s2_gt");
      case B_GE: return call("s2_ge");
      case B_EQ: return call("s2_eq");
      case B_NE: return call("s2_ne");
    }
    fail(e->line, "unsupported builtin");
  }

  void ind(int d) { for (int i = 0; i < d; ++i) out << "  "; }

  void stmt(const Stmt *s, int d) {
    switch (s->k) {
      case Stmt::Block:
        if (s->decl_kind == -1) { for (const Stmt *x : s->body) stmt(x, d); break; }
        ind(d); out << "{\n";
        for (const Stmt *x : s->body) stmt(x, d + 1);
        ind(d); out << "}\n";
        break;
      case Stmt::Empty: break;
      case Stmt::Decl: {
        const Sym *sym = s->sym;
        if (sym->k == Sym::Const && sym->cst) break;  // uses are emitted as literals
        ind(d);
        if (sym->k == Sym::Let) out << "const ";
        out << c_type(s->decl_t) << " " << sym->cname << " = ";
        if (s->init) out << ex(s->init);
        else out << c_type(s->decl_t) << "{}";
        out << ";\n";
        break;
      }
      case Stmt::Assign: {
        const Expr *l = s->lhs;
        bool multi = l->k == Expr::Swz && l->swz.size() > 1;
        ind(d);
        if (!multi) {
          out << lvalue(l) << " " << s->op << " " << ex(s->rhs) << ";\n";
        } else {
          std::string base = lvalue(l->a[0]);
          std::string v = "t" + std::to_string(tmp++);
          std::string rhs = ex(s->rhs);
          Ty lt = concrete(l->t);
          if (s->op != "=") {
            std::string cur = "s2sw<";
            for (size_t i = 0; i < l->swz.size(); ++i) cur += (i ? "," : "") + std::to_string(l->swz[i]);
            cur += ">(" + base + ")";
            rhs = "(" + cur + " " + s->op.substr(0, s->op.size() - 1) + " " + rhs + ")";
          }
          out << "{ const " << c_type(lt) << " " << v << " = " << rhs << "; ";
          static const char *nm[] = {"x", "y", "z", "w"};
          for (size_t i = 0; i < l->swz.size(); ++i) out << base << "." << nm[l->swz[i]] << " = " << v << "." << nm[i] << "; ";
          out << "}\n";
        }
        break;
      }
      case Stmt::IncDec:
        ind(d);
        if (s->prefix) out << s->op << lvalue(s->lhs) << ";\n";
        else out << lvalue(s->lhs) << s->op << ";\n";
        break;
      case Stmt::ExprS:
        ind(d); out << "(void)(" << ex(s->val) << ");\n";
        break;
      case Stmt::If:
        ind(d); out << "if (" << ex(s->cond) << ")\n";
        stmt(s->then_s, d);
        if (s->else_s) { ind(d); out << "else\n"; stmt(s->else_s, d); }
        break;
      case Stmt::For: {
        ind(d); out << "{\n";
        if (s->init_s) stmt(s->init_s, d + 1);
        ind(d + 1); out << "for (; " << (s->cond ? ex(s->cond) : std::string("true")) << "; ";
        if (s->update_s) {
          std::ostringstream save;
          save.swap(out);
          stmt(s->update_s, 0);
          std::string u = out.str();
          out.swap(save);
          while (!u.empty() && (u.back() == '\n' || u.back() == ';' || u.back() == ' ')) u.pop_back();
          if (u.find('\n') != std::string::npos || u.rfind("{", 0) == 0) out << "([&]() { " << u << "; }())";
          else out << u;
        }
        out << ")\n";
        loop_labels.push_back(-1);
        stmt(s->loop_body, d + 1);
        loop_labels.pop_back();
        ind(d); out << "}\n";
        break;
      }
      case Stmt::While:
        ind(d); out << "while (" << ex(s->cond) << ")\n";
        loop_labels.push_back(-1);
        stmt(s->loop_body, d);
        loop_labels.pop_back();
        break;
      case Stmt::DoWhile:
        ind(d); out << "do\n";
        loop_labels.push_back(-1);
        stmt(s->loop_body, d);
        loop_labels.pop_back();
        ind(d); out << "while (" << ex(s->cond) << ");\n";
        break;
      case Stmt::Loop: {
        int lab = label++;
        ind(d); out << "for (;;) {\n";
        loop_labels.push_back(lab);
        stmt(s->loop_body, d + 1);
        loop_labels.pop_back();
        ind(d + 1); out << "s2cont" << lab << ":;\n";
        if (s->continuing) {
          loop_labels.push_back(-2);
          stmt(s->continuing, d + 1);
          loop_labels.pop_back();
        }
        ind(d); out << "}\n";
        break;
      }
      case Stmt::BreakIf:
        ind(d); out << "if (" << ex(s->cond) << ") break;\n";
        break;
      case Stmt::Break: ind(d); out << "break;\n"; break;
      case Stmt::Continue:
        ind(d);
        if (!loop_labels.empty() && loop_labels.back() >= 0) out << "goto s2cont" << loop_labels.back() << ";\n";
        else out << "continue;\n";
        break;
      case Stmt::Return:
        ind(d);
        if (s->val) out << "return " << ex(s->val) << ";\n";
        else out << "return;\n";
        break;
    }
  }

  std::string signature(const Func *f) {
    std::string s = "S2HD " + c_type(f->ret) + " " + f->cname + "(";
    for (size_t i = 0; i < f->params.size(); ++i) {
      const Param &p = f->params[i];
      s += (i ? ", " : "") + c_type(p.t) + (p.out ? "& " : " ") + (p.sym ? p.sym->cname : "a_unused" + std::to_string(i));
    }
    return s + ")";
  }

  void function(const Func *f) {
    out << signature(f) << "\n";
    stmt(f->body, 0);
    out << "\n";
  }
};

// ---------------------------------------------------------------------------
// Run-of-4 lowering.  The lattice kernel evaluates runs of 4 points that
// share x and y and differ in z.  For a straight-line SDF (no branches or
// loops, float scalars and vectors only), this emits
//     s2m_user_sdf_run4(float x, float y, const s2x4 &z, s2x4 &out)
// with vectors split into components and user functions inlined; every
// scalar that depends only on p.x and p.y is computed once per run as a
// float, every other one as an s2x4 (4 lanes, one per point).  Each lane runs
// the same operations in the same order as s2m_user_sdf, so the values are
// identical; the shared part is simply not repeated.  Anything else throws
// RunBail and the SDF keeps only the per-point form.

struct RunBail {};
struct RVal {
  std::string code;
  bool var = false;  // depends on p.z
};
using RVec = std::vector<RVal>;

class RunEmitter {
 public:
  std::ostringstream out;
  int tmp = 0;
  int depth = 0;
  double fp_u = 0, fp_v = 0, sfu_u = 0, sfu_v = 0;  // ops per run (uniform once, varying per lane)
  std::map<const Sym *, RVec> env;

  [[noreturn]] static void bail() { throw RunBail{}; }

  static Ty out_t(const Expr *e) { return e->want.b != B::Void ? e->want : concrete(e->t); }

  RVal bind(const std::string &code, bool var, bool sfu = false) {
    std::string n = "r" + std::to_string(tmp++);
    out << "  const " << (var ? "s2x4 " : "float ") << n << " = " << code << ";\n";
    double &c = sfu ? (var ? sfu_v : sfu_u) : (var ? fp_v : fp_u);
    c += var ? 4.0 : 1.0;
    return {n, var};
  }

  static RVec lit(const Ty &t, const std::vector<double> &cv) {
    if (t.b != B::F32 || is_mat(t)) bail();
    RVec r;
    for (int i = 0; i < t.n; ++i) r.push_back({flit(float(cv.empty() ? 0.0 : (cv.size() == 1 ? cv[0] : cv[size_t(i)]))), false});
    return r;
  }

  static RVec bcast(const RVec &v, size_t n) {
    if (v.size() == n) return v;
    if (v.size() != 1) bail();
    return RVec(n, v[0]);
  }

  // fn(args...) lane-wise: the scalar builtin when every argument is uniform,
  // its run form s2r_<name> otherwise.
  RVal call(const std::string &name, const std::vector<RVal> &a, bool sfu) {
    bool var = false;
    std::string args;
    for (size_t i = 0; i < a.size(); ++i) {
      var = var || a[i].var;
      args += (i ? ", " : "") + a[i].code;
    }
    return bind((var ? "s2r_" + name.substr(3) : name) + "(" + args + ")", var, sfu);
  }

  RVec componentwise(const std::string &fn, const std::vector<RVec> &args, bool sfu) {
    size_t n = 1;
    for (const RVec &a : args) n = std::max(n, a.size());
    std::vector<RVec> b;
    for (const RVec &a : args) b.push_back(bcast(a, n));
    RVec r;
    for (size_t i = 0; i < n; ++i) {
      std::vector<RVal> ai;
      for (const RVec &a : b) ai.push_back(a[i]);
      r.push_back(call(fn, ai, sfu));
    }
    return r;
  }

  RVal arith(const std::string &op, const RVal &a, const RVal &b) {
    return bind("(" + a.code + " " + op + " " + b.code + ")", a.var || b.var, op == "/");
  }

  // dot(a, b) summed left to right, as the prelude's s2_dot
  RVal dot(const RVec &a, const RVec &b) {
    if (a.size() != b.size()) bail();
    RVal s = arith("*", a[0], b[0]);
    for (size_t i = 1; i < a.size(); ++i) s = arith("+", s, arith("*", a[i], b[i]));
    return s;
  }

  RVec expr(const Expr *e) {
    const Ty t = out_t(e);
    if (t.b != B::F32 || is_mat(t)) bail();
    if (e->cst && (is_abstract(e->t) || e->k == Expr::Lit ||
                   (e->k == Expr::Ref && e->sym && (e->sym->k == Sym::Const || e->sym->k == Sym::Global))))
      return lit(t, e->cv);
    const Ty nt = concrete(e->t);
    if (nt.b != B::F32 || is_mat(nt)) bail();
    switch (e->k) {
      case Expr::Lit: return lit(nt, e->cv);
      case Expr::Ref: {
        if (e->sym->cst && (e->sym->k == Sym::Const || e->sym->k == Sym::Global)) return lit(nt, e->sym->cv);
        auto it = env.find(e->sym);
        if (it == env.end()) bail();
        return it->second;
      }
      case Expr::Unary: {
        if (e->s != "-") bail();
        RVec a = expr(e->a[0]), r;
        for (const RVal &c : a) r.push_back(bind("(-" + c.code + ")", c.var));
        return r;
      }
      case Expr::Binary: {
        const std::string &op = e->s;
        if (op != "+" && op != "-" && op != "*" && op != "/") bail();
        RVec a = expr(e->a[0]), b = expr(e->a[1]);
        size_t n = std::max(a.size(), b.size());
        a = bcast(a, n);
        b = bcast(b, n);
        RVec r;
        for (size_t i = 0; i < n; ++i) r.push_back(arith(op, a[i], b[i]));
        return r;
      }
      case Expr::Swz: {
        RVec a = expr(e->a[0]), r;
        for (int k : e->swz) {
          if (k < 0 || size_t(k) >= a.size()) bail();
          r.push_back(a[size_t(k)]);
        }
        return r;
      }
      case Expr::Call: {
        if (e->is_ctor) {
          RVec r;
          for (const Expr *x : e->a) {
            RVec v = expr(x);
            r.insert(r.end(), v.begin(), v.end());
          }
          if (r.empty()) return lit(nt, {0.0});
          if (r.size() == 1 && nt.n > 1) return RVec(size_t(nt.n), r[0]);
          r.resize(size_t(nt.n));
          return r;
        }
        if (e->fn) return inline_call(e);
        return builtin(e);
      }
      default: bail();
    }
  }

  RVec builtin(const Expr *e) {
    const int id = int(e->lit);
    std::vector<RVec> a;
    for (const Expr *x : e->a) a.push_back(expr(x));
    switch (id) {
      case B_ABS: return componentwise("s2_abs", a, false);
      case B_FLOOR: return componentwise("s2_floor", a, false);
      case B_CEIL: return componentwise("s2_ceil", a, false);
      case B_SQRT: return componentwise("s2_sqrt", a, true);
      case B_MIN: return componentwise("s2_min", a, false);
      case B_MAX: return componentwise("s2_max", a, false);
      case B_CLAMP: return componentwise("s2_clamp", a, false);
      case B_SATURATE: return componentwise("s2_saturate", a, false);
      case B_MIX: return componentwise("s2_mix", a, false);
      case B_SIN: return componentwise("s2_sin", a, true);
      case B_COS: return componentwise("s2_cos", a, true);
      case B_EXP: return componentwise("s2_exp", a, true);
      case B_LOG: return componentwise("s2_log", a, true);
      case B_POW: return componentwise("s2_pow", a, true);
      case B_ATAN2: return componentwise("s2_atan2", a, true);
      case B_LENGTH: {
        if (a.size() != 1) bail();
        if (a[0].size() == 1) return {call("s2_abs", {a[0][0]}, false)};
        return {call("s2_sqrt", {dot(a[0], a[0])}, true)};
      }
      case B_DOT:
        if (a.size() != 2) bail();
        if (a[0].size() == 1) return {arith("*", a[0][0], a[1][0])};
        return {dot(a[0], a[1])};
      case B_DISTANCE: {
        if (a.size() != 2 || a[0].size() != a[1].size()) bail();
        RVec d;
        for (size_t i = 0; i < a[0].size(); ++i) d.push_back(arith("-", a[0][i], a[1][i]));
        if (d.size() == 1) return {call("s2_abs", {d[0]}, false)};
        return {call("s2_sqrt", {dot(d, d)}, true)};
      }
      default: bail();
    }
  }

  RVec inline_call(const Expr *e) {
    const Func *f = e->fn;
    if (++depth > 32) bail();
    std::vector<RVec> args;
    for (size_t i = 0; i < e->a.size(); ++i) {
      if (f->params[i].out) bail();
      args.push_back(expr(e->a[i]));
    }
    for (size_t i = 0; i < e->a.size(); ++i)
      if (f->params[i].sym) env[f->params[i].sym] = args[i];
    RVec ret;
    bool done = false;
    block(f->body, ret, done);
    if (!done) bail();
    --depth;
    return ret;
  }

  void block(const Stmt *s, RVec &ret, bool &done) {
    if (done) bail();  // statements after a return
    switch (s->k) {
      case Stmt::Block:
        for (const Stmt *x : s->body) {
          if (done) {
            if (x->k == Stmt::Empty) continue;
            bail();
          }
          block(x, ret, done);
        }
        return;
      case Stmt::Empty: return;
      case Stmt::Decl: {
        const Sym *sym = s->sym;
        if (sym->k == Sym::Const && sym->cst) return;
        if (s->decl_t.b != B::F32 || is_mat(s->decl_t)) bail();
        env[sym] = s->init ? expr(s->init) : lit(s->decl_t, {0.0});
        return;
      }
      case Stmt::Assign: {
        const Expr *l = s->lhs;
        if (l->k != Expr::Ref || !l->sym || l->sym->k != Sym::Var) bail();
        RVec r = expr(s->rhs);
        if (s->op != "=") {
          const std::string op = s->op.substr(0, s->op.size() - 1);
          if (op != "+" && op != "-" && op != "*" && op != "/") bail();
          RVec cur = env.at(l->sym);
          size_t n = std::max(cur.size(), r.size());
          cur = bcast(cur, n);
          r = bcast(r, n);
          RVec x;
          for (size_t i = 0; i < n; ++i) x.push_back(arith(op, cur[i], r[i]));
          r = x;
        }
        env[l->sym] = r;
        return;
      }
      case Stmt::Return:
        if (!s->val) bail();
        ret = expr(s->val);
        done = true;
        return;
      default: bail();
    }
  }
};

// ---------------------------------------------------------------------------
// Scalar expression graph of a straight-line SDF for tile pruning
// (prune.h).  The traversal and the lowering of each builtin are those of
// RunEmitter, so the graph performs the operations of s2m_user_sdf in the
// same order.  A user function whose body lowers to exactly the arithmetic of
// sdf::op's smooth union / intersection / subtraction of its three arguments
// becomes one combinator node.

struct PruneBail {};

class PruneBuilder {
 public:
  PruneIR ir;
  std::map<const Sym *, std::vector<int>> env;
  int depth = 0;

  [[noreturn]] static void bail() { throw PruneBail{}; }

  int node(POp op, int a = -1, int b = -1, int c = -1) {
    PNode n;
    n.op = op;
    n.a = a;
    n.b = b;
    n.c = c;
    ir.nodes.push_back(n);
    return int(ir.nodes.size()) - 1;
  }
  int cst(float v) {
    uint32_t bits;
    std::memcpy(&bits, &v, 4);
    auto it = consts_.find(bits);
    if (it != consts_.end()) return it->second;
    const int id = node(POp::Const);
    ir.nodes[size_t(id)].k = v;
    consts_[bits] = id;
    return id;
  }

  static Ty out_t(const Expr *e) { return e->want.b != B::Void ? e->want : concrete(e->t); }

  std::vector<int> lit(const Ty &t, const std::vector<double> &cv) {
    if (t.b != B::F32 || is_mat(t)) bail();
    std::vector<int> r;
    for (int i = 0; i < t.n; ++i)
      r.push_back(cst(float(cv.empty() ? 0.0 : (cv.size() == 1 ? cv[0] : cv[size_t(i)]))));
    return r;
  }

  static std::vector<int> bcast(const std::vector<int> &v, size_t n) {
    if (v.size() == n) return v;
    if (v.size() != 1) bail();
    return std::vector<int>(n, v[0]);
  }

  std::vector<int> componentwise(POp op, const std::vector<std::vector<int>> &args) {
    size_t n = 1;
    for (const auto &a : args) n = std::max(n, a.size());
    std::vector<std::vector<int>> b;
    for (const auto &a : args) b.push_back(bcast(a, n));
    std::vector<int> r;
    for (size_t i = 0; i < n; ++i)
      r.push_back(node(op, b[0][i], b.size() > 1 ? b[1][i] : -1, b.size() > 2 ? b[2][i] : -1));
    return r;
  }

  int dot(const std::vector<int> &a, const std::vector<int> &b) {
    if (a.size() != b.size()) bail();
    int s = node(POp::Mul, a[0], b[0]);
    for (size_t i = 1; i < a.size(); ++i) s = node(POp::Add, s, node(POp::Mul, a[i], b[i]));
    return s;
  }

  std::vector<int> expr(const Expr *e) {
    const Ty t = out_t(e);
    if (t.b != B::F32 || is_mat(t)) bail();
    if (e->cst && (is_abstract(e->t) || e->k == Expr::Lit ||
                   (e->k == Expr::Ref && e->sym && (e->sym->k == Sym::Const || e->sym->k == Sym::Global))))
      return lit(t, e->cv);
    const Ty nt = concrete(e->t);
    if (nt.b != B::F32 || is_mat(nt)) bail();
    switch (e->k) {
      case Expr::Lit: return lit(nt, e->cv);
      case Expr::Ref: {
        if (e->sym->cst && (e->sym->k == Sym::Const || e->sym->k == Sym::Global)) return lit(nt, e->sym->cv);
        auto it = env.find(e->sym);
        if (it == env.end()) bail();
        return it->second;
      }
      case Expr::Unary: {
        if (e->s != "-") bail();
        std::vector<int> a = expr(e->a[0]), r;
        for (int c : a) r.push_back(node(POp::Neg, c));
        return r;
      }
      case Expr::Binary: {
        const std::string &op = e->s;
        POp o = op == "+" ? POp::Add : op == "-" ? POp::Sub : op == "*" ? POp::Mul : op == "/" ? POp::Div : POp::X;
        if (o == POp::X) bail();
        std::vector<int> a = expr(e->a[0]), b = expr(e->a[1]);
        size_t n = std::max(a.size(), b.size());
        a = bcast(a, n);
        b = bcast(b, n);
        std::vector<int> r;
        for (size_t i = 0; i < n; ++i) r.push_back(node(o, a[i], b[i]));
        return r;
      }
      case Expr::Swz: {
        std::vector<int> a = expr(e->a[0]), r;
        for (int k : e->swz) {
          if (k < 0 || size_t(k) >= a.size()) bail();
          r.push_back(a[size_t(k)]);
        }
        return r;
      }
      case Expr::Call: {
        if (e->is_ctor) {
          std::vector<int> r;
          for (const Expr *x : e->a) {
            std::vector<int> v = expr(x);
            r.insert(r.end(), v.begin(), v.end());
          }
          if (r.empty()) return lit(nt, {0.0});
          if (r.size() == 1 && nt.n > 1) return std::vector<int>(size_t(nt.n), r[0]);
          r.resize(size_t(nt.n));
          return r;
        }
        if (e->fn) return inline_call(e);
        return builtin(e);
      }
      default: bail();
    }
  }

  std::vector<int> builtin(const Expr *e) {
    std::vector<std::vector<int>> a;
    for (const Expr *x : e->a) a.push_back(expr(x));
    switch (int(e->lit)) {
      case B_ABS: return componentwise(POp::Abs, a);
      case B_FLOOR: return componentwise(POp::Floor, a);
      case B_CEIL: return componentwise(POp::Ceil, a);
      case B_SQRT: return componentwise(POp::Sqrt, a);
      case B_MIN: return componentwise(POp::Min, a);
      case B_MAX: return componentwise(POp::Max, a);
      case B_CLAMP: return componentwise(POp::Clamp, a);
      case B_SATURATE: return componentwise(POp::Saturate, a);
      case B_MIX: return componentwise(POp::Mix, a);
      case B_SIN: return componentwise(POp::Sin, a);
      case B_COS: return componentwise(POp::Cos, a);
      case B_EXP: return componentwise(POp::Exp, a);
      case B_LOG: return componentwise(POp::Log, a);
      case B_POW: return componentwise(POp::Pow, a);
      case B_ATAN2: return componentwise(POp::Atan2, a);
      case B_LENGTH:
        if (a.size() != 1) bail();
        if (a[0].size() == 1) return {node(POp::Abs, a[0][0])};
        return {node(POp::Sqrt, dot(a[0], a[0]))};
      case B_DOT:
        if (a.size() != 2) bail();
        if (a[0].size() == 1) return {node(POp::Mul, a[0][0], a[1][0])};
        return {dot(a[0], a[1])};
      case B_DISTANCE: {
        if (a.size() != 2 || a[0].size() != a[1].size()) bail();
        std::vector<int> d;
        for (size_t i = 0; i < a[0].size(); ++i) d.push_back(node(POp::Sub, a[0][i], a[1][i]));
        if (d.size() == 1) return {node(POp::Abs, d[0])};
        return {node(POp::Sqrt, dot(d, d))};
      }
      default: bail();
    }
  }

  std::vector<int> inline_call(const Expr *e) {
    const Func *f = e->fn;
    if (++depth > 32) bail();
    std::vector<std::vector<int>> args;
    for (size_t i = 0; i < e->a.size(); ++i) {
      if (f->params[i].out) bail();
      args.push_back(expr(e->a[i]));
    }
    for (size_t i = 0; i < e->a.size(); ++i)
      if (f->params[i].sym) env[f->params[i].sym] = args[i];
    std::vector<int> ret;
    bool done = false;
    block(f->body, ret, done);
    if (!done) bail();
    --depth;
    if (args.size() == 3 && ret.size() == 1 && args[0].size() == 1 && args[1].size() == 1 && args[2].size() == 1) {
      const POp k = smooth_kind(ret[0], args[0][0], args[1][0], args[2][0]);
      if (k != POp::X) return {node(k, args[0][0], args[1][0], args[2][0])};
    }
    return ret;
  }

  void block(const Stmt *s, std::vector<int> &ret, bool &done) {
    if (done) bail();
    switch (s->k) {
      case Stmt::Block:
        for (const Stmt *x : s->body) {
          if (done) {
            if (x->k == Stmt::Empty) continue;
            bail();
          }
          block(x, ret, done);
        }
        return;
      case Stmt::Empty: return;
      case Stmt::Decl: {
        const Sym *sym = s->sym;
        if (sym->k == Sym::Const && sym->cst) return;
        if (s->decl_t.b != B::F32 || is_mat(s->decl_t)) bail();
        env[sym] = s->init ? expr(s->init) : lit(s->decl_t, {0.0});
        return;
      }
      case Stmt::Assign: {
        const Expr *l = s->lhs;
        if (l->k != Expr::Ref || !l->sym || l->sym->k != Sym::Var) bail();
        std::vector<int> r = expr(s->rhs);
        if (s->op != "=") {
          const std::string op = s->op.substr(0, s->op.size() - 1);
          POp o = op == "+" ? POp::Add : op == "-" ? POp::Sub : op == "*" ? POp::Mul : op == "/" ? POp::Div : POp::X;
          if (o == POp::X) bail();
          std::vector<int> cur = env.at(l->sym);
          size_t n = std::max(cur.size(), r.size());
          cur = bcast(cur, n);
          r = bcast(r, n);
          std::vector<int> x;
          for (size_t i = 0; i < n; ++i) x.push_back(node(o, cur[i], r[i]));
          r = x;
        }
        env[l->sym] = r;
        return;
      }
      case Stmt::Return:
        if (!s->val) bail();
        ret = expr(s->val);
        done = true;
        return;
      default: bail();
    }
  }

 private:
  std::map<uint32_t, int> consts_;

  bool is(int v, POp op) const { return v >= 0 && ir.nodes[size_t(v)].op == op; }
  bool is2(int v, POp op, int a, int b) const {
    return is(v, op) && ir.nodes[size_t(v)].a == a && ir.nodes[size_t(v)].b == b;
  }
  bool isc(int v, float x) const {
    if (!is(v, POp::Const)) return false;
    float k = ir.nodes[size_t(v)].k;
    return std::memcmp(&k, &x, 4) == 0;
  }
  const PNode &at(int v) const { return ir.nodes[size_t(v)]; }

  // r == mix(b, A2, h) OP (k * h) * (1 - h), h = clamp(t, 0, 1), t = 0.5 OPT (0.5 * (b OPD a)) / k
  POp smooth_kind(int r, int a, int b, int k) const {
    if (!is(r, POp::Sub) && !is(r, POp::Add)) return POp::X;
    const int m = at(r).a, q = at(r).b;
    if (!is(m, POp::Mix) || at(m).a != b) return POp::X;
    const int h = at(m).c;
    // q = (k * h) * (1 - h)
    if (!is(q, POp::Mul) || !is2(at(q).a, POp::Mul, k, h) || !is(at(q).b, POp::Sub) || !isc(at(at(q).b).a, 1.0f) ||
        at(at(q).b).b != h)
      return POp::X;
    if (!is(h, POp::Clamp) || !isc(at(h).b, 0.0f) || !isc(at(h).c, 1.0f)) return POp::X;
    const int t = at(h).a;
    if ((!is(t, POp::Add) && !is(t, POp::Sub)) || !isc(at(t).a, 0.5f)) return POp::X;
    const int dv = at(t).b;
    if (!is(dv, POp::Div) || at(dv).b != k) return POp::X;
    const int hm = at(dv).a;
    if (!is(hm, POp::Mul) || !isc(at(hm).a, 0.5f)) return POp::X;
    const int df = at(hm).b;
    const int a2 = at(m).b;
    if (is(r, POp::Sub) && is(t, POp::Add) && a2 == a && is2(df, POp::Sub, b, a)) return POp::SmoothUnion;
    if (is(r, POp::Add) && is(t, POp::Sub) && a2 == a && is2(df, POp::Sub, b, a)) return POp::SmoothIntersection;
    if (is(r, POp::Add) && is(t, POp::Sub) && is(a2, POp::Neg) && at(a2).a == a && is2(df, POp::Add, b, a))
      return POp::SmoothSubtraction;
    return POp::X;
  }
};

// Functions reachable from `root` in callee-first order; recursion is an error.
void collect_calls(const Stmt *s, std::vector<const Expr *> &calls);
void collect_calls(const Expr *e, std::vector<const Expr *> &calls) {
  if (!e) return;
  if (e->k == Expr::Call && e->fn) calls.push_back(e);
  for (const Expr *x : e->a) collect_calls(x, calls);
}
void collect_calls(const Stmt *s, std::vector<const Expr *> &calls) {
  if (!s) return;
  for (const Stmt *x : s->body) collect_calls(x, calls);
  collect_calls(s->init, calls);
  collect_calls(s->lhs, calls);
  collect_calls(s->rhs, calls);
  collect_calls(s->cond, calls);
  collect_calls(s->val, calls);
  collect_calls(s->then_s, calls);
  collect_calls(s->else_s, calls);
  collect_calls(s->init_s, calls);
  collect_calls(s->update_s, calls);
  collect_calls(s->loop_body, calls);
  collect_calls(s->continuing, calls);
}
void order_functions(Func *f, std::vector<Func *> &order, std::set<Func *> &done, std::set<Func *> &active) {
  if (done.count(f)) return;
  if (active.count(f)) fail(f->line, "recursive function '" + f->name + "' is not supported");
  active.insert(f);
  std::vector<const Expr *> calls;
  collect_calls(f->body, calls);
  for (const Expr *c : calls) order_functions(c->fn, order, done, active);
  active.erase(f);
  done.insert(f);
  order.push_back(f);
}

Func *find_fn(Module &M, const std::string &name, int nparams) {
  auto it = M.fn_by_name.find(name);
  if (it == M.fn_by_name.end()) return nullptr;
  for (Func *f : it->second)
    if (int(f->params.size()) == nparams) return f;
  return nullptr;
}

}  // namespace

// ---------------------------------------------------------------------------

FrontendResult translate(const std::string &source, Lang lang, const std::string &sdf_name) {
  FrontendResult r;
  Module M;
  try {
    {
      std::vector<Tok> toks = lex(source, lang);
      Parser(M, toks, lang).parse_module();
    }
    if (lang == Lang::GLSL) {
      // shader.rs:84-87: the fragment entry points go, the library normal
      // comes in.  Here `main` / `mainImage` are simply not lowered.
      const std::string &nm = sdf_name.empty() ? std::string("sdf") : sdf_name;
      Func *user = find_fn(M, nm, 1);
      if (!user || !(user->params[0].t == vec(B::F32, 3)) || !(user->ret == scalar(B::F32)))
        throw CompileError(0, "MISSING_SDF:no function 'float " + nm + "(vec3)' in the GLSL source");
      if (!find_fn(M, "sdf3d", 1)) {
        std::string wrap = "fn sdf3d(p: vec3<f32>) -> f32 { return " + nm + "(p); }\n";
        std::vector<Tok> toks = lex(wrap, Lang::WGSL);
        Parser(M, toks, Lang::WGSL).parse_module();
      }
    }
    bool std_normal = false;
    if (!find_fn(M, "sdf3d_normal", 2)) {
      std_normal = true;
      // The reference needs sdf3d_normal in scope (`use sdf3d::normal;`, or
      // appended for GLSL at shader.rs:87); supply the library one.
      std::vector<Tok> toks = lex(builtin_module_source("sdf3d::normal"), Lang::WGSL);
      Parser(M, toks, Lang::WGSL).parse_module();
      if (lang == Lang::WGSL) r.warnings.push_back("sdf3d_normal is not in scope; using the sdf3d::normal module");
    }
    Func *sdf = find_fn(M, "sdf3d", 1);
    if (!sdf) throw CompileError(0, "MISSING_SDF:no function 'fn sdf3d(p: vec3f) -> f32'");
    if (!(sdf->params[0].t == vec(B::F32, 3)) || !(sdf->ret == scalar(B::F32)))
      throw CompileError(sdf->line, "sdf3d must have the signature fn sdf3d(p: vec3f) -> f32");
    Func *nrm = find_fn(M, "sdf3d_normal", 2);
    if (!(nrm->params[0].t == vec(B::F32, 3)) || !(nrm->params[1].t == scalar(B::F32)) || !(nrm->ret == vec(B::F32, 3)))
      throw CompileError(nrm->line, "sdf3d_normal must have the signature fn sdf3d_normal(p: vec3f, eps: f32) -> vec3f");

    Sema S(M);
    for (Global *g : M.globals) S.resolve_global(g);
    for (Func *f : M.funcs) S.check_function(f);

    std::vector<Func *> order;
    std::set<Func *> done, active;
    order_functions(sdf, order, done, active);
    order_functions(nrm, order, done, active);
    // C++ names: overloads share a name (C++ resolves them by type).
    for (Func *f : M.funcs) f->cname = "u_" + f->name;

    Coster C;
    Cost c = C.func(sdf);
    r.fp32_ops = c.fp;
    r.sfu_ops = c.sfu;
    r.ops_exact = c.exact;

    Emitter E;
    E.out << "// lowered by the sdf2mesh_gb300 frontend\n";
    for (Func *f : order) E.out << E.signature(f) << ";\n";
    E.out << "\n";
    for (Func *f : order) E.function(f);
    E.out << "S2HD float s2m_user_sdf(float x, float y, float z) { return " << sdf->cname << "(s2mk(x, y, z)); }\n";
    E.out << "S2HD s2v3 s2m_user_normal(s2v3 p, float eps) { return " << nrm->cname << "(p, eps); }\n";
    // The library's tetrahedral normal (as `use` inserts it, or supplied
    // above): the kernels may then evaluate it as a loop over the four
    // directions with the same arithmetic, one sdf3d call site instead of four.
    if (!std_normal) {
      auto squash = [](const std::string &t) {
        std::string o;
        for (char ch : t)
          if (!std::isspace((unsigned char)ch)) o.push_back(ch);
        return o;
      };
      std::string lib = builtin_module_source("sdf3d::normal");
      size_t at = lib.find("fn sdf3d_normal(");
      std::string fn = squash(lib.substr(at));
      std::string src = squash(source);
      size_t first = src.find("fnsdf3d_normal(");
      std_normal = first != std::string::npos && src.find("fnsdf3d_normal(", first + 1) == std::string::npos &&
                   src.compare(first, fn.size(), fn) == 0;
    }
    if (std_normal) E.out << "#define S2M_STD_NORMAL 1\n";
    // run-of-4 form of sdf3d, when it is straight-line float code
    try {
      RunEmitter R;
      RVec p = {{"x", false}, {"y", false}, {"z", true}};
      R.env[sdf->params[0].sym] = p;
      RVec ret;
      bool done = false;
      R.block(sdf->body, ret, done);
      if (!done || ret.size() != 1) throw RunBail{};
      E.out << "S2HD void s2m_user_sdf_run4(float x, float y, const s2x4 &z, s2x4 &out)\n{\n" << R.out.str();
      if (ret[0].var) E.out << "  out = " << ret[0].code << ";\n";
      else E.out << "  out = s2x4_splat(" << ret[0].code << ");\n";
      E.out << "}\n#define S2M_HAS_RUN4 1\n";
      r.run_fp32_ops = (R.fp_u + R.fp_v) / 4.0;
      r.run_sfu_ops = (R.sfu_u + R.sfu_v) / 4.0;
    } catch (const RunBail &) {
    }
    // tile-pruning form of sdf3d, when it is straight-line float code with
    // combinators worth skipping
    try {
      PruneBuilder PB;
      const int X = PB.node(POp::X), Y = PB.node(POp::Y), Z = PB.node(POp::Z);
      PB.env[sdf->params[0].sym] = {X, Y, Z};
      std::vector<int> ret;
      bool done = false;
      PB.block(sdf->body, ret, done);
      if (!done || ret.size() != 1) throw PruneBail{};
      PB.ir.root = ret[0];
      PruneCode pc = prune_codegen(PB.ir);
      if (pc.ok) {
        E.out << pc.cuda;
        r.prune_combinators = pc.combinators;
        r.prune_words = pc.words;
      }
    } catch (const PruneBail &) {
    }
    r.cuda = E.out.str();
    for (auto &w : M.warnings) r.warnings.push_back(w);
    r.ok = true;
  } catch (const CompileError &e) {
    std::string msg = e.what();
    if (msg.rfind("MISSING_SDF:", 0) == 0) {
      r.status = S2M_E_MISSING_SDF;
      r.error = msg.substr(12);
    } else {
      r.status = S2M_E_PARSE;
      r.error = (e.line > 0 ? "line " + std::to_string(e.line) + ": " : std::string()) + msg;
    }
    r.ok = false;
  }
  return r;
}

// ---------------------------------------------------------------------------
// CSG programs from .sdf3d sources.  A source whose sdf3d is one expression
// over the library's primitives with constant arguments -- sdf3d_sphere,
// sdf3d_box, sdf3d_torus (each at p or p - constant), sdf3d_capsule at p --
// combined by min, max, negation and the sdf_op_smooth_* operators becomes
// the postfix program the batch interpreter evaluates with the same
// arithmetic (opcodes of include/sdf2mesh.h).

namespace {

struct CsgConv {
  Func *sdf = nullptr;
  std::vector<float> prog;
  std::string why;

  [[noreturn]] void no(const Expr *e, const std::string &m) {
    throw CompileError(e ? e->line : 0, "not a CSG expression: " + m);
  }
  static float as_f32(double v) { return float(v); }

  // A constant scalar: literal, negated literal, folded constant or const symbol.
  float scalar(const Expr *e) {
    if (e->k == Expr::Lit) return e->lit_b == B::F32 ? e->flit : as_f32(e->lit);
    if (e->k == Expr::Unary && e->s == "-" && e->a.size() == 1) return -scalar(e->a[0]);
    if (e->cst && e->cv.size() == 1) return as_f32(e->cv[0]);
    if (e->k == Expr::Ref && e->sym && e->sym->cst && e->sym->cv.size() == 1) return as_f32(e->sym->cv[0]);
    no(e, "argument is not a constant");
  }
  // A constant vector of n components: vecN(...) / vecNf(...) of constants (or a splat).
  std::vector<float> vector(const Expr *e, int n) {
    if (e->cst && int(e->cv.size()) == n) {
      std::vector<float> r;
      for (double v : e->cv) r.push_back(as_f32(v));
      return r;
    }
    if (e->k == Expr::Call && e->is_ctor) {
      if (int(e->a.size()) == n) {
        std::vector<float> r;
        for (const Expr *x : e->a) r.push_back(scalar(x));
        return r;
      }
      if (e->a.size() == 1) return std::vector<float>(size_t(n), scalar(e->a[0]));
    }
    no(e, "argument is not a constant vector");
  }
  bool is_p(const Expr *e) const {
    return e->k == Expr::Ref && e->sym && e->sym->k == Sym::Param && e->s == sdf->params[0].name;
  }
  // p -> (0,0,0);  p - c -> c
  std::vector<float> centre(const Expr *e) {
    if (is_p(e)) return {0.0f, 0.0f, 0.0f};
    if (e->k == Expr::Binary && e->s == "-" && e->a.size() == 2 && is_p(e->a[0])) return vector(e->a[1], 3);
    no(e, "primitive not evaluated at p or p - constant");
  }
  void put(float v) { prog.push_back(v); }
  void put(const std::vector<float> &v) { prog.insert(prog.end(), v.begin(), v.end()); }

  void expr(const Expr *e) {
    if (e->k != Expr::Call || e->is_ctor) no(e, "expected a call");
    const std::string &f = e->s;
    const size_t na = e->a.size();
    if ((f == "min" || f == "max") && na == 2) {
      expr(e->a[0]);
      if (f == "max" && e->a[1]->k == Expr::Unary && e->a[1]->s == "-") {
        expr(e->a[1]->a[0]);
        put(float(S2M_CSG_SUBTRACT));
      } else {
        expr(e->a[1]);
        put(float(f == "min" ? S2M_CSG_UNION : S2M_CSG_INTERSECT));
      }
      return;
    }
    if ((f == "sdf_op_smooth_union" || f == "sdf_op_smooth_intersection" || f == "sdf_op_smooth_subtraction") &&
        na == 3) {
      expr(e->a[0]);
      expr(e->a[1]);
      put(float(f == "sdf_op_smooth_union" ? S2M_CSG_SMOOTH_UNION
                                            : f == "sdf_op_smooth_intersection" ? S2M_CSG_SMOOTH_INTERSECTION
                                                                                 : S2M_CSG_SMOOTH_SUBTRACTION));
      put(scalar(e->a[2]));
      return;
    }
    if (f == "sdf3d_sphere" && na == 2) {
      put(float(S2M_CSG_SPHERE));
      put(centre(e->a[0]));
      put(scalar(e->a[1]));
      return;
    }
    if (f == "sdf3d_box" && na == 2) {
      put(float(S2M_CSG_BOX));
      put(centre(e->a[0]));
      put(vector(e->a[1], 3));
      return;
    }
    if (f == "sdf3d_torus" && na == 2) {
      put(float(S2M_CSG_TORUS));
      put(centre(e->a[0]));
      put(vector(e->a[1], 2));
      return;
    }
    if (f == "sdf3d_capsule" && na == 4) {
      if (!is_p(e->a[0])) no(e, "capsule not evaluated at p");
      put(float(S2M_CSG_CAPSULE));
      put(vector(e->a[1], 3));
      put(vector(e->a[2], 3));
      put(scalar(e->a[3]));
      return;
    }
    no(e, "unsupported call " + f);
  }
};

std::string squash_ws(const std::string &t) {
  std::string o;
  for (char ch : t)
    if (!std::isspace((unsigned char)ch)) o.push_back(ch);
  return o;
}

// The library function `name`, if the source defines it, must be the
// library's own text (the program's opcodes stand for the library formulas).
bool library_function_intact(const std::string &src_sq, const std::string &name) {
  const std::string key = "fn" + name + "(";
  size_t at = src_sq.find(key);
  if (at == std::string::npos) return true;
  if (src_sq.find(key, at + 1) != std::string::npos) return false;
  for (const char *mod : {"sdf3d::primitives", "sdf::op"}) {
    std::string lib = squash_ws(builtin_module_source(mod));
    size_t la = lib.find(key);
    if (la == std::string::npos) continue;
    size_t lb = lib.find("fn", la + 2);
    std::string fn = lib.substr(la, lb == std::string::npos ? std::string::npos : lb - la);
    return src_sq.compare(at, fn.size(), fn) == 0;
  }
  return true;
}

}  // namespace

bool csg_from_source(const std::string &source, std::vector<float> &prog, std::string &why) {
  Module M;
  try {
    std::vector<Tok> toks = lex(source, Lang::WGSL);
    Parser(M, toks, Lang::WGSL).parse_module();
    Func *sdf = find_fn(M, "sdf3d", 1);
    if (!sdf) throw CompileError(0, "no fn sdf3d(p: vec3f) -> f32");
    Sema S(M);
    for (Global *g : M.globals) S.resolve_global(g);
    for (Func *f : M.funcs) S.check_function(f);
    const std::string sq = squash_ws(source);
    for (const char *lib : {"sdf3d_sphere", "sdf3d_box", "sdf3d_torus", "sdf3d_capsule", "sdf_op_smooth_union",
                            "sdf_op_smooth_intersection", "sdf_op_smooth_subtraction"})
      if (!library_function_intact(sq, lib))
        throw CompileError(0, std::string("not a CSG expression: ") + lib + " is not the library function");
    const Stmt *body = sdf->body;
    const Stmt *ret = nullptr;
    for (const Stmt *st : body->body) {
      if (st->k == Stmt::Empty) continue;
      if (st->k != Stmt::Return || ret) throw CompileError(st->line, "not a CSG expression: sdf3d must be one return");
      ret = st;
    }
    if (!ret || !ret->val) throw CompileError(sdf->line, "not a CSG expression: sdf3d has no return value");
    CsgConv C;
    C.sdf = sdf;
    C.expr(ret->val);
    prog.swap(C.prog);
    return true;
  } catch (const CompileError &e) {
    why = (e.line > 0 ? "line " + std::to_string(e.line) + ": " : std::string()) + e.what();
    return false;
  }
}

}  // namespace s2m
