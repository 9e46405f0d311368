// frontend_lib.cpp -- the built-in WGSL modules and the `.sdf3d` line
// preprocessor (`use X;` / `include "f";`), after src/shader.rs:12-20,
// 44-67 and 159-203 of the reference, plus the WGSL text helpers of
// src/shadertoy.rs:248-352.
//
// The module texts are this project's own WGSL.  The arithmetic of each
// function follows the published distance formulas the reference also uses
// (I. Quilez, "distance functions"), operation for operation, because
// `.sdf3d` files call them by these names and expect the same values.
#include <climits>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <sstream>

#include "frontend.h"

namespace s2m {

static const char *kPrimitives = R"WGSL(
// sdf3d::primitives -- signed distances of basic solids centred at the origin.

// Box with full edge lengths `size`.
fn sdf3d_box(p: vec3f, size: vec3f) -> f32 {
    let q = abs(p) - 0.5 * size;
    return length(max(q, vec3f(0.0))) + min(max(q.x, max(q.y, q.z)), 0.0);
}

// Cylinder around the y axis with half height `half_h` and radius `radius`.
fn sdf3d_cylinder(p: vec3f, half_h: f32, radius: f32) -> f32 {
    let d = abs(vec2f(length(p.xz), p.y)) - vec2f(radius, half_h);
    return min(max(d.x, d.y), 0.0) + length(max(d, vec2f(0.0)));
}

// Capsule: the segment a-b swept by a ball of radius `radius`.
fn sdf3d_capsule(p: vec3f, a: vec3f, b: vec3f, radius: f32) -> f32 {
    let ap = p - a;
    let ab = b - a;
    let t = clamp(dot(ap, ab) / dot(ab, ab), 0.0, 1.0);
    return length(ap - ab * t) - radius;
}

fn sdf3d_sphere(p: vec3f, radius: f32) -> f32 {
    return length(p) - radius;
}

// Torus in the xz plane: radii.x to the tube centre, radii.y of the tube.
fn sdf3d_torus(p: vec3f, radii: vec2f) -> f32 {
    let q = vec2f(length(p.xz) - radii.x, p.y);
    return length(q) - radii.y;
}
)WGSL";

static const char *kOps = R"WGSL(
// sdf::op -- polynomial smooth boolean operations with blend width k.

fn sdf_op_smooth_union(a: f32, b: f32, k: f32) -> f32 {
    let h = clamp(0.5 + 0.5 * (b - a) / k, 0.0, 1.0);
    return mix(b, a, h) - k * h * (1.0 - h);
}

fn sdf_op_smooth_intersection(a: f32, b: f32, k: f32) -> f32 {
    let h = clamp(0.5 - 0.5 * (b - a) / k, 0.0, 1.0);
    return mix(b, a, h) + k * h * (1.0 - h);
}

fn sdf_op_smooth_subtraction(a: f32, b: f32, k: f32) -> f32 {
    let h = clamp(0.5 - 0.5 * (b + a) / k, 0.0, 1.0);
    return mix(b, -a, h) + k * h * (1.0 - h);
}
)WGSL";

static const char *kNormal = R"WGSL(
// sdf3d::normal -- tetrahedral central-difference gradient of sdf3d (not
// normalised): the sum of v * sdf3d(p + v * eps) over four tetrahedron
// directions v.
fn sdf3d_normal(p: vec3f, eps: f32) -> vec3f {
    let t0 = vec3f(1.0, -1.0, -1.0);
    let t1 = vec3f(-1.0, -1.0, 1.0);
    let t2 = vec3f(-1.0, 1.0, -1.0);
    let t3 = vec3f(1.0, 1.0, 1.0);
    return t0 * sdf3d(p + t0 * eps) + t1 * sdf3d(p + t1 * eps) + t2 * sdf3d(p + t2 * eps) + t3 * sdf3d(p + t3 * eps);
}
)WGSL";

static std::string g_all_sdf3d = std::string(kPrimitives) + kNormal;

const char *builtin_module_source(const std::string &name) {
  if (name == "sdf::op" || name == "sdf::*") return kOps;
  if (name == "sdf3d::normal") return kNormal;
  if (name == "sdf3d::primitives") return kPrimitives;
  if (name == "sdf3d::*") return g_all_sdf3d.c_str();
  return nullptr;
}

static std::string trim(const std::string &s) {
  size_t a = 0, b = s.size();
  while (a < b && (s[a] == ' ' || s[a] == '\t' || s[a] == '\r' || s[a] == '\n' || s[a] == '\f' || s[a] == '\v')) ++a;
  while (b > a && (s[b - 1] == ' ' || s[b - 1] == '\t' || s[b - 1] == '\r' || s[b - 1] == '\n' || s[b - 1] == '\f' || s[b - 1] == '\v')) --b;
  return s.substr(a, b - a);
}

// Split like Rust's str::lines(): on '\n', dropping one trailing '\r'.
static std::vector<std::string> split_lines(const std::string &s) {
  std::vector<std::string> out;
  size_t i = 0;
  while (i < s.size()) {
    size_t j = s.find('\n', i);
    if (j == std::string::npos) j = s.size();
    std::string line = s.substr(i, j - i);
    if (!line.empty() && line.back() == '\r') line.pop_back();
    out.push_back(line);
    i = j + 1;
  }
  return out;
}

// trimmed.replacen(word, "", 1).replace(['"', ';'], "").trim()
static std::string directive_arg(const std::string &trimmed, const std::string &word) {
  std::string s = trimmed;
  size_t p = s.find(word);
  if (p != std::string::npos) s.erase(p, word.size());
  std::string r;
  for (char c : s)
    if (c != '"' && c != ';') r.push_back(c);
  return trim(r);
}

static bool read_file(const std::string &path, std::string &out) {
  std::ifstream f(path, std::ios::binary);
  if (!f) return false;
  std::ostringstream ss;
  ss << f.rdbuf();
  out = ss.str();
  return true;
}

// Canonical path of an existing file, or the text itself.
static std::string canonical(const std::string &path) {
  char buf[PATH_MAX];
  if (!path.empty() && realpath(path.c_str(), buf)) return std::string(buf);
  return path;
}

static void expand(const std::string &text, const std::string &self_path, const std::string &base_dir,
                   std::string &out, std::vector<std::string> *log, int depth) {
  for (const std::string &line : split_lines(text)) {
    std::string t = trim(line);
    if (!t.empty() && t.back() == ';') {
      if (t.rfind("use", 0) == 0) {
        std::string name = directive_arg(t, "use");
        if (log) log->push_back(name);
        if (const char *m = builtin_module_source(name)) out += m;
        continue;  // unknown modules are dropped, as in shader.rs:177-180
      }
      if (t.rfind("include", 0) == 0) {
        std::string file = directive_arg(t, "include");
        // shader.rs:186-188 skips an include of the file itself; here the
        // comparison is on canonical paths, since includes also resolve
        // relative to the including file.
        if (file != self_path && depth < 64) {
          std::string body;
          std::string resolved = file;
          bool ok = read_file(file, body);
          if (!ok && !base_dir.empty() && !file.empty() && file[0] != '/') {
            resolved = base_dir + "/" + file;
            ok = read_file(resolved, body);
          }
          if (ok && !self_path.empty() && canonical(resolved) == canonical(self_path)) ok = false, body.clear(),
              resolved.clear();
          if (ok) {
            size_t slash = resolved.find_last_of('/');
            std::string dir = slash == std::string::npos ? base_dir : resolved.substr(0, slash);
            expand(body, resolved, dir, out, log, depth + 1);
          } else if (log && !resolved.empty()) {
            log->push_back("Could not include \"" + file + "\"");
          }
        }
        continue;
      }
    }
    out += line;
    out += "\n";
  }
}

// ShaderToy-style code as the site stores it (no version line, no uniform
// declarations, no main): wrapped as shadertoy.rs:154-166 does before
// conversion.  The inputs are the site's documented shader inputs; here they
// are uniforms the frontend folds to zero (there is no render loop).
std::string shadertoy_wrap(const std::string &code) {
  std::string g = "#version 450 core\n";
  g += "uniform vec3 iResolution;\nuniform float iTime;\nuniform float iTimeDelta;\nuniform int iFrame;\n";
  g += "uniform vec4 iChannelTime;\nuniform vec4 iMouse;\nuniform vec4 iDate;\nuniform float iSampleRate;\n";
  g += code;
  g += "\nvoid main() {}\n";
  return g;
}

std::string preprocess_sdf3d_text(const std::string &src, const std::string &self_path,
                                  const std::string &base_dir, std::vector<std::string> *log) {
  std::string out;
  expand(src, self_path, base_dir, out, log, 0);
  return out;
}

bool preprocess_sdf3d_file(const std::string &path, std::string &out, std::string &err,
                           std::vector<std::string> *log) {
  std::string text;
  if (!read_file(path, text)) {
    err = "could not read " + path;
    return false;
  }
  size_t slash = path.find_last_of('/');
  std::string dir = slash == std::string::npos ? std::string(".") : path.substr(0, slash);
  out = preprocess_sdf3d_text(text, path, dir, log);
  return true;
}

// shadertoy.rs:248-292: drop the function whose trimmed first line starts
// with `function_name`, by counting braces; lines are emitted trimmed.
bool wgsl_remove_function(const std::string &wgsl, const std::string &function_name, std::string &out) {
  out.clear();
  bool in_function = false, found = false;
  long braces = 0;
  for (const std::string &raw : split_lines(wgsl)) {
    std::string line = trim(raw);
    if (line.rfind(function_name, 0) == 0) {
      in_function = true;
      found = true;
    }
    if (in_function) {
      for (char c : line) {
        if (c == '{') ++braces;
        else if (c == '}') --braces;
      }
    }
    if (braces == 0) {
      if (!in_function) out += line + "\n";
      in_function = false;
    }
  }
  return found;
}

// shadertoy.rs:294-315
bool wgsl_has_function(const std::string &wgsl, const std::string &function_name) {
  std::string prefix = "fn " + function_name + "(";
  for (const std::string &raw : split_lines(wgsl))
    if (trim(raw).rfind(prefix, 0) == 0) return true;
  return false;
}

// shadertoy.rs:317-352 (the renamed line is appended without a newline, as
// the reference does).
bool wgsl_rename_function(const std::string &wgsl, const std::string &old_name,
                          const std::string &new_name, std::string &out) {
  out.clear();
  bool found = false;
  std::string prefix = "fn " + old_name + "(";
  for (const std::string &raw : split_lines(wgsl)) {
    std::string line = trim(raw);
    if (line.rfind(prefix, 0) == 0) {
      found = true;
      size_t p = line.find(old_name);
      out += line.substr(0, p) + new_name + line.substr(p + old_name.size());
    } else {
      out += line + "\n";
    }
  }
  return found;
}

}  // namespace s2m
