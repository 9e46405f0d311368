// s2m_oracle.cpp -- CPU restatement of the sdf2mesh dual-contouring rule.
//
// TEST INFRASTRUCTURE ONLY (the checker and the CPU baseline); the product
// never links or calls this file.  Built with -ffp-contract=off so binary32
// arithmetic rounds after every operation, as the WGSL source is written.
// Every function cites the reference file:line it restates (paths relative to
// the WilstonOreo/sdf2mesh sources).
#include "s2m_oracle.h"

#include <algorithm>
#include <charconv>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// ---------------------------------------------------------------------------
// Small vector types in precision T.
template <class T> struct V3 { T x, y, z; };
template <class T> struct V2 { T x, y; };
template <class T> V3<T> operator+(V3<T> a, V3<T> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class T> V3<T> operator-(V3<T> a, V3<T> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class T> V3<T> operator*(V3<T> a, T s) { return {a.x * s, a.y * s, a.z * s}; }
template <class T> V3<T> operator*(T s, V3<T> a) { return {s * a.x, s * a.y, s * a.z}; }

inline float m_sqrt(float v) { return std::sqrt(v); }
inline double m_sqrt(double v) { return std::sqrt(v); }
inline float m_abs(float v) { return std::fabs(v); }
inline double m_abs(double v) { return std::fabs(v); }
inline float m_min(float a, float b) { return std::fmin(a, b); }
inline double m_min(double a, double b) { return std::fmin(a, b); }
inline float m_max(float a, float b) { return std::fmax(a, b); }
inline double m_max(double a, double b) { return std::fmax(a, b); }

// length / dot as written in WGSL: components summed left to right.
template <class T> T dot3(V3<T> a, V3<T> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class T> T length3(V3<T> a) { return m_sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }
template <class T> T length2(T a, T b) { return m_sqrt(a * a + b * b); }
template <class T> T clampT(T v, T lo, T hi) { return m_min(m_max(v, lo), hi); }
// WGSL mix(e1, e2, e3) = e1 * (1 - e3) + e2 * e3.
template <class T> T mixT(T a, T b, T t) { return a * (T(1) - t) + b * t; }

// ---------------------------------------------------------------------------
// SDF library restated from src/sdf3d_primitives.wgsl and src/sdf_op.wgsl.

// sdf3d_primitives.wgsl:7-11 (b is the FULL box size).
template <class T> T sdf_box(V3<T> p, V3<T> b) {
  V3<T> q = {m_abs(p.x) - T(0.5) * b.x, m_abs(p.y) - T(0.5) * b.y, m_abs(p.z) - T(0.5) * b.z};
  V3<T> mq = {m_max(q.x, T(0)), m_max(q.y, T(0)), m_max(q.z, T(0))};
  return length3(mq) + m_min(m_max(q.x, m_max(q.y, q.z)), T(0));
}
// sdf3d_primitives.wgsl:13-17: d = abs(vec2(length(p.xz), p.y)) - vec2(r, h);
// min(max(d.x, d.y), 0) + length(max(d, vec2f())).
template <class T> T sdf_cylinder(V3<T> p, T h, T r) {
  T dx = m_abs(length2(p.x, p.z)) - r;
  T dy = m_abs(p.y) - h;
  return m_min(m_max(dx, dy), T(0)) + length2(m_max(dx, T(0)), m_max(dy, T(0)));
}
// sdf3d_primitives.wgsl:19-25
template <class T> T sdf_capsule(V3<T> p, V3<T> a, V3<T> b, T r) {
  V3<T> pa = p - a;
  V3<T> ba = b - a;
  T h = clampT(dot3(pa, ba) / dot3(ba, ba), T(0), T(1));
  return length3(pa - ba * h) - r;
}
// sdf3d_primitives.wgsl:27-30
template <class T> T sdf_sphere(V3<T> p, T s) { return length3(p) - s; }
// sdf3d_primitives.wgsl:32-36
template <class T> T sdf_torus(V3<T> p, V2<T> t) {
  T qx = length2(p.x, p.z) - t.x;
  T qy = p.y;
  return length2(qx, qy) - t.y;
}
// sdf_op.wgsl:7-11
template <class T> T op_smooth_union(T d1, T d2, T k) {
  T h = clampT(T(0.5) + T(0.5) * (d2 - d1) / k, T(0), T(1));
  return mixT(d2, d1, h) - k * h * (T(1) - h);
}
// sdf_op.wgsl:13-17
template <class T> T op_smooth_intersection(T d1, T d2, T k) {
  T h = clampT(T(0.5) - T(0.5) * (d2 - d1) / k, T(0), T(1));
  return mixT(d2, d1, h) + k * h * (T(1) - h);
}
// sdf_op.wgsl:19-23
template <class T> T op_smooth_subtraction(T d1, T d2, T k) {
  T h = clampT(T(0.5) - T(0.5) * (d2 + d1) / k, T(0), T(1));
  return mixT(d2, -d1, h) + k * h * (T(1) - h);
}

// ---------------------------------------------------------------------------
// Fixture SDFs.  Parameters arrive as f32 (exactly what a .sdf3d literal
// concretises to) and are widened for the f64 oracle.
template <class T> struct Sdf {
  int kind;
  std::vector<T> prm;

  T operator()(V3<T> p) const {
    switch (kind) {
      case ORACLE_SDF_SPHERE: return sdf_sphere(p, prm[0]);
      case ORACLE_SDF_TORUS: return sdf_torus(p, V2<T>{prm[0], prm[1]});
      case ORACLE_SDF_CSG: return csg(p);
      case ORACLE_SDF_MANDELBULB: return mandelbulb(p);
      case ORACLE_SDF_TREE: return tree(p);
      case ORACLE_SDF_MARTIN_CUBE: return martin_cube(p);
      case ORACLE_SDF_P_KEY: return p_key(p);
    }
    return T(0);
  }

  // WGSL `const` declarations are abstract floats: a constant expression such
  // as C*0.2 is folded in binary64 and rounded once when it meets an f32
  // operand (the WGSL conversion rules as naga applies them).
  static T ac(double v) { return T(v); }
  static V3<T> sw_yxz(V3<T> p) { return {p.y, p.x, p.z}; }
  static V3<T> sw_xzy(V3<T> p) { return {p.x, p.z, p.y}; }
  static V3<T> sw_zyx(V3<T> p) { return {p.z, p.y, p.x}; }
  static V3<T> v3(double a, double b, double c) { return {ac(a), ac(b), ac(c)}; }

  // The letter arc of examples/martin_cube.sdf3d:9-27 and examples/p_key.sdf3d:9-27
  // (the same function over a size constant S: C or KEY_SIZE).
  static T letter_arc(V3<T> p, T ra, T rb, double S) {
    V3<T> pp = sw_yxz(p);
    pp.x = m_abs(pp.x - ac(S * 0.2));
    pp.y = pp.y + ac(S * 0.25);
    const V3<T> h = v3(0.0, S * 0.15, 0.0);
    const V3<T> nh = {-h.x, -h.y, -h.z};
    const V3<T> c = {clampT(pp.x, nh.x, h.x), clampT(pp.y, nh.y, h.y), clampT(pp.z, nh.z, h.z)};
    const V3<T> q = pp - c;
    const T scx = T(1), scy = T(0);
    T k = T(0);
    if (T(0) > scx * q.y) k = q.x * scx + q.y * scy;  // dot(q.xy, sc)
    else k = length2(q.x, q.y);
    return m_sqrt(dot3(q, q) + ra * ra - T(2) * ra * k) - rb;
  }

  // examples/martin_cube.sdf3d: a smooth cube with the letters M A R T I N
  // carved into its faces (capsule segments and an arc).
  static T mc_segment(V3<T> p, V3<T> a, V3<T> b) { return sdf_capsule(p, a, b, ac(0.12)); }  // :30-32
  static T mc_letter_m(V3<T> p) {  // :34-47
    const double C = 1.0;
    V3<T> q = sw_yxz(p);
    q.y = q.y * T(-1);
    return m_min(m_min(mc_segment(q, v3(-C * 0.45, -C * 0.5, C), v3(-C * 0.45, C * 0.5, C)),
                       mc_segment(q, v3(-C * 0.45, -C * 0.5, C), v3(0.0, 0.0, C))),
                 m_min(mc_segment(q, v3(0.0, 0.0, C), v3(C * 0.45, -C * 0.5, C)),
                       mc_segment(q, v3(C * 0.45, -C * 0.5, C), v3(C * 0.45, C * 0.5, C))));
  }
  static T mc_letter_a(V3<T> p) {  // :50-61
    const double C = 1.0;
    V3<T> q = sw_zyx(p);
    q = V3<T>{-q.y, -q.x, q.z};
    return m_min(m_min(mc_segment(q, v3(0.0, -C * 0.5, -C), v3(-C * 0.4, C * 0.5, -C)),
                       mc_segment(q, v3(0.0, -C * 0.5, -C), v3(C * 0.4, C * 0.5, -C))),
                 mc_segment(q, v3(-C * 0.2, C * 0.1, -C), v3(C * 0.2, C * 0.1, -C)));
  }
  static T mc_letter_r(V3<T> p) {  // :64-75
    const double C = 1.0;
    V3<T> q = p;
    q.y = q.y * T(-1);
    q.x = q.x - ac(C * 0.15);
    return m_min(letter_arc(sw_xzy(q) - v3(0.0, 0.0, C), ac(C * 0.3), ac(0.12), C),
                 m_min(mc_segment(q, v3(-C * 0.4, C, C * 0.5), v3(-C * 0.4, C, -C * 0.5)),
                       mc_segment(q, v3(-C * 0.15, C, -C * 0.1), v3(C * 0.15, C, -C * 0.5))));
  }
  static T mc_letter_t(V3<T> p) {  // :79-84
    const double C = 1.0;
    return m_min(mc_segment(p, v3(C, 0.0, C * 0.5), v3(C, 0.0, -C * 0.5)),
                 mc_segment(p, v3(C, -C * 0.4, C * 0.5), v3(C, C * 0.4, C * 0.5)));
  }
  static T mc_letter_i(V3<T> p) {  // :88-92
    const double C = 1.0;
    V3<T> q = sw_yxz(p);
    q.x = q.x * T(-1);
    return mc_segment(q, v3(-C, 0.0, C * 0.5), v3(-C, 0.0, -C * 0.5));
  }
  static T mc_letter_n(V3<T> p) {  // :96-107
    const double C = 1.0;
    V3<T> q = sw_xzy(p);
    return m_min(mc_segment(q, v3(-C * 0.4, -C, C * 0.5), v3(-C * 0.4, -C, -C * 0.5)),
                 m_min(mc_segment(q, v3(C * 0.4, -C, C * 0.5), v3(C * 0.4, -C, -C * 0.5)),
                       mc_segment(q, v3(-C * 0.4, -C, -C * 0.5), v3(C * 0.4, -C, C * 0.5))));
  }
  static T martin_cube(V3<T> p) {  // :109-120
    const T cube = op_smooth_intersection(sdf_box(p, v3(1.0, 1.0, 1.0)), sdf_sphere(p, ac(1.0 * 1.40)), ac(0.02));
    const T letter = m_min(m_min(mc_letter_m(p), mc_letter_a(p)),
                           m_min(m_min(mc_letter_r(p), mc_letter_t(p)), m_min(mc_letter_i(p), mc_letter_n(p))));
    return op_smooth_subtraction(letter, cube, ac(0.02));
  }

  // examples/p_key.sdf3d: a key plate with a raised cylinder and the letter P.
  static T pk_letter_p(V3<T> p) {  // :33-41
    const double K = 15.0;
    V3<T> q = p;
    q.y = q.y * T(-1);
    q.x = q.x - ac(K * 0.15);
    return m_min(letter_arc(sw_xzy(q), ac(K * 0.3), ac(1.0), K),
                 sdf_capsule(q, v3(-K * 0.4, 0.0, K * 0.5), v3(-K * 0.4, 0.0, -K * 0.5), ac(1.0)));
  }
  static T p_key(V3<T> p) {  // :43-53
    const double K = 15.0, E = 2.0, H = 1.5, L = 1.0;
    const V3<T> s = sw_xzy(p) * ac(2.5);
    const V3<T> yzx = {p.y, p.z, p.x};
    return op_smooth_subtraction(
        pk_letter_p(s - v3(0.0, E * 2.5 + L, 0.0)),
        op_smooth_union(sdf_box(p, v3(K, K, H)), sdf_cylinder(yzx - v3(0.0, (E + H) * 0.5, 0.0), ac(E - H), ac(K * 0.35)),
                        ac(K * 0.15)),
        ac(0.0));
  }

  // Large-scale CSG workload: max(box(p, vec3(b)) - round, -S(p)) unioned by
  // min with a torus, S a left fold of sdf_op_smooth_union over n spheres.
  //   fn sdf3d(p) = min(max(sdf3d_box(p, vec3f(b)) - rr, -S), sdf3d_torus(p, vec2(R, r)))
  T csg(V3<T> p) const {
    T bfull = prm[0], rr = prm[1], tR = prm[2], tr = prm[3], k = prm[4];
    int n = int(prm[5]);
    const T *sp = &prm[6];
    T s = sdf_sphere(p - V3<T>{sp[0], sp[1], sp[2]}, sp[3]);
    for (int i = 1; i < n; ++i) {
      const T *c = sp + 4 * i;
      s = op_smooth_union(s, sdf_sphere(p - V3<T>{c[0], c[1], c[2]}, c[3]), k);
    }
    T box = sdf_box(p, V3<T>{bfull, bfull, bfull}) - rr;
    T carved = m_max(box, -s);
    return m_min(carved, sdf_torus(p, V2<T>{tR, tr}));
  }

  // Mandelbulb distance estimate, the published power-N formula in the form
  // of the reference's example GLSL (examples/mandelmesh.frag:3-28): the
  // input is swizzled to xzy, one-argument atan of y/x, asin of z/r, a
  // `continue` once r exceeds the bailout, and 0.5*log(r)*r/dr - offset.
  T mandelbulb(V3<T> p0) const {
    T power = prm[0];
    int iters = int(prm[1]);
    T bailout = prm[2], offset = prm[3];
    V3<T> p = {p0.x, p0.z, p0.y};
    V3<T> z = p;
    T r = T(0), theta = T(0), phi = T(0);
    T dr = T(1);
    for (int i = 0; i < iters; ++i) {
      r = length3(z);
      if (r > bailout) continue;
      theta = std::atan(z.y / z.x);
      phi = std::asin(z.z / r);
      dr = std::pow(r, power - T(1)) * dr * power + T(1);
      r = std::pow(r, power);
      theta = theta * power;
      phi = phi * power;
      V3<T> w = {std::cos(theta) * std::cos(phi), std::sin(theta) * std::cos(phi), std::sin(phi)};
      z = r * w + p;
    }
    return T(0.5) * std::log(r) * r / dr - offset;
  }

  // Random CSG tree as a postfix program (the batching workload).
  //   0 sphere  cx cy cz r           -> sdf3d_sphere(p - c, r)
  //   1 box     cx cy cz bx by bz    -> sdf3d_box(p - c, b)
  //   2 torus   cx cy cz R r         -> sdf3d_torus(p - c, vec2(R, r))
  //   3 capsule ax ay az bx by bz r  -> sdf3d_capsule(p, a, b, r)
  //   4 plane   nx ny nz d           -> dot(p, n) - d
  //   5 cylinder cx cy cz h r        -> sdf3d_cylinder(p - c, h, r)   (oracle only)
  //  10 union   (a b -> min(a, b))
  //  11 subtract(a b -> max(a, -b))
  //  12 intersect (a b -> max(a, b))
  //  13 smooth-union k (a b -> sdf_op_smooth_union(a, b, k))
  //  14 smooth-intersection k, 15 smooth-subtraction k (sdf_op.wgsl:13-23)
  T tree(V3<T> p) const {
    T stack[64];
    int sp = 0;
    size_t i = 0;
    while (i < prm.size()) {
      int op = int(prm[i++]);
      const T *a = &prm[i];
      switch (op) {
        case 0: stack[sp++] = sdf_sphere(p - V3<T>{a[0], a[1], a[2]}, a[3]); i += 4; break;
        case 1: stack[sp++] = sdf_box(p - V3<T>{a[0], a[1], a[2]}, V3<T>{a[3], a[4], a[5]}); i += 6; break;
        case 2: stack[sp++] = sdf_torus(p - V3<T>{a[0], a[1], a[2]}, V2<T>{a[3], a[4]}); i += 5; break;
        case 3: stack[sp++] = sdf_capsule(p, V3<T>{a[0], a[1], a[2]}, V3<T>{a[3], a[4], a[5]}, a[6]); i += 7; break;
        case 4: stack[sp++] = dot3(p, V3<T>{a[0], a[1], a[2]}) - a[3]; i += 4; break;
        case 5: stack[sp++] = sdf_cylinder(p - V3<T>{a[0], a[1], a[2]}, a[3], a[4]); i += 5; break;
        case 10: { T b = stack[--sp]; stack[sp - 1] = m_min(stack[sp - 1], b); } break;
        case 11: { T b = stack[--sp]; stack[sp - 1] = m_max(stack[sp - 1], -b); } break;
        case 12: { T b = stack[--sp]; stack[sp - 1] = m_max(stack[sp - 1], b); } break;
        case 13: { T b = stack[--sp]; stack[sp - 1] = op_smooth_union(stack[sp - 1], b, a[0]); i += 1; } break;
        case 14: { T b = stack[--sp]; stack[sp - 1] = op_smooth_intersection(stack[sp - 1], b, a[0]); i += 1; } break;
        case 15: { T b = stack[--sp]; stack[sp - 1] = op_smooth_subtraction(stack[sp - 1], b, a[0]); i += 1; } break;
        default: return T(NAN);
      }
    }
    return sp > 0 ? stack[sp - 1] : T(NAN);
  }
};

template <class T> Sdf<T> make_sdf(int kind, const float *p, int n) {
  Sdf<T> s;
  s.kind = kind;
  s.prm.assign(p, p + n);
  return s;
}

// ---------------------------------------------------------------------------
// Reference cell rule.

template <class T> struct Job {
  int N;
  T bmin[3], bmax[3], size[3];
  T eps;
};

// main.rs:139-175 with lib.rs:115-118: Bounds3D::cube(B, 0) -> [-B/2, B/2]
// (computed in f32 as euclid does), eps = 1e-4 carried in bb_max.w.
template <class T> Job<T> make_job(uint32_t N, float B, float eps) {
  Job<T> j;
  j.N = int(N);
  float half = B * 0.5f;          // Vec3D::splat(a) * 0.5
  float mn = 0.0f - half;         // center - v
  float mx = 0.0f + half;         // center + v
  for (int a = 0; a < 3; ++a) {
    j.bmin[a] = T(mn);
    j.bmax[a] = T(mx);
    // dualcontour.wgsl:23-24: size = (max - min) / f32(res - 1)
    j.size[a] = (j.bmax[a] - j.bmin[a]) / T(float(N - 1u));
  }
  j.eps = T(eps);
  return j;
}

template <class T> struct CellOut {
  bool has_vertex;
  uint8_t signs;
  T pos[3];
  T nrm[3];
};

// dualcontour.wgsl:22-27 (cell_bounds) and :29-43 (cell_new).
template <class T, class F>
void cell_corners(const Job<T> &j, const F &f, int x, int y, int z, T mn[3], T mx[3], T c[8]) {
  int pos[3] = {x, y, z};
  for (int a = 0; a < 3; ++a) {
    mn[a] = j.bmin[a] + j.size[a] * T(pos[a]);
    mx[a] = mn[a] + j.size[a];
  }
  // corner index = bx | by << 1 | bz << 2 (000,100,010,110,001,101,011,111)
  for (int k = 0; k < 8; ++k) {
    V3<T> p = {(k & 1) ? mx[0] : mn[0], (k & 2) ? mx[1] : mn[1], (k & 4) ? mx[2] : mn[2]};
    c[k] = f(p);
  }
}

// dualcontour.wgsl:72-74
template <class T> T adapt(T v0, T v1) { return (T(0) - v0) / (v1 - v0); }

// dualcontour.wgsl:86-131 (mass point) and :161-180 (kernel body).
template <class T, class F>
CellOut<T> eval_cell(const Job<T> &j, const F &f, int x, int y, int z) {
  T mn[3], mx[3], c[8];
  cell_corners(j, f, x, y, z, mn, mx, c);
  const T c000 = c[0], c100 = c[1], c010 = c[2], c110 = c[3];
  const T c001 = c[4], c101 = c[5], c011 = c[6], c111 = c[7];
  // Edge table in the order of dualcontour.wgsl:99-114: (a, b, fixed coords, axis of t).
  struct E { T a, b; T u, v; int axis; };
  const E edges[12] = {
      {c000, c001, 0, 0, 2}, {c010, c011, 0, 1, 2}, {c100, c101, 1, 0, 2}, {c110, c111, 1, 1, 2},
      {c000, c010, 0, 0, 1}, {c001, c011, 0, 1, 1}, {c100, c110, 1, 0, 1}, {c101, c111, 1, 1, 1},
      {c000, c100, 0, 0, 0}, {c001, c101, 0, 1, 0}, {c010, c110, 1, 0, 0}, {c011, c111, 1, 1, 0}};
  T avg[3] = {0, 0, 0};
  T count = 0;
  for (int i = 0; i < 12; ++i) {
    const E &e = edges[i];
    T v[3] = {0, 0, 0};
    if ((e.a > T(0)) != (e.b > T(0))) {
      T t = adapt(e.a, e.b);
      // z edges: (u, v, t); y edges: (u, t, v); x edges: (t, u, v)
      if (e.axis == 2) { v[0] = e.u; v[1] = e.v; v[2] = t; }
      else if (e.axis == 1) { v[0] = e.u; v[1] = t; v[2] = e.v; }
      else { v[0] = t; v[1] = e.u; v[2] = e.v; }
    }
    if (v[0] > T(0) || v[1] > T(0) || v[2] > T(0)) {  // :120
      avg[0] = avg[0] + v[0];
      avg[1] = avg[1] + v[1];
      avg[2] = avg[2] + v[2];
      count = count + T(1);
    }
  }
  CellOut<T> o;
  // dualcontour.wgsl:57-59 sign bits
  o.signs = uint8_t((c100 > T(0) ? 1 : 0) | (c010 > T(0) ? 2 : 0) | (c001 > T(0) ? 4 : 0) |
                    (c000 > T(0) ? 8 : 0));
  if (count <= T(1)) {  // :126-128
    o.has_vertex = false;
    return o;
  }
  o.has_vertex = true;
  for (int a = 0; a < 3; ++a) {
    T bsize = mx[a] - mn[a];                  // bounds_size(c.bounds)
    o.pos[a] = mn[a] + bsize * avg[a] / count;  // :130
  }
  // sdf3d_normal.wgsl:4-10, then normalize (dualcontour.wgsl:171).
  const T e = j.eps;
  V3<T> p = {o.pos[0], o.pos[1], o.pos[2]};
  V3<T> v1 = {T(1), T(-1), T(-1)}, v2 = {T(-1), T(-1), T(1)};
  V3<T> v3 = {T(-1), T(1), T(-1)}, v4 = {T(1), T(1), T(1)};
  V3<T> n = v1 * f(p + v1 * e) + v2 * f(p + v2 * e);
  n = n + v3 * f(p + v3 * e);
  n = n + v4 * f(p + v4 * e);
  T len = length3(n);
  o.nrm[0] = n.x / len;
  o.nrm[1] = n.y / len;
  o.nrm[2] = n.z / len;
  return o;
}

// ---------------------------------------------------------------------------
// Precision mode (ORACLE_FLAG_QEF).  Corners come from the lattice c(i) =
// bmin + size * i, shared by neighbouring cells, so all cells agree on every
// sign.  Each sign-change edge gives a crossing q (cell-local, in [0,1]^3, t
// as in dualcontour.wgsl:72-74) and a unit normal n (the tetrahedral
// gradient of sdf3d_normal.wgsl:4-10 at the crossing, normalised); the
// vertex minimises sum (n . (x - q))^2 around the mass point.  The sums are
// accumulated in T with Neumaier compensation; the 3x3 solve is binary64:
// cyclic Jacobi eigen-decomposition, eigenvalues below 0.1 of the largest
// dropped, x = c + V D^+ V^T (A^T b - A c), clamped to the cell.

template <class T> struct KSum {
  T s = 0, c = 0;
  void add(T x) {
    T t = s + x;
    if (m_abs(s) >= m_abs(x)) c = c + ((s - t) + x);
    else c = c + ((x - t) + s);
    s = t;
  }
  T value() const { return s + c; }
};

// Symmetric 3x3 eigen-decomposition by cyclic Jacobi rotations (binary64).
// a: row-major symmetric matrix (overwritten); v: eigenvectors in columns.
inline void jacobi3(double a[3][3], double v[3][3]) {
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) v[i][j] = i == j ? 1.0 : 0.0;
  for (int sweep = 0; sweep < 24; ++sweep) {
    double off = a[0][1] * a[0][1] + a[0][2] * a[0][2] + a[1][2] * a[1][2];
    double diag = a[0][0] * a[0][0] + a[1][1] * a[1][1] + a[2][2] * a[2][2];
    if (!(off > 1e-30 * diag)) break;
    for (int pq = 0; pq < 3; ++pq) {
      const int p = pq == 2 ? 1 : 0, q = pq == 0 ? 1 : 2;
      const double apq = a[p][q];
      if (apq == 0.0) continue;
      const double theta = (a[q][q] - a[p][p]) / (2.0 * apq);
      const double t = (theta >= 0.0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
      const double c = 1.0 / std::sqrt(t * t + 1.0);
      const double sn = t * c;
      for (int k = 0; k < 3; ++k) {  // A <- A J (columns p, q)
        const double akp = a[k][p], akq = a[k][q];
        a[k][p] = c * akp - sn * akq;
        a[k][q] = sn * akp + c * akq;
      }
      for (int k = 0; k < 3; ++k) {  // A <- J^T A (rows p, q)
        const double apk = a[p][k], aqk = a[q][k];
        a[p][k] = c * apk - sn * aqk;
        a[q][k] = sn * apk + c * aqk;
      }
      for (int k = 0; k < 3; ++k) {  // V <- V J
        const double vkp = v[k][p], vkq = v[k][q];
        v[k][p] = c * vkp - sn * vkq;
        v[k][q] = sn * vkp + c * vkq;
      }
    }
  }
}

// x = c + pinv(A) (b - A c), eigenvalues < 0.1 * max dropped; clamped to [0,1].
inline void qef_solve(const double A[6], const double b[3], const double c[3], double x[3]) {
  double a[3][3] = {{A[0], A[1], A[2]}, {A[1], A[3], A[4]}, {A[2], A[4], A[5]}};
  double r[3];
  for (int i = 0; i < 3; ++i) r[i] = b[i] - ((a[i][0] * c[0] + a[i][1] * c[1]) + a[i][2] * c[2]);
  double v[3][3];
  jacobi3(a, v);
  double lmax = std::fmax(std::fabs(a[0][0]), std::fmax(std::fabs(a[1][1]), std::fabs(a[2][2])));
  double y[3];
  for (int k = 0; k < 3; ++k) {
    double vr = (v[0][k] * r[0] + v[1][k] * r[1]) + v[2][k] * r[2];
    double l = a[k][k];
    y[k] = (lmax > 0.0 && std::fabs(l) >= 0.1 * lmax) ? vr / l : 0.0;
  }
  for (int i = 0; i < 3; ++i) {
    double d = (v[i][0] * y[0] + v[i][1] * y[1]) + v[i][2] * y[2];
    double xi = c[i] + d;
    x[i] = xi < 0.0 ? 0.0 : (xi > 1.0 ? 1.0 : xi);
  }
}

template <class T, class F> V3<T> tetra_normal(const F &f, V3<T> p, T e) {
  V3<T> v1 = {T(1), T(-1), T(-1)}, v2 = {T(-1), T(-1), T(1)};
  V3<T> v3 = {T(-1), T(1), T(-1)}, v4 = {T(1), T(1), T(1)};
  V3<T> n = v1 * f(p + v1 * e) + v2 * f(p + v2 * e);
  n = n + v3 * f(p + v3 * e);
  n = n + v4 * f(p + v4 * e);
  return n;
}

template <class T> T lattice_coord(const Job<T> &j, int a, int i) { return j.bmin[a] + j.size[a] * T(i); }

template <class T, class F>
CellOut<T> eval_cell_qef(const Job<T> &j, const F &f, int x, int y, int z) {
  int pos[3] = {x, y, z};
  T lo[3], hi[3];
  for (int a = 0; a < 3; ++a) {
    lo[a] = lattice_coord(j, a, pos[a]);
    hi[a] = lattice_coord(j, a, pos[a] + 1);
  }
  T c[8];
  for (int k = 0; k < 8; ++k)
    c[k] = f(V3<T>{(k & 1) ? hi[0] : lo[0], (k & 2) ? hi[1] : lo[1], (k & 4) ? hi[2] : lo[2]});
  static const int ea[12] = {0, 2, 1, 3, 0, 4, 1, 5, 0, 4, 2, 6};
  static const int eb[12] = {4, 6, 5, 7, 2, 6, 3, 7, 1, 5, 3, 7};
  static const int eax[12] = {2, 2, 2, 2, 1, 1, 1, 1, 0, 0, 0, 0};
  KSum<T> sA[6], sb[3], sq[3];
  int m = 0;
  for (int e = 0; e < 12; ++e) {
    T a = c[ea[e]], b = c[eb[e]];
    if ((a > T(0)) == (b > T(0))) continue;
    T t = adapt(a, b);
    T q[3], w[3];
    for (int ax = 0; ax < 3; ++ax) {
      if (ax == eax[e]) {
        q[ax] = t;
        w[ax] = lo[ax] + j.size[ax] * t;
      } else {
        bool one = (ea[e] >> ax) & 1;
        q[ax] = one ? T(1) : T(0);
        w[ax] = one ? hi[ax] : lo[ax];
      }
    }
    V3<T> n = tetra_normal(f, V3<T>{w[0], w[1], w[2]}, j.eps);
    T len = length3(n);
    ++m;
    for (int ax = 0; ax < 3; ++ax) sq[ax].add(q[ax]);
    if (!(len > T(0))) continue;
    T nn[3] = {n.x / len, n.y / len, n.z / len};
    T d = (nn[0] * q[0] + nn[1] * q[1]) + nn[2] * q[2];
    sA[0].add(nn[0] * nn[0]); sA[1].add(nn[0] * nn[1]); sA[2].add(nn[0] * nn[2]);
    sA[3].add(nn[1] * nn[1]); sA[4].add(nn[1] * nn[2]); sA[5].add(nn[2] * nn[2]);
    for (int ax = 0; ax < 3; ++ax) sb[ax].add(nn[ax] * d);
  }
  CellOut<T> o;
  o.signs = uint8_t((c[1] > T(0) ? 1 : 0) | (c[2] > T(0) ? 2 : 0) | (c[4] > T(0) ? 4 : 0) | (c[0] > T(0) ? 8 : 0));
  o.has_vertex = m > 0;
  if (!o.has_vertex) return o;
  double A[6], bb[3], cc[3], xs[3];
  for (int i = 0; i < 6; ++i) A[i] = double(sA[i].value());
  for (int ax = 0; ax < 3; ++ax) {
    bb[ax] = double(sb[ax].value());
    cc[ax] = double(sq[ax].value()) / double(m);
  }
  qef_solve(A, bb, cc, xs);
  for (int ax = 0; ax < 3; ++ax) o.pos[ax] = T(double(lo[ax]) + double(j.size[ax]) * xs[ax]);
  V3<T> n = tetra_normal(f, V3<T>{o.pos[0], o.pos[1], o.pos[2]}, j.eps);
  T len = length3(n);
  o.nrm[0] = n.x / len;
  o.nrm[1] = n.y / len;
  o.nrm[2] = n.z / len;
  return o;
}

struct Item {
  uint16_t x, y, z;
  uint8_t signs;
  uint64_t key() const { return uint64_t(x) | (uint64_t(y) << 16) | (uint64_t(z) << 32); }
};

// mesh.rs:326-331: binary search by key, u32::MAX if absent.
uint32_t vertex_index(const std::vector<Item> &items, uint16_t x, uint16_t y, uint16_t z) {
  uint64_t k = uint64_t(x) | (uint64_t(y) << 16) | (uint64_t(z) << 32);
  size_t lo = 0, hi = items.size();
  while (lo < hi) {
    size_t mid = (lo + hi) / 2;
    uint64_t mk = items[mid].key();
    if (mk < k) lo = mid + 1;
    else if (mk > k) hi = mid;
    else return uint32_t(mid);
  }
  return 0xFFFFFFFFu;
}

// mesh.rs:267-324 with Quad::swap / make_triangles / is_valid (lib.rs:190-211).
void build_triangles(const std::vector<Item> &items, std::vector<uint32_t> &tris, int64_t &invalid) {
  tris.clear();
  tris.reserve(items.size() * 6);
  invalid = 0;
  auto push = [&](uint32_t q0, uint32_t q1, uint32_t q2, uint32_t q3, bool swap) {
    if (swap) { std::swap(q0, q3); std::swap(q1, q2); }
    if (q0 == 0xFFFFFFFFu || q1 == 0xFFFFFFFFu || q2 == 0xFFFFFFFFu || q3 == 0xFFFFFFFFu) {
      ++invalid;
      return;
    }
    tris.push_back(q2); tris.push_back(q1); tris.push_back(q0);
    tris.push_back(q0); tris.push_back(q3); tris.push_back(q2);
  };
  for (const Item &it : items) {
    bool b0 = it.signs & 1, b1 = it.signs & 2, b2 = it.signs & 4, b3 = it.signs & 8;
    uint16_t x = it.x, y = it.y, z = it.z;
    if (b0 != b3 && y > 0 && z > 0)
      push(vertex_index(items, x, y - 1, z - 1), vertex_index(items, x, y, z - 1),
           vertex_index(items, x, y, z), vertex_index(items, x, y - 1, z), b0);
    if (b1 != b3 && x > 0 && z > 0)
      push(vertex_index(items, x - 1, y, z - 1), vertex_index(items, x, y, z - 1),
           vertex_index(items, x, y, z), vertex_index(items, x - 1, y, z), !b1);
    if (b2 != b3 && x > 0 && y > 0)
      push(vertex_index(items, x - 1, y - 1, z), vertex_index(items, x, y - 1, z),
           vertex_index(items, x, y, z), vertex_index(items, x - 1, y, z), b2);
  }
}

template <class T>
int run(int kind, const float *sp, int ns, const oracle_params *pp, oracle_mesh *out) {
  Sdf<T> f = make_sdf<T>(kind, sp, ns);
  Job<T> j = make_job<T>(pp->resolution, pp->bounds, pp->eps);
  const int N = j.N;
  const bool lag = pp->flags & ORACLE_FLAG_SLICE_LAG;
  const bool qef = pp->flags & ORACLE_FLAG_QEF;
  // main.rs:298-356: cells of slice z are labelled z; with the read-before-
  // submit lag, iteration z reads slice z-1, so only slices 0..N-2 surface,
  // labelled +1.
  int z_lo = 0, z_hi = lag ? N - 1 : N;
  if (pp->z_begin >= 0) z_lo = std::max(z_lo, int(pp->z_begin));
  if (pp->z_end >= 0) z_hi = std::min(z_hi, int(pp->z_end));
#ifdef _OPENMP
  if (pp->threads > 0) omp_set_num_threads(pp->threads);
#endif
  std::vector<Item> items;
  std::vector<T> pos, nrm;
  auto t0 = std::chrono::steady_clock::now();
  std::vector<std::vector<CellOut<T>>> rows(N);
  std::vector<std::vector<int>> rowx(N);
  for (int z = z_lo; z < z_hi; ++z) {
#pragma omp parallel for schedule(dynamic, 1)
    for (int y = 0; y < N; ++y) {
      rows[y].clear();
      rowx[y].clear();
      for (int x = 0; x < N; ++x) {
        CellOut<T> c = qef ? eval_cell_qef(j, f, x, y, z) : eval_cell(j, f, x, y, z);
        if (c.has_vertex) {
          rows[y].push_back(c);
          rowx[y].push_back(x);
        }
      }
    }
    uint16_t label = uint16_t(lag ? z + 1 : z);
    for (int y = 0; y < N; ++y) {
      for (size_t i = 0; i < rows[y].size(); ++i) {
        const CellOut<T> &c = rows[y][i];
        items.push_back(Item{uint16_t(rowx[y][i]), uint16_t(y), label, c.signs});
        pos.insert(pos.end(), c.pos, c.pos + 3);
        nrm.insert(nrm.end(), c.nrm, c.nrm + 3);
      }
    }
  }
  auto t1 = std::chrono::steady_clock::now();
  std::vector<uint32_t> tris;
  int64_t invalid = 0;
  if (!pp->skip_quads) build_triangles(items, tris, invalid);
  auto t2 = std::chrono::steady_clock::now();

  std::memset(out, 0, sizeof(*out));
  out->nverts = int64_t(items.size());
  out->ntris = int64_t(tris.size() / 3);
  out->invalid_quads = invalid;
  out->seconds_cells = std::chrono::duration<double>(t1 - t0).count();
  out->seconds_quads = std::chrono::duration<double>(t2 - t1).count();
  size_t nv = items.size();
  T *pd = static_cast<T *>(std::malloc(sizeof(T) * (3 * nv + 1)));
  T *nd = static_cast<T *>(std::malloc(sizeof(T) * (3 * nv + 1)));
  if (nv) {
    std::memcpy(pd, pos.data(), sizeof(T) * 3 * nv);
    std::memcpy(nd, nrm.data(), sizeof(T) * 3 * nv);
  }
  if (sizeof(T) == 4) { out->pos = reinterpret_cast<float *>(pd); out->nrm = reinterpret_cast<float *>(nd); }
  else { out->pos64 = reinterpret_cast<double *>(pd); out->nrm64 = reinterpret_cast<double *>(nd); }
  out->cell = static_cast<uint16_t *>(std::malloc(sizeof(uint16_t) * (3 * nv + 1)));
  out->signs = static_cast<uint8_t *>(std::malloc(nv + 1));
  for (size_t i = 0; i < nv; ++i) {
    out->cell[3 * i] = items[i].x;
    out->cell[3 * i + 1] = items[i].y;
    out->cell[3 * i + 2] = items[i].z;
    out->signs[i] = items[i].signs;
  }
  out->tris = static_cast<uint32_t *>(std::malloc(sizeof(uint32_t) * (tris.size() + 1)));
  if (!tris.empty()) std::memcpy(out->tris, tris.data(), sizeof(uint32_t) * tris.size());
  return 0;
}

// ---------------------------------------------------------------------------
// Rust `{}` Display for f32: the shortest digits that round-trip, written
// without an exponent; "-0", "NaN", "inf", "-inf" as Rust prints them.
int format_f32(float v, char *buf, int buflen) {
  std::string s;
  if (std::isnan(v)) s = "NaN";
  else if (std::isinf(v)) s = v < 0 ? "-inf" : "inf";
  else {
    char tmp[64];
    auto r = std::to_chars(tmp, tmp + sizeof(tmp), v, std::chars_format::scientific);
    std::string sci(tmp, r.ptr);
    bool neg = std::signbit(v);
    if (neg && sci[0] == '-') sci.erase(0, 1);
    size_t epos = sci.find('e');
    std::string mant = sci.substr(0, epos);
    int ex = std::atoi(sci.c_str() + epos + 1);
    std::string digits;
    for (char c : mant) if (c != '.') digits.push_back(c);
    // value = 0.d1d2d3... * 10^(ex+1)
    int point = ex + 1;
    if (digits == "0") { s = "0"; }
    else if (point <= 0) {
      s = "0." + std::string(size_t(-point), '0') + digits;
    } else if (size_t(point) >= digits.size()) {
      s = digits + std::string(size_t(point) - digits.size(), '0');
    } else {
      s = digits.substr(0, size_t(point)) + "." + digits.substr(size_t(point));
    }
    if (neg) s = "-" + s;
  }
  int n = int(s.size());
  if (n + 1 > buflen) return -1;
  std::memcpy(buf, s.c_str(), size_t(n) + 1);
  return n;
}

std::string fmt(float v) {
  char b[64];
  format_f32(v, b, sizeof b);
  return b;
}

}  // namespace

extern "C" {

int oracle_mesh_run(int kind, const float *sp, int ns, int precision, const oracle_params *p,
                    oracle_mesh *out) {
  if (!p || !out || p->resolution < 2) return -1;
  if (precision == ORACLE_F64) return run<double>(kind, sp, ns, p, out);
  return run<float>(kind, sp, ns, p, out);
}

void oracle_mesh_free(oracle_mesh *m) {
  if (!m) return;
  std::free(m->pos); std::free(m->nrm); std::free(m->pos64); std::free(m->nrm64);
  std::free(m->cell); std::free(m->signs); std::free(m->tris);
  std::memset(m, 0, sizeof(*m));
}

int oracle_eval(int kind, const float *sp, int ns, int precision, const double *xyz, int64_t n,
                double *out) {
  if (precision == ORACLE_F64) {
    Sdf<double> f = make_sdf<double>(kind, sp, ns);
    for (int64_t i = 0; i < n; ++i) out[i] = f(V3<double>{xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]});
  } else {
    Sdf<float> f = make_sdf<float>(kind, sp, ns);
    for (int64_t i = 0; i < n; ++i)
      out[i] = f(V3<float>{float(xyz[3 * i]), float(xyz[3 * i + 1]), float(xyz[3 * i + 2])});
  }
  return 0;
}

int oracle_cell_corners(int kind, const float *sp, int ns, int precision, uint32_t N, float B,
                        int32_t x, int32_t y, int32_t z, double *out8) {
  if (precision == ORACLE_F64) {
    Sdf<double> f = make_sdf<double>(kind, sp, ns);
    Job<double> j = make_job<double>(N, B, 1e-4f);
    double mn[3], mx[3], c[8];
    cell_corners(j, f, x, y, z, mn, mx, c);
    for (int k = 0; k < 8; ++k) out8[k] = c[k];
  } else {
    Sdf<float> f = make_sdf<float>(kind, sp, ns);
    Job<float> j = make_job<float>(N, B, 1e-4f);
    float mn[3], mx[3], c[8];
    cell_corners(j, f, x, y, z, mn, mx, c);
    for (int k = 0; k < 8; ++k) out8[k] = c[k];
  }
  return 0;
}

int oracle_format_f32(float v, char *buf, int buflen) { return format_f32(v, buf, buflen); }

// mesh.rs:8-48 (STLWriter), 155-180 (fetch_triangles + write), lib.rs:181-185
// (facet normal = (v2 - v0) x (v1 - v0), not normalised).
int oracle_write_stl(const float *pos, const uint32_t *tris, int64_t ntris, const char *path) {
  FILE *fp = std::fopen(path, "wb");
  if (!fp) return -1;
  std::fputs("solid\n", fp);
  for (int64_t t = 0; t < ntris; ++t) {
    const float *a = pos + 3 * size_t(tris[3 * t]);
    const float *b = pos + 3 * size_t(tris[3 * t + 1]);
    const float *c = pos + 3 * size_t(tris[3 * t + 2]);
    float u[3] = {c[0] - a[0], c[1] - a[1], c[2] - a[2]};
    float w[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]};
    float n[3] = {u[1] * w[2] - u[2] * w[1], u[2] * w[0] - u[0] * w[2], u[0] * w[1] - u[1] * w[0]};
    std::fprintf(fp, "facet normal %s %s %s\n", fmt(n[0]).c_str(), fmt(n[1]).c_str(), fmt(n[2]).c_str());
    std::fputs("\touter loop\n", fp);
    for (const float *v : {a, b, c})
      std::fprintf(fp, "\t\tvertex %s %s %s\n", fmt(v[0]).c_str(), fmt(v[1]).c_str(), fmt(v[2]).c_str());
    std::fputs("\tendloop\nendfacet\n", fp);
  }
  std::fputs("endsolid\n", fp);
  return std::fclose(fp) == 0 ? 0 : -1;
}

// mesh.rs:50-141 (PLYWriter) and 198-210 (write_ply_to_file).
int oracle_write_ply(const float *pos, const float *nrm, int64_t nverts, const uint32_t *tris,
                     int64_t ntris, const char *path) {
  FILE *fp = std::fopen(path, "wb");
  if (!fp) return -1;
  std::fprintf(fp, "ply\nformat ascii 1.0\ncomment written by rust-sdf\n");
  std::fprintf(fp, "element vertex %lld\n", (long long)nverts);
  std::fputs("property float x\nproperty float y\nproperty float z\n"
             "property float nx\nproperty float ny\nproperty float nz\n", fp);
  std::fprintf(fp, "element face %lld\n", (long long)ntris);
  std::fputs("property list uchar int vertex_index\nend_header\n", fp);
  for (int64_t i = 0; i < nverts; ++i)
    std::fprintf(fp, "%s %s %s %s %s %s\n", fmt(pos[3 * i]).c_str(), fmt(pos[3 * i + 1]).c_str(),
                 fmt(pos[3 * i + 2]).c_str(), fmt(nrm[3 * i]).c_str(), fmt(nrm[3 * i + 1]).c_str(),
                 fmt(nrm[3 * i + 2]).c_str());
  for (int64_t t = 0; t < ntris; ++t)
    std::fprintf(fp, "3 %u %u %u\n", tris[3 * t], tris[3 * t + 1], tris[3 * t + 2]);
  return std::fclose(fp) == 0 ? 0 : -1;
}

}  // extern "C"
