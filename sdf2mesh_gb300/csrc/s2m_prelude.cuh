// s2m_prelude.cuh -- vector types and shader builtins for SDF code lowered
// from WGSL / GLSL by the sdf2mesh_gb300 frontend.
//
// The same header is compiled by NVRTC (device) and by a host C++ compiler
// (frontend tests), so every function is __host__ __device__.  Arithmetic is
// written out operation by operation in the order the WGSL builtin
// definitions give (e.g. dot sums components left to right, mix is
// e1 * (1 - t) + e2 * t, normalize divides by length), so that with FMA
// contraction disabled the device and the host round identically.
#pragma once

#if defined(__CUDACC_RTC__) || defined(__CUDACC__)
#define S2HD __host__ __device__ __forceinline__
#define S2M_PRUNED_FN __host__ __device__ __noinline__
#define S2I_FN __host__ __device__ __noinline__
#else
#define S2M_PRUNED_FN inline
#define S2I_FN inline
#include <cmath>
#include <cstring>
#define S2HD inline
using std::sqrt;
inline float __int_as_float(unsigned x) { float f; std::memcpy(&f, &x, 4); return f; }
#endif

template <class T, int N> struct s2vec;

template <class T> struct s2vec<T, 2> {
  T x, y;
  S2HD T &operator[](int i) { return i == 0 ? x : y; }
  S2HD T operator[](int i) const { return i == 0 ? x : y; }
};
template <class T> struct s2vec<T, 3> {
  T x, y, z;
  S2HD T &operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
  S2HD T operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};
template <class T> struct s2vec<T, 4> {
  T x, y, z, w;
  S2HD T &operator[](int i) { return i == 0 ? x : (i == 1 ? y : (i == 2 ? z : w)); }
  S2HD T operator[](int i) const { return i == 0 ? x : (i == 1 ? y : (i == 2 ? z : w)); }
};

typedef s2vec<float, 2> s2v2;
typedef s2vec<float, 3> s2v3;
typedef s2vec<float, 4> s2v4;

// Constructors from a component list.
template <class T> S2HD s2vec<T, 2> s2mk(T a, T b) { s2vec<T, 2> r; r.x = a; r.y = b; return r; }
template <class T> S2HD s2vec<T, 3> s2mk(T a, T b, T c) { s2vec<T, 3> r; r.x = a; r.y = b; r.z = c; return r; }
template <class T> S2HD s2vec<T, 4> s2mk(T a, T b, T c, T d) { s2vec<T, 4> r; r.x = a; r.y = b; r.z = c; r.w = d; return r; }
template <class T, int N> S2HD s2vec<T, N> s2splat(T a) { s2vec<T, N> r; for (int i = 0; i < N; ++i) r[i] = a; return r; }

// Swizzle read: s2sw<0, 2, 1>(v) is v.xzy.
template <int A, int B, class T, int N> S2HD s2vec<T, 2> s2sw(const s2vec<T, N> &v) { return s2mk(v[A], v[B]); }
template <int A, int B, int C, class T, int N> S2HD s2vec<T, 3> s2sw(const s2vec<T, N> &v) { return s2mk(v[A], v[B], v[C]); }
template <int A, int B, int C, int D, class T, int N> S2HD s2vec<T, 4> s2sw(const s2vec<T, N> &v) { return s2mk(v[A], v[B], v[C], v[D]); }

// Component-wise operators.
#define S2_VV_OP(op)                                                                         \
  template <class T, int N> S2HD s2vec<T, N> operator op(const s2vec<T, N> &a, const s2vec<T, N> &b) { \
    s2vec<T, N> r; for (int i = 0; i < N; ++i) r[i] = a[i] op b[i]; return r; }              \
  template <class T, int N> S2HD s2vec<T, N> operator op(const s2vec<T, N> &a, T b) {        \
    s2vec<T, N> r; for (int i = 0; i < N; ++i) r[i] = a[i] op b; return r; }                 \
  template <class T, int N> S2HD s2vec<T, N> operator op(T a, const s2vec<T, N> &b) {        \
    s2vec<T, N> r; for (int i = 0; i < N; ++i) r[i] = a op b[i]; return r; }                 \
  template <class T, int N> S2HD s2vec<T, N> &operator op##=(s2vec<T, N> &a, const s2vec<T, N> &b) { \
    for (int i = 0; i < N; ++i) a[i] = a[i] op b[i]; return a; }                             \
  template <class T, int N> S2HD s2vec<T, N> &operator op##=(s2vec<T, N> &a, T b) {          \
    for (int i = 0; i < N; ++i) a[i] = a[i] op b; return a; }
S2_VV_OP(+)
S2_VV_OP(-)
S2_VV_OP(*)
S2_VV_OP(/)
#undef S2_VV_OP

template <class T, int N> S2HD s2vec<T, N> operator-(const s2vec<T, N> &a) {
  s2vec<T, N> r; for (int i = 0; i < N; ++i) r[i] = -a[i]; return r;
}

#define S2_CMP_OP(name, op)                                                                     \
  template <class T, int N> S2HD s2vec<bool, N> name(const s2vec<T, N> &a, const s2vec<T, N> &b) { \
    s2vec<bool, N> r; for (int i = 0; i < N; ++i) r[i] = a[i] op b[i]; return r; }
S2_CMP_OP(s2_lt, <)
S2_CMP_OP(s2_le, <=)
S2_CMP_OP(s2_gt, >)
S2_CMP_OP(s2_ge, >=)
S2_CMP_OP(s2_eq, ==)
S2_CMP_OP(s2_ne, !=)
#undef S2_CMP_OP
S2HD bool s2_lt(float a, float b) { return a < b; }
S2HD bool s2_le(float a, float b) { return a <= b; }
S2HD bool s2_gt(float a, float b) { return a > b; }
S2HD bool s2_ge(float a, float b) { return a >= b; }
S2HD bool s2_eq(float a, float b) { return a == b; }
S2HD bool s2_ne(float a, float b) { return a != b; }
S2HD bool s2_lt(int a, int b) { return a < b; }
S2HD bool s2_le(int a, int b) { return a <= b; }
S2HD bool s2_gt(int a, int b) { return a > b; }
S2HD bool s2_ge(int a, int b) { return a >= b; }
S2HD bool s2_eq(int a, int b) { return a == b; }
S2HD bool s2_ne(int a, int b) { return a != b; }
S2HD bool s2_lt(unsigned a, unsigned b) { return a < b; }
S2HD bool s2_le(unsigned a, unsigned b) { return a <= b; }
S2HD bool s2_gt(unsigned a, unsigned b) { return a > b; }
S2HD bool s2_ge(unsigned a, unsigned b) { return a >= b; }
S2HD bool s2_eq(unsigned a, unsigned b) { return a == b; }
S2HD bool s2_ne(unsigned a, unsigned b) { return a != b; }
S2HD bool s2_eq(bool a, bool b) { return a == b; }
S2HD bool s2_ne(bool a, bool b) { return a != b; }

template <int N> S2HD bool s2_all(const s2vec<bool, N> &v) { bool r = true; for (int i = 0; i < N; ++i) r = r && v[i]; return r; }
template <int N> S2HD bool s2_any(const s2vec<bool, N> &v) { bool r = false; for (int i = 0; i < N; ++i) r = r || v[i]; return r; }
S2HD bool s2_all(bool v) { return v; }
S2HD bool s2_any(bool v) { return v; }

// Conversions between element types (WGSL vec3<f32>(vec3<i32>), GLSL vec3(ivec3)).
template <class U, class T, int N> S2HD s2vec<U, N> s2cvt(const s2vec<T, N> &v) {
  s2vec<U, N> r; for (int i = 0; i < N; ++i) r[i] = U(v[i]); return r;
}

// Matrices: C columns of R-component float vectors (WGSL matCxR, GLSL matC / matCxR).
template <int C, int R> struct s2mat {
  s2vec<float, R> c[C];
  S2HD s2vec<float, R> &operator[](int i) { return c[i]; }
  S2HD const s2vec<float, R> &operator[](int i) const { return c[i]; }
};
template <int C, int R> S2HD s2vec<float, R> operator*(const s2mat<C, R> &m, const s2vec<float, C> &v) {
  s2vec<float, R> r;
  for (int j = 0; j < R; ++j) {
    float s = m.c[0][j] * v[0];
    for (int i = 1; i < C; ++i) s = s + m.c[i][j] * v[i];
    r[j] = s;
  }
  return r;
}
template <int C, int R> S2HD s2vec<float, C> operator*(const s2vec<float, R> &v, const s2mat<C, R> &m) {
  s2vec<float, C> r;
  for (int i = 0; i < C; ++i) {
    float s = v[0] * m.c[i][0];
    for (int j = 1; j < R; ++j) s = s + v[j] * m.c[i][j];
    r[i] = s;
  }
  return r;
}
template <int K, int C, int R> S2HD s2mat<C, R> operator*(const s2mat<K, R> &a, const s2mat<C, K> &b) {
  s2mat<C, R> r;
  for (int i = 0; i < C; ++i) r.c[i] = a * b.c[i];
  return r;
}
template <int C, int R> S2HD s2mat<C, R> operator*(const s2mat<C, R> &a, float s) {
  s2mat<C, R> r; for (int i = 0; i < C; ++i) r.c[i] = a.c[i] * s; return r;
}
template <int C, int R> S2HD s2mat<C, R> operator*(float s, const s2mat<C, R> &a) {
  s2mat<C, R> r; for (int i = 0; i < C; ++i) r.c[i] = s * a.c[i]; return r;
}
template <int C, int R> S2HD s2mat<C, R> operator+(const s2mat<C, R> &a, const s2mat<C, R> &b) {
  s2mat<C, R> r; for (int i = 0; i < C; ++i) r.c[i] = a.c[i] + b.c[i]; return r;
}
template <int C, int R> S2HD s2mat<C, R> operator-(const s2mat<C, R> &a, const s2mat<C, R> &b) {
  s2mat<C, R> r; for (int i = 0; i < C; ++i) r.c[i] = a.c[i] - b.c[i]; return r;
}
template <int C, int R> S2HD s2mat<C, R> operator-(const s2mat<C, R> &a) {
  s2mat<C, R> r; for (int i = 0; i < C; ++i) r.c[i] = -a.c[i]; return r;
}
template <int C> S2HD s2vec<float, C> &operator*=(s2vec<float, C> &v, const s2mat<C, C> &m) { v = v * m; return v; }
template <int C> S2HD s2mat<C, C> &operator*=(s2mat<C, C> &a, const s2mat<C, C> &b) { a = a * b; return a; }
template <int C, int R> S2HD s2mat<R, C> s2_transpose(const s2mat<C, R> &m) {
  s2mat<R, C> r;
  for (int i = 0; i < C; ++i) for (int j = 0; j < R; ++j) r.c[j][i] = m.c[i][j];
  return r;
}
// Matrix from column-major scalars / columns; diagonal from a scalar (GLSL mat2(s)).
template <int C, int R> S2HD s2mat<C, R> s2mat_diag(float s) {
  s2mat<C, R> r;
  for (int i = 0; i < C; ++i) for (int j = 0; j < R; ++j) r.c[i][j] = (i == j) ? s : 0.0f;
  return r;
}
S2HD s2mat<2, 2> s2mat22(float a, float b, float c, float d) { s2mat<2, 2> m; m.c[0] = s2mk(a, b); m.c[1] = s2mk(c, d); return m; }
S2HD s2mat<2, 2> s2mat22(s2v2 a, s2v2 b) { s2mat<2, 2> m; m.c[0] = a; m.c[1] = b; return m; }
S2HD s2mat<3, 3> s2mat33(float a, float b, float c, float d, float e, float f, float g, float h, float i) {
  s2mat<3, 3> m; m.c[0] = s2mk(a, b, c); m.c[1] = s2mk(d, e, f); m.c[2] = s2mk(g, h, i); return m;
}
S2HD s2mat<3, 3> s2mat33(s2v3 a, s2v3 b, s2v3 c) { s2mat<3, 3> m; m.c[0] = a; m.c[1] = b; m.c[2] = c; return m; }

// ---------------------------------------------------------------------------
// Scalar builtins (binary32).
S2HD float s2_abs(float x) { return fabsf(x); }
S2HD int s2_abs(int x) { return x < 0 ? -x : x; }
S2HD unsigned s2_abs(unsigned x) { return x; }
S2HD float s2_sign(float x) { return x > 0.0f ? 1.0f : (x < 0.0f ? -1.0f : 0.0f); }
S2HD int s2_sign(int x) { return x > 0 ? 1 : (x < 0 ? -1 : 0); }
S2HD float s2_floor(float x) { return floorf(x); }
S2HD float s2_ceil(float x) { return ceilf(x); }
S2HD float s2_trunc(float x) { return truncf(x); }
S2HD float s2_round(float x) { return rintf(x); }
S2HD float s2_fract(float x) { return x - floorf(x); }
S2HD float s2_sqrt(float x) { return sqrtf(x); }
S2HD float s2_inversesqrt(float x) { return 1.0f / sqrtf(x); }
S2HD float s2_exp(float x) { return expf(x); }
S2HD float s2_exp2(float x) { return exp2f(x); }
S2HD float s2_log(float x) { return logf(x); }
S2HD float s2_log2(float x) { return log2f(x); }
S2HD float s2_pow(float x, float y) { return powf(x, y); }
S2HD float s2_sin(float x) { return sinf(x); }
S2HD float s2_cos(float x) { return cosf(x); }
S2HD float s2_tan(float x) { return tanf(x); }
S2HD float s2_asin(float x) { return asinf(x); }
S2HD float s2_acos(float x) { return acosf(x); }
S2HD float s2_atan(float x) { return atanf(x); }
S2HD float s2_atan2(float y, float x) { return atan2f(y, x); }
S2HD float s2_sinh(float x) { return sinhf(x); }
S2HD float s2_cosh(float x) { return coshf(x); }
S2HD float s2_tanh(float x) { return tanhf(x); }
S2HD float s2_min(float a, float b) { return fminf(a, b); }
S2HD float s2_max(float a, float b) { return fmaxf(a, b); }
S2HD int s2_min(int a, int b) { return a < b ? a : b; }
S2HD int s2_max(int a, int b) { return a > b ? a : b; }
S2HD unsigned s2_min(unsigned a, unsigned b) { return a < b ? a : b; }
S2HD unsigned s2_max(unsigned a, unsigned b) { return a > b ? a : b; }
S2HD float s2_clamp(float e, float lo, float hi) { return fminf(fmaxf(e, lo), hi); }
// x + (+0): -0 becomes +0, every other value is unchanged (the pruned code's
// result of a decided smooth operator).
S2HD float s2_canon(float x) {
#ifdef __CUDA_ARCH__
  return __fadd_rn(x, 0.0f);
#else
  return x + 0.0f;
#endif
}
S2HD int s2_clamp(int e, int lo, int hi) { return s2_min(s2_max(e, lo), hi); }
S2HD unsigned s2_clamp(unsigned e, unsigned lo, unsigned hi) { return s2_min(s2_max(e, lo), hi); }
S2HD float s2_saturate(float e) { return fminf(fmaxf(e, 0.0f), 1.0f); }
S2HD float s2_mix(float a, float b, float t) { return a * (1.0f - t) + b * t; }
S2HD float s2_step(float edge, float x) { return edge <= x ? 1.0f : 0.0f; }
S2HD float s2_smoothstep(float lo, float hi, float x) {
  float t = s2_clamp((x - lo) / (hi - lo), 0.0f, 1.0f);
  return t * t * (3.0f - 2.0f * t);
}
S2HD float s2_fmod_glsl(float x, float y) { return x - y * floorf(x / y); }
S2HD float s2_fmod_wgsl(float x, float y) { return x - y * truncf(x / y); }
S2HD int s2_imod(int x, int y) { return y == 0 ? 0 : x % y; }
S2HD unsigned s2_imod(unsigned x, unsigned y) { return y == 0 ? 0u : x % y; }
S2HD float s2_fma(float a, float b, float c) { return fmaf(a, b, c); }
S2HD float s2_radians(float x) { return x * 0.017453292519943295f; }
S2HD float s2_degrees(float x) { return x * 57.29577951308232f; }
S2HD float s2_length(float x) { return fabsf(x); }
S2HD float s2_distance(float a, float b) { return fabsf(a - b); }
S2HD float s2_dot(float a, float b) { return a * b; }

// Component-wise vector variants of the scalar builtins.
#define S2_VEC1(name)                                                                     \
  template <class T, int N> S2HD s2vec<T, N> name(const s2vec<T, N> &a) {                 \
    s2vec<T, N> r; for (int i = 0; i < N; ++i) r[i] = name(a[i]); return r; }
#define S2_VEC2(name)                                                                     \
  template <class T, int N> S2HD s2vec<T, N> name(const s2vec<T, N> &a, const s2vec<T, N> &b) { \
    s2vec<T, N> r; for (int i = 0; i < N; ++i) r[i] = name(a[i], b[i]); return r; }      \
  template <class T, int N> S2HD s2vec<T, N> name(const s2vec<T, N> &a, T b) {            \
    s2vec<T, N> r; for (int i = 0; i < N; ++i) r[i] = name(a[i], b); return r; }
#define S2_VEC3(name)                                                                     \
  template <class T, int N> S2HD s2vec<T, N> name(const s2vec<T, N> &a, const s2vec<T, N> &b, const s2vec<T, N> &c) { \
    s2vec<T, N> r; for (int i = 0; i < N; ++i) r[i] = name(a[i], b[i], c[i]); return r; } \
  template <class T, int N> S2HD s2vec<T, N> name(const s2vec<T, N> &a, T b, T c) {       \
    s2vec<T, N> r; for (int i = 0; i < N; ++i) r[i] = name(a[i], b, c); return r; }
S2_VEC1(s2_abs) S2_VEC1(s2_sign) S2_VEC1(s2_floor) S2_VEC1(s2_ceil) S2_VEC1(s2_trunc)
S2_VEC1(s2_round) S2_VEC1(s2_fract) S2_VEC1(s2_sqrt) S2_VEC1(s2_inversesqrt) S2_VEC1(s2_exp)
S2_VEC1(s2_exp2) S2_VEC1(s2_log) S2_VEC1(s2_log2) S2_VEC1(s2_sin) S2_VEC1(s2_cos) S2_VEC1(s2_tan)
S2_VEC1(s2_asin) S2_VEC1(s2_acos) S2_VEC1(s2_atan) S2_VEC1(s2_sinh) S2_VEC1(s2_cosh)
S2_VEC1(s2_tanh) S2_VEC1(s2_saturate) S2_VEC1(s2_radians) S2_VEC1(s2_degrees)
S2_VEC2(s2_pow) S2_VEC2(s2_atan2) S2_VEC2(s2_min) S2_VEC2(s2_max) S2_VEC2(s2_fmod_glsl)
S2_VEC2(s2_fmod_wgsl) S2_VEC2(s2_imod)
S2_VEC3(s2_clamp) S2_VEC3(s2_fma) S2_VEC3(s2_mix)

// The sdf::op smooth operators, operation for operation as their WGSL text
// (0.5 * (b - a) / k is (0.5 * (b - a)) / k; k * h * (1 - h) is (k * h) * (1 - h)).
S2HD float s2_op_smooth_union(float a, float b, float k) {
  const float h = s2_clamp(0.5f + 0.5f * (b - a) / k, 0.0f, 1.0f);
  return s2_mix(b, a, h) - k * h * (1.0f - h);
}
S2HD float s2_op_smooth_intersection(float a, float b, float k) {
  const float h = s2_clamp(0.5f - 0.5f * (b - a) / k, 0.0f, 1.0f);
  return s2_mix(b, a, h) + k * h * (1.0f - h);
}
S2HD float s2_op_smooth_subtraction(float a, float b, float k) {
  const float h = s2_clamp(0.5f - 0.5f * (b + a) / k, 0.0f, 1.0f);
  return s2_mix(b, -a, h) + k * h * (1.0f - h);
}
// Out-of-line copies for the pruned code: one body each instead of one per
// combinator keeps its code (and instruction-cache footprint) small.
S2M_PRUNED_FN float s2_op_smooth_union_call(float a, float b, float k) { return s2_op_smooth_union(a, b, k); }
S2M_PRUNED_FN float s2_op_smooth_intersection_call(float a, float b, float k) {
  return s2_op_smooth_intersection(a, b, k);
}
S2M_PRUNED_FN float s2_op_smooth_subtraction_call(float a, float b, float k) {
  return s2_op_smooth_subtraction(a, b, k);
}

// ---------------------------------------------------------------------------
// Intervals for tile pruning.  [lo, hi] bounds the binary32 value that the
// point code computes for every point of a tile: each operation below applies
// the point code's own round-to-nearest operation to the endpoints (or, for
// products and quotients, to the four corners), which is sound because the
// exact operation is monotone in each argument there and rounding is
// monotone.  An interval with a NaN endpoint is unknown: every comparison on
// it is false, so no decision rests on it.  Results with an infinite
// endpoint become unknown as well, so a known interval always bounds finite
// values.  The larger helpers are out of line on the device (S2I_FN): the
// tile function calls them once per node, and inlining them all made its
// compilation slower than the rest of the module together.
struct s2i {
  float lo, hi;
};
// The quiet NaN 0x7fc00000 (device code, host code of nvcc and of a host compiler).
S2HD float s2_qnan() {
#ifdef __CUDA_ARCH__
  return __int_as_float(0x7fc00000u);
#else
  return __builtin_nanf("");
#endif
}
S2HD s2i s2i_unknown() { s2i r; r.lo = r.hi = s2_qnan(); return r; }
S2HD bool s2i_ok(s2i a) { return fabsf(a.lo) <= 3.40282347e38f && fabsf(a.hi) <= 3.40282347e38f; }
S2HD s2i s2i_pt(float v) { s2i r; r.lo = v; r.hi = v; return r; }
S2HD s2i s2i_fin(float lo, float hi) {
  s2i r; r.lo = lo; r.hi = hi;
  return s2i_ok(r) ? r : s2i_unknown();
}
S2HD float s2i_min4(float a, float b, float c, float d) { return fminf(fminf(a, b), fminf(c, d)); }
S2HD float s2i_max4(float a, float b, float c, float d) { return fmaxf(fmaxf(a, b), fmaxf(c, d)); }
S2HD s2i s2i_neg(s2i a) { return s2i_ok(a) ? s2i_fin(-a.hi, -a.lo) : s2i_unknown(); }
S2HD s2i s2i_add(s2i a, s2i b) { return s2i_ok(a) && s2i_ok(b) ? s2i_fin(a.lo + b.lo, a.hi + b.hi) : s2i_unknown(); }
S2HD s2i s2i_sub(s2i a, s2i b) { return s2i_ok(a) && s2i_ok(b) ? s2i_fin(a.lo - b.hi, a.hi - b.lo) : s2i_unknown(); }
S2I_FN s2i s2i_mul(s2i a, s2i b) {
  if (!s2i_ok(a) || !s2i_ok(b)) return s2i_unknown();
  const float p = a.lo * b.lo, q = a.lo * b.hi, r = a.hi * b.lo, s = a.hi * b.hi;
  return s2i_fin(s2i_min4(p, q, r, s), s2i_max4(p, q, r, s));
}
// x * x of one value (both factors equal at every point): never negative.
S2I_FN s2i s2i_sq(s2i a) {
  if (!s2i_ok(a)) return s2i_unknown();
  const float l = a.lo * a.lo, h = a.hi * a.hi;
  if (a.lo >= 0.0f) return s2i_fin(l, h);
  if (a.hi <= 0.0f) return s2i_fin(h, l);
  return s2i_fin(0.0f, fmaxf(l, h));
}
S2I_FN s2i s2i_div(s2i a, s2i b) {
  if (!s2i_ok(a) || !s2i_ok(b) || !(b.lo > 0.0f || b.hi < 0.0f)) return s2i_unknown();
  const float p = a.lo / b.lo, q = a.lo / b.hi, r = a.hi / b.lo, s = a.hi / b.hi;
  return s2i_fin(s2i_min4(p, q, r, s), s2i_max4(p, q, r, s));
}
S2I_FN s2i s2i_abs(s2i a) {
  if (!s2i_ok(a)) return s2i_unknown();
  if (a.lo >= 0.0f) return a;
  if (a.hi <= 0.0f) return s2i_fin(-a.hi, -a.lo);
  return s2i_fin(0.0f, fmaxf(-a.lo, a.hi));
}
S2HD s2i s2i_floor(s2i a) { return s2i_ok(a) ? s2i_fin(floorf(a.lo), floorf(a.hi)) : s2i_unknown(); }
S2HD s2i s2i_ceil(s2i a) { return s2i_ok(a) ? s2i_fin(ceilf(a.lo), ceilf(a.hi)) : s2i_unknown(); }
S2I_FN s2i s2i_sqrt(s2i a) {
  return s2i_ok(a) && a.lo >= 0.0f ? s2i_fin(sqrtf(a.lo), sqrtf(a.hi)) : s2i_unknown();
}
S2HD s2i s2i_min(s2i a, s2i b) {
  return s2i_ok(a) && s2i_ok(b) ? s2i_fin(fminf(a.lo, b.lo), fminf(a.hi, b.hi)) : s2i_unknown();
}
S2HD s2i s2i_max(s2i a, s2i b) {
  return s2i_ok(a) && s2i_ok(b) ? s2i_fin(fmaxf(a.lo, b.lo), fmaxf(a.hi, b.hi)) : s2i_unknown();
}
S2I_FN s2i s2i_clamp(s2i e, s2i lo, s2i hi) { return s2i_min(s2i_max(e, lo), hi); }
S2I_FN s2i s2i_mix(s2i a, s2i b, s2i t) { return s2i_add(s2i_mul(a, s2i_sub(s2i_pt(1.0f), t)), s2i_mul(b, t)); }
// sin / cos of a finite argument: within [-1, 1] (with a margin for the
// implementation's rounding).  atan2: within [-pi, pi], likewise.
S2HD s2i s2i_unit(s2i a) { return s2i_ok(a) ? s2i_fin(-1.0009765625f, 1.0009765625f) : s2i_unknown(); }
S2HD s2i s2i_angle(s2i a, s2i b) {
  return s2i_ok(a) && s2i_ok(b) ? s2i_fin(-3.1416015625f, 3.1416015625f) : s2i_unknown();
}

// Combinators.  *d = 1 when the result is operand a (for the smooth
// subtraction: -a) bit for bit at every point, 2 when it is operand b, 0
// otherwise; the interval returned bounds the result.
//   min / max: strictly separated operands.
//   smooth operators: the blend weight h clamps to exactly 1 (or +0) at every
//   point, k > 0, and no operand can be a zero whose sign the blend
//   arithmetic would change (mix adds b * (+0) or a * (+0), and the k term
//   adds or subtracts +0).
S2I_FN s2i s2i_min_sel(s2i a, s2i b, int *d) {
  if (d) *d = 0;
  if (!s2i_ok(a) || !s2i_ok(b)) return s2i_unknown();
  if (a.hi < b.lo) { if (d) *d = 1; return a; }
  if (b.hi < a.lo) { if (d) *d = 2; return b; }
  return s2i_min(a, b);
}
S2I_FN s2i s2i_max_sel(s2i a, s2i b, int *d) {
  if (d) *d = 0;
  if (!s2i_ok(a) || !s2i_ok(b)) return s2i_unknown();
  if (a.lo > b.hi) { if (d) *d = 1; return a; }
  if (b.lo > a.hi) { if (d) *d = 2; return b; }
  return s2i_max(a, b);
}
S2HD bool s2i_nonzero(s2i a) { return a.lo > 0.0f || a.hi < 0.0f; }
// Smooth operators keeping both operands.  r(h) = b (1 - h) + a h -/+
// k h (1 - h) is quadratic in the blend weight h, with its extremum at the
// unclamped weight h* = 0.5 +/- (b - a) / 2k.  The computed h is within a few
// ulps of clamp(h*), which moves r by k (h - h*)^2, and the binary32
// evaluation adds at most a few ulps of |a| + |b| + k: `slack` covers both
// with a wide margin.
S2HD float s2i_mag(s2i a) { return fmaxf(fabsf(a.lo), fabsf(a.hi)); }
S2HD float s2i_slack(s2i a, s2i b, s2i k) { return (s2i_mag(a) + s2i_mag(b) + k.hi) * 0x1p-20f; }
// Bounds of the smooth minimum and maximum where neither operand is proven
// to win.  With d = |a - b| / k, smin(a, b) = min(a, b) - k/4 (1 - d)^2 for
// d < 1 and min(a, b) beyond: non-decreasing in a and in b (its partial
// derivatives are h and 1 - h) and non-increasing in k; smax(a, b) =
// -smin(-a, -b) likewise in a and b, non-decreasing in k.  So the exact
// range over the box of the operands is the formula at its corners.  The
// binary32 formula (8 operations) is within E = 2^-20 (|a| + |b| + k) of the
// exact one, so a corner value moved outward by 2 E bounds the binary32
// value at every point of the box.  (A single bound of -k/4 below min(a, b)
// lets the error grow by k/4 per link of a long chain of smooth unions.)
S2HD s2i s2i_smooth_min_bound(s2i a, s2i b, s2i k) {
  const float e = 2.0f * s2i_slack(a, b, k);
  return s2i_fin(s2_op_smooth_union(a.lo, b.lo, k.hi) - e, s2_op_smooth_union(a.hi, b.hi, k.lo) + e);
}
S2HD s2i s2i_smooth_max_bound(s2i a, s2i b, s2i k) {
  const float e = 2.0f * s2i_slack(a, b, k);
  return s2i_fin(s2_op_smooth_intersection(a.lo, b.lo, k.lo) - e, s2_op_smooth_intersection(a.hi, b.hi, k.hi) + e);
}
// A decided smooth operator returns its kept operand through s2_canon (x +
// +0: -0 becomes +0, every other value is unchanged), which reproduces the
// operator's arithmetic at h = 1 or h = +0 bit for bit where the conditions
// below hold.  (b * (+0) is +0 for b > 0; the terms k h (1 - h) are +0.)
//   union         h = 1: (b * (+0) + a) - (+0)    = s2_canon(a) if a != 0 or b > 0
//                 h = 0: (b + a * (+0)) - (+0)    = s2_canon(b) if b != 0 or a > 0
//   intersection  h = 1: (b * (+0) + a) + (+0)    = s2_canon(a)
//                 h = 0: (b + a * (+0)) + (+0)    = s2_canon(b)
//   subtraction   h = 1: (b * (+0) + (-a)) + (+0) = s2_canon(-a)
//                 h = 0: (b + (-a) * (+0)) + (+0) = s2_canon(b)
// (Operands are finite: intervals with a non-finite end are unknown.)
S2I_FN s2i s2i_smooth_union_sel(s2i a, s2i b, s2i k, int *d) {
  if (d) *d = 0;
  const s2i t = s2i_add(s2i_pt(0.5f), s2i_div(s2i_mul(s2i_pt(0.5f), s2i_sub(b, a)), k));
  if (s2i_ok(t) && k.lo > 0.0f) {
    if (t.lo >= 1.0f && (s2i_nonzero(a) || b.lo > 0.0f)) { if (d) *d = 1; return a; }
    if (t.hi < 0.0f && (s2i_nonzero(b) || a.lo > 0.0f)) { if (d) *d = 2; return b; }
  }
  if (!s2i_ok(a) || !s2i_ok(b) || !s2i_ok(k) || !(k.lo > 0.0f)) return s2i_unknown();
  return s2i_smooth_min_bound(a, b, k);
}
S2I_FN s2i s2i_smooth_intersection_sel(s2i a, s2i b, s2i k, int *d) {
  if (d) *d = 0;
  const s2i t = s2i_sub(s2i_pt(0.5f), s2i_div(s2i_mul(s2i_pt(0.5f), s2i_sub(b, a)), k));
  if (s2i_ok(t) && k.lo > 0.0f) {
    if (t.lo >= 1.0f) { if (d) *d = 1; return a; }
    if (t.hi < 0.0f) { if (d) *d = 2; return b; }
  }
  if (!s2i_ok(a) || !s2i_ok(b) || !s2i_ok(k) || !(k.lo > 0.0f)) return s2i_unknown();
  return s2i_smooth_max_bound(a, b, k);
}
S2I_FN s2i s2i_smooth_subtraction_sel(s2i a, s2i b, s2i k, int *d) {
  if (d) *d = 0;
  const s2i t = s2i_sub(s2i_pt(0.5f), s2i_div(s2i_mul(s2i_pt(0.5f), s2i_add(b, a)), k));
  if (s2i_ok(t) && k.lo > 0.0f) {
    if (t.lo >= 1.0f) { if (d) *d = 1; return s2i_neg(a); }
    if (t.hi < 0.0f) { if (d) *d = 2; return b; }
  }
  if (!s2i_ok(a) || !s2i_ok(b) || !s2i_ok(k) || !(k.lo > 0.0f)) return s2i_unknown();
  return s2i_smooth_max_bound(s2i_neg(a), b, k);
}
#undef S2_VEC1
#undef S2_VEC2
#undef S2_VEC3
// mix(vec, vec, scalar), step(scalar, vec), step(vec, vec), smoothstep variants.
template <int N> S2HD s2vec<float, N> s2_mix(const s2vec<float, N> &a, const s2vec<float, N> &b, float t) {
  s2vec<float, N> r; for (int i = 0; i < N; ++i) r[i] = s2_mix(a[i], b[i], t); return r;
}
template <int N> S2HD s2vec<float, N> s2_step(const s2vec<float, N> &e, const s2vec<float, N> &x) {
  s2vec<float, N> r; for (int i = 0; i < N; ++i) r[i] = s2_step(e[i], x[i]); return r;
}
template <int N> S2HD s2vec<float, N> s2_step(float e, const s2vec<float, N> &x) {
  s2vec<float, N> r; for (int i = 0; i < N; ++i) r[i] = s2_step(e, x[i]); return r;
}
template <int N> S2HD s2vec<float, N> s2_smoothstep(const s2vec<float, N> &lo, const s2vec<float, N> &hi, const s2vec<float, N> &x) {
  s2vec<float, N> r; for (int i = 0; i < N; ++i) r[i] = s2_smoothstep(lo[i], hi[i], x[i]); return r;
}
template <int N> S2HD s2vec<float, N> s2_smoothstep(float lo, float hi, const s2vec<float, N> &x) {
  s2vec<float, N> r; for (int i = 0; i < N; ++i) r[i] = s2_smoothstep(lo, hi, x[i]); return r;
}
template <class T, int N> S2HD s2vec<T, N> s2_select(const s2vec<T, N> &f, const s2vec<T, N> &t, const s2vec<bool, N> &c) {
  s2vec<T, N> r; for (int i = 0; i < N; ++i) r[i] = c[i] ? t[i] : f[i]; return r;
}
template <class T, int N> S2HD s2vec<T, N> s2_select(const s2vec<T, N> &f, const s2vec<T, N> &t, bool c) { return c ? t : f; }
template <class T> S2HD T s2_select(T f, T t, bool c) { return c ? t : f; }

// Geometric builtins.
template <int N> S2HD float s2_dot(const s2vec<float, N> &a, const s2vec<float, N> &b) {
  float s = a[0] * b[0];
  for (int i = 1; i < N; ++i) s = s + a[i] * b[i];
  return s;
}
template <int N> S2HD int s2_dot(const s2vec<int, N> &a, const s2vec<int, N> &b) {
  int s = a[0] * b[0];
  for (int i = 1; i < N; ++i) s = s + a[i] * b[i];
  return s;
}
template <int N> S2HD float s2_length(const s2vec<float, N> &a) { return sqrtf(s2_dot(a, a)); }
template <int N> S2HD float s2_distance(const s2vec<float, N> &a, const s2vec<float, N> &b) { return s2_length(a - b); }
template <int N> S2HD s2vec<float, N> s2_normalize(const s2vec<float, N> &a) {
  float l = s2_length(a);
  s2vec<float, N> r; for (int i = 0; i < N; ++i) r[i] = a[i] / l; return r;
}
S2HD float s2_normalize(float a) { return a / fabsf(a); }
S2HD s2v3 s2_cross(const s2v3 &a, const s2v3 &b) {
  return s2mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
template <int N> S2HD s2vec<float, N> s2_reflect(const s2vec<float, N> &e1, const s2vec<float, N> &e2) {
  return e1 - 2.0f * s2_dot(e2, e1) * e2;
}

// ---------------------------------------------------------------------------
// Runs of 4 points sharing x and y (s2m_user_sdf_run4): s2x4 holds the 4
// lanes of a value that depends on z; values that do not are plain floats.
// Every operation is the scalar one applied lane by lane.
struct s2x4 {
  float v[4];
};
S2HD s2x4 s2x4_splat(float a) { s2x4 r; for (int i = 0; i < 4; ++i) r.v[i] = a; return r; }
S2HD float s2_lane(float a, int) { return a; }
S2HD float s2_lane(const s2x4 &a, int i) { return a.v[i]; }
#define S2_X4_OP(op)                                                                       \
  S2HD s2x4 operator op(const s2x4 &a, const s2x4 &b) { s2x4 r; for (int i = 0; i < 4; ++i) r.v[i] = a.v[i] op b.v[i]; return r; } \
  S2HD s2x4 operator op(const s2x4 &a, float b) { s2x4 r; for (int i = 0; i < 4; ++i) r.v[i] = a.v[i] op b; return r; } \
  S2HD s2x4 operator op(float a, const s2x4 &b) { s2x4 r; for (int i = 0; i < 4; ++i) r.v[i] = a op b.v[i]; return r; }
S2_X4_OP(+)
S2_X4_OP(-)
S2_X4_OP(*)
S2_X4_OP(/)
#undef S2_X4_OP
S2HD s2x4 operator-(const s2x4 &a) { s2x4 r; for (int i = 0; i < 4; ++i) r.v[i] = -a.v[i]; return r; }
S2HD s2x4 s2_canon(const s2x4 &a) { s2x4 r; for (int i = 0; i < 4; ++i) r.v[i] = s2_canon(a.v[i]); return r; }
#define S2_X4_F1(name) \
  template <class A> S2HD s2x4 s2r_##name(const A &a) { s2x4 r; for (int i = 0; i < 4; ++i) r.v[i] = s2_##name(s2_lane(a, i)); return r; }
#define S2_X4_F2(name)                                                                       \
  template <class A, class B> S2HD s2x4 s2r_##name(const A &a, const B &b) {                 \
    s2x4 r; for (int i = 0; i < 4; ++i) r.v[i] = s2_##name(s2_lane(a, i), s2_lane(b, i)); return r; }
#define S2_X4_F3(name)                                                                       \
  template <class A, class B, class C> S2HD s2x4 s2r_##name(const A &a, const B &b, const C &c) { \
    s2x4 r; for (int i = 0; i < 4; ++i) r.v[i] = s2_##name(s2_lane(a, i), s2_lane(b, i), s2_lane(c, i)); return r; }
S2_X4_F1(abs) S2_X4_F1(floor) S2_X4_F1(ceil) S2_X4_F1(sqrt) S2_X4_F1(saturate) S2_X4_F1(sin) S2_X4_F1(cos)
S2_X4_F1(exp) S2_X4_F1(log)
S2_X4_F2(min) S2_X4_F2(max) S2_X4_F2(pow) S2_X4_F2(atan2)
S2_X4_F3(clamp) S2_X4_F3(mix) S2_X4_F3(op_smooth_union) S2_X4_F3(op_smooth_intersection)
S2_X4_F3(op_smooth_subtraction)
// Out-of-line run forms of the smooth operators for the pruned code.
S2M_PRUNED_FN s2x4 s2r_op_smooth_union_call(s2x4 a, s2x4 b, s2x4 k) { return s2r_op_smooth_union(a, b, k); }
S2M_PRUNED_FN s2x4 s2r_op_smooth_intersection_call(s2x4 a, s2x4 b, s2x4 k) {
  return s2r_op_smooth_intersection(a, b, k);
}
S2M_PRUNED_FN s2x4 s2r_op_smooth_subtraction_call(s2x4 a, s2x4 b, s2x4 k) {
  return s2r_op_smooth_subtraction(a, b, k);
}
#undef S2_X4_F1
#undef S2_X4_F2
#undef S2_X4_F3
