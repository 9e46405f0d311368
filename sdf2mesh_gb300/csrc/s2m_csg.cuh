// s2m_csg.cuh -- CSG programs of the batch engine: the point interpreter, its
// tile-pruned form, and the interval pass that prunes it.
//
// A program is a postfix list of floats (opcodes S2M_CSG_* of
// include/sdf2mesh.h, each followed by its operands).  The arithmetic of each
// opcode is that of the library function it names
// (src/sdf3d_primitives.wgsl:7-36, src/sdf_op.wgsl:7-23), operation for
// operation, so a program and the equivalent .sdf3d source give the same bits.
//
// Tile pruning, as for compiled SDFs: per tile of lattice points an interval
// pass over the program decides, for each min / max / smooth operator,
// whether one operand gives the result bit for bit at every point of the
// tile, and records a 2-bit code per program node (node n = the n-th opcode):
//   0  skipped: the node's value is not needed;
//   1  evaluated;
//   2  a combinator whose result is its first operand (the second operand's
//      nodes are skipped), returned as the interval rules prescribe
//      (unchanged for min / max, s2_canon for the smooth operators, negated
//      for the smooth subtraction);
//   3  the same with the second operand (negated for max(a, -b)).
// The decisions are the interval library's (s2m_prelude.cuh: s2i_*_sel),
// whose soundness arguments hold for this interpreter because each interval
// operation applies the same round-to-nearest operation the point code does.
//
// The same header compiles for the host (tests), where the operations are
// plain binary32 arithmetic built without contraction.
#pragma once
#include "../../include/sdf2mesh.h"
#include "s2m_prelude.cuh"

#define S2_CSG_STACK 32
#define S2_CSG_MAX_NODES 256                     // nodes a tile record can prune
#define S2_CSG_CODE_WORDS (S2_CSG_MAX_NODES / 16)  // 2 bits per node
#define S2_CSG_TILE_WORDS (1 + S2_CSG_CODE_WORDS)  // flag word, then the codes

#if defined(__CUDACC__)
#define S2C_FN __host__ __device__ __forceinline__
#define S2C_TILE_FN __host__ __device__ __noinline__
#else
#define S2C_FN inline
#define S2C_TILE_FN inline
#endif
#ifdef __CUDA_ARCH__
#define S2C_RN(dev, host) return dev
#else
#define S2C_RN(dev, host) return host
#endif
// Round-to-nearest binary32 operations that never contract into an FMA.
S2C_FN float s2c_add(float a, float b) { S2C_RN(__fadd_rn(a, b), a + b); }
S2C_FN float s2c_sub(float a, float b) { S2C_RN(__fsub_rn(a, b), a - b); }
S2C_FN float s2c_mul(float a, float b) { S2C_RN(__fmul_rn(a, b), a * b); }
S2C_FN float s2c_div(float a, float b) { S2C_RN(__fdiv_rn(a, b), a / b); }
S2C_FN float s2c_sqrt(float a) { S2C_RN(__fsqrt_rn(a), sqrtf(a)); }
S2C_FN float s2c_ld(const float *p) { S2C_RN(__ldg(p), *p); }
#undef S2C_RN

// Operands of an opcode (-1: unknown opcode).
S2HD int s2c_operands(int op) {
  switch (op) {
    case S2M_CSG_SPHERE: return 4;
    case S2M_CSG_BOX: return 6;
    case S2M_CSG_TORUS: return 5;
    case S2M_CSG_CAPSULE: return 7;
    case S2M_CSG_PLANE: return 4;
    case S2M_CSG_UNION:
    case S2M_CSG_SUBTRACT:
    case S2M_CSG_INTERSECT: return 0;
    case S2M_CSG_SMOOTH_UNION:
    case S2M_CSG_SMOOTH_INTERSECTION:
    case S2M_CSG_SMOOTH_SUBTRACTION: return 1;
  }
  return -1;
}

// Where the pruned interpreter reads a tile's code words: plain loads
// (shared memory, host), or L2 loads of a record that other blocks of the
// same launch wrote.
struct S2CodesPtr {
  const unsigned *p;
  S2C_FN unsigned word(int i) const { return p[i]; }
};
#if defined(__CUDACC__)
struct S2CodesL2 {
  const unsigned *p;
  __device__ __forceinline__ unsigned word(int i) const { return __ldcg(p + i); }
};
#endif

struct S2CsgSdf {
  static constexpr bool kStdNormal = true;
  const float *prog;
  int len;

  S2C_FN static float len3(float x, float y, float z) {
    return s2c_sqrt(s2c_add(s2c_add(s2c_mul(x, x), s2c_mul(y, y)), s2c_mul(z, z)));
  }
  S2C_FN static float len2(float x, float y) { return s2c_sqrt(s2c_add(s2c_mul(x, x), s2c_mul(y, y))); }
  S2C_FN static float clamp01(float v) { return fminf(fmaxf(v, 0.0f), 1.0f); }
  // mix(e1, e2, t) = e1 * (1 - t) + e2 * t
  S2C_FN static float mix(float a, float b, float t) { return s2c_add(s2c_mul(a, s2c_sub(1.0f, t)), s2c_mul(b, t)); }
  // x + (+0): the smooth operators' result when the interval pass kept one operand
  S2C_FN static float canon(float x) { return s2c_add(x, 0.0f); }

  // W points (x, y, z[w]) per decoded opcode, W independent stacks
  // (instruction-level parallelism, one decode for W evaluations).  With
  // `codes` (PRUNED), nodes coded 0 are skipped and combinators coded 2 / 3
  // return their kept operand.
  template <int W, bool PRUNED, class C>
  S2C_FN void run(float x, float y, const float z[W], float out[W], const C &codes) const {
    float st[S2_CSG_STACK][W];
    int sp = 0;
    int i = 0, node = 0;
    unsigned cw = 0x55555555u;  // the code word of nodes node & ~15 ..
    while (i < len) {
      const int op = (int)s2c_ld(prog + i);
      const float *a = prog + i + 1;
      unsigned code = 1u;
      if (PRUNED) {
        if ((node & 15) == 0) cw = node < S2_CSG_MAX_NODES ? codes.word(node >> 4) : 0x55555555u;
        code = (cw >> (2 * (node & 15))) & 3u;
        if (code == 0u) {  // a node of a skipped operand: nothing pushed or popped
          i += 1 + s2c_operands(op);
          ++node;
          continue;
        }
      }
      ++node;
      switch (op) {
        case S2M_CSG_SPHERE: {  // sdf3d_sphere(p - c, r)
          const float cx = s2c_ld(a), cy = s2c_ld(a + 1), cz = s2c_ld(a + 2), r = s2c_ld(a + 3);
          const float dx = s2c_sub(x, cx), dy = s2c_sub(y, cy);
#pragma unroll
          for (int w = 0; w < W; ++w) st[sp][w] = s2c_sub(len3(dx, dy, s2c_sub(z[w], cz)), r);
          ++sp;
          i += 5;
          break;
        }
        case S2M_CSG_BOX: {  // sdf3d_box(p - c, b), b the full size
          const float qx = s2c_sub(fabsf(s2c_sub(x, s2c_ld(a))), s2c_mul(0.5f, s2c_ld(a + 3)));
          const float qy = s2c_sub(fabsf(s2c_sub(y, s2c_ld(a + 1))), s2c_mul(0.5f, s2c_ld(a + 4)));
          const float cz = s2c_ld(a + 2), hz = s2c_mul(0.5f, s2c_ld(a + 5));
#pragma unroll
          for (int w = 0; w < W; ++w) {
            const float qz = s2c_sub(fabsf(s2c_sub(z[w], cz)), hz);
            const float outside = len3(fmaxf(qx, 0.0f), fmaxf(qy, 0.0f), fmaxf(qz, 0.0f));
            st[sp][w] = s2c_add(outside, fminf(fmaxf(qx, fmaxf(qy, qz)), 0.0f));
          }
          ++sp;
          i += 7;
          break;
        }
        case S2M_CSG_TORUS: {  // sdf3d_torus(p - c, vec2(R, r))
          const float dx = s2c_sub(x, s2c_ld(a)), dy = s2c_sub(y, s2c_ld(a + 1)), cz = s2c_ld(a + 2);
          const float R = s2c_ld(a + 3), r = s2c_ld(a + 4);
#pragma unroll
          for (int w = 0; w < W; ++w) {
            const float qx = s2c_sub(len2(dx, s2c_sub(z[w], cz)), R);
            st[sp][w] = s2c_sub(len2(qx, dy), r);
          }
          ++sp;
          i += 6;
          break;
        }
        case S2M_CSG_CAPSULE: {  // sdf3d_capsule(p, a, b, r)
          const float ax = s2c_ld(a), ay = s2c_ld(a + 1), az = s2c_ld(a + 2);
          const float bax = s2c_sub(s2c_ld(a + 3), ax), bay = s2c_sub(s2c_ld(a + 4), ay),
                      baz = s2c_sub(s2c_ld(a + 5), az), r = s2c_ld(a + 6);
          const float pax = s2c_sub(x, ax), pay = s2c_sub(y, ay);
          const float d2 = s2c_add(s2c_add(s2c_mul(bax, bax), s2c_mul(bay, bay)), s2c_mul(baz, baz));
#pragma unroll
          for (int w = 0; w < W; ++w) {
            const float paz = s2c_sub(z[w], az);
            const float d1 = s2c_add(s2c_add(s2c_mul(pax, bax), s2c_mul(pay, bay)), s2c_mul(paz, baz));
            const float h = clamp01(s2c_div(d1, d2));
            st[sp][w] = s2c_sub(len3(s2c_sub(pax, s2c_mul(bax, h)), s2c_sub(pay, s2c_mul(bay, h)),
                                     s2c_sub(paz, s2c_mul(baz, h))),
                                r);
          }
          ++sp;
          i += 8;
          break;
        }
        case S2M_CSG_PLANE: {  // dot(p, n) - d
          const float dxy = s2c_add(s2c_mul(x, s2c_ld(a)), s2c_mul(y, s2c_ld(a + 1)));
          const float nz = s2c_ld(a + 2), d = s2c_ld(a + 3);
#pragma unroll
          for (int w = 0; w < W; ++w) st[sp][w] = s2c_sub(s2c_add(dxy, s2c_mul(z[w], nz)), d);
          ++sp;
          i += 5;
          break;
        }
        case S2M_CSG_UNION:
          if (PRUNED && code != 1u) {  // min: the kept operand as it is
            i += 1;
            break;
          }
          --sp;
#pragma unroll
          for (int w = 0; w < W; ++w) st[sp - 1][w] = fminf(st[sp - 1][w], st[sp][w]);
          i += 1;
          break;
        case S2M_CSG_SUBTRACT:  // max(a, -b)
          if (PRUNED && code != 1u) {
            if (code == 3u)
#pragma unroll
              for (int w = 0; w < W; ++w) st[sp - 1][w] = -st[sp - 1][w];
            i += 1;
            break;
          }
          --sp;
#pragma unroll
          for (int w = 0; w < W; ++w) st[sp - 1][w] = fmaxf(st[sp - 1][w], -st[sp][w]);
          i += 1;
          break;
        case S2M_CSG_INTERSECT:
          if (PRUNED && code != 1u) {
            i += 1;
            break;
          }
          --sp;
#pragma unroll
          for (int w = 0; w < W; ++w) st[sp - 1][w] = fmaxf(st[sp - 1][w], st[sp][w]);
          i += 1;
          break;
        case S2M_CSG_SMOOTH_UNION: {  // sdf_op_smooth_union(a, b, k)
          if (PRUNED && code != 1u) {
#pragma unroll
            for (int w = 0; w < W; ++w) st[sp - 1][w] = canon(st[sp - 1][w]);
            i += 2;
            break;
          }
          --sp;
          const float k = s2c_ld(a);
#pragma unroll
          for (int w = 0; w < W; ++w) {
            const float b = st[sp][w], d1 = st[sp - 1][w];
            const float h = clamp01(s2c_add(0.5f, s2c_div(s2c_mul(0.5f, s2c_sub(b, d1)), k)));
            st[sp - 1][w] = s2c_sub(mix(b, d1, h), s2c_mul(s2c_mul(k, h), s2c_sub(1.0f, h)));
          }
          i += 2;
          break;
        }
        case S2M_CSG_SMOOTH_INTERSECTION: {  // sdf_op_smooth_intersection(a, b, k)
          if (PRUNED && code != 1u) {
#pragma unroll
            for (int w = 0; w < W; ++w) st[sp - 1][w] = canon(st[sp - 1][w]);
            i += 2;
            break;
          }
          --sp;
          const float k = s2c_ld(a);
#pragma unroll
          for (int w = 0; w < W; ++w) {
            const float b = st[sp][w], d1 = st[sp - 1][w];
            const float h = clamp01(s2c_sub(0.5f, s2c_div(s2c_mul(0.5f, s2c_sub(b, d1)), k)));
            st[sp - 1][w] = s2c_add(mix(b, d1, h), s2c_mul(s2c_mul(k, h), s2c_sub(1.0f, h)));
          }
          i += 2;
          break;
        }
        case S2M_CSG_SMOOTH_SUBTRACTION: {  // sdf_op_smooth_subtraction(a, b, k)
          if (PRUNED && code != 1u) {
#pragma unroll
            for (int w = 0; w < W; ++w) st[sp - 1][w] = canon(code == 2u ? -st[sp - 1][w] : st[sp - 1][w]);
            i += 2;
            break;
          }
          --sp;
          const float k = s2c_ld(a);
#pragma unroll
          for (int w = 0; w < W; ++w) {
            const float b = st[sp][w], d1 = st[sp - 1][w];
            const float h = clamp01(s2c_sub(0.5f, s2c_div(s2c_mul(0.5f, s2c_add(b, d1)), k)));
            st[sp - 1][w] = s2c_add(mix(b, -d1, h), s2c_mul(s2c_mul(k, h), s2c_sub(1.0f, h)));
          }
          i += 2;
          break;
        }
        default:
#pragma unroll
          for (int w = 0; w < W; ++w) out[w] = s2_qnan();  // rejected on the host
          return;
      }
    }
#pragma unroll
    for (int w = 0; w < W; ++w) out[w] = st[sp - 1][w];
  }

  template <int W>
  S2C_FN void eval_run(float x, float y, const float z[W], float out[W]) const {
    run<W, false>(x, y, z, out, S2CodesPtr{nullptr});
  }
  template <int W>
  S2C_FN void eval_run_pruned(float x, float y, const float z[W], float out[W], const unsigned *codes) const {
    run<W, true>(x, y, z, out, S2CodesPtr{codes});
  }
  S2C_FN float eval(float x, float y, float z) const {
    float zz[1] = {z}, v[1];
    run<1, false>(x, y, zz, v, S2CodesPtr{nullptr});
    return v[0];
  }
#if defined(__CUDACC__)
  __device__ __noinline__ float operator()(float x, float y, float z) const { return eval(x, y, z); }
  // One point with a tile's codes, read from L2 (a record of this launch).
  __device__ __noinline__ float eval_tile(float x, float y, float z, const unsigned *codes) const {
    float zz[1] = {z}, v[1];
    run<1, true>(x, y, zz, v, S2CodesL2{codes});
    return v[0];
  }
  __device__ __forceinline__ void normal(float px, float py, float pz, float eps, float n[3]) const {
    s2_tetra_normal(*this, px, py, pz, eps, n);
  }
#endif
};

// ---------------------------------------------------------------------------
// The interval pass of one tile: X, Y, Z bound the coordinates of every
// point the codes will be used at.  Writes the nodes' codes
// (S2_CSG_CODE_WORDS words) and the interval of the program's value, and
// returns 1; 0 (every code 1, root unknown) for a program of more than
// S2_CSG_MAX_NODES nodes.
S2HD void s2c_set_code(unsigned *codes, int n, unsigned c) {
  unsigned &w = codes[n >> 4];
  w = (w & ~(3u << (2 * (n & 15)))) | (c << (2 * (n & 15)));
}
S2HD void s2c_skip(unsigned *codes, int from, int to) {  // nodes from .. to inclusive
  for (int n = from; n <= to; ++n) s2c_set_code(codes, n, 0u);
}
S2HD s2i s2c_len3(s2i x, s2i y, s2i z) { return s2i_sqrt(s2i_add(s2i_add(s2i_sq(x), s2i_sq(y)), s2i_sq(z))); }
S2HD s2i s2c_len2(s2i x, s2i y) { return s2i_sqrt(s2i_add(s2i_sq(x), s2i_sq(y))); }

S2C_TILE_FN int s2c_tile(const float *prog, int len, s2i X, s2i Y, s2i Z, unsigned *codes, s2i *root) {
  for (int w = 0; w < S2_CSG_CODE_WORDS; ++w) codes[w] = 0x55555555u;
  s2i st[S2_CSG_STACK];
  int first[S2_CSG_STACK];  // the first node of each stack entry's subtree
  int sp = 0, node = 0, i = 0;
  const s2i zero = s2i_pt(0.0f);
  while (i < len) {
    if (node >= S2_CSG_MAX_NODES) {
      for (int w = 0; w < S2_CSG_CODE_WORDS; ++w) codes[w] = 0x55555555u;
      *root = s2i_unknown();
      return 0;
    }
    const int op = (int)prog[i];
    const float *a = prog + i + 1;
    int d = 0, fa = 0, fb = 0;
    s2i A, Bv;
    if (op >= S2M_CSG_UNION) {
      Bv = st[--sp];
      fb = first[sp];
      A = st[sp - 1];
      fa = first[sp - 1];
    }
    switch (op) {
      case S2M_CSG_SPHERE:
        st[sp] = s2i_sub(s2c_len3(s2i_sub(X, s2i_pt(a[0])), s2i_sub(Y, s2i_pt(a[1])), s2i_sub(Z, s2i_pt(a[2]))),
                         s2i_pt(a[3]));
        break;
      case S2M_CSG_BOX: {
        const s2i qx = s2i_sub(s2i_abs(s2i_sub(X, s2i_pt(a[0]))), s2i_pt(s2c_mul(0.5f, a[3])));
        const s2i qy = s2i_sub(s2i_abs(s2i_sub(Y, s2i_pt(a[1]))), s2i_pt(s2c_mul(0.5f, a[4])));
        const s2i qz = s2i_sub(s2i_abs(s2i_sub(Z, s2i_pt(a[2]))), s2i_pt(s2c_mul(0.5f, a[5])));
        const s2i outside = s2c_len3(s2i_max(qx, zero), s2i_max(qy, zero), s2i_max(qz, zero));
        st[sp] = s2i_add(outside, s2i_min(s2i_max(qx, s2i_max(qy, qz)), zero));
        break;
      }
      case S2M_CSG_TORUS: {
        const s2i dx = s2i_sub(X, s2i_pt(a[0])), dy = s2i_sub(Y, s2i_pt(a[1])), dz = s2i_sub(Z, s2i_pt(a[2]));
        st[sp] = s2i_sub(s2c_len2(s2i_sub(s2c_len2(dx, dz), s2i_pt(a[3])), dy), s2i_pt(a[4]));
        break;
      }
      case S2M_CSG_CAPSULE: {
        const float bax = s2c_sub(a[3], a[0]), bay = s2c_sub(a[4], a[1]), baz = s2c_sub(a[5], a[2]);
        const float d2 = s2c_add(s2c_add(s2c_mul(bax, bax), s2c_mul(bay, bay)), s2c_mul(baz, baz));
        const s2i pax = s2i_sub(X, s2i_pt(a[0])), pay = s2i_sub(Y, s2i_pt(a[1])), paz = s2i_sub(Z, s2i_pt(a[2]));
        const s2i d1 = s2i_add(s2i_add(s2i_mul(pax, s2i_pt(bax)), s2i_mul(pay, s2i_pt(bay))),
                               s2i_mul(paz, s2i_pt(baz)));
        const s2i h = s2i_clamp(s2i_div(d1, s2i_pt(d2)), zero, s2i_pt(1.0f));
        st[sp] = s2i_sub(s2c_len3(s2i_sub(pax, s2i_mul(s2i_pt(bax), h)), s2i_sub(pay, s2i_mul(s2i_pt(bay), h)),
                                  s2i_sub(paz, s2i_mul(s2i_pt(baz), h))),
                         s2i_pt(a[6]));
        break;
      }
      case S2M_CSG_PLANE:
        st[sp] = s2i_sub(s2i_add(s2i_add(s2i_mul(X, s2i_pt(a[0])), s2i_mul(Y, s2i_pt(a[1]))), s2i_mul(Z, s2i_pt(a[2]))),
                         s2i_pt(a[3]));
        break;
      case S2M_CSG_UNION: st[sp - 1] = s2i_min_sel(A, Bv, &d); break;
      case S2M_CSG_SUBTRACT: st[sp - 1] = s2i_max_sel(A, s2i_neg(Bv), &d); break;
      case S2M_CSG_INTERSECT: st[sp - 1] = s2i_max_sel(A, Bv, &d); break;
      case S2M_CSG_SMOOTH_UNION: st[sp - 1] = s2i_smooth_union_sel(A, Bv, s2i_pt(a[0]), &d); break;
      case S2M_CSG_SMOOTH_INTERSECTION: st[sp - 1] = s2i_smooth_intersection_sel(A, Bv, s2i_pt(a[0]), &d); break;
      case S2M_CSG_SMOOTH_SUBTRACTION: st[sp - 1] = s2i_smooth_subtraction_sel(A, Bv, s2i_pt(a[0]), &d); break;
      default:
        *root = s2i_unknown();
        return 0;
    }
    if (op < S2M_CSG_UNION) {
      first[sp] = node;
      ++sp;
    } else if (d == 1) {  // the first operand: the second's nodes are not needed
      s2c_skip(codes, fb, node - 1);
      s2c_set_code(codes, node, 2u);
    } else if (d == 2) {  // the second operand
      s2c_skip(codes, fa, fb - 1);
      s2c_set_code(codes, node, 3u);
    }
    i += 1 + s2c_operands(op);
    ++node;
  }
  *root = st[0];
  return 1;
}
