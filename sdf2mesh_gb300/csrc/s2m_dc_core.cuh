// s2m_dc_core.cuh -- the dual-contouring rule on one cell, independent of
// how the SDF is evaluated: lattice coordinates, candidate classification,
// the reference's mass-point vertex (dualcontour.wgsl:22-180) and the
// precision-mode QEF vertex.  Every function that evaluates the SDF takes an
// evaluator `f` with
//     float f(float x, float y, float z) const;            // sdf3d
//     void f.normal(float x, float y, float z, float eps, float n[3]) const;
//                                                           // sdf3d_normal, not normalised
// NVRTC instantiates it with the lowered user SDF (s2m_dc_kernels.cuh); the
// batch engine with its CSG program interpreter (batch.cu).
// All arithmetic of the rule is explicitly rounded binary32 / binary64.
#pragma once

__device__ __forceinline__ float s2_coord(const S2Job &j, int i) {
  return __fadd_rn(j.bmin, __fmul_rn(j.size, (float)i));
}
// 1 if mn(i - 1) + size differs (bitwise) from the lattice coordinate c(i).
__device__ __forceinline__ unsigned s2_off_lattice(const S2Job &j, int i) {
  float hi = __fadd_rn(s2_coord(j, i - 1), j.size);
  return __float_as_uint(hi) != __float_as_uint(s2_coord(j, i)) ? 1u : 0u;
}

struct S2Cell {
  int x, y, z;
};

// Slab s evaluates lattice planes k0 .. k0 + nk - 1 (k0 = zb for the first
// slab, else zb + s * D + 1; the last plane is min(zb + nzc, zb + (s + 1) * D):
// the job's cells are planes zb .. zb + nzc - 1).  The tile
// pruning cuts them into tiles of S2_PT_XY x S2_PT_XY points by
// s2_tile_depth(nk) planes.
__device__ __forceinline__ void s2_slab_planes(const S2Job &j, int s, int D, int nzc, int &k0, int &nk) {
  const int zc0 = j.zb + s * D;
  const int zc1 = min(j.zb + nzc, zc0 + D);
  k0 = s == 0 ? j.zb : zc0 + 1;
  nk = zc1 - k0 + 1;
}
__device__ __forceinline__ int s2_tile_depth(int nk) {
  const int parts = (nk + S2_PT_ZMAX - 1) / S2_PT_ZMAX;
  return (nk + parts - 1) / parts;
}
// Index, among all tiles of the job, of the pruning tile whose box covers
// cell c (its corners and normal samples): the tile of the cell's lattice
// point (x, y, z + 1), whose box reaches one point further in +x, +y and -z.
// tbase[s] is slab s's first tile.
__device__ __forceinline__ unsigned long long s2_cell_prune_tile(const S2Job &job, S2Cell c,
                                                                 const unsigned long long *tbase, int D, int nzc) {
  const int s = (c.z - job.zb) / D;
  int k0, nk;
  s2_slab_planes(job, s, D, nzc, k0, nk);
  const int tz = (c.z + 1 - k0) / s2_tile_depth(nk);
  const int ntx = (job.P + S2_PT_XY - 1) / S2_PT_XY;
  const unsigned long long t = ((unsigned long long)tz * ntx + c.y / S2_PT_XY) * ntx + c.x / S2_PT_XY;
  return tbase[s] + t - tbase[0];
}

__device__ __forceinline__ S2Cell s2_cell_of(const S2Job &j, long long c, int zc0) {
  S2Cell r;
  if (c < 0x100000000ll) {
    const unsigned cu = (unsigned)c, n = (unsigned)j.N;
    const unsigned q = s2_udiv(cu, n, j.magic_n);
    r.x = (int)(cu - q * n);
    const unsigned z = s2_udiv(q, n, j.magic_n);
    r.y = (int)(q - z * n);
    r.z = zc0 + (int)z;
  } else {
    r.x = (int)(c % j.N);
    long long q = c / j.N;
    r.y = (int)(q % j.N);
    r.z = zc0 + (int)(q / j.N);
  }
  return r;
}

// The 8 lattice values of a cell, corner index bx | by << 1 | bz << 2.
// CG: read through L2 only (lattices written earlier in the same launch by
// other blocks, as in the persistent batch kernel).
template <bool CG = false>
__device__ __forceinline__ void s2_load_corners(const S2Job &j, const float *__restrict__ ring, S2Cell c, float v[8]) {
  const float *p0 = ring + (long long)(c.z % j.ring) * j.plane + (long long)c.y * j.pitch + c.x;
  const float *p1 = ring + (long long)((c.z + 1) % j.ring) * j.plane + (long long)c.y * j.pitch + c.x;
  const float *p[8] = {p0, p0 + 1, p0 + j.pitch, p0 + j.pitch + 1, p1, p1 + 1, p1 + j.pitch, p1 + j.pitch + 1};
#pragma unroll
  for (int k = 0; k < 8; ++k) v[k] = CG ? __ldcg(p[k]) : __ldg(p[k]);
}

// Mask of corners whose reference coordinates are not lattice points.
__device__ __forceinline__ unsigned s2_off_mask(const S2Job &j, S2Cell c) {
  unsigned ox = s2_off_lattice(j, c.x + 1), oy = s2_off_lattice(j, c.y + 1), oz = s2_off_lattice(j, c.z + 1);
  unsigned m = 0;
  for (int k = 1; k < 8; ++k)
    if (((k & 1) && ox) || ((k & 2) && oy) || ((k & 4) && oz)) m |= 1u << k;
  return m;
}

// A cell is a candidate when it may carry a vertex: its lattice corners do
// not all share a sign, or one of its off-lattice corners is within the
// guard band of zero (its reference value could then have the other sign).
template <bool CG = false>
__device__ __forceinline__ bool s2_classify(const S2Job &j, const float *__restrict__ ring, S2Cell c) {
  float v[8];
  s2_load_corners<CG>(j, ring, c, v);
  unsigned pos = 0;
  for (int k = 0; k < 8; ++k) pos |= (v[k] > 0.0f ? 1u : 0u) << k;
  if (pos != 0u && pos != 0xffu) return true;
  if (j.qef) return false;  // precision mode uses the lattice values as they are
  unsigned off = s2_off_mask(j, c);
  if (!off) return false;
  if (j.exact) return true;
  for (int k = 1; k < 8; ++k)
    if ((off >> k) & 1u)
      if (!(fabsf(v[k]) >= j.guard)) return true;
  return false;
}

// Classification from values already loaded (same rule as s2_classify).
__device__ __forceinline__ bool s2_classify_values(const S2Job &j, S2Cell c, const float v[8]) {
  unsigned pos = 0;
#pragma unroll
  for (int k = 0; k < 8; ++k) pos |= (v[k] > 0.0f ? 1u : 0u) << k;
  if (pos != 0u && pos != 0xffu) return true;
  if (j.qef) return false;
  const unsigned off = s2_off_mask(j, c);
  if (!off) return false;
  if (j.exact) return true;
  bool near = false;
#pragma unroll
  for (int k = 1; k < 8; ++k) near |= ((off >> k) & 1u) && !(fabsf(v[k]) >= j.guard);
  return near;
}

template <bool CG>
__device__ __forceinline__ float4 s2_ld4(const float *p) {
  return CG ? __ldcg(reinterpret_cast<const float4 *>(p)) : __ldg(reinterpret_cast<const float4 *>(p));
}
template <bool CG>
__device__ __forceinline__ float s2_ld1(const float *p) {
  return CG ? __ldcg(p) : __ldg(p);
}

// Four consecutive cells of the linear order starting at cell c0 (z, y, x):
// their candidate bits (bit m for cell c0 + m, cells past `ncells` excluded)
// and their corner values.  When N is a multiple of 4 the four cells share
// a row and start at a multiple of 4, so each of the 4 corner rows is one
// 16-byte load plus one scalar (8 loads for 4 cells instead of 32).
template <bool CG>
__device__ __forceinline__ unsigned s2_classify4(const S2Job &j, const float *__restrict__ ring, long long c0,
                                                 long long ncells, int zc0, float v[4][8]) {
  unsigned mask = 0;
  if (c0 >= ncells) return 0u;
  const S2Cell c = s2_cell_of(j, c0, zc0);
  if ((j.N & 3) == 0 && c0 + 3 < ncells) {
    const float *p0 = ring + (long long)(c.z % j.ring) * j.plane + (long long)c.y * j.pitch + c.x;
    const float *p1 = ring + (long long)((c.z + 1) % j.ring) * j.plane + (long long)c.y * j.pitch + c.x;
    const float *rows[4] = {p0, p0 + j.pitch, p1, p1 + j.pitch};  // (y, z) = 00, 10, 01, 11
    float r[4][5];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const float4 a = s2_ld4<CG>(rows[q]);
      r[q][0] = a.x; r[q][1] = a.y; r[q][2] = a.z; r[q][3] = a.w;
      r[q][4] = s2_ld1<CG>(rows[q] + 4);
    }
#pragma unroll
    for (int m = 0; m < 4; ++m) {
      // corner index bx | by << 1 | bz << 2
#pragma unroll
      for (int k = 0; k < 8; ++k) v[m][k] = r[((k >> 1) & 1) | (((k >> 2) & 1) << 1)][m + (k & 1)];
      S2Cell cm = c;
      cm.x = c.x + m;
      if (s2_classify_values(j, cm, v[m])) mask |= 1u << m;
    }
    return mask;
  }
#pragma unroll 1
  for (int m = 0; m < 4; ++m) {
    if (c0 + m >= ncells) break;
    const S2Cell cm = s2_cell_of(j, c0 + m, zc0);
    s2_load_corners<CG>(j, ring, cm, v[m]);
    if (s2_classify_values(j, cm, v[m])) mask |= 1u << m;
  }
  return mask;
}

// sdf3d_normal.wgsl:4-10 as a loop with one sdf3d call site:
// n = ((t0 + t1) + t2) + t3 with t_i = d_i * sdf3d(p + d_i * eps), the order
// the library function adds in.
template <class F>
__device__ __forceinline__ void s2_tetra_normal(const F &f, float px, float py, float pz, float eps, float n[3]) {
#pragma unroll 1
  for (int i = 0; i < 4; ++i) {
    const float dx = (i == 0 || i == 3) ? 1.0f : -1.0f;
    const float dy = (i >= 2) ? 1.0f : -1.0f;
    const float dz = (i == 1 || i == 3) ? 1.0f : -1.0f;
    const float v = f(__fadd_rn(px, __fmul_rn(dx, eps)), __fadd_rn(py, __fmul_rn(dy, eps)),
                      __fadd_rn(pz, __fmul_rn(dz, eps)));
    const float tx = __fmul_rn(dx, v), ty = __fmul_rn(dy, v), tz = __fmul_rn(dz, v);
    if (i == 0) {
      n[0] = tx; n[1] = ty; n[2] = tz;
    } else {
      n[0] = __fadd_rn(n[0], tx); n[1] = __fadd_rn(n[1], ty); n[2] = __fadd_rn(n[2], tz);
    }
  }
}

__device__ __forceinline__ float s2_len3(const float n[3]) {
  return __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(n[0], n[0]), __fmul_rn(n[1], n[1])), __fmul_rn(n[2], n[2])));
}

// dualcontour.wgsl:72-131 (crossings, counting rule, mass point) and
// :161-180 (normal, sign bits) on one candidate cell.  `v` holds the cell's
// lattice values; corners whose reference coordinates are off the lattice are
// re-evaluated here at those coordinates, so the rule sees exactly the
// reference's 8 values.  Writes the vertex and returns the final key
// (x | y << 16 | label << 32 | signs << 48 | has_vertex << 63).
template <class F>
__device__ __forceinline__ unsigned long long s2_vertex(const F &sdf, const S2Job &j, S2Cell c, float v[8],
                                                        float pos[3], float nrm[3]) {
  float mn[3] = {s2_coord(j, c.x), s2_coord(j, c.y), s2_coord(j, c.z)};
  float mx[3] = {__fadd_rn(mn[0], j.size), __fadd_rn(mn[1], j.size), __fadd_rn(mn[2], j.size)};
  // Off-lattice corners, one sdf3d call site in a loop (a warp runs the
  // largest count among its lanes instead of every inlined copy).
  unsigned off = s2_off_mask(j, c) & 0xfeu;
#pragma unroll 1
  while (off) {
    const int k = __ffs(off) - 1;
    off &= off - 1u;
    const float f = sdf((k & 1) ? mx[0] : mn[0], (k & 2) ? mx[1] : mn[1], (k & 4) ? mx[2] : mn[2]);
#pragma unroll
    for (int q = 1; q < 8; ++q)
      if (q == k) v[q] = f;
  }

  // 12 edges in the reference order: 4 along z, 4 along y, 4 along x.
  // Each: corner a, corner b, axis of t, the two fixed local coordinates.
  const int ea[12] = {0, 2, 1, 3, 0, 4, 1, 5, 0, 4, 2, 6};
  const int eb[12] = {4, 6, 5, 7, 2, 6, 3, 7, 1, 5, 3, 7};
  const int eax[12] = {2, 2, 2, 2, 1, 1, 1, 1, 0, 0, 0, 0};
  const float eu[12] = {0, 0, 1, 1, 0, 0, 1, 1, 0, 0, 1, 1};
  const float ev[12] = {0, 1, 0, 1, 0, 1, 0, 1, 0, 1, 0, 1};
  float avg[3] = {0.0f, 0.0f, 0.0f};
  float count = 0.0f;
#pragma unroll
  for (int e = 0; e < 12; ++e) {
    float a = v[ea[e]], b = v[eb[e]];
    if ((a > 0.0f) != (b > 0.0f)) {
      float t = __fdiv_rn(__fsub_rn(0.0f, a), __fsub_rn(b, a));
      float w[3];
      if (eax[e] == 2) { w[0] = eu[e]; w[1] = ev[e]; w[2] = t; }
      else if (eax[e] == 1) { w[0] = eu[e]; w[1] = t; w[2] = ev[e]; }
      else { w[0] = t; w[1] = eu[e]; w[2] = ev[e]; }
      if (w[0] > 0.0f || w[1] > 0.0f || w[2] > 0.0f) {
        avg[0] = __fadd_rn(avg[0], w[0]);
        avg[1] = __fadd_rn(avg[1], w[1]);
        avg[2] = __fadd_rn(avg[2], w[2]);
        count = __fadd_rn(count, 1.0f);
      }
    }
  }
  const unsigned signs = (v[1] > 0.0f ? 1u : 0u) | (v[2] > 0.0f ? 2u : 0u) | (v[4] > 0.0f ? 4u : 0u) | (v[0] > 0.0f ? 8u : 0u);
  const unsigned long long zl = (unsigned long long)(j.lag ? c.z + 1 : c.z);
  unsigned long long key = (unsigned long long)c.x | ((unsigned long long)c.y << 16) | (zl << 32) |
                           ((unsigned long long)signs << 48);
  if (!(count > 1.0f)) return key;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    float bsize = __fsub_rn(mx[a], mn[a]);
    pos[a] = __fadd_rn(mn[a], __fdiv_rn(__fmul_rn(bsize, avg[a]), count));
  }
  float n[3];
  sdf.normal(pos[0], pos[1], pos[2], j.eps, n);
  float len = s2_len3(n);
  nrm[0] = __fdiv_rn(n[0], len);
  nrm[1] = __fdiv_rn(n[1], len);
  nrm[2] = __fdiv_rn(n[2], len);
  return key | (1ull << 63);
}

// ---------------------------------------------------------------------------
// Precision mode.  Corners are the lattice values (shared by neighbouring
// cells, so signs agree and the mesh closes).  Every sign-change edge gives a
// crossing q in cell-local coordinates (t as in dualcontour.wgsl:72-74) and
// a unit normal (the SDF's gradient there); the vertex minimises
// sum (n . (x - q))^2 around the mass point.  The normal-equation sums are
// binary32 with Neumaier compensation; the 3x3 solve is binary64 (cyclic
// Jacobi eigen-decomposition, eigenvalues below 0.1 of the largest dropped,
// x = c + V D^+ V^T (A^T b - A c), clamped to the cell).

struct S2KSum {
  float s, c;
  __device__ __forceinline__ void init() { s = 0.0f; c = 0.0f; }
  __device__ __forceinline__ void add(float x) {
    float t = __fadd_rn(s, x);
    if (fabsf(s) >= fabsf(x)) c = __fadd_rn(c, __fadd_rn(__fsub_rn(s, t), x));
    else c = __fadd_rn(c, __fadd_rn(__fsub_rn(x, t), s));
    s = t;
  }
  __device__ __forceinline__ float value() const { return __fadd_rn(s, c); }
};

__device__ __forceinline__ void s2_jacobi3(double a[3][3], double v[3][3]) {
  for (int i = 0; i < 3; ++i)
    for (int k = 0; k < 3; ++k) v[i][k] = i == k ? 1.0 : 0.0;
#pragma unroll 1
  for (int sweep = 0; sweep < 24; ++sweep) {
    double off = __dadd_rn(__dadd_rn(__dmul_rn(a[0][1], a[0][1]), __dmul_rn(a[0][2], a[0][2])), __dmul_rn(a[1][2], a[1][2]));
    double diag = __dadd_rn(__dadd_rn(__dmul_rn(a[0][0], a[0][0]), __dmul_rn(a[1][1], a[1][1])), __dmul_rn(a[2][2], a[2][2]));
    if (!(off > __dmul_rn(1e-30, diag))) break;
#pragma unroll
    for (int pq = 0; pq < 3; ++pq) {
      const int p = pq == 2 ? 1 : 0, q = pq == 0 ? 1 : 2;
      const double apq = a[p][q];
      if (apq == 0.0) continue;
      const double theta = __ddiv_rn(__dsub_rn(a[q][q], a[p][p]), __dmul_rn(2.0, apq));
      const double t = __ddiv_rn(theta >= 0.0 ? 1.0 : -1.0,
                                 __dadd_rn(fabs(theta), __dsqrt_rn(__dadd_rn(__dmul_rn(theta, theta), 1.0))));
      const double cs = __ddiv_rn(1.0, __dsqrt_rn(__dadd_rn(__dmul_rn(t, t), 1.0)));
      const double sn = __dmul_rn(t, cs);
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const double akp = a[k][p], akq = a[k][q];
        a[k][p] = __dsub_rn(__dmul_rn(cs, akp), __dmul_rn(sn, akq));
        a[k][q] = __dadd_rn(__dmul_rn(sn, akp), __dmul_rn(cs, akq));
      }
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const double apk = a[p][k], aqk = a[q][k];
        a[p][k] = __dsub_rn(__dmul_rn(cs, apk), __dmul_rn(sn, aqk));
        a[q][k] = __dadd_rn(__dmul_rn(sn, apk), __dmul_rn(cs, aqk));
      }
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const double vkp = v[k][p], vkq = v[k][q];
        v[k][p] = __dsub_rn(__dmul_rn(cs, vkp), __dmul_rn(sn, vkq));
        v[k][q] = __dadd_rn(__dmul_rn(sn, vkp), __dmul_rn(cs, vkq));
      }
    }
  }
}

__device__ __forceinline__ void s2_qef_solve(const double A[6], const double b[3], const double c[3], double x[3]) {
  double a[3][3] = {{A[0], A[1], A[2]}, {A[1], A[3], A[4]}, {A[2], A[4], A[5]}};
  double r[3];
#pragma unroll
  for (int i = 0; i < 3; ++i)
    r[i] = __dsub_rn(b[i], __dadd_rn(__dadd_rn(__dmul_rn(a[i][0], c[0]), __dmul_rn(a[i][1], c[1])), __dmul_rn(a[i][2], c[2])));
  double v[3][3];
  s2_jacobi3(a, v);
  const double lmax = fmax(fabs(a[0][0]), fmax(fabs(a[1][1]), fabs(a[2][2])));
  double y[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const double vr = __dadd_rn(__dadd_rn(__dmul_rn(v[0][k], r[0]), __dmul_rn(v[1][k], r[1])), __dmul_rn(v[2][k], r[2]));
    const double l = a[k][k];
    y[k] = (lmax > 0.0 && fabs(l) >= __dmul_rn(0.1, lmax)) ? __ddiv_rn(vr, l) : 0.0;
  }
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    const double d = __dadd_rn(__dadd_rn(__dmul_rn(v[i][0], y[0]), __dmul_rn(v[i][1], y[1])), __dmul_rn(v[i][2], y[2]));
    const double xi = __dadd_rn(c[i], d);
    x[i] = xi < 0.0 ? 0.0 : (xi > 1.0 ? 1.0 : xi);
  }
}

template <class F>
__device__ __forceinline__ unsigned long long s2_vertex_qef(const F &sdf, const S2Job &j, S2Cell c, const float v[8],
                                                            float pos[3], float nrm[3]) {
  const float lo[3] = {s2_coord(j, c.x), s2_coord(j, c.y), s2_coord(j, c.z)};
  const float hi[3] = {s2_coord(j, c.x + 1), s2_coord(j, c.y + 1), s2_coord(j, c.z + 1)};
  S2KSum sA[6], sb[3], sq[3];
#pragma unroll
  for (int i = 0; i < 6; ++i) sA[i].init();
#pragma unroll
  for (int i = 0; i < 3; ++i) { sb[i].init(); sq[i].init(); }
  int m = 0;
#pragma unroll 1
  for (int e = 0; e < 12; ++e) {
    // edges in the reference order: 4 along z, 4 along y, 4 along x
    // corner indices of edge e's ends, one nibble per edge (dualcontour.wgsl:99-114)
    const unsigned long long EA = 0x624051403120ull, EB = 0x735173627564ull;
    const int a_ = int((EA >> (4 * e)) & 0xfull), b_ = int((EB >> (4 * e)) & 0xfull);
    const int ax = e < 4 ? 2 : (e < 8 ? 1 : 0);
    float va = 0.0f, vb = 0.0f;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      if (k == a_) va = v[k];
      if (k == b_) vb = v[k];
    }
    if ((va > 0.0f) == (vb > 0.0f)) continue;
    const float t = __fdiv_rn(__fsub_rn(0.0f, va), __fsub_rn(vb, va));
    float q[3], w[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      if (d == ax) {
        q[d] = t;
        w[d] = __fadd_rn(lo[d], __fmul_rn(j.size, t));
      } else {
        const bool one = (a_ >> d) & 1;
        q[d] = one ? 1.0f : 0.0f;
        w[d] = one ? hi[d] : lo[d];
      }
    }
    float n[3];
    sdf.normal(w[0], w[1], w[2], j.eps, n);
    const float len = s2_len3(n);
    ++m;
#pragma unroll
    for (int d = 0; d < 3; ++d) sq[d].add(q[d]);
    if (!(len > 0.0f)) continue;
    const float nn[3] = {__fdiv_rn(n[0], len), __fdiv_rn(n[1], len), __fdiv_rn(n[2], len)};
    const float dd = __fadd_rn(__fadd_rn(__fmul_rn(nn[0], q[0]), __fmul_rn(nn[1], q[1])), __fmul_rn(nn[2], q[2]));
    sA[0].add(__fmul_rn(nn[0], nn[0]));
    sA[1].add(__fmul_rn(nn[0], nn[1]));
    sA[2].add(__fmul_rn(nn[0], nn[2]));
    sA[3].add(__fmul_rn(nn[1], nn[1]));
    sA[4].add(__fmul_rn(nn[1], nn[2]));
    sA[5].add(__fmul_rn(nn[2], nn[2]));
#pragma unroll
    for (int d = 0; d < 3; ++d) sb[d].add(__fmul_rn(nn[d], dd));
  }
  const unsigned signs = (v[1] > 0.0f ? 1u : 0u) | (v[2] > 0.0f ? 2u : 0u) | (v[4] > 0.0f ? 4u : 0u) | (v[0] > 0.0f ? 8u : 0u);
  const unsigned long long zl = (unsigned long long)(j.lag ? c.z + 1 : c.z);
  const unsigned long long key = (unsigned long long)c.x | ((unsigned long long)c.y << 16) | (zl << 32) |
                                 ((unsigned long long)signs << 48);
  if (m == 0) return key;
  double A[6], b[3], cc[3], xs[3];
#pragma unroll
  for (int i = 0; i < 6; ++i) A[i] = (double)sA[i].value();
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    b[d] = (double)sb[d].value();
    cc[d] = __ddiv_rn((double)sq[d].value(), (double)m);
  }
  s2_qef_solve(A, b, cc, xs);
#pragma unroll
  for (int d = 0; d < 3; ++d) pos[d] = __double2float_rn(__dadd_rn((double)lo[d], __dmul_rn((double)j.size, xs[d])));
  float n[3];
  sdf.normal(pos[0], pos[1], pos[2], j.eps, n);
  const float len = s2_len3(n);
  nrm[0] = __fdiv_rn(n[0], len);
  nrm[1] = __fdiv_rn(n[1], len);
  nrm[2] = __fdiv_rn(n[2], len);
  return key | (1ull << 63);
}


// Decided tiles of a pruned evaluation, for classification: the flag word of
// the tile of 8 x 8 x 8 lattice points holding a cell's lower corner sits at
// flags[stride * t], t = ((z / 8) * ntx + y / 8) * ntx + x / 8.  A decided
// tile's interval bounds every corner of its cells (its box reaches one point
// past the tile's points), at or beyond +-guard with one sign: no such cell
// is a candidate, unless S2M_JOB_EXACT_CORNERS makes every cell with an
// off-lattice corner one.
struct S2CellSkip {
  const unsigned *flags;  // null: no decided tiles
  unsigned stride;
  int ntx;
};

// Classification of the batch engine in three stages that never wait on one
// another inside a stage (a decoupled look-back over a job's tiles walked
// far back behind the many tiles in flight):
//   s2_cell_mark_tiles  tiles tile0 .. tile0 + M - 1 (S2_CELL_TILE cells each,
//                       S2_CELL_BLOCK threads, S2_CELL_CPT consecutive cells
//                       per thread in groups of 4): each thread's candidate
//                       bits go to words[tile * S2_CELL_BLOCK + thread], the
//                       tile's count to tcnt[tile];
//   s2_scan_tiles       (one block) the counts into each tile's first slot;
//   s2_cell_emit_tiles  each tile's candidates in (z, y, x) order, with their
//                       8 corner values.
// With `skip`, a group of 4 cells that lies in one decided tile (N a multiple
// of 4: a group is then 4 cells of one row, x from a multiple of 4) is not
// loaded at all.
template <bool CG, int M>
__device__ __forceinline__ void s2_cell_mark_tiles(const S2Job &job, const float *__restrict__ ring, unsigned tile0,
                                                   unsigned ntiles, long long ncells, int zc0, S2CellSkip skip,
                                                   unsigned *words, unsigned *tcnt) {
  __shared__ unsigned s_warp[32];
  const unsigned tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
#pragma unroll 1
  for (int t = 0; t < M; ++t) {
    const unsigned tile = tile0 + (unsigned)t;
    if (tile >= ntiles) break;  // the same in every thread
    const long long c0 = (long long)tile * S2_CELL_TILE + (long long)S2_CELL_CPT * tid;
    unsigned decided = 0;  // bit g: group g lies in a decided tile
    if (skip.flags && !job.exact && (job.N & 3) == 0) {
      unsigned f[S2_CELL_CPT / 4];
#pragma unroll
      for (int g = 0; g < S2_CELL_CPT / 4; ++g) {  // the flag loads first, in flight together
        f[g] = 0u;
        if (c0 + 4 * g + 3 < ncells) {
          const S2Cell c = s2_cell_of(job, c0 + 4 * g, zc0);
          const unsigned ti = ((unsigned)(c.z >> 3) * (unsigned)skip.ntx + (unsigned)(c.y >> 3)) *
                                  (unsigned)skip.ntx + (unsigned)(c.x >> 3);
          f[g] = __ldcg(skip.flags + (size_t)ti * skip.stride);
        }
      }
#pragma unroll
      for (int g = 0; g < S2_CELL_CPT / 4; ++g) decided |= (f[g] & S2_TILE_DECIDED ? 1u : 0u) << g;
    }
    unsigned mk = 0u;  // bit g * 4 + m: cell c0 + 4g + m
#pragma unroll
    for (int g = 0; g < S2_CELL_CPT / 4; ++g) {
      if ((decided >> g) & 1u) continue;
      float v[4][8];
      mk |= s2_classify4<CG>(job, ring, c0 + 4 * g, ncells, zc0, v) << (4 * g);
    }
    words[(size_t)tile * S2_CELL_BLOCK + tid] = mk;
    unsigned cnt = __popc(mk);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(S2_FULL, cnt, o);
    if (lane == 0) s_warp[warp] = cnt;
    __syncthreads();
    if (warp == 0) {
      unsigned tot = lane < S2_CELL_BLOCK / 32 ? s_warp[lane] : 0u;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) tot += __shfl_xor_sync(S2_FULL, tot, o);
      if (lane == 0) tcnt[tile] = tot;
    }
    __syncthreads();  // s_warp is reused
  }
}

template <bool CG, int M>
__device__ __forceinline__ void s2_cell_emit_tiles(const S2Job &job, const float *__restrict__ ring,
                                                   const S2Cand &cand, unsigned *err, unsigned tile0, unsigned ntiles,
                                                   int zc0, const unsigned *words, const unsigned *tcnt,
                                                   const unsigned long long *toff) {
  __shared__ unsigned s_warp[32];
  __shared__ unsigned short s_cl[S2_CELL_TILE];
  const unsigned tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
#pragma unroll 1
  for (int t = 0; t < M; ++t) {
    const unsigned tile = tile0 + (unsigned)t;
    if (tile >= ntiles) break;  // the same in every thread
    const unsigned total = __ldcg(tcnt + tile);
    if (total == 0u) continue;  // the same in every thread
    const unsigned mk = __ldcg(words + (size_t)tile * S2_CELL_BLOCK + tid);
    const unsigned cnt = __popc(mk);
    unsigned inc = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned x = __shfl_up_sync(S2_FULL, inc, o);
      if ((int)lane >= o) inc += x;
    }
    if (lane == 31) s_warp[warp] = inc;
    if (tid < 32 && tid >= S2_CELL_BLOCK / 32) s_warp[tid] = 0u;
    __syncthreads();
    if (warp == 0) s2_warp_exclusive32(s_warp);
    __syncthreads();
    {  // the tile's candidates in order (cell offsets within the tile)
      unsigned r = s_warp[warp] + (inc - cnt), rem = mk;
      while (rem) {
        const unsigned m = (unsigned)__ffs(rem) - 1u;
        rem &= rem - 1u;
        s_cl[r++] = (unsigned short)(S2_CELL_CPT * tid + m);
      }
    }
    __syncthreads();
    // written one per thread: every thread's corner loads are in flight
    // together, however the candidates fall among the threads
    const unsigned long long first = __ldcg(toff + tile);
#pragma unroll 1
    for (unsigned r = tid; r < total; r += S2_CELL_BLOCK) {
      const unsigned long long o = first + r;
      if (o >= cand.cap) {
        atomicOr(err, S2_ERR_CAND_OVF);
        continue;
      }
      const S2Cell cell = s2_cell_of(job, (long long)tile * S2_CELL_TILE + s_cl[r], zc0);
      float v[8];
      s2_load_corners<CG>(job, ring, cell, v);
      cand.key[o] = (unsigned long long)cell.x | ((unsigned long long)cell.y << 16) | ((unsigned long long)cell.z << 32);
      float4 *dst = reinterpret_cast<float4 *>(cand.val + 8 * o);
      dst[0] = make_float4(v[0], v[1], v[2], v[3]);
      dst[1] = make_float4(v[4], v[5], v[6], v[7]);
    }
    __syncthreads();  // s_warp / s_cl are reused by the next tile
  }
}

// ---------------------------------------------------------------------------
// Vertices of the reference rule for a warp's 32 candidates at once.  The
// evaluations a candidate needs -- its off-lattice corners, then the four
// normal samples -- differ in number from lane to lane; here each warp lists
// them in shared memory and evaluates the list 32 at a time, so every lane
// evaluates the SDF on every pass.  Same coordinates, same arithmetic, same
// order of the normal sum as s2_vertex: the same bits.  F::kStdNormal says
// whether F's normal is the library's tetrahedral one (otherwise, and in
// precision mode, the per-lane s2_vertex path runs).
// The SDF at a point requested by lane l of the warp (s2_vertex_warp
// evaluates other lanes' requests): plain evaluators ignore l; an evaluator
// with per-lane state (the tile-pruned one) overloads this.
template <class F>
__device__ __forceinline__ float s2_sdf_for(const F &f, unsigned l, float x, float y, float z) {
  (void)l;
  return f(x, y, z);
}

struct S2WarpScratch {
  unsigned short req[32 * 8];
  float val[32][8];
  float lo[32][3], hi[32][3];
  float pos[32][3];
  float nv[32][4];
};
// Dynamic shared memory of the vertex kernel (s2m_vertices).
#define S2_VX_SMEM_BYTES (sizeof(S2WarpScratch) * (S2_VX_BLOCK / 32) + sizeof(void *) * S2_VX_BLOCK)

// Lane by lane, the corners in `req` (bit k: corner k) evaluated at the
// cell's reference coordinates (ws.lo / ws.hi), 32 requests of the warp at a
// time, whichever lanes they come from; the values replace v[k].
template <class F>
__device__ __forceinline__ void s2_corner_requests(const F &sdf, unsigned req, float v[8], S2WarpScratch &ws) {
  const unsigned lane = threadIdx.x & 31u;
  unsigned cnt = __popc(req), inc = cnt;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned t = __shfl_up_sync(S2_FULL, inc, o);
    if ((int)lane >= o) inc += t;
  }
  const unsigned total = __shfl_sync(S2_FULL, inc, 31);
  if (total == 0u) return;  // the same on the whole warp
  {
    unsigned slot = inc - cnt, rem = req;
    while (rem) {
      const unsigned k = __ffs(rem) - 1;
      rem &= rem - 1u;
      ws.req[slot++] = (unsigned short)((lane << 3) | k);
    }
  }
  __syncwarp();
#pragma unroll 1
  for (unsigned r0 = 0; r0 < total; r0 += 32) {
    const unsigned r = r0 + lane;
    if (r < total) {
      const unsigned q = ws.req[r], l = q >> 3, k = q & 7u;
      const float x = (k & 1) ? ws.hi[l][0] : ws.lo[l][0];
      const float y = (k & 2) ? ws.hi[l][1] : ws.lo[l][1];
      const float z = (k & 4) ? ws.hi[l][2] : ws.lo[l][2];
      ws.val[l][k] = s2_sdf_for(sdf, l, x, y, z);
    }
  }
  __syncwarp();
#pragma unroll
  for (int k = 0; k < 8; ++k)
    if ((req >> k) & 1u) v[k] = ws.val[lane][k];
}

template <class F>
__device__ __forceinline__ unsigned long long s2_vertex_warp(const F &sdf, const S2Job &j, bool active, S2Cell c,
                                                             float v[8], float pos[3], float nrm[3],
                                                             S2WarpScratch &ws) {
  const unsigned lane = threadIdx.x & 31u;
  const unsigned lt = s2_lanemask_lt();
  float mn[3] = {s2_coord(j, c.x), s2_coord(j, c.y), s2_coord(j, c.z)};
  float mx[3] = {__fadd_rn(mn[0], j.size), __fadd_rn(mn[1], j.size), __fadd_rn(mn[2], j.size)};
  // Corners evaluated here: the off-lattice ones (at the cell's reference
  // coordinates) and those the lattice pass left unknown (NaN or +-inf:
  // decided tiles of the pruned evaluations; a value that really is
  // non-finite is evaluated again, to the same value).  An unknown corner
  // that is on the lattice has reference coordinates equal to its lattice
  // coordinates, so both kinds are evaluated at the cell's bounds.  (Leaving
  // out the off-lattice corners whose sign the lattice value settles and that
  // end no crossing edge, in a second round of requests, was slower: fewer
  // evaluations, but more registers and code in this latency-bound kernel.)
  unsigned off = 0u;
  if (active) {
    off = s2_off_mask(j, c) & 0xfeu;
#pragma unroll
    for (int k = 0; k < 8; ++k)
      if (!(fabsf(v[k]) <= 3.40282347e38f)) off |= 1u << k;
  }
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    ws.lo[lane][a] = mn[a];
    ws.hi[lane][a] = mx[a];
  }
  // 1. off-lattice and unknown corners
  s2_corner_requests(sdf, off, v, ws);
  // 2. crossings and mass point (dualcontour.wgsl:86-131)
  const int ea[12] = {0, 2, 1, 3, 0, 4, 1, 5, 0, 4, 2, 6};
  const int eb[12] = {4, 6, 5, 7, 2, 6, 3, 7, 1, 5, 3, 7};
  const int eax[12] = {2, 2, 2, 2, 1, 1, 1, 1, 0, 0, 0, 0};
  const float eu[12] = {0, 0, 1, 1, 0, 0, 1, 1, 0, 0, 1, 1};
  const float ev[12] = {0, 1, 0, 1, 0, 1, 0, 1, 0, 1, 0, 1};
  float avg[3] = {0.0f, 0.0f, 0.0f};
  float count = 0.0f;
#pragma unroll
  for (int e = 0; e < 12; ++e) {
    const float a = v[ea[e]], b = v[eb[e]];
    if ((a > 0.0f) != (b > 0.0f)) {
      const float t = __fdiv_rn(__fsub_rn(0.0f, a), __fsub_rn(b, a));
      float w[3];
      if (eax[e] == 2) { w[0] = eu[e]; w[1] = ev[e]; w[2] = t; }
      else if (eax[e] == 1) { w[0] = eu[e]; w[1] = t; w[2] = ev[e]; }
      else { w[0] = t; w[1] = eu[e]; w[2] = ev[e]; }
      if (w[0] > 0.0f || w[1] > 0.0f || w[2] > 0.0f) {
        avg[0] = __fadd_rn(avg[0], w[0]);
        avg[1] = __fadd_rn(avg[1], w[1]);
        avg[2] = __fadd_rn(avg[2], w[2]);
        count = __fadd_rn(count, 1.0f);
      }
    }
  }
  const unsigned signs = (v[1] > 0.0f ? 1u : 0u) | (v[2] > 0.0f ? 2u : 0u) | (v[4] > 0.0f ? 4u : 0u) | (v[0] > 0.0f ? 8u : 0u);
  const unsigned long long zl = (unsigned long long)(j.lag ? c.z + 1 : c.z);
  const unsigned long long key = (unsigned long long)c.x | ((unsigned long long)c.y << 16) | (zl << 32) |
                                 ((unsigned long long)signs << 48);
  const bool has = active && count > 1.0f;
  if (has) {
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      const float bsize = __fsub_rn(mx[a], mn[a]);
      pos[a] = __fadd_rn(mn[a], __fdiv_rn(__fmul_rn(bsize, avg[a]), count));
      ws.pos[lane][a] = pos[a];
    }
  }
  // 3. the four tetrahedral normal samples of every vertex
  const unsigned vb = __ballot_sync(S2_FULL, has);
  const unsigned nreq = 4u * __popc(vb);
  const unsigned myfirst = 4u * __popc(vb & lt);
  if (has)
    for (unsigned d = 0; d < 4; ++d) ws.req[myfirst + d] = (unsigned short)((lane << 3) | d);
  __syncwarp();
#pragma unroll 1
  for (unsigned r0 = 0; r0 < nreq; r0 += 32) {
    const unsigned r = r0 + lane;
    if (r < nreq) {
      const unsigned q = ws.req[r], l = q >> 3, d = q & 7u;
      const float dx = (d == 0 || d == 3) ? 1.0f : -1.0f;
      const float dy = (d >= 2) ? 1.0f : -1.0f;
      const float dz = (d == 1 || d == 3) ? 1.0f : -1.0f;
      ws.nv[l][d] = s2_sdf_for(sdf, l, __fadd_rn(ws.pos[l][0], __fmul_rn(dx, j.eps)),
                               __fadd_rn(ws.pos[l][1], __fmul_rn(dy, j.eps)), __fadd_rn(ws.pos[l][2], __fmul_rn(dz, j.eps)));
    }
  }
  __syncwarp();
  if (!has) return key;
  float n[3];
#pragma unroll
  for (int d = 0; d < 4; ++d) {
    const float dx = (d == 0 || d == 3) ? 1.0f : -1.0f;
    const float dy = (d >= 2) ? 1.0f : -1.0f;
    const float dz = (d == 1 || d == 3) ? 1.0f : -1.0f;
    const float f = ws.nv[lane][d];
    const float tx = __fmul_rn(dx, f), ty = __fmul_rn(dy, f), tz = __fmul_rn(dz, f);
    if (d == 0) {
      n[0] = tx; n[1] = ty; n[2] = tz;
    } else {
      n[0] = __fadd_rn(n[0], tx); n[1] = __fadd_rn(n[1], ty); n[2] = __fadd_rn(n[2], tz);
    }
  }
  const float len = s2_len3(n);
  nrm[0] = __fdiv_rn(n[0], len);
  nrm[1] = __fdiv_rn(n[1], len);
  nrm[2] = __fdiv_rn(n[2], len);
  return key | (1ull << 63);
}
