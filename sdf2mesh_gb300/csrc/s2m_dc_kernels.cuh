// s2m_dc_kernels.cuh -- the SDF-dependent kernels of the dual-contouring
// pipeline.  NVRTC compiles this text for sm_103a once per SDF, after
// s2m_device.h, s2m_lookback.cuh, s2m_prelude.cuh and the lowered user code
// (which defines s2m_user_sdf and s2m_user_normal).
//
// Reference rule (WilstonOreo/sdf2mesh, src/bin/sdf2mesh/dualcontour.wgsl):
// cell (x, y, z) spans [mn, mx] with mn = bmin + size * pos and
// mx = mn + size (:22-27); its 8 corners are evaluated independently
// (:29-43).  Here every lattice point is evaluated ONCE (s2m_eval_planes).
// A cell corner coincides with a lattice point except where, on some axis,
// mn + size rounds differently from bmin + size * (pos + 1) ("off-lattice");
// for cells that can carry a vertex, those corners are re-evaluated at the
// reference coordinates (s2m_cells), so the vertex rule sees exactly the
// reference's 8 values.  All arithmetic of the vertex rule uses explicitly
// rounded binary32 intrinsics (no contraction, whatever the SDF's flags).

__device__ __forceinline__ float s2_coord(const S2Job &j, int i) {
  return __fadd_rn(j.bmin, __fmul_rn(j.size, (float)i));
}
// 1 if mn(i - 1) + size differs (bitwise) from the lattice coordinate c(i).
__device__ __forceinline__ unsigned s2_off_lattice(const S2Job &j, int i) {
  float hi = __fadd_rn(s2_coord(j, i - 1), j.size);
  return __float_as_uint(hi) != __float_as_uint(s2_coord(j, i)) ? 1u : 0u;
}

// Evaluate planes k0 .. k0 + nk - 1 of the lattice into the ring.
// grid.x covers the P * P points of a plane, grid.y runs of RUN planes; each
// thread walks its run along z.  The variants below differ only in RUN and in
// the occupancy the compiler must allow (__launch_bounds__ minimum blocks),
// which trades registers against latency hiding; the runtime's autotuner
// times them per SDF and keeps the fastest.
template <int RUN>
__device__ __forceinline__ void s2_eval_planes(const S2Job &job, float *__restrict__ ring, int k0, int nk) {
  long long idx = (long long)blockIdx.x * S2_EVAL_BLOCK + threadIdx.x;
  long long pts = (long long)job.P * job.P;
  if (idx >= pts) return;
  int i = (int)(idx % job.P);
  int jy = (int)(idx / job.P);
  float x = s2_coord(job, i), y = s2_coord(job, jy);
  int kb = k0 + (int)blockIdx.y * RUN;
  int ke = min(kb + RUN, k0 + nk);
  long long row = (long long)jy * job.pitch + i;
#pragma unroll 1
  for (int k = kb; k < ke; ++k) {
    float z = s2_coord(job, k);
    ring[(long long)(k % job.ring) * job.plane + row] = s2m_user_sdf(x, y, z);
  }
}

#define S2_EVAL_VARIANT(NAME, MINB, RUN)                                                          \
  extern "C" __global__ void __launch_bounds__(S2_EVAL_BLOCK, MINB)                               \
  NAME(S2Job job, float *__restrict__ ring, int k0, int nk) { s2_eval_planes<RUN>(job, ring, k0, nk); }
// Keep this table in step with kEvalVariants in runtime.cu.
S2_EVAL_VARIANT(s2m_eval_b2r4, 2, 4)
S2_EVAL_VARIANT(s2m_eval_b3r4, 3, 4)
S2_EVAL_VARIANT(s2m_eval_b4r4, 4, 4)
S2_EVAL_VARIANT(s2m_eval_b4r1, 4, 1)
S2_EVAL_VARIANT(s2m_eval_b6r4, 6, 4)
S2_EVAL_VARIANT(s2m_eval_b8r4, 8, 4)

struct S2Cell {
  int x, y, z;
};

__device__ __forceinline__ S2Cell s2_cell_of(const S2Job &j, long long c, int zc0) {
  S2Cell r;
  r.x = (int)(c % j.N);
  long long q = c / j.N;
  r.y = (int)(q % j.N);
  r.z = zc0 + (int)(q / j.N);
  return r;
}

// The 8 lattice values of a cell, corner index bx | by << 1 | bz << 2.
__device__ __forceinline__ void s2_load_corners(const S2Job &j, const float *__restrict__ ring, S2Cell c, float v[8]) {
  const float *p0 = ring + (long long)(c.z % j.ring) * j.plane + (long long)c.y * j.pitch + c.x;
  const float *p1 = ring + (long long)((c.z + 1) % j.ring) * j.plane + (long long)c.y * j.pitch + c.x;
  v[0] = __ldg(p0);
  v[1] = __ldg(p0 + 1);
  v[2] = __ldg(p0 + j.pitch);
  v[3] = __ldg(p0 + j.pitch + 1);
  v[4] = __ldg(p1);
  v[5] = __ldg(p1 + 1);
  v[6] = __ldg(p1 + j.pitch);
  v[7] = __ldg(p1 + j.pitch + 1);
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
__device__ __forceinline__ bool s2_classify(const S2Job &j, const float *__restrict__ ring, S2Cell c) {
  float v[8];
  s2_load_corners(j, ring, c, v);
  unsigned pos = 0;
  for (int k = 0; k < 8; ++k) pos |= (v[k] > 0.0f ? 1u : 0u) << k;
  if (pos != 0u && pos != 0xffu) return true;
  unsigned off = s2_off_mask(j, c);
  if (!off) return false;
  if (j.exact) return true;
  for (int k = 1; k < 8; ++k)
    if ((off >> k) & 1u)
      if (!(fabsf(v[k]) >= j.guard)) return true;
  return false;
}

// dualcontour.wgsl:72-131 (crossings, counting rule, mass point) and
// :161-180 (normal, sign bits) on one candidate cell.  `v` holds the cell's
// lattice values; corners whose reference coordinates are off the lattice are
// re-evaluated here at those coordinates, so the rule sees exactly the
// reference's 8 values.  Writes the vertex and returns the final key
// (x | y << 16 | label << 32 | signs << 48 | has_vertex << 63).
__device__ __forceinline__ unsigned long long s2_vertex(const S2Job &j, S2Cell c, float v[8], float pos[3],
                                                        float nrm[3]) {
  float mn[3] = {s2_coord(j, c.x), s2_coord(j, c.y), s2_coord(j, c.z)};
  float mx[3] = {__fadd_rn(mn[0], j.size), __fadd_rn(mn[1], j.size), __fadd_rn(mn[2], j.size)};
  // Off-lattice corners, one sdf3d call site in a loop (a warp runs the
  // largest count among its lanes instead of every inlined copy).
  unsigned off = s2_off_mask(j, c) & 0xfeu;
#pragma unroll 1
  while (off) {
    const int k = __ffs(off) - 1;
    off &= off - 1u;
    const float f = s2m_user_sdf((k & 1) ? mx[0] : mn[0], (k & 2) ? mx[1] : mn[1], (k & 4) ? mx[2] : mn[2]);
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
#ifdef S2M_STD_NORMAL
  // sdf3d_normal.wgsl:4-10 as a loop: n = ((t0 + t1) + t2) + t3 with
  // t_i = d_i * sdf3d(p + d_i * eps), the order the library function adds in.
  s2v3 n;
#pragma unroll 1
  for (int i = 0; i < 4; ++i) {
    const float dx = (i == 0 || i == 3) ? 1.0f : -1.0f;
    const float dy = (i >= 2) ? 1.0f : -1.0f;
    const float dz = (i == 1 || i == 3) ? 1.0f : -1.0f;
    const float f = s2m_user_sdf(__fadd_rn(pos[0], __fmul_rn(dx, j.eps)), __fadd_rn(pos[1], __fmul_rn(dy, j.eps)),
                                 __fadd_rn(pos[2], __fmul_rn(dz, j.eps)));
    const float tx = __fmul_rn(dx, f), ty = __fmul_rn(dy, f), tz = __fmul_rn(dz, f);
    if (i == 0) {
      n.x = tx; n.y = ty; n.z = tz;
    } else {
      n.x = __fadd_rn(n.x, tx); n.y = __fadd_rn(n.y, ty); n.z = __fadd_rn(n.z, tz);
    }
  }
#else
  s2v3 n = s2m_user_normal(s2mk(pos[0], pos[1], pos[2]), j.eps);
#endif
  float len = __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(n.x, n.x), __fmul_rn(n.y, n.y)), __fmul_rn(n.z, n.z)));
  nrm[0] = __fdiv_rn(n.x, len);
  nrm[1] = __fdiv_rn(n.y, len);
  nrm[2] = __fdiv_rn(n.z, len);
  return key | (1ull << 63);
}

// Cell pass of one slab (cell slices zc0 .. zc1 - 1): classify every cell and
// append the candidates, in (z, y, x) order, to the job's candidate list at
// cand.base[slab] + (look-back prefix over tiles), each with its 8 lattice
// corner values.  The last tile publishes cand.base[slab + 1].
extern "C" __global__ void __launch_bounds__(S2_CELL_BLOCK)
s2m_cells(S2Job job, S2Slab slab, S2Cand cand, int zc0, int zc1, int slab_index) {
  __shared__ unsigned s_tile;
  __shared__ unsigned s_warp[32];
  __shared__ unsigned long long s_excl;
  const unsigned tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
  if (tid == 0) s_tile = atomicAdd(slab.tile_counter, 1u);
  __syncthreads();
  const unsigned tile = s_tile;
  const long long ncells = (long long)(zc1 - zc0) * job.N * job.N;
  const unsigned ntiles = (unsigned)((ncells + S2_CELL_TILE - 1) / S2_CELL_TILE);
  if (tile >= ntiles) return;
  const unsigned long long base = cand.base[slab_index];

  unsigned ballots[S2_CELL_CPT];
#pragma unroll
  for (int m = 0; m < S2_CELL_CPT; ++m) {
    long long c = (long long)tile * S2_CELL_TILE + m * S2_CELL_BLOCK + tid;
    bool is_cand = c < ncells && s2_classify(job, slab.ring, s2_cell_of(job, c, zc0));
    ballots[m] = __ballot_sync(S2_FULL, is_cand);
    if (lane == 0) s_warp[m * 8 + warp] = __popc(ballots[m]);
  }
  __syncthreads();
  if (warp == 0) {
    unsigned tot = s2_warp_exclusive32(s_warp);
    unsigned long long excl = s2_lookback(slab.status, tile, tot, slab.err);
    if (lane == 0) {
      s_excl = excl;
      if (tile == ntiles - 1) cand.base[slab_index + 1] = base + excl + tot;
    }
  }
  __syncthreads();
  const unsigned lt = s2_lanemask_lt();
#pragma unroll
  for (int m = 0; m < S2_CELL_CPT; ++m) {
    if (!((ballots[m] >> lane) & 1u)) continue;
    unsigned long long o = base + s_excl + s_warp[m * 8 + warp] + __popc(ballots[m] & lt);
    if (o >= cand.cap) {
      atomicOr(slab.err, S2_ERR_CAND_OVF);
      continue;
    }
    long long c = (long long)tile * S2_CELL_TILE + m * S2_CELL_BLOCK + tid;
    S2Cell cell = s2_cell_of(job, c, zc0);
    float v[8];
    s2_load_corners(job, slab.ring, cell, v);
    cand.key[o] = (unsigned long long)cell.x | ((unsigned long long)cell.y << 16) | ((unsigned long long)cell.z << 32);
    float4 *dst = reinterpret_cast<float4 *>(cand.val + 8 * o);
    dst[0] = make_float4(v[0], v[1], v[2], v[3]);
    dst[1] = make_float4(v[4], v[5], v[6], v[7]);
  }
}

// Vertices of every candidate of the job, one candidate per thread (dense:
// candidates are a small fraction of the cells).  Rewrites cand.key with the
// final key and writes cand.pos / cand.nrm for cells with a vertex.
extern "C" __global__ void __launch_bounds__(S2_VX_BLOCK)
s2m_vertices(S2Job job, S2Cand cand, int nslabs) {
  const unsigned long long n = min(cand.base[nslabs], cand.cap);
  for (unsigned long long o = (unsigned long long)blockIdx.x * S2_VX_BLOCK + threadIdx.x; o < n;
       o += (unsigned long long)gridDim.x * S2_VX_BLOCK) {
    unsigned long long k = cand.key[o];
    S2Cell c;
    c.x = (int)(k & 0xffffull);
    c.y = (int)((k >> 16) & 0xffffull);
    c.z = (int)((k >> 32) & 0xffffull);
    const float4 *src = reinterpret_cast<const float4 *>(cand.val + 8 * o);
    float4 a = src[0], b = src[1];
    float v[8] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
    float pos[3], nrm[3];
    unsigned long long key = s2_vertex(job, c, v, pos, nrm);
    cand.key[o] = key;
    if (key >> 63) {
      cand.pos[3 * o] = pos[0];
      cand.pos[3 * o + 1] = pos[1];
      cand.pos[3 * o + 2] = pos[2];
      cand.nrm[3 * o] = nrm[0];
      cand.nrm[3 * o + 1] = nrm[1];
      cand.nrm[3 * o + 2] = nrm[2];
    }
  }
}
