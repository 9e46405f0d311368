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
// reference coordinates (s2m_vertices), so the vertex rule sees exactly the
// reference's 8 values.  All arithmetic of the vertex rule uses explicitly
// rounded binary32 intrinsics (no contraction, whatever the SDF's flags).

// One out-of-line copy of the SDF for the vertex kernels: they evaluate it at
// several call sites (off-lattice corners, normal samples, crossings), and
// inlining each would multiply a large body beyond the instruction cache.
__device__ __noinline__ float s2_user_sdf_call(float x, float y, float z) { return s2m_user_sdf(x, y, z); }

struct S2UserSdfCall {
#ifdef S2M_STD_NORMAL
  static constexpr bool kStdNormal = true;
#else
  static constexpr bool kStdNormal = false;
#endif
  __device__ __forceinline__ float operator()(float x, float y, float z) const { return s2_user_sdf_call(x, y, z); }
  __device__ __forceinline__ void normal(float px, float py, float pz, float eps, float n[3]) const {
#ifdef S2M_STD_NORMAL
    s2_tetra_normal(*this, px, py, pz, eps, n);
#else
    s2v3 r = s2m_user_normal(s2mk(px, py, pz), eps);
    n[0] = r.x; n[1] = r.y; n[2] = r.z;
#endif
  }
};

// The lowered user SDF as the evaluator of s2m_dc_core.cuh.
struct S2UserSdf {
#ifdef S2M_STD_NORMAL
  static constexpr bool kStdNormal = true;
#else
  static constexpr bool kStdNormal = false;
#endif
  __device__ __forceinline__ float operator()(float x, float y, float z) const { return s2m_user_sdf(x, y, z); }
  __device__ __forceinline__ void normal(float px, float py, float pz, float eps, float n[3]) const {
#ifdef S2M_STD_NORMAL
    s2_tetra_normal(*this, px, py, pz, eps, n);
#else
    s2v3 r = s2m_user_normal(s2mk(px, py, pz), eps);
    n[0] = r.x; n[1] = r.y; n[2] = r.z;
#endif
  }
};

// Evaluate planes k0 .. k0 + nk - 1 of the lattice into the ring.
// grid.x covers the P * P points of a plane, grid.y runs of RUN planes; each
// thread walks its run along z.  The variants below differ only in RUN and in
// the occupancy the compiler must allow (__launch_bounds__ minimum blocks),
// which trades registers against latency hiding; the runtime's autotuner
// times them per SDF and keeps the fastest.
template <int RUN, bool VEC>
__device__ __forceinline__ void s2_eval_planes(const S2Job &job, float *__restrict__ ring, int k0, int nk) {
  const unsigned idx = blockIdx.x * S2_EVAL_BLOCK + threadIdx.x;  // P * P < 2^32
  const unsigned pts = (unsigned)job.P * (unsigned)job.P;
  if (idx >= pts) return;
  const int jy = (int)s2_udiv(idx, (unsigned)job.P, job.magic_p);
  const int i = (int)(idx - (unsigned)jy * (unsigned)job.P);
  float x = s2_coord(job, i), y = s2_coord(job, jy);
  int kb = k0 + (int)blockIdx.y * RUN;
  int ke = min(kb + RUN, k0 + nk);
  long long row = (long long)jy * job.pitch + i;
  int k = kb;
#ifdef S2M_HAS_RUN4
  if (VEC) {
    // 4 planes at once: the x/y-only part of the SDF once, the rest per lane
#pragma unroll 1
    for (; k + 3 < ke; k += 4) {
      s2x4 z, f;
#pragma unroll
      for (int w = 0; w < 4; ++w) z.v[w] = s2_coord(job, k + w);
      s2m_user_sdf_run4(x, y, z, f);
#pragma unroll
      for (int w = 0; w < 4; ++w) ring[(long long)((k + w) % job.ring) * job.plane + row] = f.v[w];
    }
  }
#endif
#pragma unroll 1
  for (; k < ke; ++k) {
    float z = s2_coord(job, k);
    ring[(long long)(k % job.ring) * job.plane + row] = s2m_user_sdf(x, y, z);
  }
}

#define S2_EVAL_VARIANT(NAME, MINB, RUN, PAIR)                                                    \
  extern "C" __global__ void __launch_bounds__(S2_EVAL_BLOCK, MINB)                               \
  NAME(S2Job job, float *__restrict__ ring, int k0, int nk) {                                        \
    S2_PDL_WAIT();                                                                                 \
    s2_eval_planes<RUN, PAIR>(job, ring, k0, nk);                                                  \
  }
// Kernel selection: the runtime compiles an SDF's kernels as several NVRTC
// programs on parallel host threads.  Each program defines S2M_SELECT and the
// S2M_WANT_* macros of the kernels it holds; a program without S2M_SELECT
// holds them all.
// Keep this table in step with kEvalVariants in runtime.cu.
#ifndef S2M_QEF_MODULE
#if !defined(S2M_SELECT) || defined(S2M_WANT_EVAL_B2R4)
S2_EVAL_VARIANT(s2m_eval_b2r4, 2, 4, false)
#endif
#if !defined(S2M_SELECT) || defined(S2M_WANT_EVAL_B3R4)
S2_EVAL_VARIANT(s2m_eval_b3r4, 3, 4, false)
#endif
#if !defined(S2M_SELECT) || defined(S2M_WANT_EVAL_B4R4)
S2_EVAL_VARIANT(s2m_eval_b4r4, 4, 4, false)
#endif
#if !defined(S2M_SELECT) || defined(S2M_WANT_EVAL_B2V4)
S2_EVAL_VARIANT(s2m_eval_b2v4, 2, 4, true)
#endif
#if !defined(S2M_SELECT) || defined(S2M_WANT_EVAL_B3V4)
S2_EVAL_VARIANT(s2m_eval_b3v4, 3, 4, true)
#endif
#endif

#if defined(S2M_HAS_PRUNE) && !defined(S2M_QEF_MODULE)
// Tile pruning (the generated s2m_user_sdf_tile / s2m_user_sdf_pruned).
// Slab s evaluates planes k0 .. k0 + nk - 1 (s2_slab_planes: from the job's
// first cell plane zb).  Its planes are cut
// into tiles of 8 x 8 points by `tzs` planes (at most S2_PT_ZMAX, balanced),
// nzt tiles in z; tile t = (tz * nty + ty) * ntx + tx.  slab_base[s] is the
// index of slab s's first tile among all tiles of the job.  (s2_slab_planes,
// s2_tile_depth and s2_cell_prune_tile are in s2m_dc_core.cuh.)

struct S2PruneTile {
  int i0, i1, j0, j1, kb, ke;  // inclusive point ranges
};

// A tile's record: S2M_PRUNE_WORDS activity words, then a flag word.  Flag
// S2_TILE_DECIDED: the interval of the SDF's value over the tile's box lies
// at or beyond +guard (with S2_TILE_POSITIVE) or -guard, so every point's
// sign bit is known and its near-zero bit is 0 -- all that classification
// reads -- and the points are not evaluated.  Their values are not written:
// their unknown-value bits (S2PointBits::unk) are set instead, the candidate
// records get NaN for such corners, and the vertex kernel evaluates those
// exactly, so the mesh does not change.
#define S2M_TILE_WORDS (S2M_PRUNE_WORDS + 1)
// v = (c * n + b) * n + a with a, b < n: (a, b, c), in 32-bit arithmetic when
// v fits (a 64-bit division is a long instruction sequence).
__device__ __forceinline__ void s2_split3(long long v, int n, int &a, int &b, int &c) {
  if (v >= 0 && v < 0x100000000ll) {
    const unsigned u = (unsigned)v, un = (unsigned)n, q = u / un;
    a = (int)(u - q * un);
    b = (int)(q % un);
    c = (int)(q / un);
  } else {
    a = (int)(v % n);
    const long long q = v / n;
    b = (int)(q % n);
    c = (int)(q / n);
  }
}
__device__ __forceinline__ S2PruneTile s2_prune_tile(const S2Job &job, long long t, int k0, int nk, int tzs) {
  const int ntx = (job.P + S2_PT_XY - 1) / S2_PT_XY;
  S2PruneTile r;
  int tx, ty, tz;
  s2_split3(t, ntx, tx, ty, tz);
  r.i0 = tx * S2_PT_XY;
  r.i1 = min(r.i0 + S2_PT_XY, job.P) - 1;
  r.j0 = ty * S2_PT_XY;
  r.j1 = min(r.j0 + S2_PT_XY, job.P) - 1;
  r.kb = k0 + tz * tzs;
  r.ke = min(r.kb + tzs, k0 + nk) - 1;
  return r;
}

// The tile pass of slabs s_begin .. s_end - 1, in two launches of one thread
// per box, each covering many slabs so that the grid fills the GPU:
//   s2m_tiles_coarse  boxes of 4 x 4 tiles by 2 layers of tiles (32 x 32
//                     points by twice the tile depth): the full interval
//                     evaluation -> sbits and the box's flag word
//   s2m_tiles         each tile inside its coarse box: only the segments
//                     active in the box are evaluated -> bits, and the SDF
//                     operations that remain (ops[0] FP32, ops[1] SFU, per
//                     lattice point).  A tile of a decided box is decided
//                     with it (the box's interval bounds every point of the
//                     tile's box) and takes the box's bits, without an
//                     evaluation of its own.
// Coarse box c of the job is at sbits[(c - cbase[s_begin]) * S2M_TILE_WORDS],
// tile g at bits[(g - tbase[s_begin]) * S2M_TILE_WORDS]; cbase / tbase hold
// each slab's first index.
// Coordinate range of a tile's box along one axis: lattice indices a .. b,
// widened by a margin.  The boxes reach one lattice point past the tile's
// points in +x, +y and -z, and the margin (more than the normal epsilon plus
// thousands of ulps of the coordinates) covers every point the vertex kernel
// evaluates for the cells whose tile this is (cell x in [i0, i1] spans points
// x .. x + 1; cell z with plane z + 1 in the tile spans z .. z + 1): the
// off-lattice corners mn + size and the normal samples p +/- eps around a
// vertex inside its cell.  So the bits serve both the lattice evaluation and
// the vertices.
__device__ __forceinline__ s2i s2_prune_box(const S2Job &job, int a, int b) {
  const float mg = __fadd_rn(__fmul_rn(fabsf(job.eps), 1.0625f),
                             __fmul_rn(__fadd_rn(fabsf(job.bmin), fabsf(job.size)), 0x1p-12f));
  s2i r;
  r.lo = __fsub_rn(s2_coord(job, a), mg);
  r.hi = __fadd_rn(s2_coord(job, b), mg);
  return r;
}

__device__ __forceinline__ int s2_find_slab(const unsigned long long *base, int s_begin, int s_end,
                                            unsigned long long g) {
  int lo = s_begin, hi = s_end - 1;  // largest s with base[s] <= g
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (base[mid] <= g) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// S2_TILE_DECIDED (| S2_TILE_POSITIVE) when a box's root interval lies at or
// beyond +-guard; 0 otherwise, and for an unknown (NaN) interval.
__device__ __forceinline__ unsigned s2_root_flag(const S2Job &job, s2i root) {
  if (root.lo >= job.guard) return S2_TILE_DECIDED | S2_TILE_POSITIVE;
  if (root.hi <= -job.guard) return S2_TILE_DECIDED;
  return 0u;
}

#if !defined(S2M_SELECT) || defined(S2M_WANT_TILES_COARSE)
extern "C" __global__ void __launch_bounds__(S2_PT_BLOCK, 8)
s2m_tiles_coarse(S2Job job, unsigned *__restrict__ sbits, const unsigned long long *__restrict__ cbase, int s_begin,
                 int s_end, int D, int nzc) {
  S2_PDL_WAIT();
  const unsigned long long b0 = cbase[s_begin];
  const unsigned long long c = b0 + (unsigned long long)blockIdx.x * S2_PT_BLOCK + threadIdx.x;
  if (c >= cbase[s_end]) return;
  const int s = s2_find_slab(cbase, s_begin, s_end, c);
  int k0, nk;
  s2_slab_planes(job, s, D, nzc, k0, nk);
  const int tzs = s2_tile_depth(nk);
  const int ntx = (job.P + S2_PT_XY - 1) / S2_PT_XY;
  const int ncx = (ntx + S2_PT_COARSE - 1) / S2_PT_COARSE;
  int cx, cy, cz;
  s2_split3((long long)(c - cbase[s]), ncx, cx, cy, cz);
  const int span = S2_PT_XY * S2_PT_COARSE;
  const int i0 = cx * span, i1 = min(i0 + span, job.P) - 1;
  const int j0 = cy * span, j1 = min(j0 + span, job.P) - 1;
  const int kb = k0 + cz * S2_PT_COARSE_Z * tzs, ke = min(kb + S2_PT_COARSE_Z * tzs, k0 + nk) - 1;
  const s2i X = s2_prune_box(job, i0, i1 + 1), Y = s2_prune_box(job, j0, j1 + 1), Z = s2_prune_box(job, kb - 1, max(kb, ke));
  unsigned m[S2M_PRUNE_WORDS];
  float fp, sfu;
  s2i root;
  s2m_user_sdf_tile(X, Y, Z, m, &fp, &sfu, &root);
  unsigned *dst = sbits + (c - b0) * S2M_TILE_WORDS;
#pragma unroll
  for (int w = 0; w < S2M_PRUNE_WORDS; ++w) dst[w] = m[w];
  dst[S2M_PRUNE_WORDS] = s2_root_flag(job, root);
}
#endif  // S2M_WANT_TILES_COARSE

#if !defined(S2M_SELECT) || defined(S2M_WANT_TILES_FINE)
extern "C" __global__ void __launch_bounds__(S2_PT_BLOCK, 8)
s2m_tiles(S2Job job, unsigned *__restrict__ bits, unsigned long long *__restrict__ ops,
          const unsigned *__restrict__ sbits, const unsigned long long *__restrict__ tbase,
          const unsigned long long *__restrict__ cbase, int s_begin, int s_end, int D, int nzc,
          unsigned *__restrict__ list, unsigned *__restrict__ list_count, unsigned char *__restrict__ tflags,
          int fpitch) {
  S2_PDL_WAIT();
  // Thread q takes tile q % kPerBox (S2_PT_COARSE x S2_PT_COARSE along x, y,
  // by S2_PT_COARSE_Z layers along z: 32 tiles) of coarse box q / kPerBox,
  // so a warp's tiles share one box's bits and take one path through the
  // interval code.
  constexpr unsigned kPerBox = S2_PT_COARSE * S2_PT_COARSE * S2_PT_COARSE_Z;
  const unsigned long long b0 = tbase[s_begin];
  const unsigned long long q = (unsigned long long)blockIdx.x * S2_PT_BLOCK + threadIdx.x;
  const unsigned long long c = cbase[s_begin] + q / kPerBox;
  const unsigned sub = (unsigned)(q % kPerBox);
  const int ntx = (job.P + S2_PT_XY - 1) / S2_PT_XY;
  const int ncx = (ntx + S2_PT_COARSE - 1) / S2_PT_COARSE;
  int tx = 0, ty = 0, tz = 0, s = s_begin;
  bool live = c < cbase[s_end];
  if (live) {
    s = s2_find_slab(cbase, s_begin, s_end, c);
    int k0s, nks;
    s2_slab_planes(job, s, D, nzc, k0s, nks);
    const int tzs = s2_tile_depth(nks), nzt = (nks + tzs - 1) / tzs;
    int cx, cy, cz;
    s2_split3((long long)(c - cbase[s]), ncx, cx, cy, cz);
    tx = cx * S2_PT_COARSE + (int)(sub % S2_PT_COARSE);
    ty = cy * S2_PT_COARSE + (int)((sub / S2_PT_COARSE) % S2_PT_COARSE);
    tz = cz * S2_PT_COARSE_Z + (int)(sub / (S2_PT_COARSE * S2_PT_COARSE));
    live = tx < ntx && ty < ntx && tz < nzt;
  }
  unsigned long long fp_ops = 0, sfu_ops = 0;
  if (live) {
    int k0, nk;
    s2_slab_planes(job, s, D, nzc, k0, nk);
    const long long t = ((long long)tz * ntx + ty) * ntx + tx;
    const unsigned long long g = tbase[s] + (unsigned long long)t;
    const S2PruneTile tl = s2_prune_tile(job, t, k0, nk, s2_tile_depth(nk));
    const unsigned *pm = sbits + (c - cbase[s_begin]) * S2M_TILE_WORDS;
    unsigned m[S2M_PRUNE_WORDS];
    float fp = 0.0f, sfu = 0.0f;
    unsigned flag = pm[S2M_PRUNE_WORDS];
    if (flag) {
#pragma unroll
      for (int w = 0; w < S2M_PRUNE_WORDS; ++w) m[w] = pm[w];
    } else {
      const s2i X = s2_prune_box(job, tl.i0, tl.i1 + 1), Y = s2_prune_box(job, tl.j0, tl.j1 + 1),
                Z = s2_prune_box(job, tl.kb - 1, max(tl.kb, tl.ke));
      s2i root;
      s2m_user_sdf_tile_in(X, Y, Z, pm, m, &fp, &sfu, &root);
      flag = s2_root_flag(job, root);
    }
    if (flag) fp = sfu = 0.0f;  // nothing of the SDF is evaluated there
    unsigned *dst = bits + (g - b0) * S2M_TILE_WORDS;
#pragma unroll
    for (int w = 0; w < S2M_PRUNE_WORDS; ++w) dst[w] = m[w];
    dst[S2M_PRUNE_WORDS] = flag;
    // the flag as a byte, rows of fpitch bytes per (layer, tile row) of the
    // chunk; bytes past the last tile of a row read S2_TILE_DECIDED (they
    // cover no cell)
    unsigned char *frow = tflags + (g - b0) / (unsigned long long)ntx * (unsigned long long)fpitch;
    frow[tx] = (unsigned char)(flag & (S2_TILE_DECIDED | S2_TILE_POSITIVE));
    if (tx == ntx - 1)
      for (int x = ntx; x < fpitch; ++x) frow[x] = (unsigned char)S2_TILE_DECIDED;
    // the slab's list of tiles to evaluate (in any order): one atomic per slab
    // and warp, since every thread of a slab adds to the same counter
    const unsigned am = __activemask();
    const unsigned und = __ballot_sync(am, !flag);
    if (!flag) {
      const unsigned peers = __match_any_sync(und, s);
      const int leader = __ffs(peers) - 1;
      unsigned first = 0;
      if ((int)(threadIdx.x & 31u) == leader) first = atomicAdd(list_count + s, (unsigned)__popc(peers));
      first = __shfl_sync(peers, first, leader);
      const unsigned i = first + (unsigned)__popc(peers & s2_lanemask_lt());
      list[(tbase[s] - b0) + i] = (unsigned)t;
    }
    const unsigned long long npts = (unsigned long long)(tl.i1 - tl.i0 + 1) * (unsigned long long)(tl.j1 - tl.j0 + 1) *
                                    (unsigned long long)max(0, tl.ke - tl.kb + 1);
    fp_ops = (unsigned long long)fp * npts;
    sfu_ops = (unsigned long long)sfu * npts;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    fp_ops += __shfl_down_sync(0xffffffffu, fp_ops, o);
    sfu_ops += __shfl_down_sync(0xffffffffu, sfu_ops, o);
  }
  if ((threadIdx.x & 31u) == 0 && (fp_ops | sfu_ops)) {
    atomicAdd(ops, fp_ops);
    atomicAdd(ops + 1, sfu_ops);
  }
}
#endif  // S2M_WANT_TILES_FINE

// Point bits of one warp-wide step of a tile: the 32 lanes hold 8 points
// along x times 4 rows from `y0` in the plane at ring slot `slot`, so each
// ballot holds one byte (8 points) per row.  Lanes 0-3 store the sign bytes
// of rows y0 .. y0 + 3, lanes 4-7 the near-zero bytes, lanes 8-11 the
// unknown-value bytes.
__device__ __forceinline__ void s2_tile_bits(const S2Job &job, S2PointBits pb, const S2PruneTile &tl, int y0,
                                             int slot, bool is_pos, bool is_near, bool is_unk) {
  const unsigned pos = __ballot_sync(S2_FULL, is_pos);
  const unsigned near = __ballot_sync(S2_FULL, is_near);
  const unsigned unk = __ballot_sync(S2_FULL, is_unk);
  const int lane = (int)(threadIdx.x & 31u);
  const int r = lane & 3, y = y0 + r;
  if (lane < 12 && y <= tl.j1) {
    const int WP = (job.P + 31) >> 5;
    unsigned char *base = reinterpret_cast<unsigned char *>(lane < 4 ? pb.pos : lane < 8 ? pb.near : pb.unk);
    base[(((long long)slot * job.P + y) * WP) * 4 + (tl.i0 >> 3)] =
        (unsigned char)(((lane < 4 ? pos : lane < 8 ? near : unk) >> (8 * r)) & 0xffu);
  }
}

// Pruned evaluation of one tile by one warp, writing the values and their
// point bits.  Lane l takes x = i0 + l % 8 and the rows j0 + l / 8 and
// j0 + l / 8 + 4, and walks the tile's planes (RUN4: runs of 4 planes, which
// share the bit tests and the x/y-only arithmetic; a run past the tile's last
// plane repeats that plane and stores only its own planes).  `m` (shared
// memory) holds the tile's activity bits, the same for the whole warp, so the
// pruned function's branches never diverge and every lane takes part in the
// ballots.  Points past the lattice edge (tiles are 8 x 8) evaluate a
// clamped point and store nothing.
template <bool RUN4>
__device__ __forceinline__ void s2_eval_tile(const S2Job &job, float *__restrict__ ring, S2PointBits pb,
                                             const S2PruneTile &tl, const unsigned *m) {
  const int lane = (int)(threadIdx.x & 31u);
  const int i = tl.i0 + (lane & 7), ja = tl.j0 + (lane >> 3);
  const unsigned flag = m[S2M_PRUNE_WORDS];
  if (flag & S2_TILE_DECIDED) {  // the same on the whole warp: bits only, no values
    const bool pos = (flag & S2_TILE_POSITIVE) != 0u;
    int slot = tl.kb % job.ring;
#pragma unroll 1
    for (int k = tl.kb; k <= tl.ke; ++k) {
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int j = ja + 4 * h;
        const bool store = i <= tl.i1 && j <= tl.j1;
        s2_tile_bits(job, pb, tl, tl.j0 + 4 * h, slot, store && pos, false, store);
      }
      if (++slot == job.ring) slot = 0;
    }
    return;
  }
  const float x = s2_coord(job, min(i, tl.i1));
  const float y0 = s2_coord(job, min(ja, tl.j1)), y1 = s2_coord(job, min(ja + 4, tl.j1));
  const bool xin = i <= tl.i1;
  float *const col = ring + (long long)min(i, tl.i1);
  int slot = tl.kb % job.ring;  // the tile spans at most S2_PT_ZMAX <= ring planes
  if (RUN4) {
#pragma unroll 1
    for (int k = tl.kb; k <= tl.ke; k += 4) {
      s2x4 z;
#pragma unroll
      for (int w = 0; w < 4; ++w) z.v[w] = s2_coord(job, min(k + w, tl.ke));
#pragma unroll 1
      for (int h = 0; h < 2; ++h) {
        const int j = ja + 4 * h;
        const bool store = xin && j <= tl.j1;
        const s2x4 f = s2m_user_sdf_pruned_run4(x, h ? y1 : y0, z, m);
        int sw = slot;
#pragma unroll
        for (int w = 0; w < 4; ++w) {
          if (k + w <= tl.ke) {  // the same on every lane
            if (store) col[(long long)sw * job.plane + (long long)j * job.pitch] = f.v[w];
            s2_tile_bits(job, pb, tl, tl.j0 + 4 * h, sw, store && f.v[w] > 0.0f,
                         store && !(fabsf(f.v[w]) >= job.guard), false);
          }
          if (++sw == job.ring) sw = 0;
        }
      }
      slot += 4;
      if (slot >= job.ring) slot -= job.ring;
    }
    return;
  }
#pragma unroll 1
  for (int k = tl.kb; k <= tl.ke; ++k) {
    const float z = s2_coord(job, k);
#pragma unroll 1
    for (int h = 0; h < 2; ++h) {
      const int j = ja + 4 * h;
      const bool store = xin && j <= tl.j1;
      const float f = s2m_user_sdf_pruned(x, h ? y1 : y0, z, m);
      if (store) col[(long long)slot * job.plane + (long long)j * job.pitch] = f;
      s2_tile_bits(job, pb, tl, tl.j0 + 4 * h, slot, store && f > 0.0f, store && !(fabsf(f) >= job.guard), false);
    }
    if (++slot == job.ring) slot = 0;
  }
}

// One tile per warp, 4 warps per block, tile t = block * 4 + warp.
template <bool RUN4>
__device__ __forceinline__ void s2_eval_pruned(const S2Job &job, float *__restrict__ ring, S2PointBits pb,
                                               const unsigned *__restrict__ bits, int k0, int nk, int tzs, int nzt) {
  const int ntx = (job.P + S2_PT_XY - 1) / S2_PT_XY;
  const long long ntiles = (long long)ntx * ntx * nzt;
  const long long t = (long long)blockIdx.x * (S2_PT_BLOCK / 32) + (threadIdx.x >> 5);
  if (t >= ntiles) return;
  const S2PruneTile tl = s2_prune_tile(job, t, k0, nk, tzs);
  if (tl.kb > tl.ke) return;
  __shared__ unsigned s_bits[S2_PT_BLOCK / 32][S2M_TILE_WORDS];
  const int lane = (int)(threadIdx.x & 31u);
  if (lane < S2M_TILE_WORDS) s_bits[threadIdx.x >> 5][lane] = __ldg(bits + t * S2M_TILE_WORDS + lane);
  __syncwarp();
  s2_eval_tile<RUN4>(job, ring, pb, tl, s_bits[threadIdx.x >> 5]);
}

// The listed form: only the slab's undecided tiles (the tile pass's list),
// one per warp; s2m_fill_decided has written the decided ones.  Every warp
// then has real work, so the blocks are about equally long.
template <bool RUN4>
__device__ __forceinline__ void s2_eval_pruned_listed(const S2Job &job, float *__restrict__ ring, S2PointBits pb,
                                                      const unsigned *__restrict__ bits, int k0, int nk, int tzs,
                                                      const unsigned *__restrict__ list,
                                                      const unsigned *__restrict__ list_count, unsigned *chunk_ctr) {
  // The list's length is known only on the device.  One block of S2_PL_BLOCK
  // threads per SM takes chunks of S2_PL_BLOCK / 32 consecutive listed tiles
  // from `chunk_ctr` (zero at launch), one tile per warp: every warp on an SM
  // then runs neighbouring tiles, whose pruned paths share code.  (With 16
  // blocks of 4 warps per SM striding over the list, the SM's warps ran 64
  // different places of the pruned SDF and stalled on instruction fetch.)
  __shared__ unsigned s_bits[S2_PL_BLOCK / 32][S2M_TILE_WORDS];
  __shared__ unsigned s_chunk;
  const int lane = (int)(threadIdx.x & 31u);
  const unsigned n = __ldg(list_count);
  for (;;) {
    __syncthreads();  // every thread has read the previous chunk's number
    if (threadIdx.x == 0) s_chunk = atomicAdd(chunk_ctr, 1u);
    __syncthreads();
    const unsigned long long first = (unsigned long long)s_chunk * (S2_PL_BLOCK / 32);
    if (first >= n) break;
    const unsigned long long i = first + (threadIdx.x >> 5);  // whole warps
    if (i >= n) continue;
    const unsigned t = __ldg(list + i);
    const S2PruneTile tl = s2_prune_tile(job, (long long)t, k0, nk, tzs);
    if (tl.kb > tl.ke) continue;
    if (lane < S2M_TILE_WORDS) s_bits[threadIdx.x >> 5][lane] = __ldg(bits + (unsigned long long)t * S2M_TILE_WORDS + lane);
    __syncwarp();
    s2_eval_tile<RUN4>(job, ring, pb, tl, s_bits[threadIdx.x >> 5]);
  }
}

#define S2_EVALPL_VARIANT(NAME, MINB, RUN4)                                                       \
  extern "C" __global__ void __launch_bounds__(S2_PL_BLOCK, 1)                                    \
  NAME(S2Job job, float *__restrict__ ring, S2PointBits pb, const unsigned *__restrict__ bits, int k0, int nk,  \
       int tzs, const unsigned *__restrict__ list, const unsigned *__restrict__ list_count,       \
       unsigned *chunk_ctr) {                                                                     \
    S2_PDL_WAIT();                                                                                 \
    s2_eval_pruned_listed<RUN4>(job, ring, pb, bits, k0, nk, tzs, list, list_count, chunk_ctr);   \
  }
#define S2_EVALP_VARIANT(NAME, MINB, RUN4)                                                        \
  extern "C" __global__ void __launch_bounds__(S2_PT_BLOCK, MINB)                                 \
  NAME(S2Job job, float *__restrict__ ring, S2PointBits pb, const unsigned *__restrict__ bits, int k0, int nk,  \
       int tzs, int nzt) {                                                                        \
    S2_PDL_WAIT();                                                                                 \
    s2_eval_pruned<RUN4>(job, ring, pb, bits, k0, nk, tzs, nzt);                                  \
  }
// Keep this table in step with kEvalVariants in runtime.cu.
#if !defined(S2M_SELECT) || defined(S2M_WANT_EVALP_B8)
S2_EVALP_VARIANT(s2m_evalp_b8, 8, false)
#endif
#if !defined(S2M_SELECT) || defined(S2M_WANT_EVALPL_B8)
S2_EVALPL_VARIANT(s2m_evalpl_b8, 8, false)
#endif
#if !defined(S2M_SELECT) || defined(S2M_WANT_EVALPL_B8V4)
S2_EVALPL_VARIANT(s2m_evalpl_b8v4, 8, true)
#endif
#endif



#if defined(S2M_HAS_PRUNE) && !defined(S2M_QEF_MODULE)
// The SDF for the vertex kernel with the lattice evaluation's tile bits:
// lane l's requests use the bits of lane l's cell (the tile boxes cover the
// corners and normal samples of their cells), or the full SDF when it has
// none.
struct S2UserSdfPruned {
  static constexpr bool kStdNormal = S2UserSdfCall::kStdNormal;
  const unsigned *const *mp;  // per lane of the block
  __device__ __forceinline__ float operator()(float x, float y, float z) const { return s2_user_sdf_call(x, y, z); }
  __device__ __forceinline__ float at(unsigned l, float x, float y, float z) const {
    const unsigned *m = mp[(threadIdx.x & ~31u) + l];
    return m ? s2m_user_sdf_pruned(x, y, z, m) : s2_user_sdf_call(x, y, z);
  }
};
__device__ __forceinline__ float s2_sdf_for(const S2UserSdfPruned &f, unsigned l, float x, float y, float z) {
  return f.at(l, x, y, z);
}

// The activity bits of the tile of cell c (all slabs' tiles in one buffer).
__device__ __forceinline__ const unsigned *s2_cell_bits(const S2Job &job, S2Cell c, const unsigned *tbits,
                                                        const unsigned long long *tbase, int D, int nzc) {
  return tbits + s2_cell_prune_tile(job, c, tbase, D, nzc) * S2M_TILE_WORDS;
}
#endif

// Lattice corners left unknown (NaN) by a decided tile of the pruned
// evaluation: evaluated here at their lattice coordinates, exactly as the
// lattice pass would have.  (A corner whose SDF value is NaN is evaluated
// again, to the same NaN.)  For the precision mode and SDFs with their own
// normal; s2_vertex_warp evaluates them with its other requests.
__device__ __forceinline__ void s2_fill_unknown_corners(const S2Job &job, S2Cell c, float v[8]) {
#pragma unroll 1
  for (int k = 0; k < 8; ++k)
    if (v[k] != v[k])
      v[k] = s2_user_sdf_call(s2_coord(job, c.x + (k & 1)), s2_coord(job, c.y + ((k >> 1) & 1)),
                              s2_coord(job, c.z + ((k >> 2) & 1)));
}

// The 8 lattice corners of cell c from a ring that holds every plane of the
// job (one slab), NaN where the point lies in a decided tile of the pruned
// evaluation (its value was never written): tflags holds the tiles' flags as
// bytes, rows of 4 * ceil(P / 32) bytes per (layer, tile row), layers of tzs
// planes from tk0, as the tile pass writes them.
__device__ __forceinline__ void s2_ring_corners(const S2Job &job, const float *__restrict__ ring,
                                                const unsigned char *__restrict__ tflags, int tk0, int tzs, S2Cell c,
                                                float v[8]) {
  const int ntx = (job.P + S2_PT_XY - 1) / S2_PT_XY, fpitch = 4 * ((job.P + 31) >> 5);
  // ring slots and tile layers of planes z and z + 1 (one modulo, one division)
  const int s0 = c.z % job.ring, d0 = c.z - tk0, l0 = d0 / tzs;
  const int sl[2] = {s0, s0 + 1 == job.ring ? 0 : s0 + 1};
  const int ly[2] = {l0, d0 - l0 * tzs + 1 == tzs ? l0 + 1 : l0};
  const bool even = (c.x & 1) == 0;  // the row's two corners as one 8-byte load (rows start 128-byte aligned)
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    const float *p = ring + (long long)sl[h] * job.plane + (long long)c.y * job.pitch + c.x;
    const unsigned char *fr = tflags + (long long)ly[h] * ntx * fpitch;
#pragma unroll
    for (int by = 0; by < 2; ++by) {
      const unsigned char *f = fr + (long long)((c.y + by) >> 3) * fpitch;
      const float *q = p + by * job.pitch;
      float a, b;
      if (even) {
        const float2 t = __ldg(reinterpret_cast<const float2 *>(q));
        a = t.x;
        b = t.y;
      } else {
        a = __ldg(q);
        b = __ldg(q + 1);
      }
      const bool u0 = __ldg(f + (c.x >> 3)) & S2_TILE_DECIDED, u1 = __ldg(f + ((c.x + 1) >> 3)) & S2_TILE_DECIDED;
      v[4 * h + 2 * by] = u0 ? __int_as_float(0x7fc00000) : a;
      v[4 * h + 2 * by + 1] = u1 ? __int_as_float(0x7fc00000) : b;
    }
  }
}

// Vertices of every candidate of the job, one candidate per thread (dense:
// candidates are a small fraction of the cells).  Rewrites cand.key with the
// final key and writes cand.pos / cand.nrm for cells with a vertex.  With
// tbits (tile pruning, every slab's bits resident), the SDF evaluations use
// the bits of each cell's tile, and `perm` (when given) lists the candidates
// grouped by tile (s2m_vtile_*), so that a warp's evaluations take one path
// through the pruned SDF.  (The coarse box's bits, shared by more
// candidates, activate more segments; per-tile bits were faster.)  vc_cnt[t]
// counts the vertices of candidates t * S2_VC_TILE .. (t + 1) * S2_VC_TILE -
// 1 (for s2m_vc_scan).
//   Modules with a pruning form (reference rule): one block of S2_VX_BLOCK
// threads per SM takes chunks of S2_VX_CHUNK consecutive candidates (in tile
// order) from `chunk_ctr` (zero at launch), and its warps take the chunk's
// warp-sized runs from a shared counter as they come free: every warp on an
// SM evaluates neighbouring tiles, whose pruned paths share code, and a warp
// with cheap candidates does not wait at a barrier for one with costly ones
// (one run per warp and chunk left the warps stalled at the chunk's barrier;
// with chunks of 2048, 4096 and 8192 candidates the vertex phase of a 1024^3
// CSG job took 0.415, 0.406 and 0.403 ms).  (With 8 blocks of 128 threads per SM, each taking runs a grid
// stride apart, the SM's warps ran 32 different places of the pruned SDF and
// stalled on instruction fetch.)  Dynamic shared memory: S2_VX_SMEM_BYTES.
// Other modules (full SDF; precision mode, whose per-lane QEF work varies
// too much for a block-wide step): blocks of S2_VX_SMALL threads, 8 per SM,
// striding over the runs.
#if defined(S2M_HAS_PRUNE) && !defined(S2M_QEF_MODULE)
#define S2_VX_CHUNKED 1
#define S2_VX_CHUNK (8 * S2_VX_BLOCK)
#define S2_VX_THREADS S2_VX_BLOCK
#define S2_VX_MINB 1
#else
#define S2_VX_THREADS S2_VX_SMALL
#define S2_VX_MINB 8
#endif
#if !defined(S2M_SELECT) || defined(S2M_WANT_VERTICES)
extern "C" __global__ void __launch_bounds__(S2_VX_THREADS, S2_VX_MINB)
s2m_vertices(S2Job job, S2Cand cand, int nslabs, const unsigned *tbits, const unsigned long long *tbase, int D,
             int nzc, const unsigned *perm, unsigned *vc_cnt, unsigned *chunk_ctr, const float *__restrict__ ring,
             const unsigned char *__restrict__ tflags, int tk0, int tzs) {
  S2_PDL_WAIT();
  const unsigned long long n = min(cand.base[nslabs], cand.cap);
#ifdef S2_VX_CHUNKED
  extern __shared__ __align__(16) unsigned char s2_vx_smem[];
  __shared__ unsigned s_chunk;
  S2WarpScratch *const s_ws = reinterpret_cast<S2WarpScratch *>(s2_vx_smem);
  const unsigned **const s_mp =
      reinterpret_cast<const unsigned **>(s2_vx_smem + sizeof(S2WarpScratch) * (S2_VX_BLOCK / 32));
  S2UserSdfPruned psdf;
  psdf.mp = s_mp;
  __shared__ unsigned s_run;
  constexpr unsigned kRuns = S2_VX_CHUNK / 32;
  const unsigned long long nchunks = (n + S2_VX_CHUNK - 1) / S2_VX_CHUNK;
  for (;;) {
    __syncthreads();  // every thread has read the previous chunk's number and left its runs
    if (threadIdx.x == 0) {
      s_chunk = atomicAdd(chunk_ctr, 1u);
      s_run = 0u;
    }
    __syncthreads();
    const unsigned long long chunk = s_chunk;
    if (chunk >= nchunks) break;
   for (;;) {  // the chunk's warp-sized runs, taken by whichever warp is free
    unsigned run = 0u;
    if ((threadIdx.x & 31u) == 0u) run = atomicAdd(&s_run, 1u);
    run = __shfl_sync(0xffffffffu, run, 0);
    if (run >= kRuns) break;
    const unsigned long long base = chunk * S2_VX_CHUNK + 32ull * run;
#else
  __shared__ S2WarpScratch s_ws[S2_VX_SMALL / 32];
  (void)tbits; (void)tbase; (void)D; (void)nzc; (void)chunk_ctr;
  // grid-stride over warp-sized runs of candidates, all lanes together
  const unsigned long long stride = (unsigned long long)gridDim.x * S2_VX_SMALL;
  for (unsigned long long base = (unsigned long long)blockIdx.x * S2_VX_SMALL + (threadIdx.x & ~31u); base < n;
       base += stride) {
#endif
    const S2UserSdfCall sdf;
    const unsigned long long i = base + (threadIdx.x & 31u);
    const bool active = i < n;
    const unsigned long long o = active && perm ? (unsigned long long)perm[i] : i;
    unsigned long long k = active ? cand.key[o] : 0ull;
    S2Cell c;
    c.x = (int)(k & 0xffffull);
    c.y = (int)((k >> 16) & 0xffffull);
    c.z = (int)((k >> 32) & 0xffffull);
    float v[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    if (active) {
      if (ring) {  // the job's lattice is resident: corners from the ring, NaN in decided tiles
        s2_ring_corners(job, ring, tflags, tk0, tzs, c, v);
      } else {
        const float4 *src = reinterpret_cast<const float4 *>(cand.val + 8 * o);
        const float4 a = src[0], b = src[1];
        v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w; v[4] = b.x; v[5] = b.y; v[6] = b.z; v[7] = b.w;
      }
#ifndef S2M_QEF_MODULE
      if (!S2UserSdfCall::kStdNormal)  // s2_vertex_warp evaluates unknown corners with its requests
#endif
        s2_fill_unknown_corners(job, c, v);
    }
    float pos[3], nrm[3];
    unsigned long long key;
#ifdef S2M_QEF_MODULE
    // precision-mode module (compiled on the first QEF job of this SDF)
    key = active ? s2_vertex_qef(sdf, job, c, v, pos, nrm) : 0ull;
#else
#ifdef S2M_HAS_PRUNE
    if (S2UserSdfCall::kStdNormal && tbits) {
      s_mp[threadIdx.x] = active ? s2_cell_bits(job, c, tbits, tbase, D, nzc) : nullptr;
      __syncwarp();
      key = s2_vertex_warp(psdf, job, active, c, v, pos, nrm, s_ws[threadIdx.x >> 5]);
      __syncwarp();
    } else
#endif
    if (S2UserSdfCall::kStdNormal) key = s2_vertex_warp(sdf, job, active, c, v, pos, nrm, s_ws[threadIdx.x >> 5]);
    else key = active ? s2_vertex(sdf, job, c, v, pos, nrm) : 0ull;
#endif
    {  // one atomic per group of lanes whose candidates share a compaction tile
      const bool has = active && (key >> 63) != 0ull;
      const unsigned long long vt = has ? o / S2_VC_TILE : ~0ull;
      const unsigned peers = __match_any_sync(0xffffffffu, vt);
      if (has && (unsigned)(__ffs(peers) - 1) == (threadIdx.x & 31u)) atomicAdd(vc_cnt + vt, (unsigned)__popc(peers));
    }
    if (!active) continue;
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
#ifdef S2_VX_CHUNKED
  }
#endif
}
#endif  // S2M_WANT_VERTICES
