// s2m_workers.cuh -- the SDF-independent stages of the pipeline as block-level
// workers: ordered vertex compaction, the row-start scan and quad emission.
// The per-job kernels (static_kernels.cuh) and the persistent batch kernel
// (batch.cu) both run them; every worker takes its tiles from an atomic
// counter, so any number of worker blocks may run one stage.
#pragma once
#include "s2m_device.h"
#include "s2m_lookback.cuh"

// Keep the candidates that carry a vertex, in order (z, then y, then x, as
// the reference's VertexList), in the mesh's vertex arrays; count vertices
// per (z label, y) row.  Persistent grid; tiles are taken in order from
// cand.tile_counter, the prefix comes from the look-back over tiles.
// One worker block (256 threads); `leader` is true for exactly one worker.
__device__ __forceinline__ void s2_vcompact_worker(const S2Job &job, const S2Cand &cand, const S2MeshDev &mesh,
                                                   int nslabs, bool leader) {
  __shared__ unsigned s_tile;
  __shared__ unsigned s_warp[32];
  __shared__ unsigned long long s_excl;
  const unsigned tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
  const unsigned long long ncand = min(s2_ldcg(cand.base + nslabs), cand.cap);
  const unsigned ntiles = (unsigned)((ncand + S2_VC_TILE - 1) / S2_VC_TILE);
  if (ntiles == 0) {
    if (leader && tid == 0) *mesh.vtotal = 0;
    return;
  }
  const unsigned lt = s2_lanemask_lt();
  for (;;) {
    if (tid == 0) s_tile = atomicAdd(cand.tile_counter, 1u);
    __syncthreads();
    const unsigned tile = s_tile;
    if (tile >= ntiles) break;
    unsigned long long keys[S2_VC_CPT];
    unsigned ballots[S2_VC_CPT];
#pragma unroll
    for (int m = 0; m < S2_VC_CPT; ++m) {
      unsigned long long o = (unsigned long long)tile * S2_VC_TILE + m * S2_VC_BLOCK + tid;
      keys[m] = o < ncand ? s2_ldcg(cand.key + o) : 0ull;
      ballots[m] = __ballot_sync(S2_FULL, (keys[m] >> 63) != 0ull);
      if (lane == 0) s_warp[m * 8 + warp] = __popc(ballots[m]);
    }
    __syncthreads();
    if (warp == 0) {
      unsigned tot = s2_warp_exclusive32(s_warp);
      unsigned long long excl = s2_lookback(cand.status, tile, tot, mesh.err, mesh.wait_ns);
      if (lane == 0) {
        s_excl = excl;
        if (tile == ntiles - 1) *mesh.vtotal = excl + tot;
      }
    }
    __syncthreads();
#pragma unroll
    for (int m = 0; m < S2_VC_CPT; ++m) {
      if ((ballots[m] >> lane) & 1u) {
        unsigned long long o = (unsigned long long)tile * S2_VC_TILE + m * S2_VC_BLOCK + tid;
        unsigned long long v = s_excl + s_warp[m * 8 + warp] + __popc(ballots[m] & lt);
        unsigned long long key = keys[m] & ~(1ull << 63);
        unsigned y = (unsigned)((key >> 16) & 0xffffu), zl = (unsigned)((key >> 32) & 0xffffu);
        atomicAdd(mesh.rowcnt + (unsigned long long)zl * job.N + y, 1u);
        if (v >= 0xFFFFFFFEull) atomicOr(mesh.err, S2_ERR_INDEX_OVF);
        if (v >= mesh.vcap) {
          atomicOr(mesh.err, S2_ERR_VERT_OVF);
          continue;
        }
        mesh.key[v] = key;
        mesh.pos[3 * v] = s2_ldcg(cand.pos + 3 * o);
        mesh.pos[3 * v + 1] = s2_ldcg(cand.pos + 3 * o + 1);
        mesh.pos[3 * v + 2] = s2_ldcg(cand.pos + 3 * o + 2);
        mesh.nrm[3 * v] = s2_ldcg(cand.nrm + 3 * o);
        mesh.nrm[3 * v + 1] = s2_ldcg(cand.nrm + 3 * o + 1);
        mesh.nrm[3 * v + 2] = s2_ldcg(cand.nrm + 3 * o + 2);
      }
    }
    __syncthreads();
  }
}



// Block-wide exclusive scan of one u32 per thread (256 threads); returns the
// thread's exclusive prefix and writes the block total to *total.
__device__ __forceinline__ unsigned s2_block_exclusive(unsigned v, unsigned *s_warp, unsigned *total) {
  const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  unsigned inc = v;
  for (int o = 1; o < 32; o <<= 1) {
    unsigned t = __shfl_up_sync(S2_FULL, inc, o);
    if ((int)lane >= o) inc += t;
  }
  if (lane == 31) s_warp[warp] = inc;
  __syncthreads();
  if (warp == 0) {
    unsigned w = lane < (blockDim.x >> 5) ? s_warp[lane] : 0u;
    unsigned wi = w;
    for (int o = 1; o < 32; o <<= 1) {
      unsigned t = __shfl_up_sync(S2_FULL, wi, o);
      if ((int)lane >= o) wi += t;
    }
    if (lane < (blockDim.x >> 5)) s_warp[lane] = wi - w;
    if (lane == 31) *total = wi;
  }
  __syncthreads();
  return s_warp[warp] + inc - v;
}

// rowstart[r] = number of vertices in rows < r (rows ordered by z label,
// then y), rowstart[R] = total.  Persistent grid, look-back over tiles.
__device__ __forceinline__ void s2_rowscan_worker(const S2MeshDev &mesh, unsigned long long R) {
  __shared__ unsigned s_tile;
  __shared__ unsigned s_warp[32];
  __shared__ unsigned s_total;
  __shared__ unsigned long long s_excl;
  const unsigned tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
  const unsigned ntiles = (unsigned)((R + S2_SCAN_TILE - 1) / S2_SCAN_TILE);
  for (;;) {
    if (tid == 0) s_tile = atomicAdd(mesh.counters + 2, 1u);
    __syncthreads();
    const unsigned tile = s_tile;
    if (tile >= ntiles) break;
    unsigned long long e0 = (unsigned long long)tile * S2_SCAN_TILE + (unsigned long long)tid * S2_SCAN_CPT;
    unsigned v[S2_SCAN_CPT];
    unsigned sum = 0;
#pragma unroll
    for (int m = 0; m < S2_SCAN_CPT; ++m) {
      v[m] = e0 + m < R ? s2_ldcg(mesh.rowcnt + e0 + m) : 0u;
      sum += v[m];
    }
    unsigned pre = s2_block_exclusive(sum, s_warp, &s_total);
    if (warp == 0) {
      // S2_HOLD_ROWSCAN_TILE0 (tests): tile 0 keeps its status word at 0, so
      // every later tile's look-back waits until its limit
      const bool hold = tile == 0 && (mesh.hold & S2_HOLD_ROWSCAN_TILE0);
      unsigned long long excl =
          hold ? 0ull : s2_lookback(mesh.scan_status, tile, s_total, mesh.err, mesh.wait_ns);
      if (lane == 0) {
        s_excl = excl;
        if (tile == ntiles - 1) mesh.rowstart[R] = (unsigned)(excl + s_total);
      }
    }
    __syncthreads();
    unsigned run = (unsigned)s_excl + pre;
#pragma unroll
    for (int m = 0; m < S2_SCAN_CPT; ++m) {
      if (e0 + m < R) mesh.rowstart[e0 + m] = run;
      run += v[m];
    }
    __syncthreads();
  }
}



// Loads of the vertex keys and row starts: NC (a kernel launched after the
// ones that wrote them) through the read-only cache, where neighbouring
// vertices' searches of the same rows hit; else from L2 (the persistent
// batch kernel, where they were written earlier in the same launch).
template <bool NC, class T>
__device__ __forceinline__ T s2_ldq(const T *p) {
  return NC ? __ldg(p) : s2_ldcg(p);
}

// The vertices of cells (x - 1, y, z label) and (x, y, z label): the row of
// (z, y) is a contiguous run of the vertex list sorted by x, as the sorted
// VertexList the reference binary-searches (mesh.rs:326-331); one
// lower-bound search for x gives both.  S2_NO_VERTEX where there is none.
struct S2RowHit {
  unsigned xm1, x;
};
template <bool NC>
__device__ __forceinline__ S2RowHit s2_row_find(const S2MeshDev &m, int N, int x, int y, int z) {
  const unsigned long long r = (unsigned long long)z * N + y;
  const unsigned start = s2_ldq<NC>(m.rowstart + r);
  unsigned end = s2_ldq<NC>(m.rowstart + r + 1);
  if (end > m.vcap) end = (unsigned)m.vcap;
  unsigned lo = start, hi = end;
  while (lo < hi) {
    const unsigned mid = (lo + hi) >> 1;
    if ((int)(s2_ldq<NC>(m.key + mid) & 0xffffull) < x) lo = mid + 1;
    else hi = mid;
  }
  S2RowHit h;
  h.x = (lo < end && (int)(s2_ldq<NC>(m.key + lo) & 0xffffull) == x) ? lo : S2_NO_VERTEX;
  h.xm1 = (lo > start && (int)(s2_ldq<NC>(m.key + lo - 1) & 0xffffull) == x - 1) ? lo - 1 : S2_NO_VERTEX;
  return h;
}

// Quads of one vertex (mesh.rs:280-321): x, y and z edges in that order,
// each a Quad(...).swap(flag) split into triangles (q2, q1, q0), (q0, q3, q2)
// (lib.rs:531-546); a quad with a missing vertex is dropped (invalid).  The
// six neighbouring cells lie in three rows and the vertex's own row, where
// cell (x - 1, y, z) can only be vertex v - 1.
struct S2Quads {
  unsigned q[3][4];
  unsigned valid;    // bit per quad
  unsigned invalid;  // quads dropped
};

// The neighbour lookups of one vertex's quads: row a = (., y - 1, z) at x and
// x - 1, row b = (., y, z - 1) at x and x - 1, row c = (., y - 1, z - 1) at
// x, and (x - 1, y, z) in the vertex's own row; S2_NO_VERTEX where the cell
// has no vertex or no wanted quad needs the lookup.
struct S2QuadLookups {
  unsigned ax, axm1, bx, bxm1, cx, own;
};

// zq: vertices labelled below plane zq make no quads (0: every vertex).
__device__ __forceinline__ unsigned s2_quad_want(unsigned long long key, unsigned zq) {
  const int x = (int)(key & 0xffffull), y = (int)((key >> 16) & 0xffffull), z = (int)((key >> 32) & 0xffffull);
  const unsigned s = (unsigned)((key >> 48) & 0xfull);
  const bool b0 = s & 1u, b1 = s & 2u, b2 = s & 4u, b3 = s & 8u;
  if ((unsigned)z < zq) return 0u;
  return (b0 != b3 && y > 0 && z > 0 ? 1u : 0u) | (b1 != b3 && x > 0 && z > 0 ? 2u : 0u) |
         (b2 != b3 && x > 0 && y > 0 ? 4u : 0u);
}

template <bool NC>
__device__ __forceinline__ S2QuadLookups s2_quad_lookups(const S2MeshDev &m, int N, unsigned v,
                                                         unsigned long long key) {
  const int x = (int)(key & 0xffffull), y = (int)((key >> 16) & 0xffffull), z = (int)((key >> 32) & 0xffffull);
  const unsigned want = s2_quad_want(key, m.zq);
  const S2RowHit none = {S2_NO_VERTEX, S2_NO_VERTEX};
  const S2RowHit ra = (want & 5u) ? s2_row_find<NC>(m, N, x, y - 1, z) : none;      // (., y - 1, z)
  const S2RowHit rb = (want & 3u) ? s2_row_find<NC>(m, N, x, y, z - 1) : none;      // (., y, z - 1)
  const S2RowHit rc = (want & 1u) ? s2_row_find<NC>(m, N, x, y - 1, z - 1) : none;  // (., y - 1, z - 1)
  S2QuadLookups l;
  l.ax = ra.x;
  l.axm1 = ra.xm1;
  l.bx = rb.x;
  l.bxm1 = rb.xm1;
  l.cx = rc.x;
  l.own = S2_NO_VERTEX;  // (x - 1, y, z): in the vertex's own row, only vertex v - 1 can be it
  if ((want & 6u) && v > 0) {
    const unsigned long long kp = s2_ldq<NC>(m.key + v - 1);
    if (((kp ^ key) & 0x0000ffffffff0000ull) == 0ull && (int)(kp & 0xffffull) == x - 1) l.own = v - 1;
  }
  return l;
}

// Quads of one vertex from its lookups (mesh.rs:280-321).
__device__ __forceinline__ S2Quads s2_quads_from(const S2QuadLookups &l, unsigned v, unsigned long long key,
                                                 unsigned zq) {
  S2Quads r;
  r.valid = 0;
  r.invalid = 0;
  const unsigned s = (unsigned)((key >> 48) & 0xfull);
  const bool b0 = s & 1u, b1 = s & 2u, b2 = s & 4u;
  const unsigned want = s2_quad_want(key, zq);
  auto put = [&](int qi, unsigned a, unsigned b, unsigned c, unsigned d, bool swap) {
    if (swap) { unsigned t = a; a = d; d = t; t = b; b = c; c = t; }
    r.q[qi][0] = a; r.q[qi][1] = b; r.q[qi][2] = c; r.q[qi][3] = d;
    if (a != S2_NO_VERTEX && b != S2_NO_VERTEX && c != S2_NO_VERTEX && d != S2_NO_VERTEX) r.valid |= 1u << qi;
    else r.invalid++;
  };
  if (want & 1u) put(0, l.cx, l.bx, v, l.ax, b0);
  if (want & 2u) put(1, l.bxm1, l.bx, v, l.own, !b1);
  if (want & 4u) put(2, l.axm1, l.ax, v, l.own, b2);
  return r;
}

template <bool NC>
__device__ __forceinline__ S2Quads s2_vertex_quads(const S2MeshDev &m, int N, unsigned v, unsigned long long key) {
  return s2_quads_from(s2_quad_lookups<NC>(m, N, v, key), v, key, m.zq);
}

template <bool NC>
__device__ __forceinline__ void s2_quads_worker(const S2Job &job, const S2MeshDev &mesh, unsigned scan_tiles,
                                                bool leader) {
  __shared__ unsigned s_tile;
  __shared__ unsigned s_warp[32];
  __shared__ unsigned s_total;
  __shared__ unsigned long long s_excl;
  const unsigned tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
  const unsigned long long V = s2_ldcg(mesh.vtotal);
  if (V > mesh.vcap) return;  // vertex overflow: the host re-runs with larger buffers
  unsigned long long *status = mesh.scan_status + scan_tiles;
  const unsigned ntiles = (unsigned)((V + S2_Q_TILE - 1) / S2_Q_TILE);
  if (ntiles == 0) {
    if (leader && tid == 0) *mesh.ntris = 0;
    return;
  }
  const unsigned lt = s2_lanemask_lt();
  unsigned invalid = 0;
  for (;;) {
    if (tid == 0) s_tile = atomicAdd(mesh.counters + 3, 1u);
    __syncthreads();
    const unsigned tile = s_tile;
    if (tile >= ntiles) break;
    S2Quads qd[S2_Q_VPT];
    unsigned ntri[S2_Q_VPT];
#pragma unroll
    for (int m = 0; m < S2_Q_VPT; ++m) {
      unsigned long long v = (unsigned long long)tile * S2_Q_TILE + m * S2_Q_BLOCK + tid;
      qd[m].valid = 0;
      ntri[m] = 0;
      if (v < V) {
        qd[m] = s2_vertex_quads<NC>(mesh, job.N, (unsigned)v, s2_ldq<NC>(mesh.key + v));
        ntri[m] = 2u * __popc(qd[m].valid);
        invalid += qd[m].invalid;
      }
      // warp inclusive scan of ntri
      unsigned inc = ntri[m];
      for (int o = 1; o < 32; o <<= 1) {
        unsigned t = __shfl_up_sync(S2_FULL, inc, o);
        if ((int)lane >= o) inc += t;
      }
      if (lane == 31) s_warp[m * 8 + warp] = inc;
      ntri[m] = (inc - ntri[m]) | (ntri[m] << 24);  // pack: exclusive prefix, own count
    }
    if (tid < 32 - S2_Q_VPT * 8) s_warp[S2_Q_VPT * 8 + tid] = 0u;
    __syncthreads();
    if (warp == 0) {
      unsigned tot = s2_warp_exclusive32(s_warp);
      if (lane == 0) s_total = tot;
    }
    __syncthreads();
    if (warp == 0) {
      unsigned long long excl = s2_lookback(status, tile, s_total, mesh.err, mesh.wait_ns);
      if (lane == 0) {
        s_excl = excl;
        if (tile == ntiles - 1) *mesh.ntris = excl + s_total;
      }
    }
    __syncthreads();
#pragma unroll
    for (int m = 0; m < S2_Q_VPT; ++m) {
      unsigned long long t = s_excl + s_warp[m * 8 + warp] + (ntri[m] & 0xffffffu);
      for (int qi = 0; qi < 3; ++qi) {
        if (!((qd[m].valid >> qi) & 1u)) continue;
        const unsigned *q = qd[m].q[qi];
        if (t + 2 > mesh.tcap) {
          atomicOr(mesh.err, S2_ERR_TRI_OVF);
          t += 2;
          continue;
        }
        unsigned *o = mesh.tris + 3 * t;
        o[0] = q[2]; o[1] = q[1]; o[2] = q[0];
        o[3] = q[0]; o[4] = q[3]; o[5] = q[2];
        t += 2;
      }
    }
    __syncthreads();
  }
  (void)lt;
  for (int o = 16; o > 0; o >>= 1) invalid += __shfl_xor_sync(S2_FULL, invalid, o);
  if (lane == 0 && invalid) atomicAdd(mesh.invalid, (unsigned long long)invalid);
}



