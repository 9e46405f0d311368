// static_kernels.cuh -- SDF-independent kernels of the per-job pipeline,
// compiled by nvcc into libsdf2mesh_gb300.so: vertex compaction, the
// row-start scan, quad emission (thin wrappers over s2m_workers.cuh), and the
// FP32 issue-rate probe used as the evaluation roofline.
#pragma once
#include "s2m_workers.cuh"
#include "s2m_dc_core.cuh"

// Classification of one slab, bit-parallel over 32 cells along x, in passes
// that never wait on one another:
//   s2m_cells_bits     per lattice point of the slab's new planes, a sign bit
//                      (v > 0) and a near-zero bit (!(|v| >= guard)), 32
//                      points per word, each point read once (the pruned
//                      evaluation writes these bits itself)
//   s2m_cells_mark     per word of 32 cells, the candidate bits from the
//                      corner bits of the 4 point rows around it (a few dozen
//                      bitwise operations for 32 cells), and the tile counts
//                      (the last block to finish scans them into offsets)
//   s2m_cells_emit     the candidates of each tile, in (z, y, x) order
// The rule is s2_classify_values' (s2m_dc_core.cuh): a cell is a candidate
// when its 8 lattice corners do not share a sign, or (reference rule) when a
// corner whose reference coordinates are off the lattice is near zero (every
// cell with such a corner when S2M_JOB_EXACT_CORNERS).

// tile_off[t] = cand.base[slab] + (candidates of tiles < t); cand.base[slab + 1]
// = the slab's running total.  Run by one block of NT threads, any tile
// count; the counts are read from L2 (other blocks wrote them).
template <int NT>
__device__ __forceinline__ void s2_scan_tiles(const unsigned *tile_cnt, unsigned ntiles,
                                              unsigned long long *__restrict__ tile_off, unsigned long long *base,
                                              int slab_index) {
  __shared__ unsigned long long s_warp[32];
  __shared__ unsigned long long s_carry;
  const unsigned tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
  if (tid == 0) s_carry = __ldcg(base + slab_index);
  if (tid < 32) s_warp[tid] = 0ull;
  __syncthreads();
  for (unsigned t0 = 0; t0 < ntiles; t0 += NT) {
    const unsigned t = t0 + tid;
    const unsigned long long v = t < ntiles ? __ldcg(tile_cnt + t) : 0ull;
    unsigned long long inc = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned long long x = __shfl_up_sync(S2_FULL, inc, o);
      if ((int)lane >= o) inc += x;
    }
    if (lane == 31) s_warp[warp] = inc;
    __syncthreads();
    if (warp == 0) {
      const unsigned long long w = s_warp[lane];
      unsigned long long wi = w;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const unsigned long long x = __shfl_up_sync(S2_FULL, wi, o);
        if ((int)lane >= o) wi += x;
      }
      s_warp[lane] = wi - w;
    }
    __syncthreads();
    const unsigned long long carry = s_carry;
    if (t < ntiles) tile_off[t] = carry + s_warp[warp] + inc - v;
    __syncthreads();
    if (tid == NT - 1) s_carry = carry + s_warp[NT / 32 - 1] + inc;  // last thread's inclusive total
    __syncthreads();
  }
  if (tid == 0) base[slab_index + 1] = s_carry;
}

// Off-lattice bit of every cell column x: bit x % 32 of word x / 32 is
// s2_off_lattice(x + 1).
__global__ void __launch_bounds__(256) s2m_offx(S2Job job, unsigned *__restrict__ offx) {
  const int x = (int)(blockIdx.x * 256u + threadIdx.x);
  const unsigned b = __ballot_sync(S2_FULL, x < job.N && s2_off_lattice(job, x + 1));
  if ((threadIdx.x & 31u) == 0 && x < job.N) offx[x >> 5] = b;
}

// Point bits of planes k0 .. k0 + gridDim.y - 1 (for evaluation variants
// that do not write them themselves).  Grid (ceil(P / 8), planes), 8 warps
// per block, one row per warp: the warp walks the row's words (a 128-byte
// load and two ballots each).
__global__ void __launch_bounds__(256) s2m_cells_bits(S2Job job, const float *__restrict__ ring, S2PointBits pb,
                                                      int k0) {
  const int WP = (job.P + 31) >> 5;
  const int slot = (k0 + (int)blockIdx.y) % job.ring;
  const int y = (int)blockIdx.x * 8 + (int)(threadIdx.x >> 5);
  if (y >= job.P) return;  // whole warps
  const int lane = (int)(threadIdx.x & 31u);
  const float *row = ring + (long long)slot * job.plane + (long long)y * job.pitch;
  const long long o = ((long long)slot * job.P + y) * WP;
#pragma unroll 4
  for (int w = 0; w < WP; ++w) {
    const int x = w * 32 + lane;
    const bool in = x < job.P;
    const float v = in ? __ldg(row + x) : 0.0f;
    const unsigned pos = __ballot_sync(S2_FULL, in && v > 0.0f);
    const unsigned near = __ballot_sync(S2_FULL, in && !(fabsf(v) >= job.guard));
    if (lane == 0) {
      pb.pos[o + w] = pos;
      pb.near[o + w] = near;
    }
  }
}

// The point bits of a slab's planes k0 .. k0 + gridDim.y - 1 in its decided
// tiles (the pruned evaluation's tile pass proved |f| >= guard there with a
// known sign): sign from the tile's flag word, near-zero 0, unknown value 1;
// no values.  One thread per 32-point word of a row (4 tiles along x), grid
// (ceil(P * WP / 256), planes): every word of the planes is written, the
// undecided tiles' bytes as 0, which s2m_evalpl_* overwrites afterwards.
__global__ void __launch_bounds__(256) s2m_fill_decided(S2Job job, S2PointBits pb,
                                                        const unsigned *__restrict__ tiles, int tile_words, int k0,
                                                        int tzs) {
  const int WP = (job.P + 31) >> 5;
  const int q = (int)(blockIdx.x * 256u + threadIdx.x);  // word (y, w) of the plane
  if (q >= job.P * WP) return;
  const int y = q / WP, w = q - y * WP;
  const int ntx = (job.P + S2_PT_XY - 1) / S2_PT_XY;
  const unsigned long long trow = ((unsigned long long)(blockIdx.y / (unsigned)tzs) * ntx + y / S2_PT_XY) * ntx;
  unsigned pos = 0u, unk = 0u;
#pragma unroll
  for (int b = 0; b < 4; ++b) {
    const int tx = 4 * w + b;
    if (tx >= ntx) break;
    const unsigned flag = __ldg(tiles + (trow + tx) * tile_words + (tile_words - 1));
    if (!(flag & 1u)) continue;  // S2_TILE_DECIDED
    const unsigned bits = (1u << min(8, job.P - 8 * tx)) - 1u;
    unk |= bits << (8 * b);
    if (flag & 2u) pos |= bits << (8 * b);  // S2_TILE_POSITIVE
  }
  const long long o = ((long long)((k0 + (int)blockIdx.y) % job.ring) * job.P + y) * WP + w;
  pb.pos[o] = pos;
  pb.near[o] = 0u;
  pb.unk[o] = unk;
}

// Word l of cells (z = zc0 + dz, y, x = 32 w ..): l = (dz * N + y) * WN + w.
// Its coordinates from the block's first word (one 64-bit division per
// block; 32-bit ones per thread).
struct S2CellWord {
  int w, y, dz;
};
__device__ __forceinline__ S2CellWord s2_cell_word(const S2Job &job, int WN) {
  __shared__ unsigned long long s_row0;
  __shared__ int s_w0;
  const unsigned long long l0 = (unsigned long long)blockIdx.x * S2_CW_BLOCK;
  if (threadIdx.x == 0) {
    s_row0 = l0 / (unsigned long long)WN;
    s_w0 = (int)(l0 - s_row0 * (unsigned long long)WN);
  }
  __syncthreads();
  const unsigned q = (unsigned)s_w0 + threadIdx.x;  // < WN + S2_CW_BLOCK
  const unsigned row = (unsigned)s_row0 + q / (unsigned)WN;  // < slab depth * N < 2^32
  S2CellWord c;
  c.w = (int)(q % (unsigned)WN);
  c.y = (int)(row % (unsigned)job.N);
  c.dz = (int)(row / (unsigned)job.N);
  return c;
}

// The last block to finish (a fence, then an atomic count of finished blocks)
// also scans the tile counts into the slab's candidate offsets (tile_off,
// base[slab + 1]), so no separate launch is needed; `done` returns to 0.
__global__ void __launch_bounds__(S2_CW_BLOCK) s2m_cells_mark(S2Job job, S2PointBits pb,
                                                            const unsigned *__restrict__ offx,
                                                            unsigned *__restrict__ words, unsigned *tile_cnt,
                                                            unsigned *done, unsigned long long *__restrict__ tile_off,
                                                            unsigned long long *base, int slab_index, int zc0,
                                                            int zc1) {
  __shared__ unsigned s_warp[S2_CW_BLOCK / 32];
  const int WN = (job.N + 31) >> 5, WP = (job.P + 31) >> 5;
  const long long nw = (long long)(zc1 - zc0) * job.N * WN;
  const long long l = (long long)blockIdx.x * S2_CW_BLOCK + threadIdx.x;
  const S2CellWord cw = s2_cell_word(job, WN);
  unsigned cand = 0;
  if (l < nw) {
    const int w = cw.w, y = cw.y, dz = cw.dz;
    // corner k = bx | by << 1 | bz << 2 lies in point row q = by | bz << 1
    // (k = 2 q + bx); bx = 1 takes the row's bits shifted by one point
    unsigned pbit[8], nbit[8];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int slot = (zc0 + dz + (q >> 1)) % job.ring;
      const long long base = ((long long)slot * job.P + (y + (q & 1))) * WP + w;
      const bool more = w + 1 < WP;
      const unsigned plo = __ldg(pb.pos + base), phi = more ? __ldg(pb.pos + base + 1) : 0u;
      const unsigned nlo = __ldg(pb.near + base), nhi = more ? __ldg(pb.near + base + 1) : 0u;
      pbit[2 * q] = plo;
      pbit[2 * q + 1] = __funnelshift_r(plo, phi, 1);
      nbit[2 * q] = nlo;
      nbit[2 * q + 1] = __funnelshift_r(nlo, nhi, 1);
    }
    unsigned all = ~0u, any = 0u;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      all &= pbit[k];
      any |= pbit[k];
    }
    cand = any & ~all;
    if (!job.qef) {
      const unsigned ox = offx[w];
      const unsigned oy = s2_off_lattice(job, y + 1) ? ~0u : 0u;
      const unsigned oz = s2_off_lattice(job, zc0 + dz + 1) ? ~0u : 0u;
      if (job.exact) {
        cand |= ox | oy | oz;
      } else {
#pragma unroll
        for (int k = 1; k < 8; ++k)
          cand |= nbit[k] & (((k & 1) ? ox : 0u) | ((k & 2) ? oy : 0u) | ((k & 4) ? oz : 0u));
      }
    }
    if (w == WN - 1 && (job.N & 31)) cand &= (1u << (job.N & 31)) - 1u;
    words[l] = cand;
  }
  unsigned cnt = __popc(cand);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(S2_FULL, cnt, o);
  if ((threadIdx.x & 31u) == 0) s_warp[threadIdx.x >> 5] = cnt;
  __syncthreads();
  __shared__ bool s_last;
  if (threadIdx.x == 0) {
    unsigned t = 0;
    for (int i = 0; i < S2_CW_BLOCK / 32; ++i) t += s_warp[i];
    tile_cnt[blockIdx.x] = t;
    __threadfence();
    s_last = atomicAdd(done, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  s2_scan_tiles<S2_CW_BLOCK>(tile_cnt, gridDim.x, tile_off, base, slab_index);
  if (threadIdx.x == 0) *done = 0u;
}

// The candidates of each tile in order: key (x | y << 16 | z << 32) and the
// 8 lattice corner values (NaN where the point's unknown-value bit is set: a
// decided tile of the pruned evaluation wrote no value there).  A warp takes its words with candidates one at a
// time, lane l writing the cell of bit l: the corner loads of a word's cells
// are then coalesced rows, and every lane works.
__global__ void __launch_bounds__(S2_CW_BLOCK) s2m_cells_emit(S2Job job, const float *__restrict__ ring,
                                                            const unsigned *__restrict__ unk,
                                                            const unsigned *__restrict__ words,
                                                            const unsigned long long *__restrict__ tile_off,
                                                            S2Cand cand, unsigned *err, int zc0, int zc1) {
  __shared__ unsigned s_warp[32];
  const unsigned tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
  const int WN = (job.N + 31) >> 5;
  const long long nw = (long long)(zc1 - zc0) * job.N * WN;
  const long long l = (long long)blockIdx.x * S2_CW_BLOCK + tid;
  const S2CellWord cw = s2_cell_word(job, WN);
  const unsigned mask = l < nw ? words[l] : 0u;
  const unsigned cnt = __popc(mask);
  unsigned inc = cnt;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned t = __shfl_up_sync(S2_FULL, inc, o);
    if ((int)lane >= o) inc += t;
  }
  if (lane == 31) s_warp[warp] = inc;
  if (tid < 32 && tid >= S2_CW_BLOCK / 32) s_warp[tid] = 0u;
  __syncthreads();
  if (warp == 0) s2_warp_exclusive32(s_warp);
  __syncthreads();
  const unsigned long long first = tile_off[blockIdx.x] + s_warp[warp] + (inc - cnt);
  unsigned todo = __ballot_sync(S2_FULL, mask != 0u);
  while (todo) {
    const int src = __ffs(todo) - 1;
    todo &= todo - 1u;
    const unsigned m = __shfl_sync(S2_FULL, mask, src);
    const unsigned long long o = __shfl_sync(S2_FULL, first, src) + __popc(m & ((1u << lane) - 1u));
    S2Cell cell;
    cell.x = 32 * __shfl_sync(S2_FULL, cw.w, src) + (int)lane;
    cell.y = __shfl_sync(S2_FULL, cw.y, src);
    cell.z = zc0 + __shfl_sync(S2_FULL, cw.dz, src);
    if (!((m >> lane) & 1u)) continue;
    if (o >= cand.cap) {
      atomicOr(err, S2_ERR_CAND_OVF);
      continue;
    }
    float v[8];
    s2_load_corners<false>(job, ring, cell, v);
    if (unk) {  // corners of decided tiles: no value in the ring
      const int WP = (job.P + 31) >> 5, w = cell.x >> 5;
      const bool more = w + 1 < WP;
#pragma unroll
      for (int q = 0; q < 4; ++q) {  // corner k = 2 q + bx lies in point row q = by | bz << 1
        const long long base = ((long long)((cell.z + (q >> 1)) % job.ring) * job.P + (cell.y + (q & 1))) * WP + w;
        const unsigned lo = __ldg(unk + base), hi = more ? __ldg(unk + base + 1) : 0u;
        if ((lo >> lane) & 1u) v[2 * q] = __int_as_float(0x7fc00000);
        if ((__funnelshift_r(lo, hi, 1) >> lane) & 1u) v[2 * q + 1] = __int_as_float(0x7fc00000);
      }
    }
    cand.key[o] = (unsigned long long)cell.x | ((unsigned long long)cell.y << 16) | ((unsigned long long)cell.z << 32);
    float4 *dst = reinterpret_cast<float4 *>(cand.val + 8 * o);
    dst[0] = make_float4(v[0], v[1], v[2], v[3]);
    dst[1] = make_float4(v[4], v[5], v[6], v[7]);
  }
}

// Vertex work in tile order (tile pruning).  The vertex kernel evaluates the
// SDF with the activity bits of each candidate's tile; lanes of a warp whose
// candidates lie in different tiles take different paths through the pruned
// SDF, one after the other.  Candidates are listed in (z, y, x) order, so 32
// consecutive ones span several tiles.  A counting sort by tile gives the
// vertex kernel a permutation that groups them:
//   s2m_vtile_count    each candidate's tile and its rank among the tile's
//   s2m_vtile_scan     exclusive scan of the per-tile counts
//   s2m_vtile_scatter  perm[first of the tile + rank] = candidate
// The mesh does not depend on the order: a candidate's vertex is a function
// of its cell and its tile's bits alone.
__global__ void __launch_bounds__(256) s2m_vtile_count(S2Job job, S2Cand cand, int nslabs,
                                                       const unsigned long long *__restrict__ tbase, int D, int nzc,
                                                       unsigned *tcnt, unsigned long long *__restrict__ trank) {
  const unsigned long long n = min(cand.base[nslabs], cand.cap);
  for (unsigned long long i = (unsigned long long)blockIdx.x * 256u + threadIdx.x; i < n;
       i += (unsigned long long)gridDim.x * 256u) {
    const unsigned long long k = cand.key[i];
    S2Cell c;
    c.x = (int)(k & 0xffffull);
    c.y = (int)((k >> 16) & 0xffffull);
    c.z = (int)((k >> 32) & 0xffffull);
    const unsigned long long t = s2_cell_prune_tile(job, c, tbase, D, nzc);
    trank[i] = (t << 16) | atomicAdd(tcnt + t, 1u);  // a tile covers at most 8 x 8 x 8 cells
  }
}

// tcnt[0 .. T) becomes each tile's first position within its block of
// S2_VT_TILE tiles; part_cnt[b] = block b's total.  The last block to finish
// scans the totals into part_off (part_base[0] = 0 on entry); `done` returns
// to 0.
__global__ void __launch_bounds__(256) s2m_vtile_scan(unsigned *tcnt, unsigned long long T, unsigned *part_cnt,
                                                      unsigned long long *part_off, unsigned long long *part_base,
                                                      unsigned *done) {
  __shared__ unsigned s_warp[32];
  const unsigned tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
  const unsigned long long b0 = (unsigned long long)blockIdx.x * S2_VT_TILE + 8ull * tid;
  unsigned v[8], sum = 0;
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    v[q] = b0 + q < T ? tcnt[b0 + q] : 0u;
    sum += v[q];
  }
  unsigned inc = sum;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned t = __shfl_up_sync(S2_FULL, inc, o);
    if ((int)lane >= o) inc += t;
  }
  if (lane == 31) s_warp[warp] = inc;
  if (tid < 32 && tid >= 8) s_warp[tid] = 0u;
  __syncthreads();
  if (warp == 0) s2_warp_exclusive32(s_warp);
  __syncthreads();
  unsigned run = s_warp[warp] + inc - sum;
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    if (b0 + q < T) tcnt[b0 + q] = run;
    run += v[q];
  }
  __shared__ bool s_last;
  if (tid == 255) {
    part_cnt[blockIdx.x] = run;  // the block's total
    __threadfence();
    s_last = atomicAdd(done, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  s2_scan_tiles<256>(part_cnt, gridDim.x, part_off, part_base, 0);
  if (tid == 0) *done = 0u;
}

__global__ void __launch_bounds__(256) s2m_vtile_scatter(S2Cand cand, int nslabs, const unsigned *__restrict__ tcnt,
                                                         const unsigned long long *__restrict__ part_off,
                                                         const unsigned long long *__restrict__ trank,
                                                         unsigned *__restrict__ perm) {
  const unsigned long long n = min(cand.base[nslabs], cand.cap);
  for (unsigned long long i = (unsigned long long)blockIdx.x * 256u + threadIdx.x; i < n;
       i += (unsigned long long)gridDim.x * 256u) {
    const unsigned long long tr = trank[i], t = tr >> 16;
    perm[part_off[t / S2_VT_TILE] + tcnt[t] + (tr & 0xffffull)] = (unsigned)i;
  }
}

__global__ void __launch_bounds__(S2_VC_BLOCK) s2m_vcompact(S2Job job, S2Cand cand, S2MeshDev mesh, int nslabs) {
  s2_vcompact_worker(job, cand, mesh, nslabs, blockIdx.x == 0);
}

__global__ void __launch_bounds__(S2_SCAN_BLOCK) s2m_rowscan(S2MeshDev mesh, unsigned long long R) {
  s2_rowscan_worker(mesh, R);
}

__global__ void __launch_bounds__(S2_Q_BLOCK) s2m_quads(S2Job job, S2MeshDev mesh, unsigned scan_tiles) {
  s2_quads_worker<true>(job, mesh, scan_tiles, blockIdx.x == 0);
}

// FP32 issue-rate probe: 8 independent dependent chains per thread of
// separately rounded multiply and add (mode 0, the instruction mix of the
// evaluation kernels, which are compiled without contraction) or of fused
// multiply-add (mode 1).  Each chain step is 2 FP32 operations.
__global__ void __launch_bounds__(256) s2m_fp32_probe(float *out, int iters, int mode, float a, float b) {
  float x[8];
#pragma unroll
  for (int c = 0; c < 8; ++c) x[c] = (float)(threadIdx.x + c) * 1e-3f;
  if (mode == 0) {
    for (int i = 0; i < iters; ++i) {
#pragma unroll
      for (int c = 0; c < 8; ++c) x[c] = __fadd_rn(__fmul_rn(x[c], a), b);
    }
  } else {
    for (int i = 0; i < iters; ++i) {
#pragma unroll
      for (int c = 0; c < 8; ++c) x[c] = __fmaf_rn(x[c], a, b);
    }
  }
  float s = 0.0f;
#pragma unroll
  for (int c = 0; c < 8; ++c) s += x[c];
  if (s == 1234.5f) out[blockIdx.x] = s;  // keeps the chains live
}

// SFU issue-rate probe: 8 independent dependent chains of reciprocal square
// root (one MUFU operation each) and one FP32 add per step.
__global__ void __launch_bounds__(256) s2m_sfu_probe(float *out, int iters, float c) {
  float x[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) x[k] = 1.0f + (float)(threadIdx.x + k) * 1e-3f;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 8; ++k) x[k] = rsqrtf(__fadd_rn(x[k], c));
  }
  float s = 0.0f;
#pragma unroll
  for (int k = 0; k < 8; ++k) s += x[k];
  if (s == 1234.5f) out[blockIdx.x] = s;
}
