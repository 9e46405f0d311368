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


// The end of one z part of a job (s2m_mesh_generate): its vertices from index
// skip = *skip_at on (its context plane, which the part below it has already
// delivered, comes first in (z, y, x) order; skip_at null: none) become host
// vertices vbase .. vbase + vcount - 1, and its triangles host triangles
// tbase .., every index shifted in place here by vbase - skip.  Block 0
// writes the part's copy plan and the running totals to *cur (pinned host
// memory mapped into the device's address space); the host then copies with
// the copy engines while the next part's kernels run.  A part that
// overflowed its buffers or the host arrays shifts nothing and leaves its
// flags in cur->err: the host meshes the job again in one piece.
struct S2HostTotals {
  unsigned long long nverts, ntris, invalid;       // running totals after this part
  unsigned long long vfirst, vcount, vbase;        // copy: device vertices vfirst .. -> host vbase ..
  unsigned long long tcount, tbase;                // copy: device triangles 0 .. tcount -> host tbase ..
  unsigned long long ncand;                        // the part's candidate cells
  unsigned err, pad;
};
__global__ void __launch_bounds__(256) s2m_part_finish(S2MeshDev mesh, const unsigned *skip_at,
                                                       const unsigned long long *ncand,
                                                       const S2HostTotals *prev, S2HostTotals *cur,
                                                       unsigned long long hvcap, unsigned long long htcap) {
  S2_PDL_WAIT();
  const unsigned long long V = *mesh.vtotal, T = *mesh.ntris;
  const unsigned long long skip = skip_at ? (unsigned long long)*skip_at : 0ull;
  const unsigned long long vb = prev ? prev->nverts : 0ull, tb = prev ? prev->ntris : 0ull;
  unsigned err = (prev ? prev->err : 0u) | *mesh.err;
  if (V > mesh.vcap || T > mesh.tcap || skip > V || skip > vb) err |= S2_ERR_VERT_OVF;
  else if (vb + (V - skip) > hvcap || tb + T > htcap) err |= S2_ERR_HOST_OVF;
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    cur->nverts = err ? 0ull : vb + (V - skip);
    cur->ntris = err ? 0ull : tb + T;
    cur->invalid = (prev ? prev->invalid : 0ull) + *mesh.invalid;
    cur->vfirst = skip;
    cur->vcount = err ? 0ull : V - skip;
    cur->vbase = vb;
    cur->tcount = err ? 0ull : T;
    cur->tbase = tb;
    cur->ncand = *ncand;
    cur->err = err;
    cur->pad = 0u;
  }
  if (err || vb == skip) return;
  const unsigned shift = (unsigned)(vb - skip);  // indices stay below 2^32 - 1 (S2_ERR_INDEX_OVF otherwise)
  for (unsigned long long i = (unsigned long long)blockIdx.x * 256u + threadIdx.x; i < 3ull * T;
       i += (unsigned long long)gridDim.x * 256u)
    mesh.tris[i] += shift;
}

// Off-lattice bit of every cell column x: bit x % 32 of word x / 32 is
// s2_off_lattice(x + 1).
__global__ void __launch_bounds__(256) s2m_offx(S2Job job, unsigned *__restrict__ offx) {
  S2_PDL_WAIT();
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
  S2_PDL_WAIT();
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
// no values.  One thread per 32-point word of a row (4 tiles along x) and
// per layer of tiles (tzs planes, nk planes in all), grid (ceil(P * WP /
// 256), layers): every word of the planes is written, the undecided tiles'
// bytes as 0, which s2m_evalpl_* overwrites afterwards.  Before
// s2m_cells_mark_tiles the per-job pipeline fills only a slab's last plane
// this way, which the next slab's classification reads as its first (within
// its own planes the classification takes decided tiles' bits from the tile
// flags), and clears the slab's cell tile counts (zero[0 .. nzero - 1]).
__global__ void __launch_bounds__(256) s2m_fill_decided(S2Job job, S2PointBits pb,
                                                        const unsigned *__restrict__ tiles, int tile_words, int k0,
                                                        int nk, int tzs, unsigned *chunk_reset, unsigned *zero,
                                                        unsigned nzero) {
  S2_PDL_WAIT();
  // the listed evaluation that follows this launch takes its chunks from zero
  if (blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0) *chunk_reset = 0u;
  // and s2m_cells_mark_tiles adds to cleared cell tile counts
  if (blockIdx.y == 0)
    for (unsigned i = blockIdx.x * 256u + threadIdx.x; i < nzero; i += gridDim.x * 256u) zero[i] = 0u;
  const int WP = (job.P + 31) >> 5;
  const int q = (int)(blockIdx.x * 256u + threadIdx.x);  // word (y, w) of the plane
  if (q >= job.P * WP) return;
  const int y = q / WP, w = q - y * WP;
  const int ntx = (job.P + S2_PT_XY - 1) / S2_PT_XY;
  const unsigned long long trow = ((unsigned long long)blockIdx.y * ntx + y / S2_PT_XY) * ntx;
  unsigned pos = 0u, unk = 0u;
#pragma unroll
  for (int b = 0; b < 4; ++b) {
    const int tx = 4 * w + b;
    if (tx >= ntx) break;
    const unsigned flag = __ldg(tiles + (trow + tx) * tile_words + (tile_words - 1));
    if (!(flag & S2_TILE_DECIDED)) continue;
    const unsigned bits = (1u << min(8, job.P - 8 * tx)) - 1u;
    unk |= bits << (8 * b);
    if (flag & S2_TILE_POSITIVE) pos |= bits << (8 * b);
  }
  const int kb = k0 + (int)blockIdx.y * tzs, ke = min(kb + tzs, k0 + nk);
  const long long plane = (long long)job.P * WP;
  long long o = ((long long)(kb % job.ring) * job.P + y) * WP + w;
  const long long wrap = (long long)job.ring * plane;
#pragma unroll 1
  for (int k = kb; k < ke; ++k) {
    pb.pos[o] = pos;
    pb.near[o] = 0u;
    pb.unk[o] = unk;
    o += plane;
    if (o >= wrap) o -= wrap;
  }
}

// Cell words and tiles of a slab: word yw = y * WN + w of cell plane dz
// holds the cells (x = 32 w .., y, z = zc0 + dz), at words[dz * N * WN + yw].
// Tile t = dz * nbp + b (nbp = ceil(N * WN / S2_CW_BLOCK) tiles per plane)
// holds the plane's words b * S2_CW_BLOCK ..; tile order is (z, y, x) order.
//
// s2m_cells_mark: grid (nbp, ceil(planes / S2_MARK_PLANES)); a thread takes
// one word position over S2_MARK_PLANES cell planes, so each point row it
// reads serves the planes above and below it.  Each block writes its tile
// counts and adds them to the count of their cell plane (plane_cnt, zero on
// entry).  The last block to finish (a fence, then an atomic count of
// finished blocks) scans the slab's plane counts into plane offsets
// (plane_off[dz] = base[slab] + candidates of planes < dz, base[slab + 1] =
// the running total) and zeroes plane_cnt and `done` again.  (Scanning every
// tile count in that one block made it run as long as the rest of the launch
// together; s2m_cells_emit sums the counts before its tile within the plane
// instead.)
#define S2_MARK_PLANES 4
// Sign and near-zero words of one point row's 32 points (lo) and its next
// point (bit 0 of hi) with the bytes of decided tiles replaced by their flags:
// f / fn hold the flags of the row's 4 tiles and of the 4 after them, one byte
// each (bit 0 decided, bit 1 positive).
__device__ __forceinline__ void s2_decided_bytes(unsigned f, unsigned fn, unsigned &pos_lo, unsigned &pos_hi,
                                                 unsigned &near_lo, unsigned &near_hi) {
  const unsigned dm = (f & 0x01010101u) * 0xffu, pm = ((f >> 1) & f & 0x01010101u) * 0xffu;
  const unsigned dmn = fn & 1u, pmn = (fn >> 1) & fn & 1u;
  pos_lo = (pos_lo & ~dm) | pm;
  near_lo &= ~dm;
  pos_hi = (pos_hi & ~dmn) | pmn;
  near_hi &= ~dmn;
}
__global__ void __launch_bounds__(S2_CW_BLOCK) s2m_cells_mark(S2Job job, S2PointBits pb,
                                                            const unsigned *__restrict__ offx,
                                                            unsigned *__restrict__ words, unsigned *tile_cnt,
                                                            unsigned *done, unsigned *plane_cnt,
                                                            unsigned long long *__restrict__ plane_off,
                                                            unsigned long long *base, int slab_index, int zc0,
                                                            int zc1) {
  S2_PDL_WAIT();
  __shared__ unsigned s_cnt[S2_MARK_PLANES][S2_CW_BLOCK / 32];
  const int WN = (job.N + 31) >> 5, WP = (job.P + 31) >> 5, NW = job.N * WN;
  const int yw = (int)(blockIdx.x * S2_CW_BLOCK + threadIdx.x);
  const int dz0 = (int)blockIdx.y * S2_MARK_PLANES;
  const int ncp = min(S2_MARK_PLANES, zc1 - zc0 - dz0);  // cell planes of this block, >= 1
  unsigned cand[S2_MARK_PLANES];
#pragma unroll
  for (int i = 0; i < S2_MARK_PLANES; ++i) cand[i] = 0u;
  if (yw < NW) {
    const int y = yw / WN, w = yw - y * WN;
    const bool more = w + 1 < WP;
    const bool nearrule = !job.qef && !job.exact;
    const unsigned ox = job.qef ? 0u : offx[w];
    const unsigned oy = (!job.qef && s2_off_lattice(job, y + 1)) ? ~0u : 0u;
    // per point plane p: AND and OR of its 4 corner words, and (reference
    // rule) the near-zero corners that count when the plane is a cell's
    // bottom (tb: corners k = 1, 2, 3) or top (tt: k = 4 .. 7).  Corner k =
    // bx | by << 1 | bz << 2; bx = 1 takes the row's bits shifted by one.
    unsigned andp[S2_MARK_PLANES + 1], orp[S2_MARK_PLANES + 1], tb[S2_MARK_PLANES + 1], tt[S2_MARK_PLANES + 1];
    // all loads first (planes past ncp repeat the last one, unused), so that
    // they are in flight together
    long long rb[S2_MARK_PLANES + 1];
    {
      int slot = (zc0 + dz0) % job.ring;
#pragma unroll
      for (int p = 0; p <= S2_MARK_PLANES; ++p) {
        rb[p] = ((long long)slot * job.P + y) * WP + w;
        if (p < ncp && ++slot == job.ring) slot = 0;
      }
    }
    const int dw = more ? 1 : 0;
    unsigned pw[S2_MARK_PLANES + 1][4], nw[S2_MARK_PLANES + 1][4];
#pragma unroll
    for (int p = 0; p <= S2_MARK_PLANES; ++p) {
      pw[p][0] = __ldg(pb.pos + rb[p]);
      pw[p][1] = __ldg(pb.pos + rb[p] + dw);
      pw[p][2] = __ldg(pb.pos + rb[p] + WP);
      pw[p][3] = __ldg(pb.pos + rb[p] + WP + dw);
      if (nearrule) {
        nw[p][0] = __ldg(pb.near + rb[p]);
        nw[p][1] = __ldg(pb.near + rb[p] + dw);
        nw[p][2] = __ldg(pb.near + rb[p] + WP);
        nw[p][3] = __ldg(pb.near + rb[p] + WP + dw);
      }
    }
#pragma unroll
    for (int p = 0; p <= S2_MARK_PLANES; ++p) {
      const unsigned p0 = pw[p][0], p1 = pw[p][2];
      const unsigned p0s = __funnelshift_r(p0, more ? pw[p][1] : 0u, 1);
      const unsigned p1s = __funnelshift_r(p1, more ? pw[p][3] : 0u, 1);
      andp[p] = p0 & p0s & p1 & p1s;
      orp[p] = p0 | p0s | p1 | p1s;
      tb[p] = tt[p] = 0u;
      if (nearrule) {
        const unsigned n0 = nw[p][0], n1 = nw[p][2];
        const unsigned n0s = __funnelshift_r(n0, more ? nw[p][1] : 0u, 1);
        const unsigned n1s = __funnelshift_r(n1, more ? nw[p][3] : 0u, 1);
        const unsigned oz = s2_off_lattice(job, zc0 + dz0 + p) ? ~0u : 0u;
        tb[p] = (n0s & ox) | (n1 & oy) | (n1s & (ox | oy));
        tt[p] = (n0 & oz) | (n0s & (ox | oz)) | (n1 & (oy | oz)) | (n1s & (ox | oy | oz));
      }
    }
    const unsigned edge = (w == WN - 1 && (job.N & 31)) ? (1u << (job.N & 31)) - 1u : ~0u;
#pragma unroll
    for (int i = 0; i < S2_MARK_PLANES; ++i) {
      if (i >= ncp) break;
      unsigned c = (orp[i] | orp[i + 1]) & ~(andp[i] & andp[i + 1]);
      if (nearrule) c |= tb[i] | tt[i + 1];
      else if (!job.qef) c |= ox | oy | (s2_off_lattice(job, zc0 + dz0 + i + 1) ? ~0u : 0u);
      c &= edge;
      words[(long long)(dz0 + i) * NW + yw] = c;
      cand[i] = c;
    }
  }
  const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
#pragma unroll
  for (int i = 0; i < S2_MARK_PLANES; ++i) {
    unsigned cnt = __popc(cand[i]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(S2_FULL, cnt, o);
    if (lane == 0) s_cnt[i][warp] = cnt;
  }
  __syncthreads();
  if ((int)threadIdx.x < ncp) {
    unsigned t = 0;
    for (int k = 0; k < S2_CW_BLOCK / 32; ++k) t += s_cnt[threadIdx.x][k];
    tile_cnt[(unsigned long long)(dz0 + (int)threadIdx.x) * gridDim.x + blockIdx.x] = t;
    if (t) atomicAdd(plane_cnt + dz0 + (int)threadIdx.x, t);
    __threadfence();
  }
  __syncthreads();
  __shared__ bool s_last;
  if (threadIdx.x == 0) s_last = atomicAdd(done, 1u) == gridDim.x * gridDim.y - 1;
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  const unsigned nplanes = (unsigned)(zc1 - zc0);
  s2_scan_tiles<S2_CW_BLOCK, 4>(plane_cnt, nplanes, plane_off, base, slab_index);
  __syncthreads();  // every count read before it is cleared for the next slab
  for (unsigned p = threadIdx.x; p < nplanes; p += S2_CW_BLOCK) plane_cnt[p] = 0u;
  if (threadIdx.x == 0) *done = 0u;
}

// Sign and near-zero words (lo: the row's 32 points from 32 w, hi: bit 0 =
// the next point) of lattice row y in the plane at ring slot `slot`, with the
// bytes of decided tiles taken from their flags when the plane is one of the
// slab's own (layer >= 0: its layer of tiles).
struct S2RowBits {
  unsigned plo, phi, nlo, nhi;
};
__device__ __forceinline__ S2RowBits s2_row_bits(const S2Job &job, S2PointBits pb, const unsigned *__restrict__ tflags,
                                                 int ntx, int WP, int slot, int layer, int y, int w, bool more,
                                                 bool nearrule) {
  const long long rb = ((long long)slot * job.P + y) * WP + w;
  S2RowBits r;
  r.plo = __ldg(pb.pos + rb);
  r.phi = more ? __ldg(pb.pos + rb + 1) : 0u;
  r.nlo = nearrule ? __ldg(pb.near + rb) : 0u;
  r.nhi = (nearrule && more) ? __ldg(pb.near + rb + 1) : 0u;
  if (layer >= 0) {
    const long long fo = ((long long)layer * ntx + (y >> 3)) * WP + w;
    const unsigned f = __ldg(tflags + fo), fn = more ? __ldg(tflags + fo + 1) : 0u;
    s2_decided_bytes(f, fn, r.plo, r.phi, r.nlo, r.nhi);
  }
  return r;
}
__device__ __forceinline__ S2RowBits s2_shfl_row(S2RowBits v, int src) {
  S2RowBits r;
  r.plo = __shfl_sync(S2_FULL, v.plo, src);
  r.phi = __shfl_sync(S2_FULL, v.phi, src);
  r.nlo = __shfl_sync(S2_FULL, v.nlo, src);
  r.nhi = __shfl_sync(S2_FULL, v.nhi, src);
  return r;
}
// The terms of a point plane for the 32 cells of a word (as s2m_cells_mark):
// AND / OR of the 4 corner words, near-zero corners counting as a cell's
// bottom (tb) or top (tt) plane; rows a (y) and c (y + 1), oz the plane's
// off-lattice mask.
struct S2PlaneTerms {
  unsigned andp, orp, tb, tt;
};
__device__ __forceinline__ S2PlaneTerms s2_plane_terms(S2RowBits a, S2RowBits c, bool more, unsigned ox, unsigned oy,
                                                      unsigned oz, bool nearrule) {
  S2PlaneTerms t;
  const unsigned p0s = __funnelshift_r(a.plo, more ? a.phi : 0u, 1);
  const unsigned p1s = __funnelshift_r(c.plo, more ? c.phi : 0u, 1);
  t.andp = a.plo & p0s & c.plo & p1s;
  t.orp = a.plo | p0s | c.plo | p1s;
  t.tb = t.tt = 0u;
  if (nearrule) {
    const unsigned n0s = __funnelshift_r(a.nlo, more ? a.nhi : 0u, 1);
    const unsigned n1s = __funnelshift_r(c.nlo, more ? c.nhi : 0u, 1);
    t.tb = (n0s & ox) | (c.nlo & oy) | (n1s & (ox | oy));
    t.tt = (a.nlo & oz) | (n0s & (ox | oz)) | (c.nlo & (oy | oz)) | (n1s & (ox | oy | oz));
  }
  return t;
}

// s2m_cells_mark_tiles: classification of a slab by its undecided pruning
// tiles only (the listed evaluation, not S2M_JOB_EXACT_CORNERS).  A cell lies
// with all its corners in the box of the tile of its point (x, y, z + 1); when
// that tile is decided the signs agree on the box and no corner is near zero,
// so the cell is no candidate.  So only the cells of the slab's listed tiles
// are classified: a warp per listed tile (from the list the tile pass wrote,
// whose length is on the device), lane = row r (8) by cell plane (4 at a
// time), each forming the byte of its 8 cells with the word formulas of
// s2m_cells_mark.  A lane loads the point row of its own row and lower plane;
// the row above and the plane above come from the neighbouring lanes
// (shuffles), so each point row is loaded once per warp: a tile's rows are
// whole words apart, and loading every corner row in every lane made the
// kernel bound by L1 sectors.  Point bits are written only in undecided
// tiles of the slab's planes (and in full in the plane before them): the
// bytes of decided tiles read their flags (s2_decided_bytes).  The byte goes
// to the cell word (byte tx % 4 of word tx / 4); bytes of decided tiles are
// never written here, and s2m_cells_emit ignores them by the same flags.
// Counts: per cell tile of S2_CW_BLOCK words and per cell plane (atomic
// adds, one per group of lanes of one tile; both zero on entry:
// s2m_fill_decided clears the tile counts).  The last block to finish scans
// the plane counts into offsets, as s2m_cells_mark does.
#define S2_MT_BLOCK 256
__global__ void __launch_bounds__(S2_MT_BLOCK) s2m_cells_mark_tiles(
    S2Job job, S2PointBits pb, const unsigned *__restrict__ offx, unsigned *__restrict__ words, unsigned *tile_cnt,
    unsigned *done, unsigned *plane_cnt, unsigned long long *__restrict__ plane_off, unsigned long long *base,
    int slab_index, int zc0, int zc1, const unsigned *__restrict__ tflags, int tk0, int tzs,
    const unsigned *__restrict__ list, const unsigned *__restrict__ list_count) {
  S2_PDL_WAIT();
  const int WN = (job.N + 31) >> 5, WP = (job.P + 31) >> 5, NW = job.N * WN;
  const int ntx = (job.P + S2_PT_XY - 1) / S2_PT_XY;
  const unsigned nbp = (unsigned)((NW + S2_CW_BLOCK - 1) / S2_CW_BLOCK);
  const int last = zc1;  // the slab's last lattice plane
  const int slot0 = zc0 % job.ring;
  const unsigned lane = threadIdx.x & 31u;
  const int r = (int)(lane & 7u), pz = (int)(lane >> 3);
  const bool nearrule = !job.qef;
  const unsigned n = __ldg(list_count);
  const unsigned nwarps = gridDim.x * (S2_MT_BLOCK / 32);
  unsigned char *wb = reinterpret_cast<unsigned char *>(words);
#pragma unroll 1
  for (unsigned i = blockIdx.x * (S2_MT_BLOCK / 32) + (threadIdx.x >> 5); i < n; i += nwarps) {
    const unsigned t = __ldg(list + i);
    const int tx = (int)(t % (unsigned)ntx);
    const unsigned q = t / (unsigned)ntx;
    const int ty = (int)(q % (unsigned)ntx), tz = (int)(q / (unsigned)ntx);
    if (tx * S2_PT_XY >= job.N) continue;  // the tile of the last lattice point only: no cell
    const int kb = tk0 + tz * tzs, ke = min(kb + tzs, last + 1) - 1;
    const int y = ty * S2_PT_XY + r;
    const int ya = min(y, job.N), yc = min(y + 1, job.N);  // lattice rows (past the last: unused)
    const int w = tx >> 2, b = tx & 3;
    const bool more = w + 1 < WP;
    const unsigned ox = job.qef ? 0u : __ldg(offx + w);
    const unsigned oy = (!job.qef && y < job.N && s2_off_lattice(job, y + 1)) ? ~0u : 0u;
    const unsigned edge = (w == WN - 1 && (job.N & 31)) ? (1u << (job.N & 31)) - 1u : ~0u;
#pragma unroll 1
    for (int zb = kb - 1; zb <= ke - 1; zb += 4) {  // the same trips in every lane
      const int zc = zb + pz;  // this lane's cell plane: point planes zc, zc + 1
      const int K0 = min(max(zc, zc0), last), K1 = min(max(zc + 1, zc0), last);  // outside: unused
      // ring slots (the slab's planes zc0 .. last hold consecutive slots from
      // slot0, wrapping) and tile layers (K0, K1 lie in kb - 1 .. ke: this
      // tile's layer or the one below; -1 before the slab's first plane)
      const int s0 = slot0 + (K0 - zc0), s1 = slot0 + (K1 - zc0);
      const int slotK0 = s0 >= job.ring ? s0 - job.ring : s0, slotK1 = s1 >= job.ring ? s1 - job.ring : s1;
      const int lay0 = K0 < tk0 ? -1 : (K0 >= kb ? tz : tz - 1), lay1 = K1 < tk0 ? -1 : (K1 >= kb ? tz : tz - 1);
      // own row and plane; the row above in row 7, the plane above in plane 3
      const S2RowBits A = s2_row_bits(job, pb, tflags, ntx, WP, slotK0, lay0, ya, w, more, nearrule);
      S2RowBits C = A, B = A, Dd = A;
      if (r == 7) C = s2_row_bits(job, pb, tflags, ntx, WP, slotK0, lay0, yc, w, more, nearrule);
      if (pz == 3) B = s2_row_bits(job, pb, tflags, ntx, WP, slotK1, lay1, ya, w, more, nearrule);
      if (r == 7 && pz == 3) Dd = s2_row_bits(job, pb, tflags, ntx, WP, slotK1, lay1, yc, w, more, nearrule);
      const int up = r < 7 ? (int)lane + 1 : (int)lane;  // lane of row y + 1, same plane
      const S2RowBits A1 = s2_shfl_row(A, up), B1 = s2_shfl_row(B, up);
      const S2RowBits rowc0 = r < 7 ? A1 : C;   // plane zc, row y + 1
      const S2RowBits rowc1 = r < 7 ? B1 : Dd;  // plane zc + 1, row y + 1 (lanes of plane 3)
      const unsigned oz0 = (!job.qef && s2_off_lattice(job, K0)) ? ~0u : 0u;
      const unsigned oz1 = (!job.qef && s2_off_lattice(job, K1)) ? ~0u : 0u;
      const S2PlaneTerms T0 = s2_plane_terms(A, rowc0, more, ox, oy, oz0, nearrule);
      const S2PlaneTerms T3 = s2_plane_terms(B, rowc1, more, ox, oy, oz1, nearrule);  // used in plane 3's lanes
      const int nxt = pz < 3 ? (int)lane + 8 : (int)lane;  // lane of plane zc + 1, same row
      S2PlaneTerms T1;
      T1.andp = __shfl_sync(S2_FULL, T0.andp, nxt);
      T1.orp = __shfl_sync(S2_FULL, T0.orp, nxt);
      T1.tb = __shfl_sync(S2_FULL, T0.tb, nxt);
      T1.tt = __shfl_sync(S2_FULL, T0.tt, nxt);
      if (pz == 3) T1 = T3;
      const bool act = zc <= ke - 1 && zc >= zc0 && zc < zc1 && y < job.N;
      unsigned cb = 0u;
      if (act) {
        unsigned c = (T0.orp | T1.orp) & ~(T0.andp & T1.andp);
        if (nearrule) c |= T0.tb | T1.tt;
        cb = ((c & edge) >> (8 * b)) & 0xffu;
        wb[4 * ((long long)(zc - zc0) * NW + (long long)y * WN + w) + b] = (unsigned char)cb;
      }
      const unsigned T = act ? (unsigned)((y * WN + w) / S2_CW_BLOCK) : 0u;
      const unsigned long long key = act ? ((unsigned long long)(unsigned)(zc - zc0) << 32) | T : ~0ull;
      const unsigned peers = __match_any_sync(S2_FULL, key);
      const unsigned sum = __reduce_add_sync(peers, (unsigned)__popc(cb));
      if (act && sum && lane == (unsigned)(__ffs(peers) - 1)) {
        atomicAdd(tile_cnt + (unsigned long long)(zc - zc0) * nbp + T, sum);
        atomicAdd(plane_cnt + (zc - zc0), sum);
      }
    }
  }
  __threadfence();
  __syncthreads();
  __shared__ bool s_last;
  if (threadIdx.x == 0) s_last = atomicAdd(done, 1u) == gridDim.x - 1;
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  const unsigned nplanes = (unsigned)(zc1 - zc0);
  s2_scan_tiles<S2_MT_BLOCK, 4>(plane_cnt, nplanes, plane_off, base, slab_index);
  __syncthreads();  // every count read before it is cleared for the next slab
  for (unsigned p = threadIdx.x; p < nplanes; p += S2_MT_BLOCK) plane_cnt[p] = 0u;
  if (threadIdx.x == 0) *done = 0u;
}

// The candidates of each tile in order: key (x | y << 16 | z << 32) and the
// 8 lattice corner values (NaN where the point's unknown-value bit is set: a
// decided tile of the pruned evaluation wrote no value there).  Grid (nbp,
// cell planes), block = tile.  The block first lists the candidates of its
// words in shared memory (word << 5 | bit, in (y, x) order), then writes
// them one per thread: a word holds one or two candidates at most places of
// the surface, and a warp's 32 words (a row at N = 1024) a handful, so the
// block-wide list keeps the threads busy.  The tile's first slot is its
// plane's offset (s2m_cells_mark) plus the counts of the plane's tiles
// before it, summed by the block's threads together.  With tflags (after
// s2m_cells_mark_tiles; tk0 / tzs as there): the bytes of cells in decided
// tiles are cleared by the tiles' flags, and a corner of the slab's own planes
// has no value in the ring when its tile is decided (its unknown-value bit
// says so in the plane before them).
// One tile (cell plane dz, tile b of nbp in the plane) of s2m_cells_emit.
// Everything that depends on the plane alone (ring slots, flag rows, the
// division by the words per row) is formed once per block.
__device__ __forceinline__ void s2_emit_tile(const S2Job &job, const float *__restrict__ ring,
                                             const unsigned *__restrict__ unk, const unsigned *__restrict__ words,
                                             const unsigned long long *__restrict__ plane_off,
                                             const unsigned *__restrict__ tile_cnt, S2Cand cand, unsigned *err,
                                             int zc0, const unsigned *__restrict__ tflags, int tk0, int tzs,
                                             unsigned b, int dz, unsigned nbp, bool vals) {
  __shared__ unsigned s_warp[32];
  __shared__ unsigned s_pre[S2_CW_BLOCK / 32];
  __shared__ unsigned short s_list[S2_CW_BLOCK * 32];
  const unsigned tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
  const int WN = (job.N + 31) >> 5, NW = job.N * WN, WP = (job.P + 31) >> 5;
  const int ntx = (job.P + S2_PT_XY - 1) / S2_PT_XY;
  const unsigned magic_wn = job.magic_wn;  // word index -> (row, word): division by WN (>= 2)
  const int yw = (int)(b * S2_CW_BLOCK + tid);
  const unsigned *plane_cnt = tile_cnt + (unsigned long long)dz * nbp;
  const int Z0 = zc0 + dz;  // the cells' lower lattice plane; the upper one is Z0 + 1
  // the planes' ring slots and flag rows (for the corner values only)
  const float *rz[2] = {ring, ring};
  const unsigned *uz[2] = {unk, unk};
  const unsigned char *fz[2] = {nullptr, nullptr};
  if (vals) {
    const int s0 = Z0 % job.ring, s1 = s0 + 1 == job.ring ? 0 : s0 + 1;
    const int sl[2] = {s0, s1};
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int Z = Z0 + h;
      rz[h] = ring + (long long)sl[h] * job.plane;
      uz[h] = unk ? unk + (long long)sl[h] * job.P * WP : nullptr;
      fz[h] = (tflags && Z >= tk0)
                  ? reinterpret_cast<const unsigned char *>(tflags) + (long long)((Z - tk0) / tzs) * ntx * (4 * WP)
                  : nullptr;
    }
  }
  // every load first: the plane's offset, the counts of its tiles before this
  // one, this thread's word and its tiles' flags
  const unsigned long long poff = __ldg(plane_off + dz);
  unsigned pre = 0u;
  for (unsigned q = tid; q < b; q += S2_CW_BLOCK) pre += __ldg(plane_cnt + q);
  unsigned mask = yw < NW ? words[(long long)dz * NW + yw] : 0u;
  if (tflags && yw < NW) {  // bytes of cells in decided tiles were not written (s2m_cells_mark_tiles)
    const int y = WN > 1 ? (int)s2_udiv((unsigned)yw, (unsigned)WN, magic_wn) : yw, w = yw - y * WN;
    const int layer = (Z0 + 1 - tk0) / tzs;
    const unsigned f = __ldg(tflags + ((long long)layer * ntx + (y >> 3)) * WP + w);
    mask &= ~((f & 0x01010101u) * 0xffu);
  }
  pre = __reduce_add_sync(S2_FULL, pre);
  if (lane == 0) s_pre[warp] = pre;
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
  const unsigned total = s_warp[31];  // slots past the block's warps are 0: slot 31 gets the total
  {
    unsigned r = s_warp[warp] + inc - cnt, rem = mask;
    while (rem) {
      const unsigned bit = __ffs(rem) - 1u;
      rem &= rem - 1u;
      s_list[r++] = (unsigned short)((tid << 5) | bit);
    }
  }
  __syncthreads();
  unsigned long long first = poff;
#pragma unroll
  for (int k = 0; k < S2_CW_BLOCK / 32; ++k) first += s_pre[k];
#pragma unroll 1
  for (unsigned r = tid; r < total; r += S2_CW_BLOCK) {
    const unsigned e = s_list[r];
    const unsigned ywc = b * S2_CW_BLOCK + (e >> 5);
    const int wy = WN > 1 ? (int)s2_udiv(ywc, (unsigned)WN, magic_wn) : (int)ywc, w = (int)ywc - wy * WN;
    const unsigned bit = e & 31u;
    const int x = 32 * w + (int)bit;
    const unsigned long long o = first + r;
    if (o >= cand.cap) {
      atomicOr(err, S2_ERR_CAND_OVF);
      continue;
    }
    cand.key[o] = (unsigned long long)x | ((unsigned long long)wy << 16) | ((unsigned long long)Z0 << 32);
    if (!vals) continue;  // the vertex kernel reads the corners from the resident ring
    float v[8];
#pragma unroll
    for (int h = 0; h < 2; ++h) {  // corner k = bx | by << 1 | bz << 2
      const float *p = rz[h] + (long long)wy * job.pitch + x;
      v[4 * h + 0] = __ldg(p);
      v[4 * h + 1] = __ldg(p + 1);
      v[4 * h + 2] = __ldg(p + job.pitch);
      v[4 * h + 3] = __ldg(p + job.pitch + 1);
    }
    if (unk) {  // corners of decided tiles: no value in the ring
      const bool more = w + 1 < WP;
#pragma unroll
      for (int q = 0; q < 4; ++q) {  // corner k = 2 q + bx lies in point row q = by | bz << 1
        const int h = q >> 1, Y = wy + (q & 1);
        bool u0, u1;
        if (fz[h]) {  // the slab's own planes: the flags of the points' tiles
          const unsigned char *fr = fz[h] + (long long)(Y >> 3) * (4 * WP);
          u0 = __ldg(fr + (x >> 3)) & S2_TILE_DECIDED;
          u1 = __ldg(fr + ((x + 1) >> 3)) & S2_TILE_DECIDED;
        } else {  // unknown-value bits (planes written in full)
          const unsigned *ur = uz[h] + (long long)Y * WP + w;
          const unsigned lo = __ldg(ur), hi = more ? __ldg(ur + 1) : 0u;
          u0 = (lo >> bit) & 1u;
          u1 = (__funnelshift_r(lo, hi, 1) >> bit) & 1u;
        }
        if (u0) v[2 * q] = __int_as_float(0x7fc00000);
        if (u1) v[2 * q + 1] = __int_as_float(0x7fc00000);
      }
    }
    float4 *dst = reinterpret_cast<float4 *>(cand.val + 8 * o);
    dst[0] = make_float4(v[0], v[1], v[2], v[3]);
    dst[1] = make_float4(v[4], v[5], v[6], v[7]);
  }
}

// Grid (nbp, ceil(cell planes / S2_EMIT_PLANES)): a block takes the tile at
// the same place in S2_EMIT_PLANES consecutive planes (the upper corners of
// one plane's cells are the lower corners of the next plane's), skipping those
// without candidates.  vals = 0: keys only (the vertex kernel reads the
// corners from a ring that holds the whole job).  (Measured slower: a list of
// the non-empty tiles taken by blocks resident on every SM, since the list's
// order is the atomic order and (z, y, x) order keeps neighbouring tiles'
// corner loads together; one
// warp per tile, since a warp alone drains a dense tile's candidates long
// after the others.)
#define S2_EMIT_PLANES 2
__global__ void __launch_bounds__(S2_CW_BLOCK) s2m_cells_emit(S2Job job, const float *__restrict__ ring,
                                                            const unsigned *__restrict__ unk,
                                                            const unsigned *__restrict__ words,
                                                            const unsigned long long *__restrict__ plane_off,
                                                            const unsigned *__restrict__ tile_cnt, S2Cand cand,
                                                            unsigned *err, int zc0,
                                                            const unsigned *__restrict__ tflags, int tk0, int tzs,
                                                            int planes, int vals) {
  S2_PDL_WAIT();
  const int dz0 = (int)blockIdx.y * S2_EMIT_PLANES;
#pragma unroll 1
  for (int i = 0; i < S2_EMIT_PLANES; ++i) {
    const int dz = dz0 + i;
    if (dz >= planes) break;
    if (__ldg(tile_cnt + (unsigned long long)dz * gridDim.x + blockIdx.x) == 0u) continue;  // no candidate
    __syncthreads();  // the previous tile's shared lists are read
    s2_emit_tile(job, ring, unk, words, plane_off, tile_cnt, cand, err, zc0, tflags, tk0, tzs, blockIdx.x, dz,
                 gridDim.x, vals != 0);
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
  S2_PDL_WAIT();
  const unsigned long long n = min(cand.base[nslabs], cand.cap);
  for (unsigned long long i = (unsigned long long)blockIdx.x * 256u + threadIdx.x; i < n;
       i += (unsigned long long)gridDim.x * 256u) {
    const unsigned long long k = cand.key[i];
    S2Cell c;
    c.x = (int)(k & 0xffffull);
    c.y = (int)((k >> 16) & 0xffffull);
    c.z = (int)((k >> 32) & 0xffffull);
    const unsigned long long t = s2_cell_prune_tile(job, c, tbase, D, nzc);
    // one atomic per tile and warp (a warp's candidates share a few tiles)
    const unsigned am = __activemask();
    const unsigned peers = __match_any_sync(am, t);
    const int leader = __ffs(peers) - 1;
    unsigned first = 0;
    if ((int)(threadIdx.x & 31u) == leader) first = atomicAdd(tcnt + t, (unsigned)__popc(peers));
    first = __shfl_sync(peers, first, leader);
    const unsigned rank = first + (unsigned)__popc(peers & s2_lanemask_lt());
    trank[i] = (t << 16) | rank;  // a tile covers at most 8 x 8 x 8 cells
  }
}

// tcnt[0 .. T) becomes each tile's first position within its block of
// S2_VT_TILE tiles; part_cnt[b] = block b's total.  The last block to finish
// scans the totals into part_off (part_base[0] = 0 on entry); `done` returns
// to 0.
__global__ void __launch_bounds__(256) s2m_vtile_scan(unsigned *tcnt, unsigned long long T, unsigned *part_cnt,
                                                      unsigned long long *part_off, unsigned long long *part_base,
                                                      unsigned *done) {
  S2_PDL_WAIT();
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
  s2_scan_tiles<256, 4>(part_cnt, gridDim.x, part_off, part_base, 0);
  if (tid == 0) *done = 0u;
}

__global__ void __launch_bounds__(256) s2m_vtile_scatter(S2Cand cand, int nslabs, const unsigned *__restrict__ tcnt,
                                                         const unsigned long long *__restrict__ part_off,
                                                         const unsigned long long *__restrict__ trank,
                                                         unsigned *__restrict__ perm) {
  S2_PDL_WAIT();
  const unsigned long long n = min(cand.base[nslabs], cand.cap);
  for (unsigned long long i = (unsigned long long)blockIdx.x * 256u + threadIdx.x; i < n;
       i += (unsigned long long)gridDim.x * 256u) {
    const unsigned long long tr = trank[i], t = tr >> 16;
    perm[part_off[t / S2_VT_TILE] + tcnt[t] + (tr & 0xffffull)] = (unsigned)i;
  }
}

// Vertex compaction of the per-job pipeline in two wait-free passes.  The
// vertex kernel counts each tile's vertices (tiles of S2_VC_TILE candidates,
// vc_cnt); s2m_vc_scan (one block) turns the counts into each tile's first
// vertex (vc_off) and the job's vertex total (vc_base[1], mesh.vtotal;
// vc_base[0] = 0 on entry); s2m_vcompact then writes every tile's vertices
// in order, as s2_vcompact_worker does with its look-back (which the
// persistent batch kernel keeps).
__global__ void __launch_bounds__(256) s2m_vc_scan(S2Cand cand, int nslabs, const unsigned *vc_cnt,
                                                   unsigned long long *vc_off, unsigned long long *vc_base,
                                                   S2MeshDev mesh) {
  S2_PDL_WAIT();
  const unsigned long long ncand = min(cand.base[nslabs], cand.cap);
  const unsigned ntiles = (unsigned)((ncand + S2_VC_TILE - 1) / S2_VC_TILE);
  s2_scan_tiles<256, 16>(vc_cnt, ntiles, vc_off, vc_base, 0);
  if (threadIdx.x == 0) *mesh.vtotal = vc_base[1];  // written by this thread in the scan
}

__global__ void __launch_bounds__(S2_VC_BLOCK) s2m_vcompact(S2Job job, S2Cand cand, S2MeshDev mesh, int nslabs,
                                                          const unsigned long long *__restrict__ vc_off) {
  S2_PDL_WAIT();
  __shared__ unsigned s_warp[32];
  const unsigned tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
  const unsigned long long ncand = min(cand.base[nslabs], cand.cap);
  const unsigned ntiles = (unsigned)((ncand + S2_VC_TILE - 1) / S2_VC_TILE);
  const unsigned lt = s2_lanemask_lt();
  for (unsigned tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    unsigned long long keys[S2_VC_CPT];
    unsigned ballots[S2_VC_CPT];
#pragma unroll
    for (int m = 0; m < S2_VC_CPT; ++m) {
      const unsigned long long o = (unsigned long long)tile * S2_VC_TILE + m * S2_VC_BLOCK + tid;
      keys[m] = o < ncand ? cand.key[o] : 0ull;
      ballots[m] = __ballot_sync(S2_FULL, (keys[m] >> 63) != 0ull);
      if (lane == 0) s_warp[m * (S2_VC_BLOCK / 32) + warp] = __popc(ballots[m]);
    }
    __syncthreads();
    if (warp == 0) s2_warp_exclusive32(s_warp);
    __syncthreads();
    // every load of the tile's vertices first, so that they are in flight together
    float pn[S2_VC_CPT][6];
#pragma unroll
    for (int m = 0; m < S2_VC_CPT; ++m) {
      if (!((ballots[m] >> lane) & 1u)) continue;
      const unsigned long long o = (unsigned long long)tile * S2_VC_TILE + m * S2_VC_BLOCK + tid;
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        pn[m][c] = __ldg(cand.pos + 3 * o + c);
        pn[m][3 + c] = __ldg(cand.nrm + 3 * o + c);
      }
    }
    const unsigned long long first = vc_off[tile];
#pragma unroll
    for (int m = 0; m < S2_VC_CPT; ++m) {
      // one count per row and warp: the warp's vertices are in (z, y, x) order,
      // so a row's vertices are neighbours
      const bool has = (ballots[m] >> lane) & 1u;
      const unsigned long long row = has ? ((keys[m] >> 32) & 0xffffull) * (unsigned long long)job.N +
                                               ((keys[m] >> 16) & 0xffffull)
                                         : ~0ull;
      const unsigned peers = __match_any_sync(S2_FULL, row);
      if (has && (unsigned)(__ffs(peers) - 1) == lane) atomicAdd(mesh.rowcnt + row, (unsigned)__popc(peers));
      if (!has) continue;
      const unsigned long long v = first + s_warp[m * (S2_VC_BLOCK / 32) + warp] + __popc(ballots[m] & lt);
      const unsigned long long key = keys[m] & ~(1ull << 63);
      if (v >= 0xFFFFFFFEull) atomicOr(mesh.err, S2_ERR_INDEX_OVF);
      if (v >= mesh.vcap) {
        atomicOr(mesh.err, S2_ERR_VERT_OVF);
        continue;
      }
      mesh.key[v] = key;
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        mesh.pos[3 * v + c] = pn[m][c];
        mesh.nrm[3 * v + c] = pn[m][3 + c];
      }
    }
    __syncthreads();
  }
}

__global__ void __launch_bounds__(S2_SCAN_BLOCK) s2m_rowscan(S2MeshDev mesh, unsigned long long R) {
  S2_PDL_WAIT();
  s2_rowscan_worker(mesh, R);
}

// Quads of the per-job pipeline in three passes that never wait on one
// another (a look-back over the tiles made every tile's block wait at a
// barrier while its first warp walked back over tiles still searching):
//   s2m_quads_find   each vertex's neighbour lookups -- the row searches --
//                    stored as 6 words per vertex in the candidates' position
//                    and normal arrays (free once s2m_vcompact has copied the
//                    vertices out; the vertices never outnumber the
//                    candidates), each tile's triangle count, the invalid
//                    quads (mesh.rs:275-277)
//   s2m_quads_scan   one block: each tile's first triangle and the total
//   s2m_quads_write  each tile's triangles from the stored lookups, at its
//                    first triangle, in vertex order (mesh.rs:280-321)
// Tiles of S2_Q_TILE vertices, S2_Q_VPT per thread (v = tile * S2_Q_TILE +
// m * S2_Q_BLOCK + thread); quad scan words: tile offsets
// (u64), then tile counts (u32), then the base pair (u64).
__global__ void __launch_bounds__(S2_Q_BLOCK) s2m_quads_find(S2Job job, S2MeshDev mesh, unsigned *__restrict__ lk0,
                                                           unsigned *__restrict__ lk1, unsigned *__restrict__ tcnt) {
  S2_PDL_WAIT();
  __shared__ unsigned s_red[S2_Q_BLOCK / 32];
  const unsigned tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
  const unsigned long long V = *mesh.vtotal;
  if (V > mesh.vcap) return;  // vertex overflow: the host re-runs with larger buffers
  const unsigned ntiles = (unsigned)((V + S2_Q_TILE - 1) / S2_Q_TILE);
  unsigned invalid = 0;
  for (unsigned tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    unsigned cnt = 0;
#pragma unroll
    for (int m = 0; m < S2_Q_VPT; ++m) {
      const unsigned long long v = (unsigned long long)tile * S2_Q_TILE + m * S2_Q_BLOCK + tid;
      if (v >= V) continue;
      const unsigned long long key = __ldg(mesh.key + v);
      const S2QuadLookups l = s2_quad_lookups<true>(mesh, job.N, (unsigned)v, key);
      const S2Quads q = s2_quads_from(l, (unsigned)v, key, mesh.zq);
      cnt += 2u * __popc(q.valid);
      invalid += q.invalid;
      lk0[3 * v] = l.ax;
      lk0[3 * v + 1] = l.axm1;
      lk0[3 * v + 2] = l.bx;
      lk1[3 * v] = l.bxm1;
      lk1[3 * v + 1] = l.cx;
      lk1[3 * v + 2] = l.own;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(S2_FULL, cnt, o);
    if (lane == 0) s_red[warp] = cnt;
    __syncthreads();
    if (tid == 0) {
      unsigned t = 0;
#pragma unroll
      for (int k = 0; k < S2_Q_BLOCK / 32; ++k) t += s_red[k];
      tcnt[tile] = t;
    }
    __syncthreads();
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) invalid += __shfl_xor_sync(S2_FULL, invalid, o);
  if (lane == 0 && invalid) atomicAdd(mesh.invalid, (unsigned long long)invalid);
}

__global__ void __launch_bounds__(256) s2m_quads_scan(S2MeshDev mesh, const unsigned *tcnt,
                                                      unsigned long long *toff, unsigned long long *tbase) {
  S2_PDL_WAIT();
  const unsigned long long V = *mesh.vtotal;
  if (V > mesh.vcap) return;
  const unsigned ntiles = (unsigned)((V + S2_Q_TILE - 1) / S2_Q_TILE);
  s2_scan_tiles<256, 16>(tcnt, ntiles, toff, tbase, 0);
  if (threadIdx.x == 0) *mesh.ntris = tbase[1];  // written by this thread in the scan
}

__global__ void __launch_bounds__(S2_Q_BLOCK) s2m_quads_write(S2MeshDev mesh, const unsigned *__restrict__ lk0,
                                                            const unsigned *__restrict__ lk1,
                                                            const unsigned long long *__restrict__ toff) {
  S2_PDL_WAIT();
  __shared__ unsigned s_warp[32];
  const unsigned tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
  const unsigned long long V = *mesh.vtotal;
  if (V > mesh.vcap) return;
  const unsigned ntiles = (unsigned)((V + S2_Q_TILE - 1) / S2_Q_TILE);
  for (unsigned tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    S2Quads qd[S2_Q_VPT];
    unsigned ntri[S2_Q_VPT];
#pragma unroll
    for (int m = 0; m < S2_Q_VPT; ++m) {
      const unsigned long long v = (unsigned long long)tile * S2_Q_TILE + m * S2_Q_BLOCK + tid;
      qd[m].valid = 0;
      if (v < V) {
        S2QuadLookups l;
        l.ax = __ldg(lk0 + 3 * v);
        l.axm1 = __ldg(lk0 + 3 * v + 1);
        l.bx = __ldg(lk0 + 3 * v + 2);
        l.bxm1 = __ldg(lk1 + 3 * v);
        l.cx = __ldg(lk1 + 3 * v + 1);
        l.own = __ldg(lk1 + 3 * v + 2);
        qd[m] = s2_quads_from(l, (unsigned)v, __ldg(mesh.key + v), mesh.zq);
      }
      ntri[m] = 2u * __popc(qd[m].valid);
      unsigned inc = ntri[m];
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const unsigned t = __shfl_up_sync(S2_FULL, inc, o);
        if ((int)lane >= o) inc += t;
      }
      if (lane == 31) s_warp[m * (S2_Q_BLOCK / 32) + warp] = inc;
      ntri[m] = inc - ntri[m];  // exclusive within the warp
    }
    if (tid < 32 - S2_Q_VPT * (S2_Q_BLOCK / 32)) s_warp[S2_Q_VPT * (S2_Q_BLOCK / 32) + tid] = 0u;
    __syncthreads();
    if (warp == 0) s2_warp_exclusive32(s_warp);
    __syncthreads();
    const unsigned long long first = toff[tile];
#pragma unroll
    for (int m = 0; m < S2_Q_VPT; ++m) {
      unsigned long long t = first + s_warp[m * (S2_Q_BLOCK / 32) + warp] + ntri[m];
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
