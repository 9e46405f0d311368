// s2m_device.h -- structures shared by the host runtime, the nvcc-compiled
// kernels and the NVRTC-compiled per-SDF kernels.  Plain C types only (NVRTC
// compiles this without system headers).
#pragma once

// Lattice: grid point (i, j, k), 0 <= i, j, k <= N, has the coordinates
// c(i) = bmin + size * i, rounded in binary32 exactly as the reference
// computes a cell's lower corner (dualcontour.wgsl:22-27).  Planes of the
// lattice live in a ring of `ring` planes; plane k sits in slot k % ring,
// row j at offset j * pitch, so a z-slab of cells and its upper plane are
// resident together.
struct S2Job {
  int N;                   // cells per axis
  int P;                   // lattice points per axis (N + 1)
  int pitch;               // floats per lattice row (P rounded up to 32)
  int ring;                // planes in the ring
  long long plane;         // floats per plane (P * pitch)
  float bmin;              // lower corner of the box (same on every axis)
  float size;              // cell edge (bmax - bmin) / (N - 1)
  float eps;               // normal epsilon
  float guard;             // |f| below which off-lattice corners are re-evaluated
  int lag;                 // 1: labels are z + 1 (reference slice lag)
  int exact;               // 1: re-evaluate off-lattice corners of every cell
  int qef;                 // 1: precision mode (lattice corners, QEF vertex, FP64 solve)
  unsigned magic_n;        // floor(2^32 / N) + 1: division by N of 32-bit indices
  unsigned magic_p;        // floor(2^32 / P) + 1
  int zb;                  // first cell plane of the job's z range (0: the whole lattice)
  unsigned magic_wn;       // floor(2^32 / WN) + 1 (WN = ceil(N / 32) >= 2; else 0): division by WN
};

// Division of a 32-bit index by d (2 <= d < 2^31) with the precomputed
// magic = floor(2^32 / d) + 1: the high product overestimates the quotient by
// at most one, and the remainder's sign tells which.
#if defined(__CUDACC__) || defined(__CUDACC_RTC__)
__device__ __forceinline__ unsigned s2_udiv(unsigned c, unsigned d, unsigned magic) {
  unsigned q = __umulhi(c, magic);
  return ((int)(c - q * d) < 0) ? q - 1u : q;
}
#endif

// Per-slab buffers of the cell pass.
struct S2Slab {
  float *ring;                    // lattice ring
  unsigned long long *status;     // look-back words of s2m_cells tiles
  unsigned *tile_counter;         // [0] s2m_cells
  unsigned *err;                  // error flags (S2_ERR_*)
};

// Candidate cells of the whole job, in (z, y, x) order: cells that may carry
// a vertex.  s2m_cells appends them slab by slab; s2m_vertices places their
// vertices; s2m_vcompact keeps those with a vertex.
struct S2Cand {
  unsigned long long *key;        // x | y << 16 | z << 32; after s2m_vertices the final
                                  // key (label, signs << 48, has_vertex << 63)
  float *val;                     // 8 lattice corner values per candidate (32-byte aligned)
  float *pos;                     // 3 per candidate
  float *nrm;                     // 3 per candidate
  unsigned long long cap;         // capacity of the arrays
  unsigned long long *base;       // nslabs + 1 running offsets (exact even on overflow)
  unsigned long long *status;     // look-back words of s2_vcompact_worker's tiles (batch engine)
  unsigned *tile_counter;         // s2_vcompact_worker's tile counter (batch engine)
};

// Sign (v > 0) and near-zero (!(|v| >= guard)) bits of lattice points,
// indexed by ring slot like the lattice values: word ((k % ring) * P + y) *
// WP + x / 32 (WP = ceil(P / 32)) holds bit x % 32 of plane k, row y; in
// little-endian bytes, byte x / 8 holds bit x % 8.  Bits past the lattice
// edge are 0.  `unk` (pruned evaluation only): the point lies in a decided
// tile, so its sign and near bits are known but its value was not computed
// and the ring holds no value for it.
struct S2PointBits {
  unsigned *pos;
  unsigned *near;
  unsigned *unk;
};

// Mesh outputs and the cross-slab counters.
struct S2MeshDev {
  float *pos;                     // 3 * vcap
  float *nrm;                     // 3 * vcap
  unsigned long long *key;        // vcap: x | y << 16 | z << 32 | signs << 48
  unsigned *tris;                 // 3 * tcap
  unsigned long long vcap;
  unsigned long long tcap;
  unsigned long long *vtotal;     // out: vertices of the job (exact even on overflow)
  unsigned *rowcnt;               // N * N vertices per (z label, y) row
  unsigned *rowstart;             // N * N + 1 exclusive prefix of rowcnt
  unsigned long long *scan_status;  // look-back words (row scan, quads)
  unsigned *counters;             // [2] row scan, [3] quads tile counters
  unsigned long long *ntris;      // out: triangles (exact even on overflow)
  unsigned long long *invalid;    // out: invalid quads (mesh.rs:275-277)
  unsigned long long *ncand;      // out: candidates over all slabs
  unsigned *err;
  unsigned long long wait_ns;     // bound of each device wait (look-back), GPU global timer ns
  unsigned hold;                  // test hook: S2_HOLD_* (0 in normal runs)
  unsigned zq;                    // vertices with label z below zq make no quads (a z part's context plane)
};

// Programmatic dependent launch: the per-job pipeline launches each kernel so
// that its blocks may be scheduled while the kernel before it drains; every
// such kernel waits here, before it reads anything, until that kernel has
// finished and its writes are visible (a no-op for an ordinary launch).
#if defined(__CUDA_ARCH__)
#define S2_PDL_WAIT() asm volatile("griddepcontrol.wait;" ::: "memory")
#else
#define S2_PDL_WAIT()
#endif

// Test hooks (S2MeshDev::hold): a flag that nothing sets, so that a bounded
// device wait runs out and the run reports S2M_E_TIMEOUT.  Only the waiting
// is affected; every write stays bounds-checked.
#define S2_HOLD_ROWSCAN_TILE0 0x1u  /* tile 0 of the row-start scan never publishes its prefix */

// Flag word of a pruning tile's record (the tile pass): the SDF's interval
// over the tile's box lies at or beyond +guard (DECIDED | POSITIVE) or -guard
// (DECIDED), so every point's sign is known and its near-zero bit is 0.
#define S2_TILE_DECIDED 1u
#define S2_TILE_POSITIVE 2u

#define S2_ERR_LOOKBACK 0x1u      /* a look-back wait hit its iteration limit   */
#define S2_ERR_CAND_OVF 0x2u      /* candidate arrays too small                 */
#define S2_ERR_VERT_OVF 0x4u      /* vertex arrays too small                    */
#define S2_ERR_TRI_OVF 0x8u       /* triangle array too small                   */
#define S2_ERR_INDEX_OVF 0x10u    /* more than 2^32 - 2 vertices                */
#define S2_ERR_HOST_OVF 0x40u     /* host arrays too small for a job's z parts   */

#define S2_CELL_BLOCK 256
#define S2_CELL_CPT 32
#define S2_CELL_TILE (S2_CELL_BLOCK * S2_CELL_CPT)
#define S2_CW_BLOCK 256          /* words of 32 cells per classification tile */
#define S2_EVAL_BLOCK 256
#define S2_EVAL_RUN 4
// Tile pruning: tiles of 8 x 8 lattice points in x and y and at most 8
// planes in z; the pruned evaluation runs one tile per warp, 4 per block.
#define S2_PT_XY 8
#define S2_PT_ZMAX 8
#define S2_VT_TILE 2048  // per-tile candidate counts scanned per block of s2m_vtile_scan (256 threads x 8)
#define S2_PT_BLOCK 128
#define S2_PT_COARSE 4            /* tiles per coarse box of the tile pass, along x and y */
#define S2_PT_COARSE_Z 2          /* ... and layers of tiles along z */
#define S2_VX_BLOCK 1024          /* s2m_vertices with a pruning form: one block per SM */
#define S2_VX_SMALL 128           /* s2m_vertices otherwise: 8 blocks per SM */
#define S2_PL_BLOCK 1024          /* s2m_evalpl_*: one block per SM, one listed tile per warp */
#define S2_VC_BLOCK 256
#define S2_VC_CPT 4
#define S2_VC_TILE (S2_VC_BLOCK * S2_VC_CPT)
#define S2_SCAN_BLOCK 256
#define S2_SCAN_CPT 8
#define S2_SCAN_TILE (S2_SCAN_BLOCK * S2_SCAN_CPT)
#define S2_Q_BLOCK 256
#define S2_Q_VPT 2
#define S2_Q_TILE (S2_Q_BLOCK * S2_Q_VPT)
#define S2_NO_VERTEX 0xFFFFFFFFu
