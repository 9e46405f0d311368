// batch.cu -- many meshing jobs in one persistent launch.
//
// A batch job is a CSG program (a postfix list of the library's primitives
// and operators, evaluated by an interpreter on the device, so no per-job
// compilation) plus its own resolution and bounds.  All jobs of a batch run
// in ONE launch of s2m_batch_kernel: its blocks take tickets from a device
// work queue in which every job contributes nine stages in order --
//   T tile pass (interval pruning of the program per tile of the lattice),
//   E evaluate the job's lattice, M candidate bits per classification tile,
//   S (one item) the tiles' first candidate slots, C the candidates in
//   (z, y, x) order, X place vertices, V compact vertices, R scan row starts,
//   Q emit quads --
// each stage a run of items.  A block that takes an item of stage s of a job
// first waits until every item of stage s-1 of that job is done.  Those items
// hold lower tickets, so they were taken by blocks already running: the wait
// always ends (it is still bounded, and a block that gives up raises an error
// flag instead of hanging).  Jobs overlap on the device: while the last items
// of one job's stage finish, blocks already work on the next jobs.
//
// The dual-contouring rule is the one of the per-job pipeline
// (s2m_dc_core.cuh, s2m_workers.cuh): the reference's mass point or the
// precision-mode QEF, bit-identical to the per-job path for the same SDF.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/sdf2mesh.h"
#include "s2m_device.h"
#include "s2m_lookback.cuh"
#include "s2m_dc_core.cuh"
#include "s2m_workers.cuh"
#include "s2m_csg.cuh"

// ---------------------------------------------------------------------------
// Device-side batch description.

enum {
  S2_ST_TILES = 0,
  S2_ST_EVAL,
  S2_ST_MARK,   // candidate bits and counts per classification tile
  S2_ST_CSCAN,  // one item: the tiles' first candidate slots
  S2_ST_EMIT,   // candidates with their corner values
  S2_ST_VERT,
  S2_ST_VCOMPACT,
  S2_ST_ROWS,
  S2_ST_QUADS,
  S2_NSTAGES
};
static_assert(S2_NSTAGES == S2M_BATCH_STAGES, "stage count of the C ABI");
#define S2_B_TILE 8          // lattice points per edge of a tile
#define S2_B_TILES_ITEM 256  // tiles per item of the tile pass (one per thread)
#define S2_B_EVAL_TILES 64   // tiles per item of the evaluation (one warp per tile)
#define S2_B_CELL_TILES 4    // classification tiles per item of the mark and emit stages
#define S2_B_VERT_CHUNK 256
#define S2_ERR_BATCH_WAIT 0x20u

struct S2BatchJob {
  S2Job job;                        // ring == P: the whole lattice is resident
  const float *prog;
  int prog_len;
  int nzc;                          // cell slices emitted (N, or N - 1 with the slice lag)
  float *lattice;
  unsigned *tiles;                  // per tile: flag word, then the node codes (S2_CSG_TILE_WORDS)
  int ntx;                          // tiles per lattice axis
  int prune;                        // 0: every point with the full program (tiles unused)
  S2Cand cand;
  S2MeshDev mesh;
  unsigned *cwords;                 // candidate bits: one word per thread and classification tile
  unsigned *ctcnt;                  // candidates per classification tile
  unsigned long long *ctoff;        // first candidate slot of each classification tile
  unsigned *xcounter;               // vertex chunk counter
  unsigned *done;                   // completed items per stage
  unsigned nitems[S2_NSTAGES];
  unsigned scan_tiles;
};

struct S2BatchSeg {
  unsigned long long start;  // first ticket
  unsigned job, stage, count, pad;
};

struct S2BatchCtl {
  unsigned long long next;  // ticket counter
  unsigned err;
  unsigned pad;
  // block time (GPU global timer ns, summed over blocks) spent on each
  // stage's items, and waiting for a job's previous stage
  unsigned long long busy_ns[S2_NSTAGES];
  unsigned long long wait_ns;
};

// Results gathered for the host: ntris, invalid, vtotal, err, candidates.
struct S2BatchResult {
  unsigned long long ntris, invalid, vtotal, ncand;
  unsigned err, pad;
};

// Tile pass: one thread per tile of 8 x 8 x 8 lattice points (fewer at the
// lattice's far faces).  The program's interval pass (s2c_tile) over the
// tile's box gives the nodes' codes and the interval of the value; the tile
// is DECIDED (| POSITIVE) when that interval lies at or beyond +guard
// (-guard), as the per-job pipeline's tile pass decides.  The box reaches
// one lattice point past the tile's points on each axis and is widened by
// the per-job pipeline's margin (s2_prune_box: more than the normal epsilon
// plus thousands of ulps of the coordinates), so the codes also hold at every
// point the vertex stage evaluates for the cells whose lower corner lies in
// the tile (cell x spans points x .. x + 1; its off-lattice corners mn + size
// and normal samples p +- eps lie within the margin).
__device__ __forceinline__ s2i s2b_tile_axis(const S2Job &j, unsigned t) {
  const float mg = __fadd_rn(__fmul_rn(fabsf(j.eps), 1.0625f), __fmul_rn(__fadd_rn(fabsf(j.bmin), fabsf(j.size)), 0x1p-12f));
  s2i a;
  a.lo = __fsub_rn(s2_coord(j, (int)(S2_B_TILE * t)), mg);
  a.hi = __fadd_rn(s2_coord(j, (int)(S2_B_TILE * t) + S2_B_TILE), mg);
  return a;
}

// The tile record of cell c (the tile of its lower corner).
__device__ __forceinline__ const unsigned *s2b_cell_tile(const S2BatchJob &J, S2Cell c) {
  const unsigned nt = (unsigned)J.ntx;
  const unsigned t = ((unsigned)(c.z / S2_B_TILE) * nt + (unsigned)(c.y / S2_B_TILE)) * nt + (unsigned)(c.x / S2_B_TILE);
  return J.tiles + (size_t)t * S2_CSG_TILE_WORDS;
}

// Evaluators of the vertex stage with the tile codes of each candidate's
// cell: S2CsgLanes for s2_vertex_warp (lane l's requests with lane l's
// record, from shared memory), S2CsgCell for one lane's own cell (precision
// mode).  A null record evaluates the full program.
struct S2CsgLanes {
  static constexpr bool kStdNormal = true;
  S2CsgSdf f;
  const unsigned *const *rec;  // per thread of the block
  __device__ __forceinline__ float at(unsigned l, float x, float y, float z) const {
    const unsigned *r = rec[(threadIdx.x & ~31u) + l];
    return r ? f.eval_tile(x, y, z, r + 1) : f(x, y, z);
  }
};
__device__ __forceinline__ float s2_sdf_for(const S2CsgLanes &f, unsigned l, float x, float y, float z) {
  return f.at(l, x, y, z);
}
struct S2CsgCell {
  static constexpr bool kStdNormal = true;
  S2CsgSdf f;
  const unsigned *rec;
  __device__ __forceinline__ float operator()(float x, float y, float z) const {
    return rec ? f.eval_tile(x, y, z, rec + 1) : f(x, y, z);
  }
  __device__ __forceinline__ void normal(float px, float py, float pz, float eps, float n[3]) const {
    s2_tetra_normal(*this, px, py, pz, eps, n);
  }
};

__device__ __forceinline__ void s2b_stage_tiles(const S2BatchJob &J, unsigned item) {
  const S2Job &j = J.job;
  const unsigned nt = (unsigned)J.ntx, ntiles = nt * nt * nt;
  const unsigned t = item * S2_B_TILES_ITEM + threadIdx.x;
  if (!J.prune || t >= ntiles) return;
  const unsigned tx = t % nt, q = t / nt, ty = q % nt, tz = q / nt;
  unsigned codes[S2_CSG_CODE_WORDS];
  s2i root;
  s2c_tile(J.prog, J.prog_len, s2b_tile_axis(j, tx), s2b_tile_axis(j, ty), s2b_tile_axis(j, tz), codes, &root);
  unsigned flag = 0u;
  if (root.lo >= j.guard) flag = S2_TILE_DECIDED | S2_TILE_POSITIVE;
  else if (root.hi <= -j.guard) flag = S2_TILE_DECIDED;
  unsigned *rec = J.tiles + (size_t)t * S2_CSG_TILE_WORDS;
  rec[0] = flag;
#pragma unroll
  for (int w = 0; w < S2_CSG_CODE_WORDS; ++w) rec[1 + w] = codes[w];
}

// Evaluation: S2_B_EVAL_TILES tiles per item, one warp per tile (so a warp
// takes one path through the pruned program), S2_B_EVAL_TILES / 8 tiles per
// warp.  A decided tile stores +inf or -inf (128 float4 stores for a whole
// tile): the sign that classification needs, and a value that the vertex
// stage treats as unknown and evaluates where a cell needs it.  Other tiles
// evaluate 128 runs of 4 planes (8 x 8 columns x 2 runs), 4 runs per lane,
// with the tile's codes, which give the same bits as the full program.
#define S2_B_EVAL_RUN 4
__device__ __forceinline__ void s2b_stage_eval(const S2BatchJob &J, unsigned item) {
  __shared__ unsigned s_rec[256 / 32][S2_CSG_TILE_WORDS];
  const S2Job &j = J.job;
  const S2CsgSdf f{J.prog, J.prog_len};
  const unsigned nt = (unsigned)J.ntx, ntiles = nt * nt * nt;
  const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
#pragma unroll 1
  for (unsigned q = 0; q < S2_B_EVAL_TILES / 8; ++q) {
    const unsigned t = item * S2_B_EVAL_TILES + q * 8u + warp;  // the same on the whole warp
    if (t >= ntiles) break;
    const unsigned tx = t % nt, r = t / nt, ty = r % nt, tz = r / nt;
    const int x0 = (int)(S2_B_TILE * tx), y0 = (int)(S2_B_TILE * ty), z0 = (int)(S2_B_TILE * tz);
    unsigned flag = 0u;
    if (J.prune) {
      __syncwarp();
      if (lane < S2_CSG_TILE_WORDS) s_rec[warp][lane] = __ldcg(J.tiles + (size_t)t * S2_CSG_TILE_WORDS + lane);
      __syncwarp();
      flag = s_rec[warp][0];
    }
    if (flag & S2_TILE_DECIDED) {
      const float sv = (flag & S2_TILE_POSITIVE) ? __int_as_float(0x7f800000) : __int_as_float(0xff800000);
      if (x0 + S2_B_TILE <= j.P && y0 + S2_B_TILE <= j.P && z0 + S2_B_TILE <= j.P) {
        // rows of 8 points start at 32-byte multiples (pitch: 32 points)
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          const int u = k * 32 + (int)lane, h = u & 1, y = (u >> 1) & 7, z = u >> 4;
          float4 *dst = reinterpret_cast<float4 *>(J.lattice + (long long)(z0 + z) * j.plane +
                                                   (long long)(y0 + y) * j.pitch + x0 + 4 * h);
          *dst = make_float4(sv, sv, sv, sv);
        }
      } else {
#pragma unroll 1
        for (int u = (int)lane; u < S2_B_TILE * S2_B_TILE * S2_B_TILE; u += 32) {
          const int x = x0 + (u & 7), y = y0 + ((u >> 3) & 7), z = z0 + (u >> 6);
          if (x < j.P && y < j.P && z < j.P) J.lattice[(long long)z * j.plane + (long long)y * j.pitch + x] = sv;
        }
      }
      continue;
    }
#pragma unroll 1
    for (int k = 0; k < 4; ++k) {
      const unsigned lr = (unsigned)k * 32u + lane;
      const int x = x0 + (int)(lr & 7u), y = y0 + (int)((lr >> 3) & 7u), k0 = z0 + S2_B_EVAL_RUN * (int)(lr >> 6);
      if (x >= j.P || y >= j.P || k0 >= j.P) continue;
      float z[S2_B_EVAL_RUN], v[S2_B_EVAL_RUN];
#pragma unroll
      for (int w = 0; w < S2_B_EVAL_RUN; ++w) z[w] = s2_coord(j, min(k0 + w, j.P - 1));
      if (J.prune) f.eval_run_pruned<S2_B_EVAL_RUN>(s2_coord(j, x), s2_coord(j, y), z, v, s_rec[warp] + 1);
      else f.eval_run<S2_B_EVAL_RUN>(s2_coord(j, x), s2_coord(j, y), z, v);
      float *dst = J.lattice + (long long)k0 * j.plane + (long long)y * j.pitch + x;
#pragma unroll
      for (int w = 0; w < S2_B_EVAL_RUN; ++w)
        if (k0 + w < j.P) dst[(long long)w * j.plane] = v[w];
    }
  }
}

// Classification of the job (s2_cell_mark_tiles, s2_scan_tiles,
// s2_cell_emit_tiles): S2_B_CELL_TILES tiles per item of the mark and emit
// stages, one item for the scan.
__device__ __forceinline__ unsigned s2b_cell_tiles(const S2BatchJob &J, long long &ncells) {
  ncells = (long long)J.nzc * J.job.N * J.job.N;
  return (unsigned)((ncells + S2_CELL_TILE - 1) / S2_CELL_TILE);
}
__device__ __forceinline__ void s2b_stage_mark(const S2BatchJob &J, unsigned item) {
  long long ncells;
  const unsigned ntiles = s2b_cell_tiles(J, ncells);
  s2_cell_mark_tiles<true, S2_B_CELL_TILES>(J.job, J.lattice, item * S2_B_CELL_TILES, ntiles, ncells, 0,
                                            S2CellSkip{J.prune ? J.tiles : nullptr, (unsigned)S2_CSG_TILE_WORDS, J.ntx},
                                            J.cwords, J.ctcnt);
}
__device__ __forceinline__ void s2b_stage_cscan(const S2BatchJob &J) {
  long long ncells;
  const unsigned ntiles = s2b_cell_tiles(J, ncells);
  s2_scan_tiles<256, 16>(J.ctcnt, ntiles, J.ctoff, J.cand.base, 0);  // cand.base[1] = the job's candidates
}
__device__ __forceinline__ void s2b_stage_emit(const S2BatchJob &J, unsigned item) {
  long long ncells;
  const unsigned ntiles = s2b_cell_tiles(J, ncells);
  s2_cell_emit_tiles<true, S2_B_CELL_TILES>(J.job, J.lattice, J.cand, J.mesh.err, item * S2_B_CELL_TILES, ntiles, 0,
                                            J.cwords, J.ctcnt, J.ctoff);
}

__device__ __forceinline__ void s2b_stage_vertices(const S2BatchJob &J) {
  __shared__ unsigned s_chunk;
  __shared__ S2WarpScratch s_ws[256 / 32];
  __shared__ const unsigned *s_rec[256];
  const S2Job &job = J.job;
  const S2CsgSdf f{J.prog, J.prog_len};
  const S2CsgLanes lanes{f, s_rec};
  const unsigned long long n = min(__ldcg(J.cand.base + 1), J.cand.cap);
  const unsigned nchunks = (unsigned)((n + S2_B_VERT_CHUNK - 1) / S2_B_VERT_CHUNK);
  for (;;) {
    if (threadIdx.x == 0) s_chunk = atomicAdd(J.xcounter, 1u);
    __syncthreads();
    const unsigned chunk = s_chunk;
    __syncthreads();
    if (chunk >= nchunks) break;
    const unsigned long long o = (unsigned long long)chunk * S2_B_VERT_CHUNK + threadIdx.x;
    const bool active = o < n;
    unsigned long long k = active ? __ldcg(J.cand.key + o) : 0ull;
    S2Cell c;
    c.x = (int)(k & 0xffffull);
    c.y = (int)((k >> 16) & 0xffffull);
    c.z = (int)((k >> 32) & 0xffffull);
    float v[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    if (active) {
      const float4 *src = reinterpret_cast<const float4 *>(J.cand.val + 8 * o);
      const float4 a = __ldcg(src), b = __ldcg(src + 1);
      v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w; v[4] = b.x; v[5] = b.y; v[6] = b.z; v[7] = b.w;
    }
    float pos[3], nrm[3];
    unsigned long long key;
    const unsigned *rec = J.prune && active ? s2b_cell_tile(J, c) : nullptr;
    if (job.qef) {
      const S2CsgCell fc{f, rec};
      if (active)  // corners of decided tiles (+-inf): their values, at their lattice coordinates
#pragma unroll 1
        for (int q = 0; q < 8; ++q)
          if (!(fabsf(v[q]) <= 3.40282347e38f))
            v[q] = fc(s2_coord(job, c.x + (q & 1)), s2_coord(job, c.y + ((q >> 1) & 1)), s2_coord(job, c.z + (q >> 2)));
      key = active ? s2_vertex_qef(fc, job, c, v, pos, nrm) : 0ull;
    } else {
      s_rec[threadIdx.x] = rec;
      __syncwarp();
      key = s2_vertex_warp(lanes, job, active, c, v, pos, nrm, s_ws[threadIdx.x >> 5]);
      __syncwarp();
    }
    if (active) {
      J.cand.key[o] = key;
      if (key >> 63) {
        J.cand.pos[3 * o] = pos[0];
        J.cand.pos[3 * o + 1] = pos[1];
        J.cand.pos[3 * o + 2] = pos[2];
        J.cand.nrm[3 * o] = nrm[0];
        J.cand.nrm[3 * o + 1] = nrm[1];
        J.cand.nrm[3 * o + 2] = nrm[2];
      }
    }
  }
}

// Test hook of the batch kernel (the `hold` argument): job 0's row-scan items
// never count as done, so its quad items' stage wait runs out (a flag that
// nothing sets); they then skip their work and the launch reports
// S2_ERR_BATCH_WAIT.
#define S2_HOLD_BATCH_ROWS 0x2u

__global__ void __launch_bounds__(256) s2m_batch_kernel(const S2BatchJob *__restrict__ jobs,
                                                        const S2BatchSeg *__restrict__ segs, int nsegs,
                                                        unsigned long long total, S2BatchCtl *ctl,
                                                        unsigned long long stage_wait_ns, unsigned hold) {
  __shared__ unsigned long long s_ticket;
  __shared__ int s_ok;
  const unsigned tid = threadIdx.x;
  unsigned long long busy[S2_NSTAGES], waited = 0ull, t_item = 0ull;  // thread 0's accounting
  unsigned ready_job = ~0u, ready_stage = ~0u;  // thread 0: the last (job, stage) whose previous stage was seen done
#pragma unroll
  for (int k = 0; k < S2_NSTAGES; ++k) busy[k] = 0ull;
  for (;;) {
    if (tid == 0) s_ticket = atomicAdd(&ctl->next, 1ull);
    __syncthreads();
    const unsigned long long ticket = s_ticket;
    if (ticket >= total) break;
    int lo = 0, hi = nsegs - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (segs[mid].start <= ticket) lo = mid;
      else hi = mid - 1;
    }
    const S2BatchSeg sg = segs[lo];
    const unsigned item = (unsigned)(ticket - sg.start);
    const S2BatchJob &J = jobs[sg.job];
    if (tid == 0) {
      int ok = 1;
      const unsigned long long tw = s2_globaltimer();
      // (the stage's items come in runs of tickets: once the previous stage
      // was seen done, with acquire, later items of the run need not look again)
      if (sg.stage > 0 && !(sg.job == ready_job && sg.stage == ready_stage)) {
        // wait for every item of the previous stage of this job (lower tickets),
        // bounded by time: stage_wait_ns of the GPU's global timer
        const unsigned need = J.nitems[sg.stage - 1];
        unsigned long long t0 = 0;
        for (unsigned spins = 0;; ++spins) {
          unsigned d;
          asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(d) : "l"(J.done + sg.stage - 1) : "memory");
          if (d >= need) break;
          const unsigned long long now = s2_globaltimer();
          if (spins == 0) t0 = now;
          if (now - t0 > stage_wait_ns) {
            atomicOr(&ctl->err, S2_ERR_BATCH_WAIT);
            ok = 0;
            break;
          }
          __nanosleep(128);
        }
        if (ok) {
          ready_job = sg.job;
          ready_stage = sg.stage;
        }
      }
      t_item = s2_globaltimer();
      waited += t_item - tw;
      s_ok = ok;
    }
    __syncthreads();
    if (s_ok) {
      switch (sg.stage) {
        case S2_ST_TILES: s2b_stage_tiles(J, item); break;
        case S2_ST_EVAL: s2b_stage_eval(J, item); break;
        case S2_ST_MARK: s2b_stage_mark(J, item); break;
        case S2_ST_CSCAN: s2b_stage_cscan(J); break;
        case S2_ST_EMIT: s2b_stage_emit(J, item); break;
        case S2_ST_VERT: s2b_stage_vertices(J); break;
        case S2_ST_VCOMPACT: s2_vcompact_worker(J.job, J.cand, J.mesh, 1, item == 0); break;
        case S2_ST_ROWS: s2_rowscan_worker(J.mesh, (unsigned long long)J.job.N * J.job.N); break;
        case S2_ST_QUADS: s2_quads_worker<false>(J.job, J.mesh, J.scan_tiles, item == 0); break;
      }
    }
    __syncthreads();
    if (tid == 0) {
#pragma unroll
      for (int k = 0; k < S2_NSTAGES; ++k)
        if (k == (int)sg.stage) busy[k] += s2_globaltimer() - t_item;
    }
    if (tid == 0 && !((hold & S2_HOLD_BATCH_ROWS) && sg.job == 0 && sg.stage == S2_ST_ROWS)) {
      // the block's writes (ordered before by the barrier), then the count:
      // a release reduction that does not wait for its result
      asm volatile("red.release.gpu.global.add.u32 [%0], 1;" ::"l"(J.done + sg.stage) : "memory");
    }
  }
  if (tid == 0) {
#pragma unroll
    for (int k = 0; k < S2_NSTAGES; ++k)
      if (busy[k]) atomicAdd(&ctl->busy_ns[k], busy[k]);
    atomicAdd(&ctl->wait_ns, waited);
  }
}

__global__ void s2m_batch_results(const S2BatchJob *__restrict__ jobs, int n, S2BatchResult *out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const S2BatchJob &J = jobs[i];
  S2BatchResult r;
  r.ntris = *J.mesh.ntris;
  r.invalid = *J.mesh.invalid;
  r.vtotal = *J.mesh.vtotal;
  r.ncand = J.cand.base[1];
  r.err = *J.mesh.err;
  r.pad = 0;
  out[i] = r;
}

// ---------------------------------------------------------------------------
// Host side.

namespace {

void set_err(char *err, size_t errlen, const std::string &msg) {
  if (!err || errlen == 0) return;
  size_t n = std::min(errlen - 1, msg.size());
  std::memcpy(err, msg.data(), n);
  err[n] = 0;
}

int device_sms() {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return sms > 0 ? sms : 152;
}

// Operands per opcode, or -1 for an unknown opcode.
int csg_operands(int op) {
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

// Well-formed: known opcodes, operands present, the stack never underflows
// or exceeds S2_CSG_STACK, and one value is left.
bool csg_validate(const float *p, uint32_t n, std::string &why) {
  int sp = 0;
  uint32_t i = 0;
  while (i < n) {
    float fo = p[i];
    int op = int(fo);
    if (float(op) != fo || csg_operands(op) < 0) {
      why = "unknown opcode at " + std::to_string(i);
      return false;
    }
    int nops = csg_operands(op);
    if (i + 1 + uint32_t(nops) > n) {
      why = "missing operands at " + std::to_string(i);
      return false;
    }
    for (int k = 0; k < nops; ++k)
      if (!std::isfinite(p[i + 1 + k])) {
        why = "non-finite operand at " + std::to_string(i + 1 + k);
        return false;
      }
    if (op < 10) {
      if (++sp > S2_CSG_STACK) {
        why = "program needs more than 32 stack entries";
        return false;
      }
    } else if (--sp < 1) {
      why = "operator without two operands at " + std::to_string(i);
      return false;
    }
    i += 1 + uint32_t(nops);
  }
  if (sp != 1) {
    why = "program leaves " + std::to_string(sp) + " values on the stack";
    return false;
  }
  return true;
}

struct HostJob {
  std::vector<float> prog;
  s2m_params params;
  S2Job job{};
  int N = 0, nzc = 0;
  unsigned long long cand_cap = 0, vcap = 0, tcap = 0;
  bool prune = true;  // tile pass and pruned evaluation
  // placement in the run's arena
  size_t zero_off = 0, data_off = 0;
  int run = -1;  // index of the run (arena) holding the results, -1 = not run yet
  // results
  uint64_t nverts = 0, ntris = 0, invalid = 0, ncand = 0;
  uint32_t err = 0;
  bool ok = false;
  // device outputs
  float *pos = nullptr, *nrm = nullptr;
  unsigned long long *key = nullptr;
  unsigned *tris = nullptr;
};

size_t al(size_t b) { return (b + 255) / 256 * 256; }

unsigned tiles_per_axis(const HostJob &h) { return unsigned((h.job.P + S2_B_TILE - 1) / S2_B_TILE); }
size_t tile_records(const HostJob &h) {
  const size_t nt = tiles_per_axis(h);
  return h.prune ? nt * nt * nt : 0;
}

// Bytes of the zeroed control region and of the data region of a job.
void job_sizes(const HostJob &h, size_t &zero_bytes, size_t &data_bytes) {
  const unsigned long long N = (unsigned long long)h.N;
  const unsigned long long ncells = (unsigned long long)h.nzc * N * N;
  const size_t cell_tiles = (ncells + S2_CELL_TILE - 1) / S2_CELL_TILE;
  const size_t vc_tiles = (h.cand_cap + S2_VC_TILE - 1) / S2_VC_TILE;
  const size_t scan_tiles = (N * N + S2_SCAN_TILE - 1) / S2_SCAN_TILE;
  const size_t quad_tiles = (h.vcap + S2_Q_TILE - 1) / S2_Q_TILE;
  zero_bytes = al(2 * 8) + al(vc_tiles * 8) + al((scan_tiles + quad_tiles) * 8) + al(N * N * 4) +
               al(8 * 4) /*counters*/ + al(8 * 4) /*done*/ + al(8 * 8) /*ntris, invalid, vtotal, err*/ + al(4);
  data_bytes = al(size_t(h.job.ring) * size_t(h.job.plane) * 4) + al(h.cand_cap * 8) + al(h.cand_cap * 32) +
               al(h.cand_cap * 12) * 2 + al((N * N + 1) * 4) + al(h.vcap * 12) * 2 + al(h.vcap * 8) + al(h.tcap * 12) +
               al(tile_records(h) * S2_CSG_TILE_WORDS * 4) + al(cell_tiles * S2_CELL_BLOCK * 4) + al(cell_tiles * 4) +
               al(cell_tiles * 8);
}

}  // namespace

// Pinned host words the results of one launch are copied into (reused).
struct PinnedBlock {
  void *p = nullptr;
  size_t bytes = 0;
};

struct s2m_batch {
  std::vector<HostJob> jobs;
  std::vector<void *> arenas;  // one per launch; results of a launch's jobs live in its arena
  std::vector<PinnedBlock> pinned_free;
  uint64_t budget = 0;
  int blocks_per_sm = 0;
  double last_ms = 0;
  uint64_t last_launches = 0;
  double stage_busy_ms[S2_NSTAGES] = {};  // block time per stage, last run
  double stage_wait_ms = 0;
  // bounds of the persistent kernel's device waits (GPU global timer ns): a
  // stage waiting for its job's previous stage, and the look-backs
  unsigned long long stage_wait_ns = 30000000000ull;
  unsigned long long lookback_wait_ns = S2_WAIT_NS;
  bool prune = true;  // for jobs that have not run yet
};

namespace {

// S2M_TEST_HOLD (tests only): S2_HOLD_* bits of the kernels' test hooks.
unsigned test_hold() {
  const char *e = std::getenv("S2M_TEST_HOLD");
  return e ? unsigned(std::strtoul(e, nullptr, 0)) : 0u;
}

// One persistent launch in flight.
struct Wave {
  std::vector<int> idx;
  char *arena = nullptr;
  size_t arena_bytes = 0;
  cudaStream_t st = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  PinnedBlock res;  // S2BatchResult[idx.size()] then S2BatchCtl
};

int take_pinned(s2m_batch *b, size_t bytes, PinnedBlock &out) {
  for (size_t i = 0; i < b->pinned_free.size(); ++i)
    if (b->pinned_free[i].bytes >= bytes) {
      out = b->pinned_free[i];
      b->pinned_free.erase(b->pinned_free.begin() + long(i));
      return S2M_OK;
    }
  out.bytes = std::max<size_t>(bytes, 1 << 18);
  if (cudaHostAlloc(&out.p, out.bytes, cudaHostAllocDefault) != cudaSuccess) return S2M_E_OOM;
  return S2M_OK;
}

// Enqueue jobs `idx` as one persistent launch on `st` (arena from the
// stream-ordered allocator; nothing waits for the device).
int launch_wave(s2m_batch *b, const std::vector<int> &idx, cudaStream_t st, Wave &w, char *err, size_t errlen) {
  std::vector<size_t> zb(idx.size()), db(idx.size());
  size_t ztot = 0, dtot = 0;
  for (size_t i = 0; i < idx.size(); ++i) {
    job_sizes(b->jobs[idx[i]], zb[i], db[i]);
    ztot += zb[i];
    dtot += db[i];
  }
  size_t prog_bytes = 0;
  for (int j : idx) prog_bytes += al(b->jobs[j].prog.size() * 4);
  const size_t jobs_bytes = al(idx.size() * sizeof(S2BatchJob));
  const size_t segs_bytes = al(idx.size() * S2_NSTAGES * sizeof(S2BatchSeg));
  const size_t res_bytes = al(idx.size() * sizeof(S2BatchResult));
  const size_t ctl_bytes = al(sizeof(S2BatchCtl));
  const size_t total = ztot + ctl_bytes + dtot + prog_bytes + jobs_bytes + segs_bytes + res_bytes;
  char *arena = nullptr;
  cudaError_t e = cudaMallocAsync(reinterpret_cast<void **>(&arena), total, st);
  if (e != cudaSuccess) {
    cudaGetLastError();
    set_err(err, errlen, std::string("batch arena (") + std::to_string(total) + " bytes): " + cudaGetErrorString(e));
    return S2M_E_OOM;
  }
  b->arenas.push_back(arena);
  const int run_id = int(b->arenas.size()) - 1;
  w.idx = idx;
  w.arena = arena;
  w.arena_bytes = total;
  w.st = st;

  // host images of the job table, segments and programs
  std::vector<S2BatchJob> dj(idx.size());
  std::vector<S2BatchSeg> segs;
  std::vector<char> progs(prog_bytes);
  size_t zoff = 0, doff = ztot + ctl_bytes, poff = 0;
  unsigned long long ticket = 0;
  for (size_t i = 0; i < idx.size(); ++i) {
    HostJob &h = b->jobs[idx[i]];
    const unsigned long long N = (unsigned long long)h.N;
    const unsigned long long ncells = (unsigned long long)h.nzc * N * N;
    const size_t cell_tiles = (ncells + S2_CELL_TILE - 1) / S2_CELL_TILE;
    const size_t vc_tiles = (h.cand_cap + S2_VC_TILE - 1) / S2_VC_TILE;
    const size_t scan_tiles = (N * N + S2_SCAN_TILE - 1) / S2_SCAN_TILE;
    const size_t quad_tiles = (h.vcap + S2_Q_TILE - 1) / S2_Q_TILE;
    S2BatchJob &J = dj[i];
    std::memset(&J, 0, sizeof(J));
    J.job = h.job;
    J.nzc = h.nzc;
    char *z = arena + zoff;
    J.cand.base = reinterpret_cast<unsigned long long *>(z); z += al(2 * 8);
    J.cand.status = reinterpret_cast<unsigned long long *>(z); z += al(vc_tiles * 8);
    J.mesh.scan_status = reinterpret_cast<unsigned long long *>(z); z += al((scan_tiles + quad_tiles) * 8);
    J.mesh.rowcnt = reinterpret_cast<unsigned *>(z); z += al(N * N * 4);
    unsigned *counters = reinterpret_cast<unsigned *>(z); z += al(8 * 4);
    J.done = reinterpret_cast<unsigned *>(z); z += al(8 * 4);
    unsigned long long *ctl = reinterpret_cast<unsigned long long *>(z); z += al(8 * 8);
    z += al(4);
    zoff += zb[i];
    J.mesh.counters = counters;
    J.cand.tile_counter = counters + 0;
    J.xcounter = counters + 1;
    J.mesh.ntris = ctl + 0;
    J.mesh.invalid = ctl + 1;
    J.mesh.vtotal = ctl + 2;
    J.mesh.err = reinterpret_cast<unsigned *>(ctl + 3);
    char *d = arena + doff;
    J.lattice = reinterpret_cast<float *>(d); d += al(size_t(h.job.ring) * size_t(h.job.plane) * 4);
    J.cand.key = reinterpret_cast<unsigned long long *>(d); d += al(h.cand_cap * 8);
    J.cand.val = reinterpret_cast<float *>(d); d += al(h.cand_cap * 32);
    J.cand.pos = reinterpret_cast<float *>(d); d += al(h.cand_cap * 12);
    J.cand.nrm = reinterpret_cast<float *>(d); d += al(h.cand_cap * 12);
    J.mesh.rowstart = reinterpret_cast<unsigned *>(d); d += al((N * N + 1) * 4);
    J.mesh.pos = reinterpret_cast<float *>(d); d += al(h.vcap * 12);
    J.mesh.nrm = reinterpret_cast<float *>(d); d += al(h.vcap * 12);
    J.mesh.key = reinterpret_cast<unsigned long long *>(d); d += al(h.vcap * 8);
    J.mesh.tris = reinterpret_cast<unsigned *>(d); d += al(h.tcap * 12);
    J.tiles = reinterpret_cast<unsigned *>(d); d += al(tile_records(h) * S2_CSG_TILE_WORDS * 4);
    J.cwords = reinterpret_cast<unsigned *>(d); d += al(cell_tiles * S2_CELL_BLOCK * 4);
    J.ctcnt = reinterpret_cast<unsigned *>(d); d += al(cell_tiles * 4);
    J.ctoff = reinterpret_cast<unsigned long long *>(d); d += al(cell_tiles * 8);
    J.ntx = int(tiles_per_axis(h));
    J.prune = h.prune ? 1 : 0;
    doff += db[i];
    J.cand.cap = h.cand_cap;
    J.mesh.vcap = h.vcap;
    J.mesh.tcap = h.tcap;
    J.mesh.wait_ns = b->lookback_wait_ns;
    J.scan_tiles = unsigned(scan_tiles);
    std::memcpy(progs.data() + poff, h.prog.data(), h.prog.size() * 4);
    J.prog = reinterpret_cast<const float *>(arena + ztot + ctl_bytes + dtot + poff);
    J.prog_len = int(h.prog.size());
    poff += al(h.prog.size() * 4);
    // items per stage
    const unsigned long long n2 = N * N;
    {
      const unsigned long long nt = tiles_per_axis(h), ntiles = nt * nt * nt;
      J.nitems[S2_ST_TILES] = h.prune ? unsigned((ntiles + S2_B_TILES_ITEM - 1) / S2_B_TILES_ITEM) : 1u;
      J.nitems[S2_ST_EVAL] = unsigned((ntiles + S2_B_EVAL_TILES - 1) / S2_B_EVAL_TILES);
    }
    J.nitems[S2_ST_MARK] = unsigned(std::max<size_t>(1, (cell_tiles + S2_B_CELL_TILES - 1) / S2_B_CELL_TILES));
    J.nitems[S2_ST_CSCAN] = 1u;
    J.nitems[S2_ST_EMIT] = J.nitems[S2_ST_MARK];
    J.nitems[S2_ST_VERT] = unsigned(std::min<unsigned long long>(128, std::max<unsigned long long>(1, n2 / 2048)));
    J.nitems[S2_ST_VCOMPACT] = unsigned(std::min<unsigned long long>(64, std::max<unsigned long long>(1, n2 / 8192)));
    J.nitems[S2_ST_ROWS] = unsigned(std::min<unsigned long long>(16, std::max<unsigned long long>(1, n2 / 16384)));
    J.nitems[S2_ST_QUADS] = unsigned(std::min<unsigned long long>(64, std::max<unsigned long long>(1, n2 / 8192)));
    h.run = run_id;
    h.pos = J.mesh.pos;
    h.nrm = J.mesh.nrm;
    h.key = J.mesh.key;
    h.tris = J.mesh.tris;
  }
  // Tickets stage by stage over the wave's jobs: every job's tile pass, then
  // every job's lattice, and so on.  A job's stage still follows its previous
  // stage in ticket order, and by the time its items are taken the previous
  // stage's items were dispensed long before, so blocks rarely wait (in job
  // order, each job's stages followed one another directly and blocks waited
  // for the stage ahead of them).
  for (int s = 0; s < S2_NSTAGES; ++s)
    for (size_t i = 0; i < idx.size(); ++i) {
      S2BatchSeg sg;
      sg.start = ticket;
      sg.job = unsigned(i);
      sg.stage = unsigned(s);
      sg.count = dj[i].nitems[s];
      sg.pad = 0;
      segs.push_back(sg);
      ticket += dj[i].nitems[s];
    }
  char *d_prog = arena + ztot + ctl_bytes + dtot;
  S2BatchJob *d_jobs = reinterpret_cast<S2BatchJob *>(d_prog + prog_bytes);
  S2BatchSeg *d_segs = reinterpret_cast<S2BatchSeg *>(reinterpret_cast<char *>(d_jobs) + jobs_bytes);
  S2BatchResult *d_res = reinterpret_cast<S2BatchResult *>(reinterpret_cast<char *>(d_segs) + segs_bytes);
  S2BatchCtl *d_ctl = reinterpret_cast<S2BatchCtl *>(arena + ztot);

#define S2B_CUDA(call)                                                                 \
  do {                                                                                 \
    cudaError_t e_ = (call);                                                           \
    if (e_ != cudaSuccess) {                                                           \
      set_err(err, errlen, std::string(#call) + ": " + cudaGetErrorString(e_));        \
      return S2M_E_CUDA;                                                               \
    }                                                                                  \
  } while (0)
  S2B_CUDA(cudaMemsetAsync(arena, 0, ztot + ctl_bytes, st));
  S2B_CUDA(cudaMemcpyAsync(d_prog, progs.data(), prog_bytes, cudaMemcpyHostToDevice, st));
  S2B_CUDA(cudaMemcpyAsync(d_jobs, dj.data(), idx.size() * sizeof(S2BatchJob), cudaMemcpyHostToDevice, st));
  S2B_CUDA(cudaMemcpyAsync(d_segs, segs.data(), segs.size() * sizeof(S2BatchSeg), cudaMemcpyHostToDevice, st));
  if (b->blocks_per_sm <= 0) {
    int nb = 0;
    S2B_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, s2m_batch_kernel, 256, 0));
    b->blocks_per_sm = std::max(1, nb);
  }
  const int grid = device_sms() * b->blocks_per_sm;
  cudaEvent_t e0, e1;
  S2B_CUDA(cudaEventCreate(&e0));
  S2B_CUDA(cudaEventCreate(&e1));
  S2B_CUDA(cudaEventRecord(e0, st));
  s2m_batch_kernel<<<grid, 256, 0, st>>>(d_jobs, d_segs, int(segs.size()), ticket, d_ctl, b->stage_wait_ns,
                                         test_hold());
  S2B_CUDA(cudaGetLastError());
  S2B_CUDA(cudaEventRecord(e1, st));
  s2m_batch_results<<<unsigned((idx.size() + 127) / 128), 128, 0, st>>>(d_jobs, int(idx.size()), d_res);
  S2B_CUDA(cudaGetLastError());
  const size_t rbytes = idx.size() * sizeof(S2BatchResult);
  if (take_pinned(b, rbytes + sizeof(S2BatchCtl), w.res) != S2M_OK) {
    set_err(err, errlen, "pinned result buffer");
    return S2M_E_OOM;
  }
  S2B_CUDA(cudaMemcpyAsync(w.res.p, d_res, rbytes, cudaMemcpyDeviceToHost, st));
  S2B_CUDA(cudaMemcpyAsync(static_cast<char *>(w.res.p) + rbytes, d_ctl, sizeof(S2BatchCtl), cudaMemcpyDeviceToHost,
                           st));
  w.e0 = e0;
  w.e1 = e1;
  S2B_CUDA(cudaEventRecord(w.e1, st));  // re-recorded after the copies: completion of the whole launch
  return S2M_OK;
#undef S2B_CUDA
}

bool wave_ready(const Wave &w) { return cudaEventQuery(w.e1) != cudaErrorNotReady; }

// Wait for the launch and copy its results into the jobs.
int finish_wave(s2m_batch *b, Wave &w, char *err, size_t errlen) {
  cudaError_t e = cudaEventSynchronize(w.e1);
  float ms = 0;
  cudaEventElapsedTime(&ms, w.e0, w.e1);
  cudaEventDestroy(w.e0);
  cudaEventDestroy(w.e1);
  w.e0 = w.e1 = nullptr;
  if (e != cudaSuccess) {
    set_err(err, errlen, std::string("batch launch: ") + cudaGetErrorString(e));
    return S2M_E_CUDA;
  }
  b->last_ms += ms;
  b->last_launches += 2;
  const std::vector<int> &idx = w.idx;
  const S2BatchResult *res = static_cast<const S2BatchResult *>(w.res.p);
  const S2BatchCtl hctl = *reinterpret_cast<const S2BatchCtl *>(static_cast<const char *>(w.res.p) +
                                                                 idx.size() * sizeof(S2BatchResult));
  b->pinned_free.push_back(w.res);
  w.res = PinnedBlock();
  for (int k = 0; k < S2_NSTAGES; ++k) b->stage_busy_ms[k] += double(hctl.busy_ns[k]) * 1e-6;
  b->stage_wait_ms += double(hctl.wait_ns) * 1e-6;
  if (hctl.err & S2_ERR_BATCH_WAIT) {
    set_err(err, errlen, "a batch stage wait hit its limit");
    return S2M_E_TIMEOUT;
  }
  for (size_t i = 0; i < idx.size(); ++i) {
    HostJob &h = b->jobs[idx[i]];
    h.ntris = res[i].ntris;
    h.invalid = res[i].invalid;
    h.nverts = res[i].vtotal;
    h.ncand = res[i].ncand;
    h.err = res[i].err;
    h.ok = (h.err & (S2_ERR_CAND_OVF | S2_ERR_VERT_OVF | S2_ERR_TRI_OVF | S2_ERR_LOOKBACK | S2_ERR_INDEX_OVF)) == 0;
  }
  return S2M_OK;
}

int run_wave(s2m_batch *b, const std::vector<int> &idx, cudaStream_t st, char *err, size_t errlen) {
  Wave w;
  int rc = launch_wave(b, idx, st, w, err, errlen);
  if (rc != S2M_OK) return rc;
  return finish_wave(b, w, err, errlen);
}

}  // namespace

extern "C" {

int s2m_batch_create(s2m_batch **out, uint64_t memory_budget_bytes) {
  if (!out) return S2M_E_INVALID;
  s2m_batch *b = new s2m_batch();
  b->budget = memory_budget_bytes;
  *out = b;
  return S2M_OK;
}

int s2m_batch_add_csg(s2m_batch *b, const float *program, uint32_t len, const s2m_params *params,
                      uint32_t *job_id, char *err, size_t errlen) {
  if (!b || !program || !params) {
    set_err(err, errlen, "null argument");
    return S2M_E_INVALID;
  }
  std::string why;
  if (!csg_validate(program, len, why)) {
    set_err(err, errlen, "invalid CSG program: " + why);
    return S2M_E_INVALID;
  }
  HostJob h;
  h.prog.assign(program, program + len);
  h.params = *params;
  h.prune = b->prune;
  uint32_t N = params->resolution;
  if (params->flags & S2M_JOB_POW2_ROUNDING)
    if (__builtin_popcount(N) > 1) N = 2u << (31u - uint32_t(__builtin_clz(N)));
  if (N < 2 || N > 4096) {
    set_err(err, errlen, "batch resolution must be in [2, 4096]");
    return S2M_E_INVALID;
  }
  if (!(params->bounds > 0.0f) || !std::isfinite(params->bounds)) {
    set_err(err, errlen, "bounds must be a positive finite number");
    return S2M_E_INVALID;
  }
  h.N = int(N);
  S2Job &j = h.job;
  j.N = int(N);
  j.P = int(N) + 1;
  j.pitch = (j.P + 31) / 32 * 32;
  j.plane = (long long)j.P * j.pitch;
  j.ring = j.P;
  // Bounds3D::cube(B, 0) and dualcontour.wgsl:23-24 in binary32 (as the per-job path)
  volatile float half = params->bounds * 0.5f;
  volatile float mn = 0.0f - half;
  volatile float mx = 0.0f + half;
  volatile float ext = mx - mn;
  j.bmin = mn;
  j.size = ext / float(N - 1u);
  j.eps = params->eps > 0.0f ? params->eps : 1e-4f;
  j.guard = j.size;
  j.lag = (params->flags & S2M_JOB_SLICE_LAG) ? 1 : 0;
  j.exact = (params->flags & S2M_JOB_EXACT_CORNERS) ? 1 : 0;
  j.qef = (params->flags & S2M_JOB_QEF) ? 1 : 0;
  j.magic_n = uint32_t((1ull << 32) / uint64_t(j.N) + 1);
  j.magic_p = uint32_t((1ull << 32) / uint64_t(j.P) + 1);
  {
    const uint64_t wn = (uint64_t(j.N) + 31) / 32;
    j.magic_wn = wn >= 2 ? uint32_t((1ull << 32) / wn + 1) : 0u;
  }
  h.nzc = j.lag ? int(N) - 1 : int(N);
  const unsigned long long n3 = (unsigned long long)N * N * N, n2 = (unsigned long long)N * N;
  h.cand_cap = std::min(n3, std::max<unsigned long long>(4096, 8 * n2));
  h.vcap = params->max_vertices ? params->max_vertices : std::min(h.cand_cap, std::max<unsigned long long>(4096, 6 * n2));
  h.vcap = std::min(h.vcap, h.cand_cap);
  h.tcap = params->max_triangles ? params->max_triangles : 2 * h.vcap + 4096;
  b->jobs.push_back(std::move(h));
  if (job_id) *job_id = uint32_t(b->jobs.size() - 1);
  return S2M_OK;
}

uint64_t s2m_batch_job_footprint(const s2m_batch *b, uint32_t job) {
  if (!b || job >= b->jobs.size()) return 0;
  size_t z, d;
  job_sizes(b->jobs[job], z, d);
  return z + d + al(b->jobs[job].prog.size() * 4) + sizeof(S2BatchJob) + S2_NSTAGES * sizeof(S2BatchSeg);
}

int s2m_batch_run(s2m_batch *b, void *stream, char *err, size_t errlen) {
  if (!b) return S2M_E_INVALID;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  b->last_ms = 0;
  b->last_launches = 0;
  for (double &x : b->stage_busy_ms) x = 0;
  b->stage_wait_ms = 0;
  std::vector<int> pending;
  for (size_t i = 0; i < b->jobs.size(); ++i)
    if (b->jobs[i].run < 0) pending.push_back(int(i));
  for (int round = 0; round < 4 && !pending.empty(); ++round) {
    // waves under the memory budget, in submission order
    size_t w0 = 0;
    while (w0 < pending.size()) {
      std::vector<int> wave;
      uint64_t used = 0;
      for (size_t i = w0; i < pending.size(); ++i) {
        uint64_t fp = s2m_batch_job_footprint(b, uint32_t(pending[i]));
        if (!wave.empty() && b->budget && used + fp > b->budget) break;
        wave.push_back(pending[i]);
        used += fp;
      }
      int rc = run_wave(b, wave, st, err, errlen);
      if (rc != S2M_OK) return rc;
      w0 += wave.size();
    }
    // jobs whose buffers overflowed run again with their exact totals
    std::vector<int> again;
    for (int i : pending) {
      HostJob &h = b->jobs[i];
      if (h.ok) continue;
      if (h.err & (S2_ERR_LOOKBACK | S2_ERR_INDEX_OVF)) {
        set_err(err, errlen, "job " + std::to_string(i) + ": device error flags " + std::to_string(h.err));
        return (h.err & S2_ERR_LOOKBACK) ? S2M_E_TIMEOUT : S2M_E_OVERFLOW;
      }
      const unsigned long long n3 = (unsigned long long)h.N * h.N * h.N;
      if (h.err & S2_ERR_CAND_OVF) {
        h.cand_cap = std::min<unsigned long long>(n3, h.ncand + h.ncand / 16 + 4096);
        h.vcap = h.cand_cap;
      } else if (h.err & S2_ERR_VERT_OVF) {
        h.vcap = std::min<unsigned long long>(h.cand_cap, h.nverts + h.nverts / 16 + 4096);
      }
      if (h.err & S2_ERR_TRI_OVF) h.tcap = h.ntris + h.ntris / 16 + 4096;
      h.tcap = std::max<unsigned long long>(h.tcap, 2 * h.vcap + 4096);
      h.run = -1;
      again.push_back(i);
    }
    pending.swap(again);
  }
  if (!pending.empty()) {
    set_err(err, errlen, "batch jobs still overflow after resizing");
    return S2M_E_OVERFLOW;
  }
  return S2M_OK;
}

int s2m_batch_job_info(const s2m_batch *b, uint32_t job, s2m_mesh_info *info) {
  if (!b || !info || job >= b->jobs.size()) return S2M_E_INVALID;
  const HostJob &h = b->jobs[job];
  std::memset(info, 0, sizeof(*info));
  if (h.run < 0) return S2M_E_INVALID;
  info->nverts = h.nverts;
  info->ntris = h.ntris;
  info->invalid_quads = h.invalid;
  info->cells = (uint64_t)h.N * h.N * h.N;
  info->candidate_cells = h.ncand;
  info->resolution = uint32_t(h.N);
  info->slab_depth = uint32_t(h.N);
  info->d_pos = h.pos;
  info->d_nrm = h.nrm;
  info->d_cell = reinterpret_cast<const uint64_t *>(h.key);
  info->d_tris = h.tris;
  info->kernel_launches = 0;
  return S2M_OK;
}

int s2m_batch_job_copy_to_host(const s2m_batch *b, uint32_t job, float *pos, float *nrm, uint64_t *cell,
                               uint32_t *tris, void *stream) {
  if (!b || job >= b->jobs.size() || b->jobs[job].run < 0) return S2M_E_INVALID;
  const HostJob &h = b->jobs[job];
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  cudaError_t e = cudaSuccess;
  if (pos && h.nverts) e = cudaMemcpyAsync(pos, h.pos, h.nverts * 12, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess && nrm && h.nverts) e = cudaMemcpyAsync(nrm, h.nrm, h.nverts * 12, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess && cell && h.nverts) e = cudaMemcpyAsync(cell, h.key, h.nverts * 8, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess && tris && h.ntris) e = cudaMemcpyAsync(tris, h.tris, h.ntris * 12, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  return e == cudaSuccess ? S2M_OK : S2M_E_CUDA;
}

int s2m_batch_stats(const s2m_batch *b, double *kernel_ms, uint64_t *launches, uint32_t *njobs) {
  if (!b) return S2M_E_INVALID;
  if (kernel_ms) *kernel_ms = b->last_ms;
  if (launches) *launches = b->last_launches;
  if (njobs) *njobs = uint32_t(b->jobs.size());
  return S2M_OK;
}

int s2m_batch_set_wait_limit(s2m_batch *b, double stage_seconds, double lookback_seconds) {
  if (!b || !(stage_seconds > 0.0) || !(lookback_seconds > 0.0) || stage_seconds > 3600.0 || lookback_seconds > 3600.0)
    return S2M_E_INVALID;
  b->stage_wait_ns = (unsigned long long)(stage_seconds * 1e9);
  b->lookback_wait_ns = (unsigned long long)(lookback_seconds * 1e9);
  return S2M_OK;
}

int s2m_batch_stage_profile(const s2m_batch *b, double *busy_ms, uint32_t nstages, double *wait_ms) {
  if (!b || (nstages && !busy_ms)) return S2M_E_INVALID;
  for (uint32_t k = 0; k < nstages; ++k) busy_ms[k] = k < S2_NSTAGES ? b->stage_busy_ms[k] : 0.0;
  if (wait_ms) *wait_ms = b->stage_wait_ms;
  return S2M_OK;
}

int s2m_batch_set_pruning(s2m_batch *b, int enabled) {
  if (!b) return S2M_E_INVALID;
  b->prune = enabled != 0;
  for (HostJob &h : b->jobs)
    if (h.run < 0) h.prune = b->prune;
  return S2M_OK;
}

void s2m_batch_free(s2m_batch *b) {
  if (!b) return;
  for (void *a : b->arenas) cudaFreeAsync(a, nullptr);
  cudaStreamSynchronize(nullptr);
  for (PinnedBlock &p : b->pinned_free) cudaFreeHost(p.p);
  delete b;
}

}  // extern "C"

// ===========================================================================
// Serving: continuous batching.
//
// Requests (CSG programs, or compiled SDFs) are queued by any host thread.
// The server thread admits queued requests while their device footprint fits
// the memory budget and fewer than `max_inflight` persistent launches are
// running, and launches each admitted group as one persistent kernel on its
// own stream.  Requests that arrive while launches run are admitted as soon
// as a slot and memory free up; the new launch then runs beside the one still
// finishing, so their work overlaps on the device.  Compiled-SDF requests run
// the per-job pipeline on a third stream from a second host thread.  A
// request's latency is completion minus submission (host clock).

#include <atomic>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <memory>
#include <set>
#include <thread>

namespace {

double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

struct SReq {
  uint64_t id = 0;
  int kind = 0;  // 0 CSG program, 1 compiled SDF
  std::vector<float> prog;
  const s2m_sdf *sdf = nullptr;
  s2m_params params{};
  double t_submit = 0, t_done = 0;
  int state = 0;  // 0 queued, 1 running, 2 done, 3 failed
  int status = S2M_OK;
  std::string msg;
  uint64_t footprint = 0;
  s2m_mesh_info info{};
  int wave = -1;        // CSG: server wave holding the results
  uint32_t job = 0;     // CSG: job index inside that wave's batch
  s2m_mesh *mesh = nullptr;  // compiled SDF: the mesh handle
  int attempts = 0;
};

struct SWave {
  s2m_batch *b = nullptr;
  Wave w;
  std::vector<uint64_t> reqs;
  int live = 0;        // requests of this wave whose results are still held
  bool finished = false;
  cudaStream_t st = nullptr;
};

}  // namespace

namespace s2m {
// Device bytes s2m_mesh_create allocates for a job (runtime.cu): its own job
// setup and buffer plan, so admission follows the resolution rounding, the
// slab depth, the tile-pruning buffers and caller-set capacities.
uint64_t mesh_job_footprint(const s2m_sdf *sdf, const s2m_params &params);
}  // namespace s2m

namespace {
// Admission footprint of a compiled-SDF request: the job's buffer plan plus
// 64 MiB for the autotuner's first run and pool rounding.
uint64_t sdf_job_footprint(const s2m_sdf *sdf, const s2m_params &p) {
  return s2m::mesh_job_footprint(sdf, p) + (64ull << 20);
}

}  // namespace

struct s2m_server {
  s2m_server_config cfg{};
  std::mutex mu;
  std::condition_variable cv, done_cv;
  std::map<uint64_t, SReq> reqs;
  std::deque<uint64_t> queue, sdf_queue;
  std::vector<SWave> waves;
  uint64_t next_id = 1;
  uint64_t used_bytes = 0, peak_bytes = 0;
  uint64_t submitted = 0, completed = 0, failed = 0, batches = 0;
  double first_submit = 0, last_done = 0;
  double voxels_done = 0;
  std::vector<double> latencies_ms;
  bool stop = false;
  int inflight = 0;
  uint64_t ran_compiled = 0, ran_interpreted = 0;
  cudaStream_t streams[2] = {nullptr, nullptr};
  std::vector<cudaStream_t> sdf_streams;  // one per per-job worker
  std::thread worker;
  std::vector<std::thread> sdf_workers;
  int device = 0;
  // compiled sources (keyed by language, name, text): non-CSG sources compiled
  // in the submitting call, CSG sources by the background compiler
  std::mutex compile_mu;
  std::condition_variable compile_cv;
  std::map<std::string, s2m_sdf *> compiled;
  std::deque<std::string> compile_queue;
  std::set<std::string> compile_pending, compile_failed;
  bool compile_stop = false;
  std::thread compiler;
};

namespace {

void server_release_locked(s2m_server *s, SReq &r) {
  if (r.state != 2 && r.state != 3) return;
  if (r.kind == 0 && r.wave >= 0) {
    SWave &sw = s->waves[size_t(r.wave)];
    if (--sw.live == 0 && sw.finished && sw.b) {
      for (void *a : sw.b->arenas) cudaFreeAsync(a, sw.st);
      sw.b->arenas.clear();
      for (PinnedBlock &p : sw.b->pinned_free) cudaFreeHost(p.p);
      sw.b->pinned_free.clear();
      delete sw.b;
      sw.b = nullptr;
    }
    r.wave = -1;
  }
  if (r.kind == 1 && r.mesh) {
    s2m_mesh_free(r.mesh);
    r.mesh = nullptr;
  }
  if (r.footprint) {
    s->used_bytes -= std::min(s->used_bytes, r.footprint);
    r.footprint = 0;
  }
}

void server_complete_locked(s2m_server *s, SReq &r, int status, const std::string &msg) {
  r.t_done = now_s();
  r.status = status;
  r.msg = msg;
  if (status == S2M_OK) {
    r.state = 2;
    ++s->completed;
    ++(r.kind == 1 ? s->ran_compiled : s->ran_interpreted);
    s->latencies_ms.push_back((r.t_done - r.t_submit) * 1e3);
    s->voxels_done += double(r.info.cells);
  } else {
    r.state = 3;
    ++s->failed;
  }
  s->last_done = r.t_done;
  if (!s->cfg.keep_results) server_release_locked(s, r);
}

void server_loop(s2m_server *s) {
  cudaSetDevice(s->device);
  std::unique_lock<std::mutex> lk(s->mu);
  char err[1024];
  int next_stream = 0;
  while (true) {
    // 1. launches that finished
    for (size_t wi = 0; wi < s->waves.size(); ++wi) {
      SWave &sw = s->waves[wi];
      if (sw.finished || !sw.b || !wave_ready(sw.w)) continue;
      int rc = finish_wave(sw.b, sw.w, err, sizeof err);
      sw.finished = true;
      --s->inflight;
      sw.live = 1;  // guard: the batch stays alive while its requests complete
      for (size_t k = 0; k < sw.reqs.size(); ++k) {
        SReq &r = s->reqs[sw.reqs[k]];
        const HostJob &h = sw.b->jobs[k];
        if (rc == S2M_OK && h.ok) {
          s2m_batch_job_info(sw.b, uint32_t(k), &r.info);
          r.wave = int(wi);
          r.job = uint32_t(k);
          ++sw.live;
          server_complete_locked(s, r, S2M_OK, "");
        } else if (rc == S2M_OK && r.attempts < 4 && !(h.err & (S2_ERR_LOOKBACK | S2_ERR_INDEX_OVF))) {
          // buffers too small: queue again with the exact totals
          const unsigned long long need_c = h.ncand + h.ncand / 16 + 4096;
          const unsigned long long need_v = std::max<unsigned long long>(h.nverts + h.nverts / 16 + 4096, need_c);
          r.params.max_vertices = need_v;
          r.params.max_triangles = std::max<unsigned long long>(h.ntris + h.ntris / 16 + 4096, 2 * need_v + 4096);
          s->used_bytes -= std::min(s->used_bytes, r.footprint);
          r.footprint = 0;
          r.state = 0;
          s->queue.push_front(r.id);
        } else {
          server_complete_locked(s, r, rc == S2M_OK ? S2M_E_OVERFLOW : rc, rc == S2M_OK ? "overflow" : err);
        }
      }
      if (--sw.live == 0 && sw.b) {
        for (void *a : sw.b->arenas) cudaFreeAsync(a, sw.st);
        sw.b->arenas.clear();
        for (PinnedBlock &p : sw.b->pinned_free) cudaFreeHost(p.p);
        sw.b->pinned_free.clear();
        delete sw.b;
        sw.b = nullptr;
      }
      s->done_cv.notify_all();
    }
    // 2. admission: a new launch when a slot is free
    if (!s->queue.empty() && s->inflight < int(s->cfg.max_inflight)) {
      s2m_batch *b = new s2m_batch();
      std::vector<uint64_t> ids;
      uint64_t add = 0;
      while (!s->queue.empty() && ids.size() < s->cfg.max_batch_jobs) {
        SReq &r = s->reqs[s->queue.front()];
        uint32_t jid = 0;
        if (s2m_batch_add_csg(b, r.prog.data(), uint32_t(r.prog.size()), &r.params, &jid, err, sizeof err) != S2M_OK) {
          s->queue.pop_front();
          server_complete_locked(s, r, S2M_E_INVALID, err);
          continue;
        }
        const uint64_t fp = s2m_batch_job_footprint(b, jid);
        if (s->cfg.memory_budget_bytes && fp > s->cfg.memory_budget_bytes) {
          b->jobs.pop_back();
          s->queue.pop_front();
          server_complete_locked(s, r, S2M_E_OOM, "request larger than the memory budget");
          continue;
        }
        if (s->cfg.memory_budget_bytes && s->used_bytes + add + fp > s->cfg.memory_budget_bytes) {
          b->jobs.pop_back();
          break;  // waits for memory: admitted when earlier requests release theirs
        }
        r.footprint = fp;
        add += fp;
        r.state = 1;
        ++r.attempts;
        ids.push_back(r.id);
        s->queue.pop_front();
      }
      if (!ids.empty()) {
        s->used_bytes += add;
        s->peak_bytes = std::max(s->peak_bytes, s->used_bytes);
        SWave sw;
        sw.b = b;
        sw.reqs = ids;
        sw.st = s->streams[next_stream];
        next_stream ^= 1;
        std::vector<int> idx(ids.size());
        for (size_t k = 0; k < ids.size(); ++k) idx[k] = int(k);
        lk.unlock();
        int rc = launch_wave(b, idx, sw.st, sw.w, err, sizeof err);
        lk.lock();
        if (rc != S2M_OK) {
          for (uint64_t id : ids) server_complete_locked(s, s->reqs[id], rc, err);
          delete b;
        } else {
          ++s->inflight;
          ++s->batches;
          s->waves.push_back(sw);
        }
        continue;
      }
      delete b;
    }
    if (s->stop && s->queue.empty() && s->inflight == 0) break;
    s->cv.wait_for(lk, std::chrono::microseconds(200));
  }
}

// One per-job worker: takes compiled-SDF requests in arrival order while
// their footprint fits the budget and runs each on its own stream, so the
// workers' jobs overlap on the device.
void server_sdf_loop(s2m_server *s, int worker) {
  cudaSetDevice(s->device);
  cudaStream_t stream = s->sdf_streams[size_t(worker)];
  std::unique_lock<std::mutex> lk(s->mu);
  char err[1024];
  while (true) {
    if (s->sdf_queue.empty()) {
      if (s->stop) break;
      s->cv.wait_for(lk, std::chrono::milliseconds(1));
      continue;
    }
    uint64_t id = s->sdf_queue.front();
    SReq &r0 = s->reqs[id];
    if (s->cfg.memory_budget_bytes && s->used_bytes + r0.footprint > s->cfg.memory_budget_bytes &&
        s->used_bytes > 0) {
      s->cv.wait_for(lk, std::chrono::microseconds(200));
      continue;
    }
    s->sdf_queue.pop_front();
    s->used_bytes += r0.footprint;
    s->peak_bytes = std::max(s->peak_bytes, s->used_bytes);
    r0.state = 1;
    const s2m_sdf *sdf = r0.sdf;
    s2m_params p = r0.params;
    lk.unlock();
    s2m_mesh *m = nullptr;
    int rc = s2m_mesh_create(sdf, &p, stream, &m, err, sizeof err);
    lk.lock();
    SReq &r = s->reqs[id];
    if (rc == S2M_OK) {
      r.mesh = m;
      s2m_mesh_get_info(m, &r.info);
    }
    server_complete_locked(s, r, rc, rc == S2M_OK ? "" : err);
    s->done_cv.notify_all();
  }
}

// The background compiler of CSG sources (tiering): each queued key is
// compiled once; its later requests then run on the compiled module.
void server_compile_loop(s2m_server *s) {
  cudaSetDevice(s->device);
  std::unique_lock<std::mutex> lk(s->compile_mu);
  char err[4096];
  while (true) {
    if (s->compile_queue.empty()) {
      if (s->compile_stop) break;
      s->compile_cv.wait_for(lk, std::chrono::milliseconds(5));
      continue;
    }
    if (s->compile_stop) break;
    const std::string key = s->compile_queue.front();
    s->compile_queue.pop_front();
    lk.unlock();
    // key: language, NUL, function name, NUL, source
    const size_t a = key.find('\0'), b = key.find('\0', a + 1);
    const int lang = std::atoi(key.substr(0, a).c_str());
    const std::string name = key.substr(a + 1, b - a - 1), source = key.substr(b + 1);
    std::string text = source;
    s2m_sdf *sdf = nullptr;
    int rc = S2M_OK;
    if (lang == S2M_LANG_WGSL) {
      char *pre = nullptr;
      rc = s2m_preprocess_source(source.c_str(), nullptr, &pre, err, sizeof err);
      if (rc == S2M_OK) {
        text = pre;
        s2m_free_string(pre);
      }
    }
    if (rc == S2M_OK) rc = s2m_compile(text.c_str(), lang, name.c_str(), 0, &sdf, err, sizeof err);
    lk.lock();
    s->compile_pending.erase(key);
    if (rc == S2M_OK && sdf) {
      auto ins = s->compiled.emplace(key, sdf);
      if (!ins.second) s2m_sdf_free(sdf);
    } else {
      s->compile_failed.insert(key);  // stays on the interpreter
    }
  }
}

double percentile(std::vector<double> v, double q) {
  if (v.empty()) return 0;
  std::sort(v.begin(), v.end());
  double pos = q * double(v.size() - 1);
  size_t i = size_t(pos);
  double f = pos - double(i);
  return i + 1 < v.size() ? v[i] * (1 - f) + v[i + 1] * f : v[i];
}

}  // namespace

extern "C" {

int s2m_server_create(const s2m_server_config *cfg, s2m_server **out, char *err, size_t errlen) {
  if (!out) return S2M_E_INVALID;
  s2m_server *s = new s2m_server();
  if (cfg) s->cfg = *cfg;
  if (s->cfg.max_inflight == 0) s->cfg.max_inflight = 2;
  if (s->cfg.max_batch_jobs == 0) s->cfg.max_batch_jobs = 1024;
  cudaGetDevice(&s->device);
  // keep freed arenas in the stream-ordered pool instead of returning them to the driver
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, s->device) == cudaSuccess) {
    uint64_t keep = ~0ull;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
  }
  for (int i = 0; i < 2; ++i)
    if (cudaStreamCreateWithFlags(&s->streams[i], cudaStreamNonBlocking) != cudaSuccess) {
      set_err(err, errlen, "cudaStreamCreate failed");
      delete s;
      return S2M_E_CUDA;
    }
  if (s->cfg.sdf_workers == 0) s->cfg.sdf_workers = 4;
  s->sdf_streams.assign(s->cfg.sdf_workers, nullptr);
  for (auto &st : s->sdf_streams)
    if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) {
      set_err(err, errlen, "cudaStreamCreate failed");
      for (auto &t : s->sdf_streams)
        if (t) cudaStreamDestroy(t);
      for (int i = 0; i < 2; ++i) cudaStreamDestroy(s->streams[i]);
      delete s;
      return S2M_E_CUDA;
    }
  s->worker = std::thread(server_loop, s);
  for (uint32_t i = 0; i < s->cfg.sdf_workers; ++i) s->sdf_workers.emplace_back(server_sdf_loop, s, int(i));
  s->compiler = std::thread(server_compile_loop, s);
  *out = s;
  return S2M_OK;
}

int s2m_server_submit_csg(s2m_server *s, const float *program, uint32_t len, const s2m_params *params,
                          uint64_t *request_id, char *err, size_t errlen) {
  if (!s || !program || !params) return S2M_E_INVALID;
  std::string why;
  if (!csg_validate(program, len, why)) {
    set_err(err, errlen, "invalid CSG program: " + why);
    return S2M_E_INVALID;
  }
  std::lock_guard<std::mutex> lk(s->mu);
  SReq r;
  r.id = s->next_id++;
  r.kind = 0;
  r.prog.assign(program, program + len);
  r.params = *params;
  r.t_submit = now_s();
  if (s->submitted == 0) s->first_submit = r.t_submit;
  ++s->submitted;
  s->queue.push_back(r.id);
  if (request_id) *request_id = r.id;
  s->reqs.emplace(r.id, std::move(r));
  s->cv.notify_all();
  return S2M_OK;
}

int s2m_server_submit_sdf(s2m_server *s, const s2m_sdf *sdf, const s2m_params *params, uint64_t *request_id,
                          char *err, size_t errlen) {
  if (!s || !sdf || !params) return S2M_E_INVALID;
  uint64_t fp = sdf_job_footprint(sdf, *params);
  if (s->cfg.memory_budget_bytes && fp > s->cfg.memory_budget_bytes) {
    set_err(err, errlen, "request larger than the memory budget");
    return S2M_E_OOM;
  }
  std::lock_guard<std::mutex> lk(s->mu);
  SReq r;
  r.id = s->next_id++;
  r.kind = 1;
  r.sdf = sdf;
  r.params = *params;
  r.footprint = fp;
  r.t_submit = now_s();
  if (s->submitted == 0) s->first_submit = r.t_submit;
  ++s->submitted;
  s->sdf_queue.push_back(r.id);
  if (request_id) *request_id = r.id;
  s->reqs.emplace(r.id, std::move(r));
  s->cv.notify_all();
  return S2M_OK;
}

int s2m_server_submit_source(s2m_server *s, const char *source, int lang, const char *sdf_name,
                             const s2m_params *params, uint64_t *request_id, char *err, size_t errlen) {
  if (!s || !source || !params) return S2M_E_INVALID;
  const std::string key = std::to_string(lang) + '\0' + (sdf_name ? sdf_name : "sdf") + '\0' + source;
  s2m_sdf *sdf = nullptr;
  {
    std::lock_guard<std::mutex> lk(s->compile_mu);
    auto it = s->compiled.find(key);
    if (it != s->compiled.end()) sdf = it->second;
  }
  if (!sdf && lang == S2M_LANG_WGSL) {
    // a CSG source without a compiled module yet: the interpreter now, and
    // (tiering) its module compiled in the background for later requests
    uint32_t n = 0;
    if (s2m_csg_from_source(source, nullptr, 0, &n, nullptr, 0) == S2M_OK && n > 0) {
      std::vector<float> prog(n);
      if (s2m_csg_from_source(source, prog.data(), n, &n, err, errlen) == S2M_OK) {
        if (!(s->cfg.flags & S2M_SERVER_INTERPRET_ONLY)) {
          std::lock_guard<std::mutex> lk(s->compile_mu);
          if (!s->compile_pending.count(key) && !s->compile_failed.count(key) && !s->compiled.count(key)) {
            s->compile_pending.insert(key);
            s->compile_queue.push_back(key);
            s->compile_cv.notify_all();
          }
        }
        return s2m_server_submit_csg(s, prog.data(), n, params, request_id, err, errlen);
      }
    }
  }
  if (!sdf) {
    std::string text = source;
    if (lang == S2M_LANG_WGSL) {
      char *pre = nullptr;
      if (s2m_preprocess_source(source, nullptr, &pre, err, errlen) != S2M_OK) return S2M_E_PARSE;
      text = pre;
      s2m_free_string(pre);
    }
    int rc = s2m_compile(text.c_str(), lang, sdf_name, 0, &sdf, err, errlen);
    if (rc != S2M_OK) return rc;
    std::lock_guard<std::mutex> lk(s->compile_mu);
    auto ins = s->compiled.emplace(key, sdf);
    if (!ins.second) {
      s2m_sdf_free(sdf);
      sdf = ins.first->second;
    }
  }
  return s2m_server_submit_sdf(s, sdf, params, request_id, err, errlen);
}

int s2m_server_wait(s2m_server *s, uint64_t id, double timeout_s, s2m_mesh_info *info, char *err, size_t errlen) {
  if (!s) return S2M_E_INVALID;
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->reqs.find(id);
  if (it == s->reqs.end()) return S2M_E_INVALID;
  const double deadline = now_s() + timeout_s;
  while (it->second.state < 2) {
    if (now_s() > deadline) return S2M_E_TIMEOUT;
    s->done_cv.wait_for(lk, std::chrono::milliseconds(1));
  }
  if (info) *info = it->second.info;
  if (it->second.status != S2M_OK) set_err(err, errlen, it->second.msg);
  return it->second.status;
}

int s2m_server_copy_to_host(s2m_server *s, uint64_t id, float *pos, float *nrm, uint64_t *cell, uint32_t *tris) {
  if (!s) return S2M_E_INVALID;
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->reqs.find(id);
  if (it == s->reqs.end() || it->second.state != 2) return S2M_E_INVALID;
  SReq &r = it->second;
  // the mesh's work finished on its worker's stream (s2m_mesh_create synchronised it)
  if (r.kind == 1) return r.mesh ? s2m_mesh_copy_to_host(r.mesh, pos, nrm, cell, tris, nullptr) : S2M_E_INVALID;
  if (r.wave < 0 || !s->waves[size_t(r.wave)].b) return S2M_E_INVALID;
  return s2m_batch_job_copy_to_host(s->waves[size_t(r.wave)].b, r.job, pos, nrm, cell, tris,
                                    s->waves[size_t(r.wave)].st);
}

int s2m_server_release(s2m_server *s, uint64_t id) {
  if (!s) return S2M_E_INVALID;
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->reqs.find(id);
  if (it == s->reqs.end()) return S2M_E_INVALID;
  server_release_locked(s, it->second);
  s->cv.notify_all();
  return S2M_OK;
}

int s2m_server_drain(s2m_server *s, double timeout_s) {
  if (!s) return S2M_E_INVALID;
  std::unique_lock<std::mutex> lk(s->mu);
  const double deadline = now_s() + timeout_s;
  while (s->completed + s->failed < s->submitted) {
    if (now_s() > deadline) return S2M_E_TIMEOUT;
    s->done_cv.wait_for(lk, std::chrono::milliseconds(1));
  }
  return S2M_OK;
}

int s2m_server_get_stats(s2m_server *s, s2m_server_stats *out) {
  if (!s || !out) return S2M_E_INVALID;
  std::lock_guard<std::mutex> lk(s->mu);
  std::memset(out, 0, sizeof(*out));
  out->submitted = s->submitted;
  out->completed = s->completed;
  out->failed = s->failed;
  out->batches = s->batches;
  out->peak_bytes = s->peak_bytes;
  out->p50_ms = percentile(s->latencies_ms, 0.50);
  out->p99_ms = percentile(s->latencies_ms, 0.99);
  double sum = 0;
  for (double l : s->latencies_ms) sum += l;
  out->mean_ms = s->latencies_ms.empty() ? 0 : sum / double(s->latencies_ms.size());
  const double span = s->last_done - s->first_submit;
  out->span_s = span;
  out->meshes_per_s = span > 0 ? double(s->completed) / span : 0;
  out->gvoxels_per_s = span > 0 ? s->voxels_done / span / 1e9 : 0;
  out->ran_compiled = s->ran_compiled;
  out->ran_interpreted = s->ran_interpreted;
  std::lock_guard<std::mutex> ck(s->compile_mu);
  out->compiled_sources = s->compiled.size();
  out->compiles_pending = s->compile_pending.size();
  return S2M_OK;
}

int s2m_server_reset_stats(s2m_server *s) {
  if (!s) return S2M_E_INVALID;
  std::lock_guard<std::mutex> lk(s->mu);
  if (s->completed + s->failed < s->submitted) return S2M_E_INVALID;  // drain first
  s->submitted = s->completed = s->failed = s->batches = 0;
  s->ran_compiled = s->ran_interpreted = 0;
  s->peak_bytes = s->used_bytes;
  s->first_submit = s->last_done = 0;
  s->voxels_done = 0;
  s->latencies_ms.clear();
  return S2M_OK;
}

void s2m_server_free(s2m_server *s) {
  if (!s) return;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
    s->cv.notify_all();
  }
  {
    std::lock_guard<std::mutex> lk(s->compile_mu);
    s->compile_stop = true;
    s->compile_cv.notify_all();
  }
  if (s->compiler.joinable()) s->compiler.join();
  if (s->worker.joinable()) s->worker.join();
  for (auto &t : s->sdf_workers)
    if (t.joinable()) t.join();
  for (auto &kv : s->reqs) {
    kv.second.state = kv.second.state < 2 ? 3 : kv.second.state;
    server_release_locked(s, kv.second);
  }
  for (SWave &sw : s->waves)
    if (sw.b) {
      for (void *a : sw.b->arenas) cudaFreeAsync(a, sw.st);
      for (PinnedBlock &p : sw.b->pinned_free) cudaFreeHost(p.p);
      delete sw.b;
    }
  for (int i = 0; i < 2; ++i)
    if (s->streams[i]) {
      cudaStreamSynchronize(s->streams[i]);
      cudaStreamDestroy(s->streams[i]);
    }
  for (auto &st : s->sdf_streams)
    if (st) {
      cudaStreamSynchronize(st);
      cudaStreamDestroy(st);
    }
  for (auto &kv : s->compiled) s2m_sdf_free(kv.second);
  delete s;
}

}  // extern "C"
