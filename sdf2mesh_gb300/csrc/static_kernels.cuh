// static_kernels.cuh -- SDF-independent kernels of the per-job pipeline,
// compiled by nvcc into libsdf2mesh_gb300.so: vertex compaction, the
// row-start scan, quad emission (thin wrappers over s2m_workers.cuh), and the
// FP32 issue-rate probe used as the evaluation roofline.
#pragma once
#include "s2m_workers.cuh"
#include "s2m_dc_core.cuh"

// Classification of one slab in three passes that never wait on one another
// (a single pass with a look-back makes every resident tile wait for the
// aggregates of the others):
//   s2m_cells_mark     candidate bits of S2_CELL_CPT cells per thread, tile counts
//   s2m_cells_offsets  exclusive scan of the tile counts (one block)
//   s2m_cells_emit     the candidates of each tile, in (z, y, x) order
__global__ void __launch_bounds__(S2_CELL_BLOCK) s2m_cells_mark(S2Job job, const float *__restrict__ ring,
                                                                unsigned short *__restrict__ masks,
                                                                unsigned *__restrict__ tile_cnt, int zc0, int zc1) {
  __shared__ unsigned s_warp[S2_CELL_BLOCK / 32];
  const unsigned tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5, tile = blockIdx.x;
  const long long ncells = (long long)(zc1 - zc0) * job.N * job.N;
  const long long c0 = (long long)tile * S2_CELL_TILE + (long long)S2_CELL_CPT * tid;
  unsigned mask = 0;
#pragma unroll
  for (int g = 0; g < S2_CELL_CPT / 4; ++g) {
    float v[4][8];
    mask |= s2_classify4<false>(job, ring, c0 + 4 * g, ncells, zc0, v) << (4 * g);
  }
  masks[(size_t)tile * S2_CELL_BLOCK + tid] = (unsigned short)mask;
  unsigned cnt = __popc(mask);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(S2_FULL, cnt, o);
  if (lane == 0) s_warp[warp] = cnt;
  __syncthreads();
  if (tid == 0) {
    unsigned t = 0;
    for (int w = 0; w < S2_CELL_BLOCK / 32; ++w) t += s_warp[w];
    tile_cnt[tile] = t;
  }
}

// tile_off[t] = cand.base[slab] + (candidates of tiles < t); cand.base[slab + 1]
// = the slab's running total.  One block of 1024 threads, any tile count.
__global__ void __launch_bounds__(1024) s2m_cells_offsets(const unsigned *__restrict__ tile_cnt, unsigned ntiles,
                                                          unsigned long long *__restrict__ tile_off,
                                                          unsigned long long *base, int slab_index) {
  __shared__ unsigned long long s_warp[32];
  __shared__ unsigned long long s_carry;
  const unsigned tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
  if (tid == 0) s_carry = base[slab_index];
  __syncthreads();
  for (unsigned t0 = 0; t0 < ntiles; t0 += 1024) {
    const unsigned t = t0 + tid;
    const unsigned long long v = t < ntiles ? tile_cnt[t] : 0ull;
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
    if (tid == 1023) s_carry = carry + s_warp[31] + inc;  // last thread's inclusive total
    __syncthreads();
  }
  if (tid == 0) base[slab_index + 1] = s_carry;
}

__global__ void __launch_bounds__(S2_CELL_BLOCK) s2m_cells_emit(S2Job job, const float *__restrict__ ring,
                                                                const unsigned short *__restrict__ masks,
                                                                const unsigned long long *__restrict__ tile_off,
                                                                S2Cand cand, unsigned *err, int zc0) {
  __shared__ unsigned s_warp[32];
  const unsigned tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5, tile = blockIdx.x;
  const unsigned mask = masks[(size_t)tile * S2_CELL_BLOCK + tid];
  const unsigned cnt = __popc(mask);
  unsigned inc = cnt;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned t = __shfl_up_sync(S2_FULL, inc, o);
    if ((int)lane >= o) inc += t;
  }
  if (lane == 31) s_warp[warp] = inc;
  if (tid < 32 && tid >= S2_CELL_BLOCK / 32) s_warp[tid] = 0u;
  __syncthreads();
  if (warp == 0) s2_warp_exclusive32(s_warp);
  __syncthreads();
  if (!mask) return;
  unsigned long long o = tile_off[tile] + s_warp[warp] + (inc - cnt);
  const long long c0 = (long long)tile * S2_CELL_TILE + (long long)S2_CELL_CPT * tid;
  unsigned rem = mask;
  while (rem) {
    const int m = __ffs(rem) - 1;
    rem &= rem - 1u;
    if (o >= cand.cap) {
      atomicOr(err, S2_ERR_CAND_OVF);
      ++o;
      continue;
    }
    const S2Cell cell = s2_cell_of(job, c0 + m, zc0);
    float v[8];
    s2_load_corners<false>(job, ring, cell, v);
    cand.key[o] = (unsigned long long)cell.x | ((unsigned long long)cell.y << 16) | ((unsigned long long)cell.z << 32);
    float4 *dst = reinterpret_cast<float4 *>(cand.val + 8 * o);
    dst[0] = make_float4(v[0], v[1], v[2], v[3]);
    dst[1] = make_float4(v[4], v[5], v[6], v[7]);
    ++o;
  }
}

__global__ void __launch_bounds__(S2_VC_BLOCK) s2m_vcompact(S2Job job, S2Cand cand, S2MeshDev mesh, int nslabs) {
  s2_vcompact_worker(job, cand, mesh, nslabs, blockIdx.x == 0);
}

__global__ void __launch_bounds__(S2_SCAN_BLOCK) s2m_rowscan(S2MeshDev mesh, unsigned long long R) {
  s2_rowscan_worker(mesh, R);
}

__global__ void __launch_bounds__(S2_Q_BLOCK) s2m_quads(S2Job job, S2MeshDev mesh, unsigned scan_tiles) {
  s2_quads_worker(job, mesh, scan_tiles, blockIdx.x == 0);
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
