// s2m_lookback.cuh -- single-pass, order-preserving tile prefix sums
// (decoupled look-back) used by every compaction of the pipeline.
//
// Each tile publishes its aggregate, then walks back over its predecessors'
// status words (32 at a time, one per lane) until it meets an inclusive
// prefix.  Tiles take their ids from an atomic counter when they start, so a
// tile only ever waits for tiles that are already running; every wait is
// still bounded in time: once the GPU's global timer has advanced by the
// job's wait limit (S2MeshDev::wait_ns, default S2_WAIT_NS) since the tile
// began to wait, it raises S2_ERR_LOOKBACK in the job's error word and
// continues, and every write that uses the offset is bounds-checked against
// its buffer's capacity.
#pragma once

#define S2_LB_AGG 1ull
#define S2_LB_PRE 2ull
#define S2_LB_MASK ((1ull << 62) - 1ull)
#define S2_WAIT_NS 2000000000ull /* default bound of one device wait: 2 s */
#define S2_FULL 0xffffffffu

__device__ __forceinline__ unsigned long long s2_globaltimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ void s2_st_release(unsigned long long *p, unsigned long long v) {
  asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ unsigned long long s2_ld_acquire(const unsigned long long *p) {
  unsigned long long v;
  asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ unsigned s2_lanemask_lt() {
  unsigned m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

// Loads of data that other blocks of the same launch wrote: cached in L2
// only, never served from a stale L1 line.
__device__ __forceinline__ unsigned long long s2_ldcg(const unsigned long long *p) { return __ldcg(p); }
__device__ __forceinline__ unsigned s2_ldcg(const unsigned *p) { return __ldcg(p); }
__device__ __forceinline__ float s2_ldcg(const float *p) { return __ldcg(p); }

// The walk back alone (tile > 0, its aggregate already published): all 32
// lanes of one warp; the exclusive prefix over tiles 0 .. tile-1, the same in
// every lane.  Publishes nothing.
__device__ __forceinline__ unsigned long long s2_lookback_walk(const unsigned long long *status, unsigned tile,
                                                               unsigned *err, unsigned long long wait_ns) {
  const unsigned lane = threadIdx.x & 31u;
  unsigned long long excl = 0;
  long long base = (long long)tile - 1;
  unsigned long long t0 = 0;
  for (;;) {
    long long idx = base - (long long)lane;
    unsigned long long w = idx >= 0 ? s2_ld_acquire(status + idx) : (S2_LB_PRE << 62);
    unsigned flag = (unsigned)(w >> 62);
    unsigned pmask = __ballot_sync(S2_FULL, flag == 2u);
    unsigned zmask = __ballot_sync(S2_FULL, flag == 0u);
    unsigned first = pmask ? (unsigned)(__ffs(pmask) - 1) : 32u;
    unsigned need = first >= 31u ? S2_FULL : ((2u << first) - 1u);
    if (zmask & need) {
      const unsigned long long now = __shfl_sync(S2_FULL, s2_globaltimer(), 0);
      if (t0 == 0) t0 = now;
      else if (now - t0 > wait_ns) {
        if (lane == 0) atomicOr(err, S2_ERR_LOOKBACK);
        break;
      }
      __nanosleep(32);
      continue;
    }
    unsigned long long v = (lane <= first) ? (w & S2_LB_MASK) : 0ull;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(S2_FULL, v, o);
    excl += v;
    if (first < 32u) break;
    base -= 32;
  }
  return excl;
}

// Called by all 32 lanes of one warp; returns the exclusive prefix of
// `aggregate` over tiles 0 .. tile-1 (the same value in every lane).
__device__ __forceinline__ unsigned long long s2_lookback(unsigned long long *status, unsigned tile,
                                                          unsigned long long aggregate, unsigned *err,
                                                          unsigned long long wait_ns) {
  const unsigned lane = threadIdx.x & 31u;
  if (tile == 0) {
    if (lane == 0) s2_st_release(status, (S2_LB_PRE << 62) | aggregate);
    return 0ull;
  }
  if (lane == 0) s2_st_release(status + tile, (S2_LB_AGG << 62) | aggregate);
  const unsigned long long excl = s2_lookback_walk(status, tile, err, wait_ns);
  if (lane == 0) s2_st_release(status + tile, (S2_LB_PRE << 62) | (excl + aggregate));
  return excl;
}

// Exclusive scan of one value per warp-slot: `vals` holds 32 entries; warp 0
// replaces them by their exclusive prefix and returns the total.
__device__ __forceinline__ unsigned s2_warp_exclusive32(unsigned *vals) {
  const unsigned lane = threadIdx.x & 31u;
  unsigned v = vals[lane];
  unsigned inc = v;
  for (int o = 1; o < 32; o <<= 1) {
    unsigned t = __shfl_up_sync(S2_FULL, inc, o);
    if ((int)lane >= o) inc += t;
  }
  vals[lane] = inc - v;
  return __shfl_sync(S2_FULL, inc, 31);
}

// tile_off[t] = cand.base[slab] + (candidates of tiles < t); cand.base[slab + 1]
// = the slab's running total.  Run by one block of NT threads, CPT
// consecutive counts per thread and step, any tile count; the counts are
// read from L2 (other blocks wrote them).
template <int NT, int CPT>
__device__ __forceinline__ void s2_scan_tiles(const unsigned *tile_cnt, unsigned ntiles,
                                              unsigned long long *__restrict__ tile_off, unsigned long long *base,
                                              int slab_index) {
  __shared__ unsigned long long s_warp[32];
  __shared__ unsigned long long s_carry;
  const unsigned tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
  if (tid == 0) s_carry = __ldcg(base + slab_index);
  if (tid < 32) s_warp[tid] = 0ull;
  __syncthreads();
  for (unsigned t0 = 0; t0 < ntiles; t0 += NT * CPT) {
    const unsigned tb = t0 + tid * CPT;
    unsigned v[CPT];
    unsigned long long sum = 0ull;
#pragma unroll
    for (int q = 0; q < CPT; ++q) {
      v[q] = tb + q < ntiles ? __ldcg(tile_cnt + tb + q) : 0u;
      sum += v[q];
    }
    unsigned long long inc = sum;
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
    unsigned long long run = carry + s_warp[warp] + inc - sum;
#pragma unroll
    for (int q = 0; q < CPT; ++q) {
      if (tb + q < ntiles) tile_off[tb + q] = run;
      run += v[q];
    }
    __syncthreads();
    if (tid == NT - 1) s_carry = run;  // the last thread's running total
    __syncthreads();
  }
  if (tid == 0) base[slab_index + 1] = s_carry;
}
