// static_kernels.cuh -- SDF-independent kernels of the per-job pipeline,
// compiled by nvcc into libsdf2mesh_gb300.so: vertex compaction, the
// row-start scan, quad emission (thin wrappers over s2m_workers.cuh), and the
// FP32 issue-rate probe used as the evaluation roofline.
#pragma once
#include "s2m_workers.cuh"

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
