// runtime.cu -- libsdf2mesh_gb300.so: NVRTC compilation of lowered SDFs,
// the slab-streamed dual-contouring pipeline on one GB300, and the C ABI
// declared in include/sdf2mesh.h.
//
// Pipeline of one job (reference: src/bin/sdf2mesh/main.rs:298-363 and
// src/mesh.rs:267-341, which run one z-slice per dispatch with a host
// round-trip each):
//   for each slab of D cell slices:
//     s2m_eval_*        lattice planes of the slab into an L2-sized ring (NVRTC)
//     s2m_cells_mark / _offsets / _emit
//                       classify cells, append candidates in order (nvcc)
//   s2m_vertices        reference-rule (or QEF) vertices           (NVRTC)
//   s2m_vcompact        ordered vertex compaction, row counts      (nvcc)
//   s2m_rowscan         row starts of the sorted vertex list       (nvcc)
//   s2m_quads           quads -> triangles, ordered                (nvcc)
// Everything is stream-ordered; the host reads back a few counters at the end.
#include <cuda_runtime.h>
#include <nvrtc.h>

#include <errno.h>
#include <sys/stat.h>
#include <unistd.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <mutex>
#include <sstream>
#include <string>
#include <thread>
#include <vector>

#include "../../include/sdf2mesh.h"
#include "frontend.h"
#include "mesh_io.h"
#include "s2m_device.h"
#include "static_kernels.cuh"

// Sources embedded at build time (s2m_embedded.inc is generated from the
// .cuh / .h files by build.py).
#include "s2m_embedded.inc"

namespace {

void set_err(char *err, size_t errlen, const std::string &msg) {
  if (!err || errlen == 0) return;
  size_t n = std::min(errlen - 1, msg.size());
  std::memcpy(err, msg.data(), n);
  err[n] = 0;
}

char *dup_string(const std::string &s) {
  char *p = static_cast<char *>(std::malloc(s.size() + 1));
  if (p) std::memcpy(p, s.c_str(), s.size() + 1);
  return p;
}

#define S2_CUDA(call)                                                                          \
  do {                                                                                         \
    cudaError_t e_ = (call);                                                                   \
    if (e_ != cudaSuccess) {                                                                   \
      set_err(err, errlen, std::string(#call) + ": " + cudaGetErrorString(e_));                 \
      return e_ == cudaErrorMemoryAllocation ? S2M_E_OOM : S2M_E_CUDA;                         \
    }                                                                                          \
  } while (0)

int device_sm_count() {
  static int sms = 0;
  if (!sms) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms <= 0) sms = 152;
  }
  return sms;
}

}  // namespace

// Evaluation-kernel variants compiled into every SDF module (the tables in
// s2m_dc_kernels.cuh): name, z-run length, whether it evaluates the run-of-4
// form, whether it is a tile-pruned variant (present only in modules of SDFs
// with a pruning form), and whether it evaluates only the tile pass's list of
// undecided tiles (after s2m_fill_decided).
struct EvalVariant {
  const char *name;
  int run;
  bool vec;
  bool pruned;
  bool listed;
};
constexpr EvalVariant kEvalVariants[] = {
    {"s2m_eval_b2r4", 4, false, false, false}, {"s2m_eval_b3r4", 4, false, false, false},
    {"s2m_eval_b4r4", 4, false, false, false}, {"s2m_eval_b2v4", 4, true, false, false},
    {"s2m_eval_b3v4", 4, true, false, false},  {"s2m_evalp_b8", 1, false, true, false},
    {"s2m_evalpl_b8", 1, false, true, true},   {"s2m_evalpl_b8v4", 4, true, true, true}};
constexpr int kNumEvalVariants = int(sizeof(kEvalVariants) / sizeof(kEvalVariants[0]));

// The NVRTC programs of one SDF's module.  Each holds some of its kernels
// (the S2M_WANT_* selections of s2m_dc_kernels.cuh) and compiles on its own
// host thread, so a module builds in the time of its slowest program.
// `variant`: the evaluation variant it holds (-1: none); `prune`: present only
// for SDFs with a tile form; `full_only`: present only in modules without
// pruning.  The full-evaluation run-of-4 variants are the slowest programs to
// compile (12 s of a CSG module's 13 s on one core each) and are never the
// fastest variant where tile pruning runs, so pruned modules leave them out.
struct ModulePart {
  const char *defines;
  int variant;
  bool prune;
  bool full_only;
};
constexpr ModulePart kParts[] = {
    {"#define S2M_WANT_EVAL_B2R4 1\n", 0, false, false},   {"#define S2M_WANT_EVAL_B3R4 1\n", 1, false, false},
    {"#define S2M_WANT_EVAL_B4R4 1\n", 2, false, false},   {"#define S2M_WANT_EVAL_B2V4 1\n", 3, false, true},
    {"#define S2M_WANT_EVAL_B3V4 1\n", 4, false, true},    {"#define S2M_WANT_EVALP_B8 1\n", 5, true, false},
    {"#define S2M_WANT_EVALPL_B8 1\n", 6, true, false},    {"#define S2M_WANT_EVALPL_B8V4 1\n", 7, true, false},
    {"#define S2M_WANT_TILES_COARSE 1\n", -1, true, false}, {"#define S2M_WANT_TILES_FINE 1\n", -1, true, false},
    {"#define S2M_WANT_VERTICES 1\n", -1, false, false}};
constexpr int kNumParts = int(sizeof(kParts) / sizeof(kParts[0]));
constexpr int kPartTilesCoarse = 8, kPartTilesFine = 9, kPartVertices = 10;
bool part_in_module(int i, bool prune) { return prune ? !kParts[i].full_only : !kParts[i].prune; }

struct s2m_sdf {
  std::string user_cuda;
  double fp32_ops = 0, sfu_ops = 0;
  double run_fp32_ops = 0, run_sfu_ops = 0;  // per point in runs of 4 (0: no run form)
  int prune_words = 0;                        // activity words per pruning tile (0: no pruning form)
  int prune_combinators = 0;
  uint32_t flags = 0;
  cudaLibrary_t libs[kNumParts] = {};           // one loaded library per NVRTC program (kParts)
  double compile_s = 0;                         // wall time of the last module build
  int programs = 0, cache_hits = 0;             // NVRTC programs of the build, and those read from the cache
  cudaKernel_t k_eval[kNumEvalVariants] = {};  // null: variant not in this module
  cudaKernel_t k_tiles = nullptr;               // tile pass of the pruned variants (tiles,
  cudaKernel_t k_tiles_coarse = nullptr;        // and the boxes of 4 x 4 tiles first)
  cudaKernel_t k_vertices = nullptr;
  // precision mode: a second module with the QEF vertex kernel, built on the
  // first QEF job (most SDFs never need it, and it compiles slowly)
  std::mutex qef_mu;
  cudaLibrary_t qef_lib = nullptr;
  cudaKernel_t k_vertices_qef = nullptr;
  // autotuned evaluation variant (-1: not tuned yet) and its timings (ns per point)
  mutable std::mutex tune_mu;
  mutable int eval_variant = -1;
  mutable int eval_variant_plain = -1;  // fastest variant without pruning (runs with no pruning buffers)
  // full evaluation slow enough per point that deep slabs pay (set by the
  // autotuner; see kDeepSlabNsPerPoint)
  mutable bool deep_slabs = false;
  mutable double tune_ns[kNumEvalVariants] = {};
  // candidates, vertices and triangles per N^2 cells of this SDF's largest job
  // so far: the next job's initial capacities (an SDF whose surface outgrows
  // the default estimate then overflows and re-runs only once)
  mutable double seen_cand = 0, seen_vert = 0, seen_tri = 0;
  // host copy time over meshing time of the SDF's last one-piece
  // s2m_mesh_generate: sets the sizes of its z parts
  mutable double copy_ratio = 0.5;
  mutable int tune_regs[kNumEvalVariants] = {};
  mutable int tune_local[kNumEvalVariants] = {};  // local (spill/stack) bytes per thread
};

struct s2m_mesh {
  const s2m_sdf *sdf = nullptr;
  cudaStream_t stream = nullptr;  // buffers are allocated and freed in this stream's order
  s2m_params params{};
  S2Job job{};
  int N = 0, D = 0, nzc = 0, nslabs = 0;
  // workspace
  float *ring = nullptr;
  unsigned long long *slab_ctrl = nullptr;  // per cell plane of a slab: its first candidate slot
  unsigned *pt_bits = nullptr;               // sign, near-zero, then unknown-value bits of the ring's lattice points
  unsigned *offx = nullptr;                  // off-lattice bits of the cell columns
  unsigned *cell_words = nullptr;            // candidate bits, 32 cells per word
  unsigned *tile_cnt = nullptr;              // per cell tile: candidates
  // tile pruning: [ops FP32, ops SFU] (2 u64), the length of each slab's list
  // of undecided tiles (u32), the first tile and the first coarse box of
  // every slab (2 x nslabs + 1 u64), then for `prune_chunk` slabs the
  // activity words of the coarse boxes and the tiles, and the tile lists
  unsigned long long *prune_buf = nullptr;
  std::vector<unsigned long long> slab_tile_base, slab_coarse_base;  // host copies
  int prune_chunk = 0;
  size_t prune_base_off = 0;   // bytes from prune_buf to the slab tile bases
  size_t prune_cbase_off = 0;  // ... to the slab coarse-box bases
  size_t prune_sbits_off = 0;  // ... to the coarse boxes' activity words
  size_t prune_bits_off = 0;   // ... to the tiles' activity words
  size_t prune_list_off = 0;   // ... to the lists of undecided tiles
  size_t prune_flags_off = 0;  // ... to the tiles' flags as bytes (s2m_tiles -> classification)
  size_t cell_tiles = 0, vc_tiles = 0, slab_ctrl_words = 0;
  // candidate list of the whole job
  unsigned long long *cand_key = nullptr;
  float *cand_val = nullptr, *cand_pos = nullptr, *cand_nrm = nullptr;
  unsigned long long cand_cap = 0;
  unsigned long long *cand_base = nullptr;    // nslabs + 1
  unsigned long long *cand_status = nullptr;  // vc_ctrl_words(vc_tiles): s2m_vc_scan's base pair, counts, offsets
  // vertex work in tile order (s2m_vtile_*), with tile pruning when every
  // slab's tile bits stay resident: [part_base 2 u64 | tile counts (vt_tiles)
  // + done counter | block totals (vt_blocks) | block offsets (vt_blocks u64)
  // | tile and rank per candidate (u64) | permutation (u32)]
  unsigned char *vt_buf = nullptr;
  unsigned long long vt_tiles = 0;
  unsigned vt_blocks = 0;
  size_t vt_cnt_off = 0, vt_part_off = 0, vt_poff_off = 0, vt_rank_off = 0, vt_perm_off = 0;
  // outputs and job counters
  float *pos = nullptr, *nrm = nullptr;
  unsigned long long *key = nullptr;
  unsigned *tris = nullptr;
  unsigned long long vcap = 0, tcap = 0;
  unsigned *rowcnt = nullptr, *rowstart = nullptr;
  unsigned long long *scan_status = nullptr;
  size_t scan_tiles = 0, quad_tiles = 0;
  unsigned long long *jobctl = nullptr;  // [ntris, invalid, vtotal, err | counters[8]]
  // host results
  unsigned long long *h_read = nullptr;  // pinned readback
  // z part of the lattice (s2m_mesh_generate): cell planes zpart_begin ..
  // zpart_end - 1, zpart_end < 0 for the whole job; zfrac = its share of the
  // job's cell planes (for the learned capacities)
  int zpart_begin = 0, zpart_end = -1;
  double zfrac = 1.0;
  unsigned quads_from_z = 0;  // vertices with a lower label z make no quads (the context plane of a part)
  bool tiles_ready = false;   // the tile pass of every slab was enqueued elsewhere (s2m_mesh_generate)
  // host time of the last s2m_mesh_create (ms) and its pipeline runs
  double t_setup = 0, t_launch = 0, t_wait = 0;
  unsigned runs = 0;
  uint64_t nverts = 0, ntris = 0, invalid = 0, ncand = 0;
  uint32_t errflags = 0;
  uint64_t launches = 0;
  // SDF operations of the last run's lattice evaluation, and its points
  bool last_pruned = false;
  int last_variant = 0;
  double eval_points = 0, eval_fp_ops = 0, eval_sfu_ops = 0;
  // optional per-kernel timing: an event pair around each launch
  bool profile = false;
  std::vector<cudaEvent_t> ev;
  std::vector<int> ev_kind;
  std::vector<double> ev_units;
  size_t ev_used = 0;
  s2m_profile prof{};
  // bound of each device wait of a run (look-backs), GPU global timer ns
  unsigned long long wait_ns = S2_WAIT_NS;
  // CUDA graph of the whole pipeline, replayed by s2m_mesh_run_async
  bool use_graph = false;
  cudaGraphExec_t graph = nullptr;
  cudaStream_t capture_stream = nullptr;  // private stream the graph is captured on
};

namespace {

// ---------------------------------------------------------------------------
// NVRTC

// ---------------------------------------------------------------------------
// On-disk cache of compiled modules.  The key is everything the CUBIN depends
// on: the NVRTC version, the options (architecture, contraction) and the whole
// program text (pipeline sources + lowered SDF + kernel selection).  A file
// holds the key itself beside the CUBIN, so a hit is an exact match, not a
// hash match.  Directory: $S2M_CACHE_DIR (empty: no cache), else
// $XDG_CACHE_HOME/sdf2mesh_gb300, else $HOME/.cache/sdf2mesh_gb300.

std::string module_cache_dir() {
  if (const char *d = std::getenv("S2M_CACHE_DIR")) return d;
  if (const char *x = std::getenv("XDG_CACHE_HOME"))
    if (*x) return std::string(x) + "/sdf2mesh_gb300";
  if (const char *h = std::getenv("HOME"))
    if (*h) return std::string(h) + "/.cache/sdf2mesh_gb300";
  return "";
}

bool make_dirs(const std::string &dir) {
  if (dir.empty()) return false;
  for (size_t i = 1; i <= dir.size(); ++i) {
    if (i == dir.size() || dir[i] == '/') {
      const std::string sub = dir.substr(0, i);
      if (::mkdir(sub.c_str(), 0755) != 0 && errno != EEXIST) return false;
    }
  }
  return true;
}

// 128-bit file name of a key: two FNV-1a style 64-bit hashes with different
// offsets and multipliers (a name, not a proof: the file holds the key).
std::string key_name(const std::string &key) {
  uint64_t a = 1469598103934665603ull, b = 0x9e3779b97f4a7c15ull;
  for (unsigned char c : key) {
    a = (a ^ c) * 1099511628211ull;
    b = (b ^ c) * 0x100000001b3ull + 0x2545f4914f6cdd1dull;
  }
  char buf[40];
  std::snprintf(buf, sizeof buf, "%016llx%016llx", (unsigned long long)a, (unsigned long long)b);
  return buf;
}

constexpr char kCacheMagic[] = "S2MCUBIN1";

bool cache_load(const std::string &dir, const std::string &key, std::vector<char> &cubin) {
  if (dir.empty()) return false;
  std::ifstream f(dir + "/" + key_name(key) + ".cubin", std::ios::binary);
  if (!f) return false;
  char magic[sizeof kCacheMagic];
  uint64_t klen = 0, clen = 0;
  if (!f.read(magic, sizeof magic) || std::memcmp(magic, kCacheMagic, sizeof magic) != 0) return false;
  if (!f.read(reinterpret_cast<char *>(&klen), 8) || klen != key.size()) return false;
  std::string k(klen, '\0');
  if (!f.read(&k[0], std::streamsize(klen)) || k != key) return false;
  if (!f.read(reinterpret_cast<char *>(&clen), 8) || clen == 0 || clen > (1ull << 31)) return false;
  cubin.resize(size_t(clen));
  return bool(f.read(cubin.data(), std::streamsize(clen)));
}

void cache_store(const std::string &dir, const std::string &key, const std::vector<char> &cubin) {
  if (dir.empty() || !make_dirs(dir)) return;
  static std::atomic<unsigned> seq{0};
  const std::string name = dir + "/" + key_name(key) + ".cubin";
  const std::string tmp = name + ".tmp" + std::to_string(::getpid()) + "." + std::to_string(seq++);
  {
    std::ofstream f(tmp, std::ios::binary);
    if (!f) return;
    const uint64_t klen = key.size(), clen = cubin.size();
    f.write(kCacheMagic, sizeof kCacheMagic);
    f.write(reinterpret_cast<const char *>(&klen), 8);
    f.write(key.data(), std::streamsize(klen));
    f.write(reinterpret_cast<const char *>(&clen), 8);
    f.write(cubin.data(), std::streamsize(clen));
    if (!f) {
      std::remove(tmp.c_str());
      return;
    }
  }
  if (std::rename(tmp.c_str(), name.c_str()) != 0) std::remove(tmp.c_str());  // atomic publish
}

// NVRTC: the lowered SDF with the pipeline's device sources into a CUBIN for
// sm_103a (or the cached CUBIN of the same program), loaded as a library.
// `defines` selects the program's kernels; `qef` builds the precision-mode
// vertex kernel alone.  *hit tells whether the CUBIN came from the cache.
// The vertex kernel's dynamic shared memory (S2_VX_SMEM_BYTES) is above the
// 48 KB that a launch gets without asking.
int vertex_smem_attribute(cudaKernel_t k, char *err, size_t errlen) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess)
    e = cudaKernelSetAttributeForDevice(k, cudaFuncAttributeMaxDynamicSharedMemorySize, int(S2_VX_SMEM_BYTES), dev);
  if (e != cudaSuccess) {
    set_err(err, errlen, std::string("vertex kernel shared memory: ") + cudaGetErrorString(e));
    return S2M_E_CUDA;
  }
  return S2M_OK;
}

int nvrtc_build(const s2m_sdf *s, bool qef, const char *defines, cudaLibrary_t *lib, bool *hit, char *err,
                size_t errlen) {
  std::string src;
  src += "// sdf2mesh_gb300 per-SDF module\n";
  if (qef) src += "#define S2M_QEF_MODULE 1\n";
  if (defines) {
    src += "#define S2M_SELECT 1\n";
    src += defines;
  }
  src += kS2mDeviceH;
  src += kS2mLookbackCuh;
  src += kS2mPreludeCuh;
  src += kS2mDcCoreCuh;
  src += s->user_cuda;
  src += kS2mDcKernelsCuh;
  std::vector<const char *> opts = {"--gpu-architecture=sm_103a", "-std=c++17", "-default-device"};
  if (std::getenv("S2M_NVRTC_LINEINFO")) opts.push_back("-lineinfo");
  opts.push_back((s->flags & S2M_COMPILE_FMAD) ? "--fmad=true" : "--fmad=false");
  int vmaj = 0, vmin = 0;
  nvrtcVersion(&vmaj, &vmin);
  std::string key = "nvrtc " + std::to_string(vmaj) + "." + std::to_string(vmin) + "\n";
  for (const char *o : opts) key += std::string(o) + "\n";
  key += src;
  const std::string dir = module_cache_dir();
  std::vector<char> cubin;
  *hit = cache_load(dir, key, cubin);
  if (!*hit) {
    nvrtcProgram prog;
    if (nvrtcCreateProgram(&prog, src.c_str(), "s2m_module.cu", 0, nullptr, nullptr) != NVRTC_SUCCESS) {
      set_err(err, errlen, "nvrtcCreateProgram failed");
      return S2M_E_NVRTC;
    }
    nvrtcResult rc = nvrtcCompileProgram(prog, int(opts.size()), opts.data());
    if (rc != NVRTC_SUCCESS) {
      size_t n = 0;
      nvrtcGetProgramLogSize(prog, &n);
      std::string log(n, '\0');
      if (n) nvrtcGetProgramLog(prog, &log[0]);
      nvrtcDestroyProgram(&prog);
      set_err(err, errlen, std::string("NVRTC: ") + nvrtcGetErrorString(rc) + "\n" + log);
      return S2M_E_NVRTC;
    }
    size_t cubin_n = 0;
    nvrtcGetCUBINSize(prog, &cubin_n);
    cubin.resize(cubin_n);
    nvrtcGetCUBIN(prog, cubin.data());
    nvrtcDestroyProgram(&prog);
    cache_store(dir, key, cubin);
  }
  cudaError_t ce = cudaLibraryLoadData(lib, cubin.data(), nullptr, nullptr, 0, nullptr, nullptr, 0);
  if (ce != cudaSuccess) {
    set_err(err, errlen, std::string("cudaLibraryLoadData: ") + cudaGetErrorString(ce));
    return ce == cudaErrorNoDevice || ce == cudaErrorInsufficientDriver ? S2M_E_NO_DEVICE : S2M_E_CUDA;
  }
  return S2M_OK;
}

int compile_module(s2m_sdf *s, char *err, size_t errlen) {
  // Pruned variants are bit-exact only without FMA contraction (their
  // interval bounds and the skipped arithmetic assume separately rounded
  // operations), so an S2M_COMPILE_FMAD module does not use them.
  const bool prune = s->prune_words > 0 && !(s->flags & (S2M_COMPILE_FMAD | S2M_COMPILE_NO_PRUNE));
  const auto t0 = std::chrono::steady_clock::now();
  struct Result {
    int rc = S2M_OK;
    bool hit = false;
    char msg[2048] = {0};
  };
  std::vector<Result> res(kNumParts);
  std::vector<std::thread> th;
  for (int i = 0; i < kNumParts; ++i) {
    if (!part_in_module(i, prune)) continue;
    th.emplace_back([s, i, &res] {
      res[size_t(i)].rc = nvrtc_build(s, false, kParts[i].defines, &s->libs[i], &res[size_t(i)].hit,
                                      res[size_t(i)].msg, sizeof res[size_t(i)].msg);
    });
  }
  for (auto &t : th) t.join();
  s->programs = int(th.size());
  s->cache_hits = 0;
  for (int i = 0; i < kNumParts; ++i) {
    if (!part_in_module(i, prune)) continue;
    if (res[size_t(i)].rc != S2M_OK) {
      set_err(err, errlen, res[size_t(i)].msg);
      return res[size_t(i)].rc;
    }
    s->cache_hits += res[size_t(i)].hit ? 1 : 0;
  }
  s->compile_s = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  for (int i = 0; i < kNumParts; ++i) {
    const int v = kParts[i].variant;
    if (v < 0 || !part_in_module(i, prune)) continue;
    if (cudaLibraryGetKernel(&s->k_eval[v], s->libs[i], kEvalVariants[v].name) != cudaSuccess) {
      set_err(err, errlen, std::string("kernel missing from the compiled module: ") + kEvalVariants[v].name);
      return S2M_E_CUDA;
    }
  }
  if (prune && (cudaLibraryGetKernel(&s->k_tiles, s->libs[kPartTilesFine], "s2m_tiles") != cudaSuccess ||
                cudaLibraryGetKernel(&s->k_tiles_coarse, s->libs[kPartTilesCoarse], "s2m_tiles_coarse") !=
                    cudaSuccess)) {
    set_err(err, errlen, "kernel missing from the compiled module: s2m_tiles / s2m_tiles_coarse");
    return S2M_E_CUDA;
  }
  if (cudaLibraryGetKernel(&s->k_vertices, s->libs[kPartVertices], "s2m_vertices") != cudaSuccess) {
    set_err(err, errlen, "kernels missing from the compiled module");
    return S2M_E_CUDA;
  }
  return s->prune_words > 0 ? vertex_smem_attribute(s->k_vertices, err, errlen) : S2M_OK;
}

// The QEF vertex kernel of an SDF, built once on its first precision-mode job.
int ensure_qef_module(const s2m_sdf *cs, char *err, size_t errlen) {
  s2m_sdf *s = const_cast<s2m_sdf *>(cs);
  std::lock_guard<std::mutex> lock(s->qef_mu);
  if (s->k_vertices_qef) return S2M_OK;
  bool hit = false;
  int rc = nvrtc_build(s, true, nullptr, &s->qef_lib, &hit, err, errlen);
  if (rc != S2M_OK) return rc;
  if (cudaLibraryGetKernel(&s->k_vertices_qef, s->qef_lib, "s2m_vertices") != cudaSuccess) {
    set_err(err, errlen, "QEF vertex kernel missing from the compiled module");
    return S2M_E_CUDA;
  }
  return S2M_OK;
}

// ---------------------------------------------------------------------------
// Job setup

// main.rs:139-148: a resolution that is not a power of two becomes 2 << ilog2.
uint32_t reference_resolution(uint32_t r) {
  if (__builtin_popcount(r) > 1) {
    uint32_t lg = 31u - uint32_t(__builtin_clz(r));
    r = 2u << lg;
  }
  return r;
}

// Pinned 8-word read-back slots, carved from blocks that live for the process
// (pinning and unpinning host memory per job would synchronise the device).
std::mutex g_pinned_mu;
std::vector<unsigned long long *> g_pinned_free;

unsigned long long *take_pinned_slot() {
  std::lock_guard<std::mutex> lock(g_pinned_mu);
  if (g_pinned_free.empty()) {
    unsigned long long *blk = nullptr;
    if (cudaMallocHost(&blk, 512 * 64) != cudaSuccess) return nullptr;
    for (int i = 0; i < 512; ++i) g_pinned_free.push_back(blk + 8 * i);
  }
  unsigned long long *p = g_pinned_free.back();
  g_pinned_free.pop_back();
  return p;
}

void give_pinned_slot(unsigned long long *p) {
  std::lock_guard<std::mutex> lock(g_pinned_mu);
  g_pinned_free.push_back(p);
}

void free_buffers(s2m_mesh *m) {
  void *ptrs[] = {m->ring, m->slab_ctrl, m->pt_bits, m->offx, m->cell_words, m->tile_cnt, m->prune_buf, m->cand_key, m->cand_val, m->cand_pos, m->cand_nrm, m->cand_base,
                  m->cand_status, m->pos, m->nrm, m->key, m->tris, m->rowcnt, m->rowstart, m->scan_status,
                  m->jobctl, m->vt_buf};
  for (void *p : ptrs)
    if (p) cudaFreeAsync(p, m->stream);
  if (m->h_read) give_pinned_slot(m->h_read);
  m->ring = nullptr; m->slab_ctrl = nullptr; m->pt_bits = nullptr; m->offx = nullptr; m->cell_words = nullptr;
  m->tile_cnt = nullptr; m->prune_buf = nullptr; m->cand_key = nullptr; m->cand_val = nullptr; m->cand_pos = nullptr;
  m->cand_nrm = nullptr; m->cand_base = nullptr; m->cand_status = nullptr; m->pos = nullptr; m->nrm = nullptr;
  m->key = nullptr; m->tris = nullptr; m->rowcnt = nullptr; m->rowstart = nullptr; m->scan_status = nullptr;
  m->jobctl = nullptr; m->h_read = nullptr; m->vt_buf = nullptr;
}

int setup_job(s2m_mesh *m, char *err, size_t errlen) {
  const s2m_params &p = m->params;
  uint32_t N = p.resolution;
  if (p.flags & S2M_JOB_POW2_ROUNDING) N = reference_resolution(N);
  if (N < 2 || N > 65535) {
    set_err(err, errlen, "resolution must be in [2, 65535]");
    return S2M_E_INVALID;
  }
  if (!(p.bounds > 0.0f) || !std::isfinite(p.bounds)) {
    set_err(err, errlen, "bounds must be a positive finite number");
    return S2M_E_INVALID;
  }
  m->N = int(N);
  S2Job &j = m->job;
  j.N = int(N);
  j.P = int(N) + 1;
  j.pitch = (j.P + 31) / 32 * 32;
  j.plane = (long long)j.P * j.pitch;
  // Bounds3D::cube(B, 0) in binary32 (lib.rs:115-118), size per
  // dualcontour.wgsl:23-24.
  volatile float half = p.bounds * 0.5f;
  volatile float mn = 0.0f - half;
  volatile float mx = 0.0f + half;
  volatile float ext = mx - mn;
  j.bmin = mn;
  j.size = ext / float(N - 1u);
  j.eps = p.eps;
  j.guard = j.size;  // one cell: far above any rounding difference of a corner
  j.lag = (p.flags & S2M_JOB_SLICE_LAG) ? 1 : 0;
  j.exact = (p.flags & S2M_JOB_EXACT_CORNERS) ? 1 : 0;
  j.qef = (p.flags & S2M_JOB_QEF) ? 1 : 0;
  j.magic_n = uint32_t((1ull << 32) / uint64_t(j.N) + 1);
  j.magic_p = uint32_t((1ull << 32) / uint64_t(j.P) + 1);
  {
    const uint64_t wn = (uint64_t(j.N) + 31) / 32;
    j.magic_wn = wn >= 2 ? uint32_t((1ull << 32) / wn + 1) : 0u;
  }
  // cell planes of the job: the whole lattice, or the part zpart_begin ..
  // zpart_end - 1 (s2m_mesh_generate's z parts)
  const int full_nzc = j.lag ? int(N) - 1 : int(N);
  if (m->zpart_end >= 0) {
    j.zb = m->zpart_begin;
    m->nzc = std::max(0, std::min(full_nzc, m->zpart_end) - m->zpart_begin);
  } else {
    j.zb = 0;
    m->nzc = full_nzc;
  }
  m->zfrac = full_nzc > 0 ? double(m->nzc) / double(full_nzc) : 1.0;
  // Slab depth.  Full evaluation: the ring of D + 1 lattice planes is sized
  // to stay resident in the 126 MB L2 between the evaluation and the point
  // bits pass -- unless the autotuner measured the evaluation at
  // kDeepSlabNsPerPoint or more, which then runs deep slabs as below.  An SDF with a tile form: the pruned evaluation writes the
  // point bits itself and classification reads only those (and the
  // candidates' corners), so the ring need not fit in L2; deep slabs (a ring
  // of up to 4.6 GB, slabs of equal depth) amortise each slab's evaluation
  // tail, where its last heavy tiles run at low occupancy (a 1024^3 CSG job:
  // 16.3 ms with 10-plane slabs, 7.9 ms with 512).  A job in one slab (1024^3
  // and its z parts) keeps its whole lattice resident, and the vertex kernel
  // reads the candidates' corners from it.
  int D = int(p.slab_depth);
  if (D <= 0) {
    const double plane_bytes = double(j.plane) * 4.0;
    if (m->sdf && (m->sdf->k_tiles || m->sdf->deep_slabs)) {
      const int dmax = std::max(1, int(std::min(4.6e9 / plane_bytes, 1.0e9)) - 1);
      const int nz = std::max(1, m->nzc);
      const int ns = (nz + dmax - 1) / dmax;
      D = (nz + ns - 1) / ns;
    } else {
      D = int(48.0e6 / plane_bytes) - 1;
      D = std::max(1, std::min(D, 64));
    }
  }
  D = std::max(1, std::min(D, std::max(1, m->nzc)));
  m->D = D;
  j.ring = D + 1;
  m->nslabs = m->nzc > 0 ? (m->nzc + D - 1) / D : 0;
  return S2M_OK;
}

// Point bits of the ring (three arrays of ring * P * ceil(P / 32) words).
size_t pt_bits_words(const s2m_mesh *m) {  // one of the three arrays (S2PointBits)
  const size_t P = size_t(m->job.P), WP = (P + 31) / 32;
  return size_t(m->job.ring) * P * WP;
}
S2PointBits point_bits(const s2m_mesh *m) {
  S2PointBits pb;
  pb.pos = m->pt_bits;
  pb.near = m->pt_bits + pt_bits_words(m);
  pb.unk = m->pt_bits + 2 * pt_bits_words(m);
  return pb;
}

// Planes k0 .. k0 + nk - 1 that slab s evaluates.
void slab_planes(const s2m_mesh *m, int s, int &k0, int &nk) {
  const int zb = m->job.zb;
  const int zc0 = zb + s * m->D;
  const int zc1 = std::min(zb + m->nzc, zc0 + m->D);
  k0 = s == 0 ? zb : zc0 + 1;
  nk = zc1 - k0 + 1;
}

// Tiles of slab planes k0 .. k0 + nk - 1 for the pruned variants: tzs planes
// per tile (at most S2_PT_ZMAX, balanced), nzt tiles in z, none empty (the
// device computes the same in s2_tile_depth).
struct PruneGeom {
  int tzs = 0, nzt = 0;
  long long ntiles = 0;
};
PruneGeom prune_geom(const S2Job &j, int nk) {
  PruneGeom g;
  const int parts = (nk + S2_PT_ZMAX - 1) / S2_PT_ZMAX;
  g.tzs = (nk + parts - 1) / parts;
  g.nzt = (nk + g.tzs - 1) / g.tzs;
  const long long ntx = (j.P + S2_PT_XY - 1) / S2_PT_XY;
  g.ntiles = ntx * ntx * g.nzt;
  return g;
}

// The tile pass runs over chunks of prune_chunk slabs, two launches each; the
// activity words of a chunk stay within kPruneBitsBudget (all slabs of the
// job at once up to well beyond 1024^3).
constexpr size_t kPruneBitsBudget = size_t(256) << 20;
size_t prune_layout(s2m_mesh *m) {
  const int ns = m->nslabs;
  m->slab_tile_base.assign(size_t(ns) + 1, 0ull);
  m->slab_coarse_base.assign(size_t(ns) + 1, 0ull);
  const long long ntx = (m->job.P + S2_PT_XY - 1) / S2_PT_XY;
  const long long ncx = (ntx + S2_PT_COARSE - 1) / S2_PT_COARSE;
  unsigned long long max_slab = 1;
  for (int s = 0; s < ns; ++s) {
    int k0, nk;
    slab_planes(m, s, k0, nk);
    const PruneGeom g = prune_geom(m->job, nk);
    m->slab_tile_base[size_t(s) + 1] = m->slab_tile_base[size_t(s)] + (unsigned long long)g.ntiles;
    m->slab_coarse_base[size_t(s) + 1] =
        m->slab_coarse_base[size_t(s)] + (unsigned long long)(ncx * ncx * ((g.nzt + S2_PT_COARSE_Z - 1) / S2_PT_COARSE_Z));
    max_slab = std::max(max_slab, (unsigned long long)g.ntiles);
  }
  const size_t words = size_t(m->sdf->prune_words);
  m->prune_chunk = int(std::max<size_t>(1, std::min<size_t>(size_t(std::max(ns, 1)),
                                                            kPruneBitsBudget / (max_slab * (words + 1) * 4))));
  unsigned long long chunk_tiles = 0, chunk_coarse = 0;
  for (int s = 0; s < ns; s += m->prune_chunk) {
    const int e = std::min(ns, s + m->prune_chunk);
    chunk_tiles = std::max(chunk_tiles, m->slab_tile_base[size_t(e)] - m->slab_tile_base[size_t(s)]);
    chunk_coarse = std::max(chunk_coarse, m->slab_coarse_base[size_t(e)] - m->slab_coarse_base[size_t(s)]);
  }
  auto up16 = [](size_t x) { return (x + 15) / 16 * 16; };
  m->prune_base_off = up16(16 + 4 * size_t(ns));
  m->prune_cbase_off = up16(m->prune_base_off + 8 * (size_t(ns) + 1));
  m->prune_sbits_off = up16(m->prune_cbase_off + 8 * (size_t(ns) + 1));
  m->prune_bits_off = up16(m->prune_sbits_off + size_t(chunk_coarse) * (words + 1) * 4);  // + each box's flag word
  m->prune_list_off = up16(m->prune_bits_off + size_t(chunk_tiles) * (words + 1) * 4);  // + each tile's flag word
  m->prune_flags_off = up16(m->prune_list_off + size_t(chunk_tiles) * 4);
  // one byte per tile of the chunk, rows of 4 * WP bytes (one word per 32 lattice points along x)
  const size_t flag_rows = size_t(chunk_tiles / (unsigned long long)ntx);
  return m->prune_flags_off + flag_rows * size_t((m->job.P + 31) / 32) * 4;
}
template <class T> T *prune_at(const s2m_mesh *m, size_t off) {
  return reinterpret_cast<T *>(reinterpret_cast<char *>(m->prune_buf) + off);
}
unsigned long long *prune_bases(const s2m_mesh *m) { return prune_at<unsigned long long>(m, m->prune_base_off); }
unsigned *prune_list_counts(const s2m_mesh *m) { return reinterpret_cast<unsigned *>(m->prune_buf + 2); }

// Launches of the per-job pipeline with programmatic dependent launch: a
// kernel's blocks may be scheduled while the kernel before it in the stream
// drains, and wait at S2_PDL_WAIT until its writes are visible.
cudaLaunchConfig_t pdl_config(dim3 grid, dim3 block, size_t smem, cudaStream_t st, cudaLaunchAttribute *attr) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  attr->id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr->val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cfg;
}
template <typename... KArgs, typename... Args>
cudaError_t launch_pdl(void (*k)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st, Args... args) {
  cudaLaunchAttribute attr;
  const cudaLaunchConfig_t cfg = pdl_config(grid, block, smem, st, &attr);
  return cudaLaunchKernelEx(&cfg, k, static_cast<KArgs>(args)...);
}
cudaError_t launch_pdl(cudaKernel_t k, dim3 grid, dim3 block, size_t smem, cudaStream_t st, void **args) {
  cudaLaunchAttribute attr;
  const cudaLaunchConfig_t cfg = pdl_config(grid, block, smem, st, &attr);
  return cudaLaunchKernelExC(&cfg, reinterpret_cast<const void *>(k), args);
}

// Device pointers of the counters inside jobctl.
struct JobCtl {
  unsigned long long *ntris, *invalid, *vtotal;
  unsigned *err;
  unsigned *counters;
};
JobCtl jobctl(const s2m_mesh *m) {
  JobCtl c;
  c.ntris = m->jobctl + 0;
  c.invalid = m->jobctl + 1;
  c.vtotal = m->jobctl + 2;
  c.err = reinterpret_cast<unsigned *>(m->jobctl + 3);
  c.counters = reinterpret_cast<unsigned *>(m->jobctl + 4);  // 8 x u32
  return c;
}

// Tile pass over slabs [s_begin, s_end) (coarse boxes, then tiles) and the
// pruned evaluation of slab s.
cudaError_t launch_tiles(const s2m_mesh *m, int s_begin, int s_end, cudaStream_t st) {
  S2Job jj = m->job;
  unsigned *sbits = prune_at<unsigned>(m, m->prune_sbits_off);
  unsigned *bits = prune_at<unsigned>(m, m->prune_bits_off);
  unsigned long long *ops = m->prune_buf;
  const unsigned long long *tbase = prune_at<unsigned long long>(m, m->prune_base_off);
  const unsigned long long *cbase = prune_at<unsigned long long>(m, m->prune_cbase_off);
  int D = m->D, nzc = m->nzc;
  const unsigned long long nc = m->slab_coarse_base[size_t(s_end)] - m->slab_coarse_base[size_t(s_begin)];
  void *cargs[] = {&jj, &sbits, &cbase, &s_begin, &s_end, &D, &nzc};
  cudaError_t e = launch_pdl(m->sdf->k_tiles_coarse, dim3(unsigned((nc + S2_PT_BLOCK - 1) / S2_PT_BLOCK)),
                             dim3(S2_PT_BLOCK), 0, st, cargs);
  if (e != cudaSuccess) return e;
  // one thread per tile slot of each coarse box (s2m_tiles)
  const unsigned long long n = nc * S2_PT_COARSE * S2_PT_COARSE * S2_PT_COARSE_Z;
  unsigned *list = prune_at<unsigned>(m, m->prune_list_off);
  unsigned *counts = prune_list_counts(m);
  unsigned char *tflags = prune_at<unsigned char>(m, m->prune_flags_off);
  int fpitch = 4 * ((m->job.P + 31) / 32);
  void *targs[] = {&jj, &bits, &ops, &sbits, &tbase, &cbase, &s_begin, &s_end, &D, &nzc, &list, &counts, &tflags,
                   &fpitch};
  return launch_pdl(m->sdf->k_tiles, dim3(unsigned((n + S2_PT_BLOCK - 1) / S2_PT_BLOCK)), dim3(S2_PT_BLOCK), 0, st,
                    targs);
}
cudaError_t launch_evalp(const s2m_mesh *m, int v, int s, int chunk_begin, cudaStream_t st) {
  S2Job jj = m->job;
  float *ring = m->ring;
  int k0, nk;
  slab_planes(m, s, k0, nk);
  PruneGeom g = prune_geom(m->job, nk);
  const unsigned *bits = prune_at<unsigned>(m, m->prune_bits_off) + (m->slab_tile_base[size_t(s)] -
                                                                     m->slab_tile_base[size_t(chunk_begin)]) *
                                                                        (size_t(m->sdf->prune_words) + 1);
  S2PointBits pb = point_bits(m);
  if (kEvalVariants[v].listed) {
    const int W1 = m->sdf->prune_words + 1;
    const long long plane_words = (long long)m->job.P * ((m->job.P + 31) / 32);
    unsigned *chunks = jobctl(m).counters + 5;  // set to zero by the fill, taken by the listed evaluation
    cudaError_t e;
    if (!m->job.exact) {
      // classification by listed tiles (s2m_cells_mark_tiles): the bits of
      // the slab's last plane in full (the next slab's first plane), the
      // other planes' decided tiles read from the tile flags; the cell tile
      // counts cleared
      const long long ntx = (m->job.P + S2_PT_XY - 1) / S2_PT_XY;
      const unsigned *lbits = bits + size_t(g.nzt - 1) * size_t(ntx * ntx) * size_t(W1);
      e = launch_pdl(s2m_fill_decided, dim3(unsigned((plane_words + 255) / 256), 1u), dim3(256), 0, st, jj, pb, lbits,
                     W1, k0 + nk - 1, 1, 1, chunks, m->tile_cnt, unsigned(m->cell_tiles));
    } else {  // every cell is classified (s2m_cells_mark): every plane's bits
      e = launch_pdl(s2m_fill_decided, dim3(unsigned((plane_words + 255) / 256), unsigned(g.nzt)), dim3(256), 0, st,
                     jj, pb, bits, W1, k0, nk, g.tzs, chunks, static_cast<unsigned *>(nullptr), 0u);
    }
    if (e != cudaSuccess) return e;
    const unsigned *list = prune_at<unsigned>(m, m->prune_list_off) +
                           (m->slab_tile_base[size_t(s)] - m->slab_tile_base[size_t(chunk_begin)]);
    const unsigned *count = prune_list_counts(m) + s;
    void *largs[] = {&jj, &ring, &pb, &bits, &k0, &nk, &g.tzs, &list, &count, &chunks};
    // one block per SM takes chunks of the list (its length is on the device)
    const long long lblocks = std::min<long long>((g.ntiles + S2_PL_BLOCK / 32 - 1) / (S2_PL_BLOCK / 32),
                                                  (long long)device_sm_count());
    return launch_pdl(m->sdf->k_eval[v], dim3(unsigned(lblocks)), dim3(S2_PL_BLOCK), 0, st, largs);
  }
  void *pargs[] = {&jj, &ring, &pb, &bits, &k0, &nk, &g.tzs, &g.nzt};
  return launch_pdl(m->sdf->k_eval[v], dim3(unsigned((g.ntiles + 3) / 4)), dim3(S2_PT_BLOCK), 0, st, pargs);
}

// Classification buffers: words of 32 cells per slab (tiles of S2_CW_BLOCK
// words), and the point bits of a slab's D + 1 planes.
// Vertex compaction control (u64 words): [base pair | per-tile vertex counts
// (u32) | per-tile first vertex]; the first vc_ctrl_offsets words are zeroed
// per job.
size_t vc_ctrl_offsets(size_t vc_tiles) { return 2 + (vc_tiles + 1) / 2; }
size_t vc_ctrl_words(size_t vc_tiles) { return vc_ctrl_offsets(vc_tiles) + vc_tiles; }

// Scan words of a job (u64): the row-start scan's look-back words, then the
// quad passes' tile offsets, tile counts (u32, two per word) and base pair.
size_t scan_status_words(size_t scan_tiles, size_t quad_tiles) {
  return scan_tiles + quad_tiles + (quad_tiles + 1) / 2 + 2;
}

// Classification tiles: S2_CW_BLOCK words of 32 cells of one cell plane, nbp
// per plane, D planes per slab.
unsigned cell_tiles_per_plane(const s2m_mesh *m) {
  const size_t WN = size_t((m->N + 31) / 32);
  return unsigned((size_t(m->N) * WN + S2_CW_BLOCK - 1) / S2_CW_BLOCK);
}
size_t cell_word_tiles(const s2m_mesh *m) { return size_t(m->D) * cell_tiles_per_plane(m); }
// Classification counters (u32): per cell tile its candidates, the finished
// mark blocks, per cell plane its candidates.
size_t tile_cnt_words(const s2m_mesh *m) { return m->cell_tiles + 1 + size_t(m->D); }
unsigned *cls_done(const s2m_mesh *m) { return m->tile_cnt + m->cell_tiles; }
unsigned *cls_plane_cnt(const s2m_mesh *m) { return m->tile_cnt + m->cell_tiles + 1; }

void drop_graph(s2m_mesh *m) {
  if (m->graph) cudaGraphExecDestroy(m->graph);
  m->graph = nullptr;
}

// Bytes of every device buffer of a job, in allocation order.  plan_buffers
// fixes the capacities and layouts on the mesh; alloc_buffers allocates
// exactly this plan, and the server's admission sums it (mesh_job_footprint),
// so the two cannot drift apart.
struct BufPlan {
  size_t ring, slab_ctrl, pt_bits, offx, cell_words, tile_cnt, prune, cand_key, cand_val, cand_pos, cand_nrm,
      cand_base, cand_status, vt, pos, nrm, key, tris, rowcnt, rowstart, scan_status, jobctl;
  size_t total() const {
    return ring + slab_ctrl + pt_bits + offx + cell_words + tile_cnt + prune + cand_key + cand_val + cand_pos +
           cand_nrm + cand_base + cand_status + vt + pos + nrm + key + tris + rowcnt + rowstart + scan_status +
           jobctl;
  }
};

BufPlan plan_buffers(s2m_mesh *m, unsigned long long cand_cap, unsigned long long vcap, unsigned long long tcap) {
  const S2Job &j = m->job;
  const unsigned long long N = (unsigned long long)m->N;
  m->cand_cap = std::max<unsigned long long>(1024, std::min(cand_cap, N * N * N));
  m->vcap = std::max<unsigned long long>(1024, std::min(vcap, N * N * N));
  m->tcap = std::max<unsigned long long>(2048, tcap);
  m->cell_tiles = cell_word_tiles(m);
  m->vc_tiles = (m->cand_cap + S2_VC_TILE - 1) / S2_VC_TILE;
  m->slab_ctrl_words = size_t(m->D) + 1;
  m->scan_tiles = (N * N + S2_SCAN_TILE - 1) / S2_SCAN_TILE;
  m->quad_tiles = (m->vcap + S2_Q_TILE - 1) / S2_Q_TILE;
  BufPlan b{};
  b.ring = size_t(j.ring) * size_t(j.plane) * sizeof(float);
  b.slab_ctrl = m->slab_ctrl_words * 8;
  b.pt_bits = 3 * pt_bits_words(m) * 4;
  b.offx = size_t((j.N + 31) / 32) * 4;
  b.cell_words = m->cell_tiles * S2_CW_BLOCK * 4;
  b.tile_cnt = tile_cnt_words(m) * 4;
  const bool prune = m->sdf->k_tiles && m->nslabs > 0;
  b.prune = prune ? prune_layout(m) : 0;
  b.cand_key = m->cand_cap * 8;
  b.cand_val = m->cand_cap * 32;
  b.cand_pos = m->cand_cap * 12;
  b.cand_nrm = m->cand_cap * 12;
  b.cand_base = size_t(m->nslabs + 1) * 8;
  b.cand_status = vc_ctrl_words(m->vc_tiles) * 8;
  b.vt = 0;
  m->vt_tiles = 0;
  if (prune && m->prune_chunk >= m->nslabs && m->cand_cap < (1ull << 32)) {
    auto up16 = [](size_t x) { return (x + 15) / 16 * 16; };
    m->vt_tiles = m->slab_tile_base[size_t(m->nslabs)] - m->slab_tile_base[0];
    m->vt_blocks = unsigned((m->vt_tiles + S2_VT_TILE - 1) / S2_VT_TILE);
    m->vt_cnt_off = 16;
    m->vt_part_off = up16(m->vt_cnt_off + 4 * (size_t(m->vt_tiles) + 1));
    m->vt_poff_off = up16(m->vt_part_off + 4 * size_t(m->vt_blocks));
    m->vt_rank_off = up16(m->vt_poff_off + 8 * size_t(m->vt_blocks));
    m->vt_perm_off = up16(m->vt_rank_off + 8 * size_t(m->cand_cap));
    b.vt = m->vt_perm_off + 4 * size_t(m->cand_cap);
  }
  b.pos = m->vcap * 12;
  b.nrm = m->vcap * 12;
  b.key = m->vcap * 8;
  b.tris = m->tcap * 12;
  b.rowcnt = N * N * 4;
  b.rowstart = (N * N + 1) * 4;
  b.scan_status = scan_status_words(m->scan_tiles, m->quad_tiles) * 8;
  b.jobctl = 8 * 8;
  return b;
}

// Initial capacities of a job's candidate, vertex and triangle arrays (the
// pipeline regrows them to the exact totals when they overflow).
void initial_caps(const s2m_mesh *m, const s2m_params &p, unsigned long long &cand_cap, unsigned long long &vcap,
                  unsigned long long &tcap) {
  const unsigned long long N = (unsigned long long)m->N;
  const unsigned long long N3 = N * N * N;
  double sc = 0, sv = 0, st = 0;
  if (m->sdf) {
    std::lock_guard<std::mutex> lock(m->sdf->tune_mu);
    sc = m->sdf->seen_cand;
    sv = m->sdf->seen_vert;
    st = m->sdf->seen_tri;
  }
  const double n2 = double(N * N);
  auto learned = [&](double ratio) { return (unsigned long long)(ratio * n2 * m->zfrac * 1.1) + 4096; };
  cand_cap = std::min(N3, std::max<unsigned long long>({65536, 8 * N * N, learned(sc)}));
  vcap = p.max_vertices ? p.max_vertices
                        : std::min(N3, std::max<unsigned long long>({65536, 6 * N * N, learned(sv)}));
  tcap = p.max_triangles ? p.max_triangles
                         : std::max<unsigned long long>({131072, 2 * vcap + 4096, learned(st)});
  if (p.max_vertices) cand_cap = std::min(N3, std::max<unsigned long long>(1024, p.max_vertices));
}

// Remember the surface density of a finished job for the SDF's next jobs.
void learn_caps(const s2m_mesh *m) {
  const double n2 = double(m->N) * double(m->N) * m->zfrac;  // per N^2 of a whole job
  if (!m->sdf || n2 < 4096.0) return;  // tiny jobs say little about large ones
  std::lock_guard<std::mutex> lock(m->sdf->tune_mu);
  m->sdf->seen_cand = std::max(m->sdf->seen_cand, double(m->ncand) / n2);
  m->sdf->seen_vert = std::max(m->sdf->seen_vert, double(m->nverts) / n2);
  m->sdf->seen_tri = std::max(m->sdf->seen_tri, double(m->ntris) / n2);
}

// Host hook for failure tests: when S2M_TEST_FAIL_ALLOC=k is set, the k-th
// device allocation of the process (counting from 1) reports
// cudaErrorMemoryAllocation without allocating.
std::atomic<long long> g_alloc_count{0};
cudaError_t mesh_malloc(void **p, size_t bytes, cudaStream_t st) {
  static const long long fail_at = [] {
    const char *e = std::getenv("S2M_TEST_FAIL_ALLOC");
    return e ? std::atoll(e) : 0ll;
  }();
  if (fail_at > 0 && ++g_alloc_count == fail_at) {
    *p = nullptr;
    return cudaErrorMemoryAllocation;
  }
  return cudaMallocAsync(p, bytes, st);
}

int alloc_buffers(s2m_mesh *m, unsigned long long cand_cap, unsigned long long vcap, unsigned long long tcap,
                  char *err, size_t errlen) {
  drop_graph(m);
  free_buffers(m);
  const BufPlan b = plan_buffers(m, cand_cap, vcap, tcap);
  cudaStream_t st = m->stream;
  S2_CUDA(mesh_malloc((void **)&m->ring, b.ring, st));
  S2_CUDA(mesh_malloc((void **)&m->slab_ctrl, b.slab_ctrl, st));
  S2_CUDA(mesh_malloc((void **)&m->pt_bits, b.pt_bits, st));
  // the words' bits past the lattice edge are never written and must read 0
  S2_CUDA(cudaMemsetAsync(m->pt_bits, 0, b.pt_bits, st));
  S2_CUDA(mesh_malloc((void **)&m->offx, b.offx, st));
  S2_CUDA(mesh_malloc((void **)&m->cell_words, b.cell_words, st));
  S2_CUDA(mesh_malloc((void **)&m->tile_cnt, b.tile_cnt, st));
  if (b.prune) {
    S2_CUDA(mesh_malloc((void **)&m->prune_buf, b.prune, st));
    // pageable source: the call returns once the words are staged
    S2_CUDA(cudaMemcpyAsync(prune_bases(m), m->slab_tile_base.data(), m->slab_tile_base.size() * 8,
                            cudaMemcpyHostToDevice, st));
    S2_CUDA(cudaMemcpyAsync(prune_at<unsigned long long>(m, m->prune_cbase_off), m->slab_coarse_base.data(),
                            m->slab_coarse_base.size() * 8, cudaMemcpyHostToDevice, st));
  }
  S2_CUDA(mesh_malloc((void **)&m->cand_key, b.cand_key, st));
  S2_CUDA(mesh_malloc((void **)&m->cand_val, b.cand_val, st));
  S2_CUDA(mesh_malloc((void **)&m->cand_pos, b.cand_pos, st));
  S2_CUDA(mesh_malloc((void **)&m->cand_nrm, b.cand_nrm, st));
  S2_CUDA(mesh_malloc((void **)&m->cand_base, b.cand_base, st));
  S2_CUDA(mesh_malloc((void **)&m->cand_status, b.cand_status, st));
  if (b.vt) S2_CUDA(mesh_malloc((void **)&m->vt_buf, b.vt, st));
  S2_CUDA(mesh_malloc((void **)&m->pos, b.pos, st));
  S2_CUDA(mesh_malloc((void **)&m->nrm, b.nrm, st));
  S2_CUDA(mesh_malloc((void **)&m->key, b.key, st));
  S2_CUDA(mesh_malloc((void **)&m->tris, b.tris, st));
  S2_CUDA(mesh_malloc((void **)&m->rowcnt, b.rowcnt, st));
  S2_CUDA(mesh_malloc((void **)&m->rowstart, b.rowstart, st));
  S2_CUDA(mesh_malloc((void **)&m->scan_status, b.scan_status, st));
  S2_CUDA(mesh_malloc((void **)&m->jobctl, b.jobctl, st));
  m->h_read = take_pinned_slot();
  if (!m->h_read) {
    set_err(err, errlen, "pinned read-back slot");
    return S2M_E_OOM;
  }
  return S2M_OK;
}

// Two events per launch when profiling (created once, reused every run).
cudaError_t prof_mark(s2m_mesh *m, cudaStream_t st, int kind, double units, bool after) {
  if (!m->profile) return cudaSuccess;
  if (m->ev_used == m->ev.size()) {
    cudaEvent_t e;
    cudaError_t rc = cudaEventCreate(&e);
    if (rc != cudaSuccess) return rc;
    m->ev.push_back(e);
    m->ev_kind.push_back(0);
    m->ev_units.push_back(0);
  }
  if (!after) {
    m->ev_kind[m->ev_used] = kind;
    m->ev_units[m->ev_used] = units;
  }
  return cudaEventRecord(m->ev[m->ev_used++], st);
}

void prof_collect(s2m_mesh *m) {
  for (size_t i = 0; i + 1 < m->ev_used; i += 2) {
    float ms = 0;
    if (cudaEventElapsedTime(&ms, m->ev[i], m->ev[i + 1]) != cudaSuccess) continue;
    int k = m->ev_kind[i];
    m->prof.ms[k] += ms;
    m->prof.launches[k] += 1;
    if (k == 0) m->prof.eval_points += m->ev_units[i];
    if (k == 1) m->prof.cells += m->ev_units[i];
  }
  m->ev_used = 0;
}

#define S2_LAUNCH(kind, units, call)                                   \
  do {                                                                 \
    cudaError_t e_ = prof_mark(m, st, kind, double(units), false);     \
    if (e_ != cudaSuccess) return e_;                                  \
    if ((e_ = (call)) != cudaSuccess) return e_;                       \
    if ((e_ = prof_mark(m, st, kind, 0, true)) != cudaSuccess) return e_; \
    ++m->launches;                                                     \
  } while (0)

// The device view of a mesh's outputs and counters.
S2MeshDev mesh_dev(const s2m_mesh *m) {
  const JobCtl c = jobctl(m);
  S2MeshDev md;
  md.pos = m->pos;
  md.nrm = m->nrm;
  md.key = m->key;
  md.tris = m->tris;
  md.vcap = m->vcap;
  md.tcap = m->tcap;
  md.vtotal = c.vtotal;
  md.rowcnt = m->rowcnt;
  md.rowstart = m->rowstart;
  md.scan_status = m->scan_status;
  md.counters = c.counters;
  md.ntris = c.ntris;
  md.invalid = c.invalid;
  md.err = c.err;
  md.wait_ns = m->wait_ns;
  md.hold = 0;
  if (const char *h = std::getenv("S2M_TEST_HOLD")) md.hold = unsigned(std::strtoul(h, nullptr, 0));  // tests only
  md.zq = m->quads_from_z;
  return md;
}

cudaError_t enqueue(s2m_mesh *m, cudaStream_t st) {
  const S2Job &j = m->job;
  const JobCtl c = jobctl(m);
  const unsigned long long N = (unsigned long long)m->N;
  const int sms = device_sm_count();
  m->launches = 0;
  m->ev_used = 0;
  cudaError_t e;
  if ((e = cudaMemsetAsync(m->jobctl, 0, 8 * 8, st)) != cudaSuccess) return e;
  if ((e = cudaMemsetAsync(m->cand_base, 0, size_t(m->nslabs + 1) * 8, st)) != cudaSuccess) return e;
  if ((e = cudaMemsetAsync(m->cand_status, 0, vc_ctrl_offsets(m->vc_tiles) * 8, st)) != cudaSuccess) return e;
  if ((e = cudaMemsetAsync(m->rowcnt, 0, N * N * 4, st)) != cudaSuccess) return e;
  if ((e = cudaMemsetAsync(m->scan_status, 0, scan_status_words(m->scan_tiles, m->quad_tiles) * 8, st)) != cudaSuccess)
    return e;

  S2Cand cand;
  cand.key = m->cand_key;
  cand.val = m->cand_val;
  cand.pos = m->cand_pos;
  cand.nrm = m->cand_nrm;
  cand.cap = m->cand_cap;
  cand.base = m->cand_base;
  cand.status = nullptr;  // the per-job compaction is wait-free (s2m_vc_scan, s2m_vcompact)
  cand.tile_counter = nullptr;

  const S2MeshDev md = mesh_dev(m);

  const long long pts = (long long)j.P * j.P;
  const unsigned eval_blocks = unsigned((pts + S2_EVAL_BLOCK - 1) / S2_EVAL_BLOCK);
  int ev = m->sdf->eval_variant >= 0 ? m->sdf->eval_variant : 0;
  // without pruning buffers (the no-allocation entry point) the fastest plain variant
  if (kEvalVariants[ev].pruned && !m->prune_buf) ev = std::max(0, m->sdf->eval_variant_plain);
  const bool pruned = kEvalVariants[ev].pruned;
  const int run = kEvalVariants[ev].run;
  m->last_pruned = pruned;
  m->last_variant = ev;
  m->eval_points = 0;
  m->eval_fp_ops = m->eval_sfu_ops = 0;
  const bool tiles_ready = pruned && m->tiles_ready && m->prune_chunk >= m->nslabs;
  // one slab with the listed evaluation: the ring keeps the job's whole
  // lattice, so the candidates carry no corner values and the vertex kernel
  // reads them from the ring (decided tiles' points by their flags)
  const bool resident = pruned && kEvalVariants[ev].listed && !j.exact && !j.qef && m->nslabs == 1 && m->prune_buf;
  if (pruned && !tiles_ready) {  // operation counters and the slabs' list lengths
    cudaError_t e0 = cudaMemsetAsync(m->prune_buf, 0, m->prune_base_off, st);
    if (e0 != cudaSuccess) return e0;
  }
  // finished-block counter and plane counts of the classification (each slab's
  // last mark block leaves them zero for the next)
  if ((e = cudaMemsetAsync(cls_done(m), 0, (1 + size_t(m->D)) * 4, st)) != cudaSuccess) return e;
  S2_LAUNCH(1, 0, launch_pdl(s2m_offx, unsigned((N + 255) / 256), 256, 0, st, j, m->offx));
  const S2PointBits pb = point_bits(m);
  for (int s = 0; s < m->nslabs; ++s) {
    int zc0 = j.zb + s * m->D;
    int zc1 = std::min(j.zb + m->nzc, zc0 + m->D);
    int k0, nk;
    slab_planes(m, s, k0, nk);
    S2Job jj = j;
    float *ring = m->ring;
    m->eval_points += double(pts) * nk;
    if (pruned) {
      const int cb = s - s % m->prune_chunk;
      if (s == cb && !tiles_ready) S2_LAUNCH(0, 0, launch_tiles(m, cb, std::min(m->nslabs, cb + m->prune_chunk), st));
      S2_LAUNCH(0, double(pts) * nk, launch_evalp(m, ev, s, cb, st));
    } else {
      void *eargs[] = {&jj, &ring, &k0, &nk};
      dim3 eg(eval_blocks, unsigned((nk + run - 1) / run));
      S2_LAUNCH(0, double(pts) * nk, launch_pdl(m->sdf->k_eval[ev], eg, dim3(S2_EVAL_BLOCK), 0, st, eargs));
    }
    unsigned long long ncells = (unsigned long long)(zc1 - zc0) * N * N;
    if (!pruned)  // the pruned evaluation writes the point bits of its planes itself
      S2_LAUNCH(1, 0, launch_pdl(s2m_cells_bits, dim3(unsigned((j.P + 7) / 8), unsigned(nk)), 256, 0, st, j, m->ring, pb, k0));
    const unsigned nbp = cell_tiles_per_plane(m);
    const unsigned ncp = unsigned(zc1 - zc0);
    const dim3 mg(nbp, (ncp + S2_MARK_PLANES - 1) / S2_MARK_PLANES), eg(nbp, (ncp + S2_EMIT_PLANES - 1) / S2_EMIT_PLANES);
    // the listed evaluation (but for S2M_JOB_EXACT_CORNERS) writes no point
    // bits of decided tiles but those of the slab's last plane: classification
    // by the slab's listed tiles and the tiles' flags
    const unsigned *tflags = nullptr;
    const int tzs = pruned ? prune_geom(j, nk).tzs : 1;
    if (kEvalVariants[ev].listed && !j.exact) {
      const int cb = s - s % m->prune_chunk;
      const unsigned long long ntx = (unsigned long long)((j.P + S2_PT_XY - 1) / S2_PT_XY);
      tflags = reinterpret_cast<const unsigned *>(
          prune_at<unsigned char>(m, m->prune_flags_off) +
          (m->slab_tile_base[size_t(s)] - m->slab_tile_base[size_t(cb)]) / ntx * size_t(4 * ((j.P + 31) / 32)));
      const unsigned *list = prune_at<unsigned>(m, m->prune_list_off) +
                             (m->slab_tile_base[size_t(s)] - m->slab_tile_base[size_t(cb)]);
      const unsigned *count = prune_list_counts(m) + s;
      const unsigned long long stiles = m->slab_tile_base[size_t(s) + 1] - m->slab_tile_base[size_t(s)];
      const unsigned mt_grid = unsigned(std::max<unsigned long long>(
          1, std::min<unsigned long long>((stiles + S2_MT_BLOCK / 32 - 1) / (S2_MT_BLOCK / 32),
                                          (unsigned long long)sms * 4)));  // resident: 64 registers a thread
      S2_LAUNCH(1, ncells, launch_pdl(s2m_cells_mark_tiles, mt_grid, S2_MT_BLOCK, 0, st, j, pb, m->offx,
                                      m->cell_words, m->tile_cnt, cls_done(m), cls_plane_cnt(m), m->slab_ctrl,
                                      m->cand_base, s, zc0, zc1, tflags, k0, tzs, list, count));
    } else {
      S2_LAUNCH(1, ncells, launch_pdl(s2m_cells_mark, mg, S2_CW_BLOCK, 0, st, j, pb, m->offx, m->cell_words,
                                      m->tile_cnt, cls_done(m), cls_plane_cnt(m), m->slab_ctrl, m->cand_base, s,
                                      zc0, zc1));
    }
    S2_LAUNCH(1, 0, launch_pdl(s2m_cells_emit, eg, S2_CW_BLOCK, 0, st, j, m->ring, pruned ? pb.unk : nullptr,
                               m->cell_words, m->slab_ctrl, m->tile_cnt, cand, c.err, zc0, tflags, k0, tzs,
                               int(ncp), resident ? 0 : 1));
  }
  S2Job jj = j;
  int nslabs = m->nslabs;
  // the lattice evaluation's tile bits, when every slab's are still resident
  const unsigned *tbits = (pruned && m->prune_chunk >= m->nslabs && !j.qef) ? prune_at<unsigned>(m, m->prune_bits_off)
                                                                             : nullptr;
  const unsigned long long *tbase = m->prune_buf ? prune_at<unsigned long long>(m, m->prune_base_off) : nullptr;
  int D = m->D, nzc = m->nzc;
  const unsigned *perm = nullptr;
  if (tbits && m->vt_buf) {  // candidates grouped by tile for the vertex kernel
    unsigned *tcnt = reinterpret_cast<unsigned *>(m->vt_buf + m->vt_cnt_off);
    unsigned *part = reinterpret_cast<unsigned *>(m->vt_buf + m->vt_part_off);
    unsigned long long *pbase = reinterpret_cast<unsigned long long *>(m->vt_buf);
    unsigned long long *poff = reinterpret_cast<unsigned long long *>(m->vt_buf + m->vt_poff_off);
    unsigned long long *rank = reinterpret_cast<unsigned long long *>(m->vt_buf + m->vt_rank_off);
    unsigned *vperm = reinterpret_cast<unsigned *>(m->vt_buf + m->vt_perm_off);
    if ((e = cudaMemsetAsync(m->vt_buf, 0, m->vt_part_off, st)) != cudaSuccess) return e;
    const unsigned cgrid = unsigned(sms) * 8;
    S2_LAUNCH(2, 0, launch_pdl(s2m_vtile_count, cgrid, 256, 0, st, j, cand, nslabs, tbase, D, nzc, tcnt, rank));
    S2_LAUNCH(2, 0, launch_pdl(s2m_vtile_scan, m->vt_blocks, 256, 0, st, tcnt, m->vt_tiles, part, poff, pbase,
                                                                  tcnt + m->vt_tiles));
    S2_LAUNCH(2, 0, launch_pdl(s2m_vtile_scatter, cgrid, 256, 0, st, cand, nslabs, tcnt, poff, rank, vperm));
    perm = vperm;
  }
  unsigned long long *vc_base = m->cand_status;
  unsigned *vc_cnt = reinterpret_cast<unsigned *>(m->cand_status + 2);
  unsigned long long *vc_off = m->cand_status + vc_ctrl_offsets(m->vc_tiles);
  unsigned *vx_chunks = c.counters + 4;  // zeroed with jobctl at the start of the job
  const float *vring = resident ? m->ring : nullptr;
  const unsigned char *vflags = resident ? prune_at<unsigned char>(m, m->prune_flags_off) : nullptr;
  int vk0 = 0, vnk = 0;
  if (m->nslabs > 0) slab_planes(m, 0, vk0, vnk);
  int vtzs = resident ? prune_geom(j, vnk).tzs : 1;
  void *vargs[] = {&jj, &cand, &nslabs, &tbits, &tbase, &D, &nzc, &perm, &vc_cnt, &vx_chunks, &vring, &vflags, &vk0,
                   &vtzs};
  const cudaKernel_t kv = j.qef ? m->sdf->k_vertices_qef : m->sdf->k_vertices;
  if (m->sdf->prune_words > 0 && !j.qef)  // chunked form: one block per SM (S2_VX_BLOCK threads, 64 registers each)
    S2_LAUNCH(2, 0, launch_pdl(kv, dim3(unsigned(sms)), dim3(S2_VX_BLOCK), S2_VX_SMEM_BYTES, st, vargs));
  else
    S2_LAUNCH(2, 0, launch_pdl(kv, dim3(unsigned(sms) * 16), dim3(S2_VX_SMALL), 0, st, vargs));
  S2_LAUNCH(3, 0, launch_pdl(s2m_vc_scan, 1, 256, 0, st, cand, nslabs, vc_cnt, vc_off, vc_base, md));
  const unsigned vc_grid = unsigned(std::max<size_t>(1, std::min<size_t>(m->vc_tiles, size_t(sms) * 8)));
  S2_LAUNCH(3, 0, launch_pdl(s2m_vcompact, vc_grid, S2_VC_BLOCK, 0, st, j, cand, md, m->nslabs, vc_off));
  const unsigned scan_grid = unsigned(std::max<size_t>(1, std::min<size_t>(m->scan_tiles, size_t(sms) * 8)));
  S2_LAUNCH(4, 0, launch_pdl(s2m_rowscan, scan_grid, S2_SCAN_BLOCK, 0, st, md, N * N));
  const unsigned q_grid = unsigned(std::max<size_t>(1, std::min<size_t>(m->quad_tiles, size_t(sms) * 8)));
  unsigned long long *qoff = m->scan_status + m->scan_tiles;  // quad scan words (s2m_quads_find ..)
  unsigned *qcnt = reinterpret_cast<unsigned *>(qoff + m->quad_tiles);
  unsigned long long *qbase = qoff + m->quad_tiles + (m->quad_tiles + 1) / 2;
  unsigned *lk0 = reinterpret_cast<unsigned *>(m->cand_pos), *lk1 = reinterpret_cast<unsigned *>(m->cand_nrm);
  S2_LAUNCH(5, 0, launch_pdl(s2m_quads_find, q_grid, S2_Q_BLOCK, 0, st, j, md, lk0, lk1, qcnt));
  S2_LAUNCH(5, 0, launch_pdl(s2m_quads_scan, 1, 256, 0, st, md, qcnt, qoff, qbase));
  S2_LAUNCH(5, 0, launch_pdl(s2m_quads_write, q_grid, S2_Q_BLOCK, 0, st, md, lk0, lk1, qoff));
  return cudaSuccess;
}

// Deep slabs for full evaluation: a lattice point of a ring that no longer
// fits in L2 costs 8 more bytes of DRAM traffic (its value written by the
// evaluation, read back by the point-bit pass), about 0.0012 ns at 6.8 TB/s.
// An evaluation measured at 0.01 ns per point or more keeps that under 12 %,
// while the L2-sized ring would cost 4 launches and an evaluation tail per
// slab of a few planes (at 2048^3 the L2 rule gives one-plane slabs: 8192
// launches per job).
constexpr double kDeepSlabNsPerPoint = 0.01;

// Autotuner: time every evaluation variant of the module on the slabs at a
// quarter, a half and three quarters of the job (into the job's own ring,
// which the pipeline overwrites afterwards) and keep the fastest for this
// SDF.  A pruned variant is timed with its tile pass.  Runs once per SDF, on
// its first job.  (One window through the middle of a CSG scene is where
// pruning saves least; quartiles are closer to the whole job.)
int autotune_eval(s2m_mesh *m, cudaStream_t st, char *err, size_t errlen) {
  const s2m_sdf *sdf = m->sdf;
  std::lock_guard<std::mutex> lock(sdf->tune_mu);
  if (sdf->eval_variant >= 0) return S2M_OK;
  if (std::getenv("S2M_EVAL_VARIANT")) {
    int v = std::atoi(std::getenv("S2M_EVAL_VARIANT"));
    if (v < 0 || v >= kNumEvalVariants || !sdf->k_eval[v]) v = 0;
    sdf->eval_variant = v;
    sdf->eval_variant_plain = kEvalVariants[v].pruned ? 0 : v;
    return S2M_OK;
  }
  const S2Job &j = m->job;
  const long long pts = (long long)j.P * j.P;
  std::vector<int> trial;
  for (int q = 1; q <= 3 && m->nslabs > 0; ++q) {
    const int s = std::min(m->nslabs - 1, m->nslabs * q / 4);
    if (trial.empty() || trial.back() != s) trial.push_back(s);
  }
  double trial_pts = 0;
  for (int s : trial) {
    int k0, nk;
    slab_planes(m, s, k0, nk);
    trial_pts += double(pts) * nk;
  }
  // small jobs: too little work per launch to rank the variants; keep the default
  if (trial_pts < 6.0e6) {
    sdf->eval_variant = 0;
    sdf->eval_variant_plain = 0;
    return S2M_OK;
  }
  cudaEvent_t a, b;
  S2_CUDA(cudaEventCreate(&a));
  S2_CUDA(cudaEventCreate(&b));
  const unsigned eval_blocks = unsigned((pts + S2_EVAL_BLOCK - 1) / S2_EVAL_BLOCK);
  double best = 1e300, best_plain = 1e300;
  int best_v = 0, best_plain_v = 0;
  for (int v = 0; v < kNumEvalVariants; ++v) {
    if (!sdf->k_eval[v] || (kEvalVariants[v].pruned && !m->prune_buf)) {
      sdf->tune_ns[v] = 0;
      continue;
    }
    float ms_best = 1e30f;
    for (int rep = 0; rep < 3; ++rep) {
      if (kEvalVariants[v].pruned) S2_CUDA(cudaMemsetAsync(m->prune_buf, 0, m->prune_base_off, st));
      S2_CUDA(cudaEventRecord(a, st));
      for (int s : trial) {
        if (kEvalVariants[v].pruned) {
          S2_CUDA(launch_tiles(m, s, s + 1, st));
          S2_CUDA(launch_evalp(m, v, s, s, st));
        } else {
          S2Job jj = j;
          float *ring = m->ring;
          int k0, nk;
          slab_planes(m, s, k0, nk);
          void *args[] = {&jj, &ring, &k0, &nk};
          dim3 eg(eval_blocks, unsigned((nk + kEvalVariants[v].run - 1) / kEvalVariants[v].run));
          S2_CUDA(cudaLaunchKernel((const void *)sdf->k_eval[v], eg, dim3(S2_EVAL_BLOCK), args, 0, st));
        }
      }
      S2_CUDA(cudaEventRecord(b, st));
      S2_CUDA(cudaEventSynchronize(b));
      float ms = 0;
      S2_CUDA(cudaEventElapsedTime(&ms, a, b));
      if (rep > 0) ms_best = std::min(ms_best, ms);
    }
    double ns = double(ms_best) * 1e6 / trial_pts;
    sdf->tune_ns[v] = ns;
    cudaFuncAttributes fa;
    if (cudaFuncGetAttributes(&fa, (const void *)sdf->k_eval[v]) == cudaSuccess) {
      sdf->tune_regs[v] = fa.numRegs;
      sdf->tune_local[v] = int(fa.localSizeBytes);
    } else {
      cudaGetLastError();
    }
    if (ns < best) {
      best = ns;
      best_v = v;
    }
    if (!kEvalVariants[v].pruned && ns < best_plain) {
      best_plain = ns;
      best_plain_v = v;
    }
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  sdf->eval_variant = best_v;
  sdf->eval_variant_plain = best_plain_v;
  sdf->deep_slabs = !kEvalVariants[best_v].pruned && best >= kDeepSlabNsPerPoint;
  return S2M_OK;
}

int readback(s2m_mesh *m, cudaStream_t st, char *err, size_t errlen) {
  S2_CUDA(cudaMemcpyAsync(m->h_read, m->jobctl, 4 * 8, cudaMemcpyDeviceToHost, st));
  S2_CUDA(cudaMemcpyAsync(m->h_read + 4, m->cand_base + m->nslabs, 8, cudaMemcpyDeviceToHost, st));
  if (m->last_pruned) S2_CUDA(cudaMemcpyAsync(m->h_read + 5, m->prune_buf, 16, cudaMemcpyDeviceToHost, st));
  S2_CUDA(cudaStreamSynchronize(st));
  prof_collect(m);
  if (m->last_pruned) {
    m->eval_fp_ops = double(m->h_read[5]);
    m->eval_sfu_ops = double(m->h_read[6]);
  } else {
    const bool run = kEvalVariants[m->last_variant].vec;
    const double fp = run && m->sdf->run_fp32_ops > 0 ? m->sdf->run_fp32_ops : m->sdf->fp32_ops;
    const double sfu = run && m->sdf->run_fp32_ops > 0 ? m->sdf->run_sfu_ops : m->sdf->sfu_ops;
    m->eval_fp_ops = fp * m->eval_points;
    m->eval_sfu_ops = sfu * m->eval_points;
  }
  m->ntris = m->h_read[0];
  m->invalid = m->h_read[1];
  m->nverts = m->h_read[2];
  m->errflags = unsigned(m->h_read[3] & 0xffffffffull);
  m->ncand = m->h_read[4];
  return S2M_OK;
}

}  // namespace

namespace s2m {
// Device bytes that s2m_mesh_create allocates for this job at its first
// attempt: the same job setup (resolution rounding, slab depth, tile
// layout) and the same buffer plan, without allocating.  0 for a job that
// setup rejects.  Used by the server's admission (batch.cu).
uint64_t mesh_job_footprint(const s2m_sdf *sdf, const s2m_params &params) {
  s2m_mesh m;
  m.sdf = sdf;
  m.params = params;
  if (!(m.params.eps > 0.0f)) m.params.eps = 1e-4f;
  if (setup_job(&m, nullptr, 0) != S2M_OK) return 0;
  unsigned long long cand_cap, vcap, tcap;
  initial_caps(&m, m.params, cand_cap, vcap, tcap);
  return uint64_t(plan_buffers(&m, cand_cap, vcap, tcap).total());
}
}  // namespace s2m

// ===========================================================================
// Meshing without device allocation: the pipeline's scratch in one fixed
// array.  In host code `s2m_noalloc_scratch` names a host-side stand-in, not
// device memory, so its device address is looked up once per device and
// passed to the kernels as a pointer.

static __device__ __align__(256) unsigned char s2m_noalloc_scratch[S2M_NOALLOC_SCRATCH_BYTES];

namespace {

constexpr int kNoallocMaxDevices = 64;
std::mutex g_noalloc_mu;
unsigned char *g_noalloc_ptr[kNoallocMaxDevices] = {};

int noalloc_scratch(unsigned char **ptr, char *err, size_t errlen) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    set_err(err, errlen, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    return S2M_E_NO_DEVICE;
  }
  if (dev < 0 || dev >= kNoallocMaxDevices) {
    set_err(err, errlen, "device ordinal beyond the no-allocation table");
    return S2M_E_INVALID;
  }
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (!g_noalloc_ptr[dev]) {
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, s2m_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      set_err(err, errlen, std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(e));
      return S2M_E_CUDA;
    }
    g_noalloc_ptr[dev] = static_cast<unsigned char *>(p);
  }
  *ptr = g_noalloc_ptr[dev];
  return S2M_OK;
}

// Carve `bytes` (rounded up to 256) off the scratch; false when it is full.
template <class T> bool carve(unsigned char *base, size_t &used, size_t count, T **out) {
  size_t bytes = (count * sizeof(T) + 255) / 256 * 256;
  if (used + bytes > size_t(S2M_NOALLOC_SCRATCH_BYTES)) return false;
  *out = reinterpret_cast<T *>(base + used);
  used += bytes;
  return true;
}

// ---------------------------------------------------------------------------
// Pinned host arrays of s2m_mesh_generate, kept for reuse: pinning hundreds of
// MB costs tens of ms, the copy into them well under one.  Blocks are mapped
// into the device's address space (the z parts' copy kernels store into
// them).  At most kHostPoolKeep bytes stay pooled.
struct HostBlock {
  void *p = nullptr;
  size_t bytes = 0;
};
std::mutex g_host_mu;
std::vector<HostBlock> g_host_free;
size_t g_host_free_bytes = 0;
constexpr size_t kHostPoolKeep = size_t(16) << 30;

HostBlock take_host_block(size_t bytes) {
  bytes = std::max<size_t>(bytes, 4096);
  {
    std::lock_guard<std::mutex> lock(g_host_mu);
    int best = -1;
    for (size_t i = 0; i < g_host_free.size(); ++i)
      if (g_host_free[i].bytes >= bytes && g_host_free[i].bytes <= 4 * bytes &&
          (best < 0 || g_host_free[i].bytes < g_host_free[size_t(best)].bytes))
        best = int(i);
    if (best >= 0) {
      HostBlock b = g_host_free[size_t(best)];
      g_host_free.erase(g_host_free.begin() + best);
      g_host_free_bytes -= b.bytes;
      return b;
    }
  }
  HostBlock b;
  b.bytes = bytes + bytes / 4;  // room for the next job's slightly larger mesh
  if (cudaHostAlloc(&b.p, b.bytes, cudaHostAllocMapped | cudaHostAllocPortable) != cudaSuccess) {
    cudaGetLastError();
    b.p = nullptr;
    b.bytes = 0;
  }
  return b;
}

void give_host_block(HostBlock b) {
  if (!b.p) return;
  std::vector<void *> drop;
  {
    std::lock_guard<std::mutex> lock(g_host_mu);
    g_host_free.push_back(b);
    g_host_free_bytes += b.bytes;
    while (g_host_free_bytes > kHostPoolKeep && !g_host_free.empty()) {  // drop the oldest
      drop.push_back(g_host_free.front().p);
      g_host_free_bytes -= g_host_free.front().bytes;
      g_host_free.erase(g_host_free.begin());
    }
  }
  for (void *p : drop) cudaFreeHost(p);
}

struct HostMeshOwner {
  HostBlock pos, nrm, tris;
};

// Device pointer of a mapped pinned block.
template <class T> T *mapped(const HostBlock &b) {
  void *d = nullptr;
  return cudaHostGetDevicePointer(&d, b.p, 0) == cudaSuccess ? static_cast<T *>(d) : nullptr;
}

// The stream the later z parts' tile passes run on (one per device).
cudaStream_t tile_stream() {
  static std::mutex mu;
  static cudaStream_t streams[kNoallocMaxDevices] = {};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kNoallocMaxDevices) return nullptr;
  std::lock_guard<std::mutex> lock(mu);
  if (!streams[dev] && cudaStreamCreateWithFlags(&streams[dev], cudaStreamNonBlocking) != cudaSuccess)
    streams[dev] = nullptr;
  return streams[dev];
}

// The side stream the z parts' host copies run on (one per device).  (Three
// streams, one per array, moved nothing faster: device-to-host copies into
// pinned memory top out near 190 GB/s here, by one copy engine, several, or
// SM stores into mapped memory alike.)
cudaStream_t copy_stream() {
  static std::mutex mu;
  static cudaStream_t streams[kNoallocMaxDevices] = {};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kNoallocMaxDevices) return nullptr;
  std::lock_guard<std::mutex> lock(mu);
  if (!streams[dev] && cudaStreamCreateWithFlags(&streams[dev], cudaStreamNonBlocking) != cudaSuccess)
    streams[dev] = nullptr;
  return streams[dev];
}

}  // namespace

// ===========================================================================
// C ABI

extern "C" {

int s2m_abi_version(void) { return S2M_ABI_VERSION; }

const char *s2m_status_string(int s) {
  switch (s) {
    case S2M_OK: return "ok";
    case S2M_E_INVALID: return "invalid argument";
    case S2M_E_IO: return "i/o error";
    case S2M_E_PARSE: return "parse error";
    case S2M_E_MISSING_SDF: return "missing sdf function";
    case S2M_E_NVRTC: return "NVRTC compile error";
    case S2M_E_CUDA: return "CUDA error";
    case S2M_E_OOM: return "out of device memory";
    case S2M_E_OVERFLOW: return "mesh too large";
    case S2M_E_TIMEOUT: return "device wait timed out";
    case S2M_E_NO_DEVICE: return "no CUDA device";
  }
  return "unknown status";
}

void s2m_free_string(char *s) { std::free(s); }

int s2m_preprocess_file(const char *path, char **out, char *err, size_t errlen) {
  if (!path || !out) return S2M_E_INVALID;
  std::string text, e;
  if (!s2m::preprocess_sdf3d_file(path, text, e, nullptr)) {
    set_err(err, errlen, e);
    return S2M_E_IO;
  }
  *out = dup_string(text);
  return S2M_OK;
}

int s2m_preprocess_source(const char *source, const char *base_dir, char **out, char *err, size_t errlen) {
  if (!source || !out) {
    set_err(err, errlen, "null argument");
    return S2M_E_INVALID;
  }
  *out = dup_string(s2m::preprocess_sdf3d_text(source, "", base_dir ? base_dir : "", nullptr));
  return S2M_OK;
}

int s2m_csg_from_source(const char *source, float *program, uint32_t capacity, uint32_t *len, char *err,
                        size_t errlen) {
  if (!source || !len) {
    set_err(err, errlen, "null argument");
    return S2M_E_INVALID;
  }
  std::vector<float> prog;
  std::string why;
  const std::string pre = s2m::preprocess_sdf3d_text(source, "", "", nullptr);
  if (!s2m::csg_from_source(pre, prog, why)) {
    set_err(err, errlen, why);
    return S2M_E_PARSE;
  }
  *len = uint32_t(prog.size());
  if (program && capacity >= prog.size()) std::memcpy(program, prog.data(), prog.size() * sizeof(float));
  else if (program) {
    set_err(err, errlen, "program needs " + std::to_string(prog.size()) + " floats");
    return S2M_E_OVERFLOW;
  }
  return S2M_OK;
}

int s2m_translate(const char *source, int lang, const char *sdf_name, char **out, double *fp32_ops,
                  double *sfu_ops, char *err, size_t errlen) {
  if (!source) return S2M_E_INVALID;
  const std::string text = lang == S2M_LANG_SHADERTOY ? s2m::shadertoy_wrap(source) : std::string(source);
  s2m::FrontendResult r = s2m::translate(text, lang == S2M_LANG_WGSL ? s2m::Lang::WGSL : s2m::Lang::GLSL,
                                         sdf_name ? sdf_name : "sdf");
  if (!r.ok) {
    set_err(err, errlen, r.error);
    return r.status ? r.status : S2M_E_PARSE;
  }
  if (out) *out = dup_string(r.cuda);
  if (fp32_ops) *fp32_ops = r.fp32_ops;
  if (sfu_ops) *sfu_ops = r.sfu_ops;
  return S2M_OK;
}

int s2m_compile(const char *source, int lang, const char *sdf_name, uint32_t compile_flags, s2m_sdf **out,
                char *err, size_t errlen) {
  if (!source || !out) return S2M_E_INVALID;
  *out = nullptr;
  const std::string text = lang == S2M_LANG_SHADERTOY ? s2m::shadertoy_wrap(source) : std::string(source);
  s2m::FrontendResult r = s2m::translate(text, lang == S2M_LANG_WGSL ? s2m::Lang::WGSL : s2m::Lang::GLSL,
                                         sdf_name ? sdf_name : "sdf");
  if (!r.ok) {
    set_err(err, errlen, r.error);
    return r.status ? r.status : S2M_E_PARSE;
  }
  s2m_sdf *s = new s2m_sdf();
  s->user_cuda = r.cuda;
  s->fp32_ops = r.fp32_ops;
  s->sfu_ops = r.sfu_ops;
  s->run_fp32_ops = r.run_fp32_ops;
  s->run_sfu_ops = r.run_sfu_ops;
  s->prune_words = r.prune_words;
  s->prune_combinators = r.prune_combinators;
  s->flags = compile_flags;
  int rc = compile_module(s, err, errlen);
  if (rc != S2M_OK) {
    delete s;
    return rc;
  }
  *out = s;
  return S2M_OK;
}

int s2m_compile_file(const char *path, int lang, const char *sdf_name, uint32_t compile_flags, s2m_sdf **out,
                     char *err, size_t errlen) {
  if (!path || !out) return S2M_E_INVALID;
  std::string text;
  if (lang != S2M_LANG_WGSL) {
    std::ifstream f(path, std::ios::binary);
    if (!f) {
      set_err(err, errlen, std::string("could not read ") + path);
      return S2M_E_IO;
    }
    std::ostringstream ss;
    ss << f.rdbuf();
    text = ss.str();
  } else {
    std::string e;
    if (!s2m::preprocess_sdf3d_file(path, text, e, nullptr)) {
      set_err(err, errlen, e);
      return S2M_E_IO;
    }
  }
  return s2m_compile(text.c_str(), lang, sdf_name, compile_flags, out, err, errlen);
}

const char *s2m_sdf_cuda_source(const s2m_sdf *sdf) { return sdf ? sdf->user_cuda.c_str() : nullptr; }

int s2m_sdf_compile_info(const s2m_sdf *sdf, double *seconds, int *programs, int *cache_hits) {
  if (!sdf) return S2M_E_INVALID;
  if (seconds) *seconds = sdf->compile_s;
  if (programs) *programs = sdf->programs;
  if (cache_hits) *cache_hits = sdf->cache_hits;
  return S2M_OK;
}

int s2m_sdf_run_op_counts(const s2m_sdf *sdf, double *fp32_ops, double *sfu_ops) {
  if (!sdf) return S2M_E_INVALID;
  if (fp32_ops) *fp32_ops = sdf->run_fp32_ops;
  if (sfu_ops) *sfu_ops = sdf->run_sfu_ops;
  return sdf->run_fp32_ops > 0 ? S2M_OK : S2M_E_INVALID;
}

int s2m_sdf_eval_variant(const s2m_sdf *sdf, char *name, size_t namelen, double *ns_per_point) {
  if (!sdf) return S2M_E_INVALID;
  int v = sdf->eval_variant;
  if (name && namelen) set_err(name, namelen, v >= 0 ? kEvalVariants[v].name : "untuned");
  if (ns_per_point)
    for (int i = 0; i < kNumEvalVariants; ++i) ns_per_point[i] = sdf->tune_ns[i];
  return v;
}

int s2m_sdf_set_eval_variant(s2m_sdf *sdf, int variant) {
  if (!sdf || variant < 0 || variant >= kNumEvalVariants || !sdf->k_eval[variant]) return S2M_E_INVALID;
  std::lock_guard<std::mutex> lock(sdf->tune_mu);
  sdf->eval_variant = variant;
  if (!kEvalVariants[variant].pruned) sdf->eval_variant_plain = variant;
  else if (sdf->eval_variant_plain < 0) sdf->eval_variant_plain = 0;
  return S2M_OK;
}

int s2m_sdf_eval_variant_info(const s2m_sdf *sdf, int variant, char *name, size_t namelen, int *registers,
                              int *local_bytes) {
  if (!sdf || variant < 0 || variant >= kNumEvalVariants) return S2M_E_INVALID;
  if (name && namelen) set_err(name, namelen, kEvalVariants[variant].name);
  if (registers) *registers = sdf->tune_regs[variant];
  if (local_bytes) *local_bytes = sdf->tune_local[variant];
  return S2M_OK;
}

int s2m_sdf_prune_info(const s2m_sdf *sdf, int *combinators, int *words) {
  if (!sdf) return S2M_E_INVALID;
  const bool on = sdf->k_tiles != nullptr;
  if (combinators) *combinators = on ? sdf->prune_combinators : 0;
  if (words) *words = on ? sdf->prune_words : 0;
  return S2M_OK;
}

int s2m_mesh_eval_ops(const s2m_mesh *m, double *points, double *fp32_ops, double *sfu_ops) {
  if (!m) return S2M_E_INVALID;
  if (points) *points = m->eval_points;
  if (fp32_ops) *fp32_ops = m->eval_fp_ops;
  if (sfu_ops) *sfu_ops = m->eval_sfu_ops;
  return m->last_pruned ? 1 : 0;
}

int s2m_sdf_op_counts(const s2m_sdf *sdf, double *fp32_ops, double *sfu_ops) {
  if (!sdf) return S2M_E_INVALID;
  if (fp32_ops) *fp32_ops = sdf->fp32_ops;
  if (sfu_ops) *sfu_ops = sdf->sfu_ops;
  return S2M_OK;
}

void s2m_sdf_free(s2m_sdf *sdf) {
  if (!sdf) return;
  for (cudaLibrary_t l : sdf->libs)
    if (l) cudaLibraryUnload(l);
  if (sdf->qef_lib) cudaLibraryUnload(sdf->qef_lib);
  delete sdf;
}

int s2m_wgsl_remove_function(const char *wgsl, const char *fn, char **out) {
  if (!wgsl || !fn || !out) return S2M_E_INVALID;
  std::string r;
  bool found = s2m::wgsl_remove_function(wgsl, fn, r);
  *out = found ? dup_string(r) : nullptr;
  return found ? S2M_OK : S2M_E_MISSING_SDF;
}

int s2m_wgsl_rename_function(const char *wgsl, const char *old_name, const char *new_name, char **out) {
  if (!wgsl || !old_name || !new_name || !out) return S2M_E_INVALID;
  std::string r;
  bool found = s2m::wgsl_rename_function(wgsl, old_name, new_name, r);
  *out = found ? dup_string(r) : nullptr;
  return found ? S2M_OK : S2M_E_MISSING_SDF;
}

int s2m_wgsl_has_function(const char *wgsl, const char *fn) {
  if (!wgsl || !fn) return 0;
  return s2m::wgsl_has_function(wgsl, fn) ? 1 : 0;
}

int s2m_mesh_run_async(s2m_mesh *m, void *stream) {
  if (!m || !m->sdf) return S2M_E_INVALID;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (m->use_graph && !m->profile) {
    // capture the launch sequence once, on a private stream (the legacy
    // default stream cannot be captured), then replay it on the caller's
    // stream: one launch call instead of one per kernel and memset
    if (!m->graph) {
      if (!m->capture_stream && cudaStreamCreateWithFlags(&m->capture_stream, cudaStreamNonBlocking) != cudaSuccess)
        return S2M_E_CUDA;
      cudaGraph_t g = nullptr;
      cudaError_t e = cudaStreamBeginCapture(m->capture_stream, cudaStreamCaptureModeThreadLocal);
      if (e == cudaSuccess) {
        cudaError_t e2 = enqueue(m, m->capture_stream);
        e = cudaStreamEndCapture(m->capture_stream, &g);
        if (e2 != cudaSuccess) e = e2;
      }
      if (e == cudaSuccess) e = cudaGraphInstantiate(&m->graph, g, 0);
      if (g) cudaGraphDestroy(g);
      if (e != cudaSuccess) {
        cudaGetLastError();
        m->graph = nullptr;
        return S2M_E_CUDA;
      }
    }
    return cudaGraphLaunch(m->graph, st) == cudaSuccess ? S2M_OK : S2M_E_CUDA;
  }
  cudaError_t e = enqueue(m, st);
  if (e != cudaSuccess) return e == cudaErrorMemoryAllocation ? S2M_E_OOM : S2M_E_CUDA;
  return S2M_OK;
}

int s2m_mesh_sync(s2m_mesh *m, void *stream, char *err, size_t errlen) {
  if (!m) return S2M_E_INVALID;
  int rc = readback(m, static_cast<cudaStream_t>(stream), err, errlen);
  if (rc != S2M_OK) return rc;
  if (m->errflags & S2_ERR_LOOKBACK) {
    set_err(err, errlen, "a device-side look-back wait hit its limit");
    return S2M_E_TIMEOUT;
  }
  if (m->errflags & S2_ERR_INDEX_OVF) {
    set_err(err, errlen, "more than 2^32 - 2 vertices");
    return S2M_E_OVERFLOW;
  }
  if (m->errflags & (S2_ERR_CAND_OVF | S2_ERR_VERT_OVF | S2_ERR_TRI_OVF)) {
    set_err(err, errlen, "mesh buffers overflowed");
    return S2M_E_OVERFLOW;
  }
  return S2M_OK;
}

int s2m_mesh_create(const s2m_sdf *sdf, const s2m_params *params, void *stream, s2m_mesh **out, char *err,
                    size_t errlen) {
  if (!sdf || !params || !out) return S2M_E_INVALID;
  *out = nullptr;
  using clk = std::chrono::steady_clock;
  auto t = clk::now();
  auto lap = [&t]() {
    const auto now = clk::now();
    const double ms = std::chrono::duration<double, std::milli>(now - t).count();
    t = now;
    return ms;
  };
  s2m_mesh *m = new s2m_mesh();
  m->sdf = sdf;
  m->stream = static_cast<cudaStream_t>(stream);
  m->params = *params;
  static std::once_flag pool_once;
  std::call_once(pool_once, [] {
    // freed mesh buffers stay in the stream-ordered pool for the next job
    int dev = 0;
    cudaMemPool_t pool;
    if (cudaGetDevice(&dev) == cudaSuccess && cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
      uint64_t keep = ~0ull;
      cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
  });
  if (!(m->params.eps > 0.0f)) m->params.eps = 1e-4f;
  int rc = setup_job(m, err, errlen);
  if (rc == S2M_OK && m->job.qef) rc = ensure_qef_module(sdf, err, errlen);
  if (rc != S2M_OK) {
    delete m;
    return rc;
  }
  const unsigned long long N = (unsigned long long)m->N;
  const unsigned long long N3 = N * N * N;
  unsigned long long cand_cap, vcap, tcap;
  initial_caps(m, *params, cand_cap, vcap, tcap);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  for (int attempt = 0; attempt < 5; ++attempt) {
    rc = alloc_buffers(m, cand_cap, vcap, tcap, err, errlen);
    if (rc != S2M_OK) break;
    if (m->sdf->eval_variant < 0) {
      if ((rc = autotune_eval(m, st, err, errlen)) != S2M_OK) break;
      const int d0 = m->D;
      if (!params->slab_depth && setup_job(m, err, errlen) == S2M_OK && m->D != d0 &&
          (rc = alloc_buffers(m, cand_cap, vcap, tcap, err, errlen)) != S2M_OK)
        break;  // the tuned slab depth needs a ring of another size
    }
    m->t_setup += lap();
    cudaError_t e = enqueue(m, st);
    m->t_launch += lap();
    ++m->runs;
    if (e != cudaSuccess) {
      set_err(err, errlen, std::string("launch: ") + cudaGetErrorString(e));
      rc = S2M_E_CUDA;
      break;
    }
    rc = readback(m, st, err, errlen);
    m->t_wait += lap();
    if (rc != S2M_OK) break;
    if (m->errflags & S2_ERR_LOOKBACK) {
      set_err(err, errlen, "a device-side look-back wait hit its limit");
      rc = S2M_E_TIMEOUT;
      break;
    }
    if (m->errflags & S2_ERR_INDEX_OVF) {
      set_err(err, errlen, "more than 2^32 - 2 vertices");
      rc = S2M_E_OVERFLOW;
      break;
    }
    if (!(m->errflags & (S2_ERR_CAND_OVF | S2_ERR_VERT_OVF | S2_ERR_TRI_OVF))) {
      rc = S2M_OK;
      break;
    }
    // The totals of the stage that overflowed are exact (offsets are counted
    // even where the writes were dropped): grow to them and run again.
    if (m->errflags & S2_ERR_CAND_OVF) {
      cand_cap = std::min<unsigned long long>(N3, m->ncand + m->ncand / 16 + 4096);
      vcap = std::max(vcap, cand_cap);
    } else if (m->errflags & S2_ERR_VERT_OVF) {
      vcap = std::min<unsigned long long>(N3, m->nverts + m->nverts / 16 + 4096);
    }
    if (m->errflags & S2_ERR_TRI_OVF) tcap = m->ntris + m->ntris / 16 + 4096;
    tcap = std::max(tcap, 2 * vcap + 4096);
    rc = S2M_E_OVERFLOW;
    set_err(err, errlen, "mesh buffers overflowed after resizing");
  }
  if (rc != S2M_OK) {
    free_buffers(m);
    delete m;
    return rc;
  }
  learn_caps(m);
  *out = m;
  return S2M_OK;
}

int s2m_mesh_noalloc(const s2m_sdf *sdf, const s2m_params *params, s2m_noalloc_mesh *out, void *stream,
                     char *err, size_t errlen) {
  if (!sdf || !params || !out || !out->pos || !out->nrm || !out->cell || !out->tris) {
    set_err(err, errlen, "null argument");
    return S2M_E_INVALID;
  }
  s2m_mesh m;  // host bookkeeping only; every device pointer below is scratch or the caller's
  m.sdf = sdf;
  m.params = *params;
  if (!(m.params.eps > 0.0f)) m.params.eps = 1e-4f;
  // Slabs of at most 8 cell slices keep the lattice ring small.
  if (m.params.slab_depth == 0 || m.params.slab_depth > 8) m.params.slab_depth = 8;
  int rc = setup_job(&m, err, errlen);
  if (rc != S2M_OK) return rc;
  if (uint32_t(m.N) > S2M_NOALLOC_MAX_RESOLUTION) {
    set_err(err, errlen, "resolution " + std::to_string(m.N) + " exceeds the no-allocation limit of " +
                             std::to_string(S2M_NOALLOC_MAX_RESOLUTION));
    return S2M_E_INVALID;
  }
  out->resolution = uint32_t(m.N);
  if (m.job.qef && !sdf->k_vertices_qef) {
    set_err(err, errlen, "precision mode needs the SDF's QEF module, which loading allocates: run one "
                         "s2m_mesh_create with S2M_JOB_QEF for this SDF first");
    return S2M_E_INVALID;
  }
  unsigned char *base = nullptr;
  rc = noalloc_scratch(&base, err, errlen);
  if (rc != S2M_OK) return rc;

  const S2Job &j = m.job;
  const unsigned long long N = (unsigned long long)m.N;
  m.cell_tiles = cell_word_tiles(&m);
  m.slab_ctrl_words = size_t(m.D) + 1;
  m.scan_tiles = (N * N + S2_SCAN_TILE - 1) / S2_SCAN_TILE;
  size_t used = 0;
  bool ok = carve(base, used, size_t(j.ring) * size_t(j.plane), &m.ring) &&
            carve(base, used, m.slab_ctrl_words, &m.slab_ctrl) &&
            carve(base, used, 3 * pt_bits_words(&m), &m.pt_bits) && carve(base, used, size_t((N + 31) / 32), &m.offx) &&
            carve(base, used, m.cell_tiles * S2_CW_BLOCK, &m.cell_words) && carve(base, used, tile_cnt_words(&m), &m.tile_cnt) &&
            carve(base, used, size_t(m.nslabs + 1), &m.cand_base) &&
            carve(base, used, size_t(N * N), &m.rowcnt) && carve(base, used, size_t(N * N + 1), &m.rowstart) &&
            carve(base, used, size_t(8), &m.jobctl);
  if (!ok) {
    set_err(err, errlen, "no-allocation scratch too small for this job");
    return S2M_E_INVALID;
  }
  // The rest holds the candidate list and its scan words: 64 bytes per
  // candidate plus 12 bytes of compaction counts and offsets per S2_VC_TILE
  // candidates and 12 bytes of quad tile offset and count per S2_Q_TILE
  // vertices (vertices never outnumber candidates).
  size_t left = size_t(S2M_NOALLOC_SCRATCH_BYTES) - used;
  const double per_cand = 64.0 + 12.0 / S2_VC_TILE + 12.0 / S2_Q_TILE;
  unsigned long long cap =
      (unsigned long long)((double(left) - 10 * 256.0 - 8.0 * double(m.scan_tiles) - 64.0) / per_cand);
  cap = cap / 1024 * 1024;
  m.cand_cap = cap;
  m.vc_tiles = (cap + S2_VC_TILE - 1) / S2_VC_TILE;
  m.vcap = std::min<unsigned long long>(out->max_vertices, cap);
  m.tcap = out->max_triangles;
  m.quad_tiles = (m.vcap + S2_Q_TILE - 1) / S2_Q_TILE;
  ok = carve(base, used, size_t(cap), &m.cand_key) && carve(base, used, size_t(cap) * 8, &m.cand_val) &&
       carve(base, used, size_t(cap) * 3, &m.cand_pos) && carve(base, used, size_t(cap) * 3, &m.cand_nrm) &&
       carve(base, used, vc_ctrl_words(m.vc_tiles), &m.cand_status) &&
       carve(base, used, scan_status_words(m.scan_tiles, m.quad_tiles), &m.scan_status);
  if (!ok || cap == 0) {
    set_err(err, errlen, "no-allocation scratch layout failed");
    return S2M_E_INVALID;
  }
  m.pos = out->pos;
  m.nrm = out->nrm;
  m.key = reinterpret_cast<unsigned long long *>(out->cell);
  m.tris = out->tris;
  unsigned long long counts[8] = {0};
  m.h_read = counts;  // pageable host words for the count read-back
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  cudaError_t e = enqueue(&m, st);
  if (e != cudaSuccess) {
    set_err(err, errlen, std::string("launch: ") + cudaGetErrorString(e));
    return S2M_E_CUDA;
  }
  rc = readback(&m, st, err, errlen);
  m.h_read = nullptr;
  if (rc != S2M_OK) return rc;
  out->nverts = m.nverts;
  out->ntris = m.ntris;
  out->invalid_quads = m.invalid;
  out->candidate_cells = m.ncand;
  if (m.errflags & S2_ERR_LOOKBACK) {
    set_err(err, errlen, "a device-side look-back wait hit its limit");
    return S2M_E_TIMEOUT;
  }
  if (m.errflags & S2_ERR_CAND_OVF) {
    set_err(err, errlen, "the surface has " + std::to_string(m.ncand) + " candidate cells; the scratch holds " +
                             std::to_string(cap));
    return S2M_E_OVERFLOW;
  }
  if (m.errflags & (S2_ERR_VERT_OVF | S2_ERR_INDEX_OVF)) {
    set_err(err, errlen, "the mesh has " + std::to_string(m.nverts) + " vertices; the output holds " +
                             std::to_string(out->max_vertices));
    return S2M_E_OVERFLOW;
  }
  if (m.errflags & S2_ERR_TRI_OVF) {
    set_err(err, errlen, "the mesh has " + std::to_string(m.ntris) + " triangles; the output holds " +
                             std::to_string(out->max_triangles));
    return S2M_E_OVERFLOW;
  }
  return S2M_OK;
}

int s2m_mesh_footprint(const s2m_sdf *sdf, const s2m_params *params, uint64_t *bytes) {
  if (!sdf || !params || !bytes) return S2M_E_INVALID;
  *bytes = s2m::mesh_job_footprint(sdf, *params);
  return *bytes ? S2M_OK : S2M_E_INVALID;
}

int s2m_mesh_get_info(const s2m_mesh *m, s2m_mesh_info *info) {
  if (!m || !info) return S2M_E_INVALID;
  std::memset(info, 0, sizeof(*info));
  info->nverts = m->nverts;
  info->ntris = m->ntris;
  info->invalid_quads = m->invalid;
  info->cells = (uint64_t)m->N * m->N * m->N;
  info->candidate_cells = m->ncand;
  info->resolution = uint32_t(m->N);
  info->slab_depth = uint32_t(m->D);
  info->d_pos = m->pos;
  info->d_nrm = m->nrm;
  info->d_cell = reinterpret_cast<const uint64_t *>(m->key);
  info->d_tris = m->tris;
  info->kernel_launches = m->launches;
  info->host_setup_ms = m->t_setup;
  info->host_launch_ms = m->t_launch;
  info->host_wait_ms = m->t_wait;
  info->runs = m->runs;
  return S2M_OK;
}

int s2m_mesh_copy_to_host(const s2m_mesh *m, float *pos, float *nrm, uint64_t *cell, uint32_t *tris, void *stream) {
  if (!m) return S2M_E_INVALID;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  cudaError_t e = cudaSuccess;
  if (pos && m->nverts) e = cudaMemcpyAsync(pos, m->pos, m->nverts * 12, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess && nrm && m->nverts) e = cudaMemcpyAsync(nrm, m->nrm, m->nverts * 12, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess && cell && m->nverts) e = cudaMemcpyAsync(cell, m->key, m->nverts * 8, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess && tris && m->ntris) e = cudaMemcpyAsync(tris, m->tris, m->ntris * 12, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  return e == cudaSuccess ? S2M_OK : S2M_E_CUDA;
}

// s2m_mesh_generate in one part: create, copy into pooled pinned arrays, free.
static int generate_one(const s2m_sdf *sdf, const s2m_params *params, void *stream, s2m_host_mesh *out, char *err,
                        size_t errlen) {
  s2m_mesh *m = nullptr;
  const auto t0 = std::chrono::steady_clock::now();
  int rc = s2m_mesh_create(sdf, params, stream, &m, err, errlen);
  if (rc != S2M_OK) return rc;
  const auto t1 = std::chrono::steady_clock::now();
  HostMeshOwner *o = new HostMeshOwner();
  o->pos = take_host_block(m->nverts * 12);
  o->nrm = take_host_block(m->nverts * 12);
  o->tris = take_host_block(m->ntris * 12);
  if (!o->pos.p || !o->nrm.p || !o->tris.p) {
    give_host_block(o->pos); give_host_block(o->nrm); give_host_block(o->tris);
    delete o;
    s2m_mesh_free(m);
    set_err(err, errlen, "pinned host arrays");
    return S2M_E_OOM;
  }
  rc = s2m_mesh_copy_to_host(m, static_cast<float *>(o->pos.p), static_cast<float *>(o->nrm.p), nullptr,
                             static_cast<uint32_t *>(o->tris.p), stream);
  if (rc == S2M_OK && m->runs == 1) {  // (an overflow re-run would inflate the meshing time)
    const double mesh_ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
    const double copy_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t1).count();
    if (mesh_ms > 0.0) {
      std::lock_guard<std::mutex> lock(sdf->tune_mu);
      sdf->copy_ratio = std::min(2.0, std::max(0.02, copy_ms / mesh_ms));
    }
  }
  out->pos = static_cast<const float *>(o->pos.p);
  out->nrm = static_cast<const float *>(o->nrm.p);
  out->tris = static_cast<const uint32_t *>(o->tris.p);
  out->nverts = m->nverts;
  out->ntris = m->ntris;
  out->invalid_quads = m->invalid;
  out->resolution = uint32_t(m->N);
  out->parts = 1;
  out->owner = o;
  s2m_mesh_free(m);
  if (rc != S2M_OK) {
    s2m_host_mesh_free(out);
    set_err(err, errlen, "device to host copy failed");
  }
  return rc;
}

int s2m_mesh_generate(const s2m_sdf *sdf, const s2m_params *params, uint32_t parts, void *stream,
                      s2m_host_mesh *out, char *err, size_t errlen) {
  if (!sdf || !params || !out) return S2M_E_INVALID;
  std::memset(out, 0, sizeof(*out));
  // the job's geometry: resolution after rounding, cell planes, slice lag
  s2m_mesh probe;
  probe.sdf = sdf;
  probe.params = *params;
  if (!(probe.params.eps > 0.0f)) probe.params.eps = 1e-4f;
  int rc = setup_job(&probe, err, errlen);
  if (rc != S2M_OK) return rc;
  const int nzc = probe.nzc, lag = probe.job.lag;
  // automatic count (measured at 1024^3 on the CSG scene: one piece 2.57 ms,
  // two parts 2.12, three 2.07, four 2.15 per mesh in host memory)
  unsigned K = parts ? parts : (probe.N >= 1024 ? 3u : probe.N >= 512 ? 2u : 1u);
  K = std::min<unsigned>(K, unsigned(std::max(1, nzc / 16)));  // parts of at least 16 cell planes
  // an SDF's first job tunes its evaluation in one piece
  if (K <= 1 || sdf->eval_variant < 0) return generate_one(sdf, params, stream, out, err, errlen);
  if (probe.job.qef && (rc = ensure_qef_module(sdf, err, errlen)) != S2M_OK) return rc;

  cudaStream_t st = static_cast<cudaStream_t>(stream);
  cudaStream_t side = copy_stream();
  if (!side) return generate_one(sdf, params, stream, out, err, errlen);
  std::vector<s2m_mesh *> pm;
  std::vector<cudaEvent_t> ev;
  HostMeshOwner *o = new HostMeshOwner();
  HostBlock totals;
  auto cleanup = [&]() {
    for (cudaEvent_t e : ev) cudaEventDestroy(e);
    for (s2m_mesh *m : pm) {
      free_buffers(m);
      delete m;
    }
    give_host_block(o->pos); give_host_block(o->nrm); give_host_block(o->tris);
    give_host_block(totals);
    delete o;
  };
  // Part sizes: part k + 1's kernels should take as long as part k's copy, so
  // the sizes fall geometrically by r = copy time / meshing time (learned
  // from the SDF's one-piece runs): the last part, whose copy nothing hides,
  // is the smallest.  Parts keep at least 16 cell planes.
  std::vector<int> zcut(K + 1, 0);
  {
    double r;
    {
      std::lock_guard<std::mutex> lock(sdf->tune_mu);
      r = sdf->copy_ratio;
    }
    r = std::min(1.0, std::max(0.05, r));
    std::vector<double> w(K);
    double sum = 0;
    for (unsigned k = 0; k < K; ++k) sum += (w[k] = std::pow(r, double(k)));
    double acc = 0;
    for (unsigned k = 0; k < K; ++k) {
      acc += w[k];
      zcut[k + 1] = k + 1 == K ? nzc : int(std::lround(double(nzc) * acc / sum));
    }
    for (unsigned k = K - 1; k >= 1; --k) zcut[k] = std::min(zcut[k], zcut[k + 1] - 16);  // 16 planes each
    zcut[0] = 0;
    for (unsigned k = 1; k < K; ++k) zcut[k] = std::max(zcut[k], zcut[k - 1] + 16);
    zcut[K] = nzc;
  }
  unsigned long long vcap = 0, tcap = 0;
  for (unsigned k = 0; k < K; ++k) {
    const int z0 = zcut[k], z1 = zcut[k + 1];
    s2m_mesh *m = new s2m_mesh();
    pm.push_back(m);
    m->sdf = sdf;
    m->stream = st;
    m->params = probe.params;
    m->zpart_begin = k ? z0 - 1 : 0;  // a later part also meshes the plane below it (context)
    m->zpart_end = z1;
    m->quads_from_z = k ? unsigned(z0 + lag) : 0u;
    unsigned long long cc, vc, tc;
    if ((rc = setup_job(m, err, errlen)) == S2M_OK) {
      // the whole job's capacities: a part's share of the surface can be far
      // from its share of the planes (an overflow would mesh the job twice)
      const double zf = m->zfrac;
      m->zfrac = 1.0;
      initial_caps(m, m->params, cc, vc, tc);
      m->zfrac = zf;
      rc = alloc_buffers(m, cc, vc, tc, err, errlen);
    }
    if (rc != S2M_OK) {
      cleanup();
      return rc;
    }
    vcap += m->vcap;
    tcap += m->tcap;
  }
  o->pos = take_host_block(vcap * 12);
  o->nrm = take_host_block(vcap * 12);
  o->tris = take_host_block(tcap * 12);
  totals = take_host_block(K * sizeof(S2HostTotals));
  S2HostTotals *tot_d = mapped<S2HostTotals>(totals);
  if (!o->pos.p || !o->nrm.p || !o->tris.p || !tot_d) {
    cleanup();
    set_err(err, errlen, "pinned host arrays");
    return S2M_E_OOM;
  }
  // The later parts' tile passes (independent of every other part) on a third
  // stream, so that they run beside part 0's kernels; then all parts'
  // kernels (each ending with its copy plan), then, as each part finishes,
  // its copies on the side stream's copy engine: they run while the later
  // parts' kernels do.
  cudaError_t e = cudaSuccess;
  std::vector<cudaEvent_t> tev(K, nullptr), pev;
  {
    int ev_v = sdf->eval_variant >= 0 ? sdf->eval_variant : 0;
    cudaStream_t ts = tile_stream();
    for (unsigned k = 1; k < K && ts && e == cudaSuccess; ++k) {
      s2m_mesh *m = pm[k];
      if (!(kEvalVariants[ev_v].pruned && m->prune_buf && m->prune_chunk >= m->nslabs)) continue;
      if ((e = cudaEventCreateWithFlags(&tev[k], cudaEventDisableTiming)) != cudaSuccess) break;
      ev.push_back(tev[k]);
      if ((e = cudaMemsetAsync(m->prune_buf, 0, m->prune_base_off, ts)) != cudaSuccess) break;
      if ((e = launch_tiles(m, 0, m->nslabs, ts)) != cudaSuccess) break;
      if ((e = cudaEventRecord(tev[k], ts)) != cudaSuccess) break;
      m->tiles_ready = true;
    }
  }
  for (unsigned k = 0; k < K && e == cudaSuccess; ++k) {
    s2m_mesh *m = pm[k];
    cudaEvent_t done;
    if ((e = cudaEventCreateWithFlags(&done, cudaEventDisableTiming)) != cudaSuccess) break;
    ev.push_back(done);
    pev.push_back(done);
    if (tev[k] && (e = cudaStreamWaitEvent(st, tev[k], 0)) != cudaSuccess) break;
    if ((e = enqueue(m, st)) != cudaSuccess) break;
    // the part's first non-context row: its row start counts the context plane's vertices
    const unsigned *skip_at = k ? m->rowstart + (unsigned long long)m->quads_from_z * m->N : nullptr;
    if ((e = launch_pdl(s2m_part_finish, dim3(unsigned(device_sm_count()) * 4), dim3(256), 0, st, mesh_dev(m), skip_at,
                        (const unsigned long long *)(m->cand_base + m->nslabs),
                        (const S2HostTotals *)(k ? tot_d + (k - 1) : nullptr), tot_d + k, vcap, tcap)) != cudaSuccess)
      break;
    e = cudaEventRecord(done, st);
  }
  const S2HostTotals *tot_h = static_cast<const S2HostTotals *>(totals.p);
  for (unsigned k = 0; k < K && e == cudaSuccess; ++k) {
    if ((e = cudaEventSynchronize(pev[k])) != cudaSuccess) break;
    const S2HostTotals t = tot_h[k];
    if (t.err) break;  // the one-piece fallback below
    const s2m_mesh *m = pm[k];
    char *hp = static_cast<char *>(o->pos.p), *hn = static_cast<char *>(o->nrm.p), *ht = static_cast<char *>(o->tris.p);
    if (t.vcount) {
      if ((e = cudaMemcpyAsync(hp + 12 * t.vbase, m->pos + 3 * t.vfirst, 12 * t.vcount, cudaMemcpyDeviceToHost,
                               side)) != cudaSuccess ||
          (e = cudaMemcpyAsync(hn + 12 * t.vbase, m->nrm + 3 * t.vfirst, 12 * t.vcount, cudaMemcpyDeviceToHost,
                               side)) != cudaSuccess)
        break;
    }
    if (t.tcount &&
        (e = cudaMemcpyAsync(ht + 12 * t.tbase, m->tris, 12 * t.tcount, cudaMemcpyDeviceToHost, side)) != cudaSuccess)
      break;
  }
  // every stream drained before the parts' buffers can be freed, whatever failed
  for (cudaStream_t q : {side, tile_stream(), st}) {
    if (!q) continue;
    const cudaError_t es = cudaStreamSynchronize(q);
    if (e == cudaSuccess) e = es;
  }
  if (e != cudaSuccess) {
    cleanup();
    set_err(err, errlen, std::string("z parts: ") + cudaGetErrorString(e));
    return S2M_E_CUDA;
  }
  unsigned flags = 0;
  for (unsigned k = 0; k < K; ++k) {  // the parts' counts, from their copy plans (no further readback)
    s2m_mesh *m = pm[k];
    const S2HostTotals &t = tot_h[k];
    flags |= t.err;
    if (t.err) continue;
    m->ncand = t.ncand;
    m->nverts = t.vfirst + t.vcount;
    m->ntris = t.tcount;
    learn_caps(m);
  }
  const S2HostTotals t = static_cast<const S2HostTotals *>(totals.p)[K - 1];
  flags |= t.err;
  if (flags & S2_ERR_LOOKBACK) {
    cleanup();
    set_err(err, errlen, "a device-side look-back wait hit its limit");
    return S2M_E_TIMEOUT;
  }
  if (flags & S2_ERR_INDEX_OVF) {
    cleanup();
    set_err(err, errlen, "more than 2^32 - 2 vertices");
    return S2M_E_OVERFLOW;
  }
  if (flags & (S2_ERR_CAND_OVF | S2_ERR_VERT_OVF | S2_ERR_TRI_OVF | S2_ERR_HOST_OVF)) {
    // a part outgrew its buffers: the job again in one piece (which re-runs
    // with the exact totals), the parts' totals now learned for the next job
    cleanup();
    return generate_one(sdf, params, stream, out, err, errlen);
  }
  out->pos = static_cast<const float *>(o->pos.p);
  out->nrm = static_cast<const float *>(o->nrm.p);
  out->tris = static_cast<const uint32_t *>(o->tris.p);
  out->nverts = t.nverts;
  out->ntris = t.ntris;
  out->invalid_quads = t.invalid;
  out->resolution = uint32_t(probe.N);
  out->parts = K;
  out->owner = o;
  o = new HostMeshOwner();  // the arrays now belong to `out`
  cleanup();
  return S2M_OK;
}

void s2m_host_mesh_free(s2m_host_mesh *mesh) {
  if (!mesh || !mesh->owner) return;
  HostMeshOwner *o = static_cast<HostMeshOwner *>(mesh->owner);
  give_host_block(o->pos);
  give_host_block(o->nrm);
  give_host_block(o->tris);
  delete o;
  std::memset(mesh, 0, sizeof(*mesh));
}

int s2m_mesh_write(const s2m_mesh *m, const char *path, char *err, size_t errlen) {
  if (!m || !path) return S2M_E_INVALID;
  std::vector<float> pos(m->nverts * 3), nrm(m->nverts * 3);
  std::vector<uint32_t> tris(m->ntris * 3);
  int rc = s2m_mesh_copy_to_host(m, pos.data(), nrm.data(), nullptr, tris.data(), nullptr);
  if (rc != S2M_OK) {
    set_err(err, errlen, "device to host copy failed");
    return rc;
  }
  return s2m::write_mesh_file(path, pos.data(), nrm.data(), m->nverts, tris.data(), m->ntris, err, errlen);
}

int s2m_mesh_set_wait_limit(s2m_mesh *m, double seconds) {
  if (!m || !(seconds > 0.0) || seconds > 3600.0) return S2M_E_INVALID;
  m->wait_ns = (unsigned long long)(seconds * 1e9);
  drop_graph(m);  // a captured graph holds the old bound
  return S2M_OK;
}

int s2m_mesh_set_graph(s2m_mesh *m, int enable) {
  if (!m) return S2M_E_INVALID;
  m->use_graph = enable != 0;
  if (!m->use_graph) drop_graph(m);
  return S2M_OK;
}

int s2m_mesh_set_profiling(s2m_mesh *m, int enable) {
  if (!m) return S2M_E_INVALID;
  m->profile = enable != 0;
  return S2M_OK;
}

int s2m_mesh_get_profile(const s2m_mesh *m, s2m_profile *out) {
  if (!m || !out) return S2M_E_INVALID;
  *out = m->prof;
  return S2M_OK;
}

int s2m_mesh_reset_profile(s2m_mesh *m) {
  if (!m) return S2M_E_INVALID;
  m->prof = s2m_profile{};
  return S2M_OK;
}

void s2m_mesh_free(s2m_mesh *m) {
  if (!m) return;
  for (cudaEvent_t e : m->ev) cudaEventDestroy(e);
  drop_graph(m);
  free_buffers(m);
  if (m->capture_stream) cudaStreamDestroy(m->capture_stream);
  delete m;
}

int s2m_write_stl(const float *pos, const uint32_t *tris, uint64_t ntris, const char *path) {
  return s2m::write_stl(path, pos, tris, ntris) ? S2M_OK : S2M_E_IO;
}

int s2m_write_stl_binary(const float *pos, const uint32_t *tris, uint64_t ntris, const char *path) {
  if ((!pos && ntris) || (!tris && ntris) || !path) return S2M_E_INVALID;
  return s2m::write_stl_binary(path, pos, tris, ntris) ? S2M_OK : S2M_E_IO;
}

int s2m_mesh_write_stl_binary(const s2m_mesh *m, const char *path, char *err, size_t errlen) {
  if (!m || !path) return S2M_E_INVALID;
  std::vector<float> pos(m->nverts * 3);
  std::vector<uint32_t> tris(m->ntris * 3);
  int rc = s2m_mesh_copy_to_host(m, pos.data(), nullptr, nullptr, tris.data(), nullptr);
  if (rc != S2M_OK) {
    set_err(err, errlen, "device to host copy failed");
    return rc;
  }
  if (!s2m::write_stl_binary(path, pos.data(), tris.data(), m->ntris)) {
    set_err(err, errlen, std::string("could not write ") + path);
    return S2M_E_IO;
  }
  return S2M_OK;
}

int s2m_write_ply(const float *pos, const float *nrm, uint64_t nverts, const uint32_t *tris, uint64_t ntris,
                  const char *path) {
  return s2m::write_ply(path, pos, nrm, nverts, tris, ntris) ? S2M_OK : S2M_E_IO;
}

int s2m_measure_sfu_peak(double *gops, void *stream) {
  if (!gops) return S2M_E_INVALID;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int sms = device_sm_count();
  const int blocks = sms * 8, iters = 4096;
  float *out = nullptr;
  if (cudaMallocAsync(&out, size_t(blocks) * 4, st) != cudaSuccess) return S2M_E_OOM;
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  double best = 0;
  for (int rep = 0; rep < 4; ++rep) {
    cudaEventRecord(a, st);
    s2m_sfu_probe<<<blocks, 256, 0, st>>>(out, iters, 0.5f);
    cudaEventRecord(b, st);
    cudaEventSynchronize(b);
    float ms = 0;
    cudaEventElapsedTime(&ms, a, b);
    double ops = double(blocks) * 256.0 * iters * 8.0;
    if (rep > 0) best = std::max(best, ops / (double(ms) * 1e-3) / 1e9);
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  cudaFreeAsync(out, st);
  cudaStreamSynchronize(st);
  if (cudaGetLastError() != cudaSuccess) return S2M_E_CUDA;
  *gops = best;
  return S2M_OK;
}

int s2m_measure_fp32_peak(double *gops, void *stream) {
  if (!gops) return S2M_E_INVALID;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int sms = device_sm_count();
  const int blocks = sms * 8, iters = 8192;
  float *out = nullptr;
  if (cudaMalloc(&out, size_t(blocks) * 4) != cudaSuccess) return S2M_E_OOM;
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  double best = 0;
  for (int rep = 0; rep < 4; ++rep) {
    cudaEventRecord(a, st);
    s2m_fp32_probe<<<blocks, 256, 0, st>>>(out, iters, 0, 0.999f, 1e-3f);
    cudaEventRecord(b, st);
    cudaEventSynchronize(b);
    float ms = 0;
    cudaEventElapsedTime(&ms, a, b);
    double ops = double(blocks) * 256.0 * iters * 8.0 * 2.0;
    if (rep > 0) best = std::max(best, ops / (double(ms) * 1e-3) / 1e9);
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  cudaFree(out);
  if (cudaGetLastError() != cudaSuccess) return S2M_E_CUDA;
  *gops = best;
  return S2M_OK;
}

}  // extern "C"
