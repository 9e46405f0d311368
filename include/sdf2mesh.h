/*
 * sdf2mesh.h -- C ABI of libsdf2mesh_gb300.so, the GB300 (sm_103a) engine
 * that meshes signed distance functions by dual contouring.
 *
 * The reference (WilstonOreo/sdf2mesh) has no FFI: its boundary is a Rust
 * binary and a wgpu module.  Each entry point below names the reference code
 * it stands in for (paths relative to the reference sources).
 *
 * Conventions
 *   - Every function returns an s2m_status (0 = S2M_OK) unless noted; on
 *     failure, when `err` is non-null, a NUL-terminated message is written
 *     into err[0..errlen).  No exception or abort crosses this boundary.
 *   - `stream` is a cudaStream_t passed as void* (NULL = the legacy default
 *     stream).  Device work is stream-ordered.
 *   - Handles are opaque; the caller frees each with its *_free function.
 *     An s2m_sdf is immutable after compilation and may be shared between
 *     threads; an s2m_mesh is used by one thread at a time.
 */
#ifndef SDF2MESH_GB300_H
#define SDF2MESH_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define S2M_ABI_VERSION 2

typedef enum {
  S2M_OK = 0,
  S2M_E_INVALID = 1,      /* bad argument                                         */
  S2M_E_IO = 2,           /* file could not be read or written                    */
  S2M_E_PARSE = 3,        /* WGSL / GLSL source rejected by the frontend          */
  S2M_E_MISSING_SDF = 4,  /* no sdf3d / named GLSL function (shadertoy.rs MissingSdf) */
  S2M_E_NVRTC = 5,        /* NVRTC could not compile the lowered source           */
  S2M_E_CUDA = 6,         /* CUDA runtime error                                   */
  S2M_E_OOM = 7,          /* device allocation failed                             */
  S2M_E_OVERFLOW = 8,     /* mesh exceeds the largest supported buffers            */
  S2M_E_TIMEOUT = 9,      /* a bounded device wait expired (kernel error flag)    */
  S2M_E_NO_DEVICE = 10    /* no CUDA device                                       */
} s2m_status;

/* S2M_LANG_SHADERTOY: ShaderToy-style GLSL as the site stores it (no version
   line, uniforms or main), wrapped as shadertoy.rs:154-166 does; its inputs
   (iTime, iResolution, iMouse ...) are constant zero.  The HTTP fetch of the
   reference (--shadertoy-id) is not offered: files only. */
typedef enum { S2M_LANG_WGSL = 0, S2M_LANG_GLSL = 1, S2M_LANG_SHADERTOY = 2 } s2m_lang;

/* Compile flags. */
#define S2M_COMPILE_FMAD 0x1u      /* allow FMA contraction: faster, no longer bit-exact
                                      with the reference rule's binary32 arithmetic
                                      (also turns tile pruning off)                  */
#define S2M_COMPILE_NO_PRUNE 0x2u  /* evaluate every operation of the SDF at every
                                      lattice point (no tile pruning)               */

/* Job flags (s2m_params.flags). */
#define S2M_JOB_POW2_ROUNDING 0x1u  /* round resolution up to a power of two as the
                                       reference CLI does (main.rs:141-148)         */
#define S2M_JOB_SLICE_LAG 0x2u      /* reproduce the reference's read-before-submit
                                       slice lag (main.rs:324-355): only cell slices
                                       0..N-2 are emitted, labelled z+1             */
#define S2M_JOB_EXACT_CORNERS 0x4u  /* re-evaluate every off-lattice corner of every
                                       cell (verification mode; slower)             */
#define S2M_JOB_QEF 0x8u            /* precision mode (no reference counterpart; the
                                       reference places the mass point,
                                       dualcontour.wgsl:86-131): corners from the
                                       shared lattice, a QEF vertex from the crossing
                                       normals, FP32 compensated sums, FP64 solve  */

typedef struct s2m_sdf s2m_sdf;
typedef struct s2m_mesh s2m_mesh;

/* Job parameters.  Stands in for AppState (main.rs:12-64, 139-175). */
typedef struct {
  uint32_t resolution;    /* cells per axis N (>= 2)                       */
  float bounds;           /* edge of the centred cube [-B/2, B/2]^3        */
  float eps;              /* normal epsilon (reference: 1e-4)              */
  uint32_t flags;         /* S2M_JOB_*                                     */
  uint32_t slab_depth;    /* cell slices per slab; 0 = automatic: a ring of
                             lattice planes that fits in L2 (full
                             evaluation), or slabs of equal depth from a
                             ring of up to 4 GB (SDFs with a tile form)     */
  uint32_t reserved;
  uint64_t max_vertices;  /* initial vertex capacity; 0 = automatic        */
  uint64_t max_triangles; /* initial triangle capacity; 0 = automatic      */
} s2m_params;

/* Result description; device pointers stay owned by the s2m_mesh. */
typedef struct {
  uint64_t nverts;
  uint64_t ntris;
  uint64_t invalid_quads;   /* quads dropped as in mesh.rs:270-277           */
  uint64_t cells;           /* N^3 voxels of the job                         */
  uint64_t candidate_cells; /* cells whose exact corners were re-evaluated   */
  uint32_t resolution;      /* N actually used (after optional rounding)     */
  uint32_t slab_depth;
  const float *d_pos;       /* device: 3 * nverts  (x, y, z)                 */
  const float *d_nrm;       /* device: 3 * nverts  unit normals              */
  const uint64_t *d_cell;   /* device: nverts keys x | y<<16 | z<<32 | signs<<48 */
  const uint32_t *d_tris;   /* device: 3 * ntris vertex indices              */
  uint64_t kernel_launches; /* kernels launched by the last run              */
  /* Host time of the last s2m_mesh_create / s2m_mesh_run, ms: job setup and
     buffer allocation, launching the pipeline, then waiting for the device
     and reading its counters back; and the pipeline runs it took (more than
     one after a capacity overflow). */
  double host_setup_ms;
  double host_launch_ms;
  double host_wait_ms;
  uint32_t runs;
  uint32_t reserved;
} s2m_mesh_info;

/* ---- shader front end (src/shader.rs, src/shadertoy.rs) --------------- */

/* Sdf3DShader::from_path + shader_source_input (shader.rs:44-67, 159-203):
   expand `use` / `include` lines of a .sdf3d file.  *out is malloc'ed; free
   it with s2m_free_string. */
int s2m_preprocess_file(const char *path, char **out, char *err, size_t errlen);

/* The same expansion on in-memory .sdf3d text (shader.rs:159-203); `include`
   paths resolve against the working directory, then `base_dir` (may be
   NULL).  *out is malloc'ed; free it with s2m_free_string. */
int s2m_preprocess_source(const char *source, const char *base_dir, char **out, char *err, size_t errlen);

/* Compile an SDF source (WGSL .sdf3d text after preprocessing, or GLSL) to a
   device module for sm_103a: frontend -> CUDA C -> NVRTC.  Stands in for
   Sdf3DShader::add_to_source + create_shader_module (shader.rs:155-157,
   220-225) and, for GLSL, from_glsl_fragment_shader (shader.rs:73-104);
   `sdf_name` is the GLSL function (default "sdf"). */
int s2m_compile(const char *source, int lang, const char *sdf_name, uint32_t compile_flags,
                s2m_sdf **out, char *err, size_t errlen);

/* s2m_preprocess_file (WGSL) or a GLSL file read, then s2m_compile. */
int s2m_compile_file(const char *path, int lang, const char *sdf_name, uint32_t compile_flags,
                     s2m_sdf **out, char *err, size_t errlen);

/* The lowered CUDA C of a compiled SDF (for --debug-cuda); owned by sdf. */
const char *s2m_sdf_cuda_source(const s2m_sdf *sdf);

/* How the SDF's module was built: wall seconds of the NVRTC stage, the NVRTC
   programs it was split into (compiled on parallel host threads), and how
   many of them came from the on-disk module cache ($S2M_CACHE_DIR, empty to
   turn it off; default $XDG_CACHE_HOME or $HOME/.cache, sdf2mesh_gb300/),
   whose files hold the whole program text beside the CUBIN so that a hit is
   an exact match.  The reference compiles its shader per run
   (shader.rs:220-225). */
int s2m_sdf_compile_info(const s2m_sdf *sdf, double *seconds, int *programs, int *cache_hits);

/* Algorithmic FP32 and SFU operations of one sdf3d evaluation. */
int s2m_sdf_op_counts(const s2m_sdf *sdf, double *fp32_ops, double *sfu_ops);
/* Operations per point when the lattice kernel evaluates runs of 4 points
   sharing x and y (the part that depends only on x and y runs once per run);
   S2M_E_INVALID when the SDF has no run form (branches, loops). */
int s2m_sdf_run_op_counts(const s2m_sdf *sdf, double *fp32_ops, double *sfu_ops);

/* Evaluation-kernel variant the autotuner chose for this SDF on its first
   job (-1: not tuned yet): its name, and the measured ns per lattice point
   of each of the S2M_EVAL_VARIANTS variants.  No reference counterpart (the
   reference has one fixed kernel, dualcontour.wgsl:161-162). */
#define S2M_EVAL_VARIANTS 8
int s2m_sdf_eval_variant(const s2m_sdf *sdf, char *name, size_t namelen, double *ns_per_point);
/* Use `variant` for this SDF's later jobs instead of tuning (S2M_E_INVALID
   when the module has no such variant, e.g. a pruned one without a pruning
   form). */
int s2m_sdf_set_eval_variant(s2m_sdf *sdf, int variant);
/* Name, registers per thread and local (spill) bytes per thread of one
   variant, as the tuner recorded them (0 before tuning).  Variants 5 to 7
   are the tile-pruned ones; their ns per point is 0 when the SDF has no
   pruning form. */
int s2m_sdf_eval_variant_info(const s2m_sdf *sdf, int variant, char *name, size_t namelen, int *registers,
                              int *local_bytes);

/* Tile pruning (no reference counterpart).  For a straight-line SDF the
   frontend also emits an interval evaluation over a tile of 8 x 8 x <= 8
   lattice points.  Where it proves that a min, max or sdf::op smooth
   operator returns one operand bit for bit at every point of the tile, the
   other operand's exclusive operations are skipped there, so the lattice
   values stay bit-identical.  *combinators: combinators that can prune;
   *words: activity words per tile (0: no tile form, or turned off by
   S2M_COMPILE_FMAD / _NO_PRUNE; a straight-line SDF without combinators
   still has a tile form, with 0 combinators and 1 word). */
int s2m_sdf_prune_info(const s2m_sdf *sdf, int *combinators, int *words);

void s2m_sdf_free(s2m_sdf *sdf);

/* Frontend only (no device): lower a source to CUDA C.  *out is malloc'ed. */
int s2m_translate(const char *source, int lang, const char *sdf_name, char **out,
                  double *fp32_ops, double *sfu_ops, char *err, size_t errlen);

/* WGSL text surgery (shadertoy.rs:248-352).  *out is malloc'ed. */
int s2m_wgsl_remove_function(const char *wgsl, const char *function_name, char **out);
int s2m_wgsl_rename_function(const char *wgsl, const char *old_name, const char *new_name,
                             char **out);
int s2m_wgsl_has_function(const char *wgsl, const char *function_name); /* 1 / 0 */

void s2m_free_string(char *s);

/* ---- meshing (dualcontour.wgsl:161-180, main.rs:298-356, mesh.rs:267-341) */

/* Mesh an SDF: grid evaluation, sign changes, crossings, vertex placement
   and quad emission, all on the device, into buffers owned by *out.
   Synchronises `stream` at the end (the counts are read back). */
int s2m_mesh_create(const s2m_sdf *sdf, const s2m_params *params, void *stream,
                    s2m_mesh **out, char *err, size_t errlen);

/* Re-run the same job into the mesh's existing buffers, stream-ordered,
   without synchronising (for timing).  Counts become valid after
   s2m_mesh_sync. */
int s2m_mesh_run_async(s2m_mesh *mesh, void *stream);

/* Wait for `stream`, read the counts back and check the device error flags. */
int s2m_mesh_sync(s2m_mesh *mesh, void *stream, char *err, size_t errlen);

int s2m_mesh_get_info(const s2m_mesh *mesh, s2m_mesh_info *info);

/* Device bytes s2m_mesh_create allocates for this job on its first attempt
   (lattice ring, point bits, tile records, candidate, vertex and triangle
   buffers), computed by the same job setup and buffer plan without
   allocating anything.  A job whose initial capacities overflow is re-run
   with the exact totals and then holds more.  No reference counterpart (the
   reference's memory is two storage textures per slice, texture.rs:15-48). */
int s2m_mesh_footprint(const s2m_sdf *sdf, const s2m_params *params, uint64_t *bytes);

/* SDF operations the last run's lattice evaluation executed: points
   evaluated, FP32 and SFU operations in total (pruned runs: counted per tile
   by the tile pass; others: the per-point counts times the points).
   Returns 1 when the run was tile-pruned, 0 when not, < 0 on error. */
int s2m_mesh_eval_ops(const s2m_mesh *mesh, double *points, double *fp32_ops, double *sfu_ops);

/* Copy the mesh to caller-owned host buffers (any may be NULL):
   pos / nrm 3*nverts floats, cell nverts keys, tris 3*ntris indices. */
int s2m_mesh_copy_to_host(const s2m_mesh *mesh, float *pos, float *nrm, uint64_t *cell,
                          uint32_t *tris, void *stream);

/* TriangleMesh::write_to_file (mesh.rs:182-196): STL or PLY by extension. */
int s2m_mesh_write(const s2m_mesh *mesh, const char *path, char *err, size_t errlen);

/* ---- one call to a mesh in host memory -----------------------------------
   Replaces the reference's generate() returning its TriangleMesh in host
   memory (main.rs:177-364, lib.rs TriangleMesh): s2m_mesh_create +
   s2m_mesh_copy_to_host + s2m_mesh_free in one call, with the same bits.  A
   large job runs as `parts` slices of cell planes along z (0: chosen by the
   library, 1: one piece); each part's device-to-host copy then runs while the
   next part's kernels do.  A part after the first also meshes the last cell
   plane of the one below it (its quads need those vertices) and copies none
   of it.  The arrays are pinned host memory owned by the library until
   s2m_host_mesh_free. */
typedef struct {
  const float *pos;       /* 3 * nverts (x, y, z)                                  */
  const float *nrm;       /* 3 * nverts unit normals                               */
  const uint32_t *tris;   /* 3 * ntris vertex indices                              */
  uint64_t nverts;
  uint64_t ntris;
  uint64_t invalid_quads;
  uint32_t resolution;    /* N actually used                                       */
  uint32_t parts;         /* z parts the job ran as                                */
  void *owner;            /* library bookkeeping                                   */
} s2m_host_mesh;
int s2m_mesh_generate(const s2m_sdf *sdf, const s2m_params *params, uint32_t parts, void *stream,
                      s2m_host_mesh *out, char *err, size_t errlen);
void s2m_host_mesh_free(s2m_host_mesh *mesh);

void s2m_mesh_free(s2m_mesh *mesh);

/* Per-kernel device time of a mesh's runs, from CUDA events recorded on the
   launching stream around every kernel while profiling is enabled.  Kinds:
   0 grid evaluation, 1 cell classification, 2 vertex placement, 3 vertex
   compaction, 4 row scan, 5 quads.
   Accumulates over runs until reset; read after s2m_mesh_sync. */
#define S2M_KERNEL_KINDS 6
typedef struct {
  double ms[S2M_KERNEL_KINDS];
  uint64_t launches[S2M_KERNEL_KINDS];
  double eval_points;      /* lattice points evaluated by kind-0 launches */
  double cells;            /* cells classified by kind-1 launches         */
} s2m_profile;
int s2m_mesh_set_profiling(s2m_mesh *mesh, int enable);
/* Bound of every device-side wait of this mesh's runs (the look-back of the
   ordered compactions), in seconds of the GPU's global timer; default 2 s.
   A wait that runs out raises an error flag instead of spinning on: the run
   finishes with S2M_E_TIMEOUT and the context stays usable.  The reference
   has no device waits; it panics on a failed readback (main.rs:184, 196,
   texture.rs:110). */
int s2m_mesh_set_wait_limit(s2m_mesh *mesh, double seconds);
/* Replay the mesh's launch sequence as a CUDA graph in s2m_mesh_run_async
   (captured on the first run on a stream; not while profiling). */
int s2m_mesh_set_graph(s2m_mesh *mesh, int enable);
int s2m_mesh_get_profile(const s2m_mesh *mesh, s2m_profile *out);
int s2m_mesh_reset_profile(s2m_mesh *mesh);

/* ---- meshing without device allocation ---------------------------------
   No counterpart in the reference: an addition for callers that may not
   allocate device memory while they mesh -- programs that reserve the GPU's
   memory up front in their own arena (renderers, simulators, engines with a
   fixed memory plan), that run under a hard memory quota, or that must not
   pay the device-wide synchronisation a cudaMalloc / cudaFree can cause in
   the middle of a frame or a timed loop.

   s2m_mesh_noalloc meshes one job like s2m_mesh_create, but every scratch
   buffer of the pipeline (lattice planes, candidate cells, scan words,
   counters) lives in one fixed array of S2M_NOALLOC_SCRATCH_BYTES inside the
   library, which every GPU that loads the library holds until the process
   exits.  The caller allocates the outputs (device memory) and the library
   allocates nothing: no cudaMalloc, cudaFree or allocating library call.
   Compile the SDF beforehand (s2m_compile loads a module, which allocates).

   Limits: resolution <= S2M_NOALLOC_MAX_RESOLUTION (larger is rejected with
   S2M_E_INVALID before any device work); the surface must fit the scratch's
   candidate-cell capacity (S2M_E_OVERFLOW otherwise).  If the caller's
   vertex or triangle capacity is too small the call returns S2M_E_OVERFLOW
   with the exact nverts / ntris needed.
   Concurrency: every call shares the one array, so calls whose device work
   overlaps (other host threads, or other streams without ordering between
   them) race; serialise them.  The first call on a device looks up the
   array's device address (cudaGetSymbolAddress) with that device current;
   make that first call before any stream capture.  The address is kept for
   the life of the process: after cudaDeviceReset (or a release of the
   device's primary context) the array lives at a new address and the kept
   one is stale, so do not call this entry point again in that process.  The
   call synchronises `stream` (it reads the counts back). */
#define S2M_NOALLOC_SCRATCH_BYTES (64u << 20)
#define S2M_NOALLOC_MAX_RESOLUTION 256u
typedef struct {
  float *pos;              /* in: device, 3 * max_vertices floats          */
  float *nrm;              /* in: device, 3 * max_vertices floats          */
  uint64_t *cell;          /* in: device, max_vertices keys (as s2m_mesh_info.d_cell) */
  uint32_t *tris;          /* in: device, 3 * max_triangles indices        */
  uint64_t max_vertices;   /* in                                           */
  uint64_t max_triangles;  /* in                                           */
  uint64_t nverts;         /* out (exact, also on S2M_E_OVERFLOW)          */
  uint64_t ntris;          /* out (exact when the vertices fit)            */
  uint64_t invalid_quads;  /* out                                          */
  uint64_t candidate_cells;/* out                                          */
  uint32_t resolution;     /* out: N used                                  */
  uint32_t reserved;
} s2m_noalloc_mesh;
int s2m_mesh_noalloc(const s2m_sdf *sdf, const s2m_params *params, s2m_noalloc_mesh *out, void *stream,
                     char *err, size_t errlen);

/* ---- batching: many jobs in one persistent launch -----------------------
   No reference counterpart (the reference meshes one SDF per process run).
   A batch job is a CSG program: a postfix list of floats, each opcode
   followed by its operands, evaluated on the device by an interpreter whose
   arithmetic is that of the library function of the same name
   (src/sdf3d_primitives.wgsl:7-36, src/sdf_op.wgsl:7-23), so no per-job
   compilation is needed.  Operands:
     SPHERE cx cy cz r            sdf3d_sphere(p - c, r)
     BOX cx cy cz bx by bz        sdf3d_box(p - c, b)            (full size b)
     TORUS cx cy cz R r           sdf3d_torus(p - c, vec2(R, r))
     CAPSULE ax ay az bx by bz r  sdf3d_capsule(p, a, b, r)
     PLANE nx ny nz d             dot(p, n) - d
     UNION / SUBTRACT / INTERSECT  min(a, b) / max(a, -b) / max(a, b)
     SMOOTH_UNION k, SMOOTH_INTERSECTION k, SMOOTH_SUBTRACTION k
                                   sdf_op_smooth_*(a, b, k)
   s2m_batch_run meshes every job added since the last run in one launch of
   a persistent kernel over a device work queue (waves of at most
   memory_budget_bytes of device memory; 0 = no limit).  Job results stay on
   the device until s2m_batch_free. */
enum {
  S2M_CSG_SPHERE = 0, S2M_CSG_BOX = 1, S2M_CSG_TORUS = 2, S2M_CSG_CAPSULE = 3, S2M_CSG_PLANE = 4,
  S2M_CSG_UNION = 10, S2M_CSG_SUBTRACT = 11, S2M_CSG_INTERSECT = 12, S2M_CSG_SMOOTH_UNION = 13,
  S2M_CSG_SMOOTH_INTERSECTION = 14, S2M_CSG_SMOOTH_SUBTRACTION = 15
};
/* The CSG program of a .sdf3d source (raw or preprocessed) whose sdf3d is a
   single expression over sdf3d_sphere / box / torus (at p or p - constant),
   sdf3d_capsule (at p), min, max, negation and sdf_op_smooth_* with constant
   arguments -- e.g. the batching workload's sources.  *len receives the
   length; program (capacity floats) may be NULL to query it.  S2M_E_PARSE
   with the reason for any other source (compile it with s2m_compile). */
int s2m_csg_from_source(const char *source, float *program, uint32_t capacity, uint32_t *len, char *err,
                        size_t errlen);
typedef struct s2m_batch s2m_batch;
int s2m_batch_create(s2m_batch **out, uint64_t memory_budget_bytes);
int s2m_batch_add_csg(s2m_batch *b, const float *program, uint32_t len, const s2m_params *params,
                      uint32_t *job_id, char *err, size_t errlen);
/* Device bytes the job needs while it runs (lattice, candidates, mesh). */
uint64_t s2m_batch_job_footprint(const s2m_batch *b, uint32_t job);
/* Synchronises `stream`. */
int s2m_batch_run(s2m_batch *b, void *stream, char *err, size_t errlen);
int s2m_batch_job_info(const s2m_batch *b, uint32_t job, s2m_mesh_info *info);
int s2m_batch_job_copy_to_host(const s2m_batch *b, uint32_t job, float *pos, float *nrm, uint64_t *cell,
                               uint32_t *tris, void *stream);
/* Device time of the last run's persistent launches, their count, jobs in the batch. */
int s2m_batch_stats(const s2m_batch *b, double *kernel_ms, uint64_t *launches, uint32_t *njobs);
/* Bounds of the persistent kernel's device waits, in seconds of the GPU's
   global timer: a job stage waiting for the job's previous stage (default
   30 s) and the look-back of its ordered compactions (default 2 s).  A wait
   that runs out makes s2m_batch_run return S2M_E_TIMEOUT. */
int s2m_batch_set_wait_limit(s2m_batch *b, double stage_seconds, double lookback_seconds);
/* Tile pruning of the CSG programs (default on), for the batch's jobs that
   have not run yet: per tile of 8^3 lattice points an interval pass over the
   program decides the tile's sign or which operands of its min / max /
   smooth operators can be skipped; the results are bit-identical either way. */
int s2m_batch_set_pruning(s2m_batch *b, int enabled);
/* Where the last run's persistent launches spent their block time: for each
   stage (0 tile pass, 1 lattice, 2 candidate bits, 3 candidate slots, 4
   candidates, 5 vertices, 6 vertex compaction, 7 row scan, 8 quads; nstages
   entries written, 0 past the last stage) the summed block time of its items
   in ms of the GPU's global timer, and in *wait_ms the block time spent
   waiting for a job's previous stage. */
#define S2M_BATCH_STAGES 9
int s2m_batch_stage_profile(const s2m_batch *b, double *busy_ms, uint32_t nstages, double *wait_ms);
void s2m_batch_free(s2m_batch *b);

/* ---- serving: continuous batching ---------------------------------------
   No reference counterpart.  A request loop on its own host threads:
   requests (CSG programs, or compiled SDFs) from any thread are admitted in
   arrival order while their device footprint fits memory_budget_bytes.  CSG
   programs run on the batch interpreter: fewer than max_inflight persistent
   launches at a time, each admitted group one launch on its own stream, so
   requests that arrive while others are on the GPU start as soon as a slot
   and memory free up and overlap with them.  Compiled-SDF requests run the
   per-job pipeline on sdf_workers host threads, each with its own stream, so
   several jobs share the GPU at once.
   Sources (s2m_server_submit_source) are tiered: a CSG source whose compiled
   module is not ready yet runs on the interpreter while a background thread
   compiles it; its later requests run the compiled module (tile-pruned
   per-job pipeline).  Latency = completion - submission (host clock). */
typedef struct s2m_server s2m_server;
#define S2M_SERVER_INTERPRET_ONLY 0x1u  /* CSG sources always on the interpreter (no background compile) */
typedef struct {
  uint64_t memory_budget_bytes;  /* admission limit; 0 = none                         */
  uint32_t max_inflight;         /* concurrent persistent launches (default 2)        */
  uint32_t max_batch_jobs;       /* requests per launch (default 1024)                */
  uint32_t keep_results;         /* 1: meshes stay on the device until s2m_server_release */
  uint32_t sdf_workers;          /* per-job pipelines at once, one stream each (default 4) */
  uint32_t flags;                /* S2M_SERVER_*                                      */
  uint32_t reserved;
} s2m_server_config;
typedef struct {
  uint64_t submitted, completed, failed, batches, peak_bytes;
  double p50_ms, p99_ms, mean_ms;   /* latency of completed requests            */
  double span_s;                    /* first submission to last completion      */
  double meshes_per_s, gvoxels_per_s;
  uint64_t ran_compiled;            /* completed on a compiled module (per-job pipeline) */
  uint64_t ran_interpreted;         /* completed on the batch interpreter          */
  uint64_t compiled_sources;        /* sources whose module is ready               */
  uint64_t compiles_pending;        /* sources queued for or in background compilation */
} s2m_server_stats;
int s2m_server_create(const s2m_server_config *cfg, s2m_server **out, char *err, size_t errlen);
int s2m_server_submit_csg(s2m_server *s, const float *program, uint32_t len, const s2m_params *params,
                          uint64_t *request_id, char *err, size_t errlen);
int s2m_server_submit_sdf(s2m_server *s, const s2m_sdf *sdf, const s2m_params *params, uint64_t *request_id,
                          char *err, size_t errlen);
/* A request as source text, the reference's plugin surface.  WGSL whose
   sdf3d is a CSG expression (s2m_csg_from_source) runs on the batch
   interpreter until the background compile of its text finishes (unless
   S2M_SERVER_INTERPRET_ONLY), then on its compiled module; any other source
   is compiled once, in the call (cached by its text), and runs the per-job
   pipeline. */
int s2m_server_submit_source(s2m_server *s, const char *source, int lang, const char *sdf_name,
                             const s2m_params *params, uint64_t *request_id, char *err, size_t errlen);
/* S2M_OK once the request completed, S2M_E_TIMEOUT if it has not yet, or its error. */
int s2m_server_wait(s2m_server *s, uint64_t request_id, double timeout_s, s2m_mesh_info *info, char *err,
                    size_t errlen);
int s2m_server_copy_to_host(s2m_server *s, uint64_t request_id, float *pos, float *nrm, uint64_t *cell,
                            uint32_t *tris);
int s2m_server_release(s2m_server *s, uint64_t request_id);
int s2m_server_drain(s2m_server *s, double timeout_s);
int s2m_server_get_stats(s2m_server *s, s2m_server_stats *out);
/* Start a new measurement window (counts, latencies, span, peak bytes); the
   compiled-source cache and resident results stay.  S2M_E_INVALID while
   requests are still in flight (drain first). */
int s2m_server_reset_stats(s2m_server *s);
void s2m_server_free(s2m_server *s);

/* ---- host writers (mesh.rs:8-141) -------------------------------------- */

/* ASCII STL with Rust `{}` float text, facet normal (v2-v0) x (v1-v0). */
int s2m_write_stl(const float *pos, const uint32_t *tris, uint64_t ntris, const char *path);
/* Binary STL (80-byte header, u32 count, 50 bytes per facet: the same facet
   normal (v2-v0) x (v1-v0) as the ASCII writer, lib.rs:181-185, three
   vertices, a zero attribute word), written from all host threads.  Not in
   the reference, whose ASCII STL runs to GBs at 2048^3 (README.md:96);
   stands beside write_stl_to_file (mesh.rs:167-180).  S2M_E_IO also for more
   than 2^32 - 1 triangles. */
int s2m_write_stl_binary(const float *pos, const uint32_t *tris, uint64_t ntris, const char *path);
/* s2m_mesh_write's binary STL form: the mesh copied to host memory, then
   s2m_write_stl_binary. */
int s2m_mesh_write_stl_binary(const s2m_mesh *mesh, const char *path, char *err, size_t errlen);
/* ASCII PLY with per-vertex normals. */
int s2m_write_ply(const float *pos, const float *nrm, uint64_t nverts, const uint32_t *tris,
                  uint64_t ntris, const char *path);

/* ---- diagnostics --------------------------------------------------------- */

const char *s2m_status_string(int status);
int s2m_abi_version(void);
/* Measured FP32 issue rate of the current device in Gop/s (one FP32 add or
   mul per lane per cycle), from a dependent-chain microkernel. */
int s2m_measure_fp32_peak(double *gops, void *stream);
/* Measured SFU (MUFU) issue rate in Gop/s, from a reciprocal-square-root chain. */
int s2m_measure_sfu_peak(double *gops, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* SDF2MESH_GB300_H */
