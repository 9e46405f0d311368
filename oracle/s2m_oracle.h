/*
 * s2m_oracle.h -- CPU oracle for the sdf2mesh dual-contouring path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is a plain C++ restatement of the
 * reference's algorithm, used by the tests, by smoke() and by bench.py's CPU
 * baseline as the checker.  The product (libsdf2mesh_gb300.so and its CUDA
 * kernels) never links, loads or calls it.
 *
 * What it restates (paths are relative to the WilstonOreo/sdf2mesh sources):
 *   - job parameters:         src/bin/sdf2mesh/main.rs:139-175, src/lib.rs:115-118
 *   - per-cell evaluation:    src/bin/sdf2mesh/dualcontour.wgsl:22-43
 *   - sign bits:              src/bin/sdf2mesh/dualcontour.wgsl:57-69
 *   - mass-point vertex:      src/bin/sdf2mesh/dualcontour.wgsl:72-131
 *   - kernel body:            src/bin/sdf2mesh/dualcontour.wgsl:161-180
 *   - tetrahedral normal:     src/sdf3d_normal.wgsl:4-10
 *   - primitives / ops:       src/sdf3d_primitives.wgsl:7-36, src/sdf_op.wgsl:7-23
 *   - host slice loop + lag:  src/bin/sdf2mesh/main.rs:298-356
 *   - vertex list + quads:    src/mesh.rs:213-331, src/lib.rs:181-211
 *   - STL / PLY text:         src/mesh.rs:8-141, 143-211
 *
 * Parity status: the reference ships no golden vectors or known-answer tests
 * for the mesh path (its only tests cover GLSL text surgery), and it cannot be
 * built here (Rust + wgpu + a graphics stack).  Parity of this oracle is
 * therefore UNPINNED against reference outputs; it is pinned instead against
 * analytic known answers (sphere / torus surface distance, closed-manifold
 * and Euler-characteristic checks) in tests/test_oracle.py.
 *
 * Two precisions: ORACLE_F32 follows the reference rule in IEEE binary32 with
 * no FMA contraction (built with -ffp-contract=off); ORACLE_F64 runs the same
 * rule in binary64 and serves as the accuracy yardstick.
 */
#ifndef S2M_ORACLE_H
#define S2M_ORACLE_H
#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* SDF fixtures restated by hand (independent of the product's frontend). */
enum {
  ORACLE_SDF_SPHERE = 0,     /* params: r                                          */
  ORACLE_SDF_TORUS = 1,      /* params: R, r          (sdf3d_torus(p, vec2(R, r)))  */
  ORACLE_SDF_CSG = 2,        /* params: box_full, box_round, torus_R, torus_r, k,
                                n, then n x (cx, cy, cz, radius)                    */
  ORACLE_SDF_MANDELBULB = 3, /* params: power, iterations, bailout, offset          */
  ORACLE_SDF_TREE = 4,       /* params: postfix CSG program, see s2m_oracle.cpp     */
  ORACLE_SDF_MARTIN_CUBE = 5,/* no params: the reference's examples/martin_cube.sdf3d */
  ORACLE_SDF_P_KEY = 6       /* no params: the reference's examples/p_key.sdf3d       */
};

enum { ORACLE_F32 = 0, ORACLE_F64 = 1 };

enum {
  ORACLE_FLAG_SLICE_LAG = 1, /* reproduce main.rs:324-355 (read-before-submit)      */
  ORACLE_FLAG_QEF = 2        /* precision mode: corners from the shared lattice, a
                                QEF vertex (normal-equation sums with Neumaier
                                compensation in the oracle's precision, 3x3 solve
                                in binary64); not a reference rule: the reference
                                places the mass point (dualcontour.wgsl:86-131) */
};

typedef struct {
  uint32_t resolution;  /* N cells per axis (already rounded if the caller wants) */
  float bounds;         /* cube edge B; the box is [-B/2, B/2]^3                  */
  float eps;            /* normal epsilon (1e-4 in the reference)                 */
  uint32_t flags;
  int32_t z_begin;      /* restrict cell slices to [z_begin, z_end); -1 = all     */
  int32_t z_end;
  int32_t threads;      /* OpenMP threads; 0 = library default                    */
  int32_t skip_quads;   /* 1 = vertices only                                      */
} oracle_params;

typedef struct {
  int64_t nverts;
  int64_t ntris;
  int64_t invalid_quads;
  /* exactly one of the f32 / f64 pairs is set, by precision */
  float *pos, *nrm;           /* 3 * nverts */
  double *pos64, *nrm64;      /* 3 * nverts */
  uint16_t *cell;             /* 3 * nverts : label (x, y, z) as in mesh.rs:214 */
  uint8_t *signs;             /* nverts: bit0 c100>0, bit1 c010>0, bit2 c001>0, bit3 c000>0 */
  uint32_t *tris;             /* 3 * ntris */
  double seconds_cells;       /* wall time of the cell pass      */
  double seconds_quads;       /* wall time of the quad assembly  */
} oracle_mesh;

int oracle_mesh_run(int sdf_kind, const float *sdf_params, int n_params,
                    int precision, const oracle_params *params, oracle_mesh *out);
void oracle_mesh_free(oracle_mesh *m);

/* Evaluate the fixture SDF at n points (xyz interleaved). */
int oracle_eval(int sdf_kind, const float *sdf_params, int n_params, int precision,
                const double *xyz, int64_t n, double *out);

/* The 8 corner values of one cell exactly as the reference computes them
   (dualcontour.wgsl:22-43), in the given precision, returned as doubles. */
int oracle_cell_corners(int sdf_kind, const float *sdf_params, int n_params, int precision,
                        uint32_t resolution, float bounds, int32_t x, int32_t y, int32_t z,
                        double *out8);

/* ASCII writers with Rust `{}` float formatting (mesh.rs:8-48, 50-141). */
int oracle_write_stl(const float *pos, const uint32_t *tris, int64_t ntris, const char *path);
int oracle_write_ply(const float *pos, const float *nrm, int64_t nverts,
                     const uint32_t *tris, int64_t ntris, const char *path);
/* Rust `{}` Display of one f32 into buf; returns the length. */
int oracle_format_f32(float v, char *buf, int buflen);

#ifdef __cplusplus
}
#endif
#endif
