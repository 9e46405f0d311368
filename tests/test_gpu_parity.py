"""GPU parity: the CUDA path through the C ABI against the CPU oracle.

Every case below runs libsdf2mesh_gb300.so on the GPU (NVRTC-compiled
evaluation + cell kernels, nvcc-compiled compaction and quad kernels) and the
oracle's restatement of the reference rule (dualcontour.wgsl:22-180,
main.rs:298-356, mesh.rs:213-331) on the same SDF, bounds and resolution.
SDFs built from correctly rounded operations must match bit for bit:
vertex cells, sign bits, positions, normals, triangle indices and the
invalid-quad count.
"""
from __future__ import annotations

import numpy as np
import pytest

import oracle
import sdf2mesh_gb300 as s2m
from sdf2mesh_gb300 import workloads
from tests.parity import assert_bit_exact, compare_with_ties, keys_of, same_bits

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torus_sdf(lib):
    src, prm = workloads.torus(0.5, 0.2)
    return s2m.Sdf3DShader.from_source(src).compile(), prm


def run(sdf, N, B=2.0, **kw):
    return s2m.generate(sdf, s2m.AppState(resolution=N, bounds=B, **kw))


def test_torus_128_plain(torus_sdf):
    sdf, prm = torus_sdf
    gpu = run(sdf, 128)
    ref = oracle.mesh(oracle.TORUS, prm, 128, 2.0)
    assert ref.nverts > 10000
    assert_bit_exact(gpu, ref, "torus 128")


def test_torus_reference_file(lib):
    """examples/torus.sdf3d text as the reference ships it, through the file path."""
    import os
    import tempfile
    d = tempfile.mkdtemp()
    p = os.path.join(d, "torus.sdf3d")
    with open(p, "w") as f:
        f.write("use sdf3d::*;\n\nfn sdf3d(p: vec3f) -> f32 {\n    return sdf3d_torus(p, vec2(0.5, 0.2));\n}\n")
    sdf = s2m.Sdf3DShader.from_path(p).compile()
    gpu = run(sdf, 64)
    ref = oracle.mesh(oracle.TORUS, [0.5, 0.2], 64, 2.0)
    assert_bit_exact(gpu, ref, "torus file 64")


@pytest.mark.parametrize("N", [2, 3, 5, 17, 33, 100])
def test_torus_odd_sizes(torus_sdf, N):
    sdf, prm = torus_sdf
    assert_bit_exact(run(sdf, N), oracle.mesh(oracle.TORUS, prm, N, 2.0), f"torus {N}")


def test_slice_lag_and_rounding(torus_sdf):
    """The reference CLI: pow2 rounding (96 -> 128) and the read-before-submit slice lag."""
    sdf, prm = torus_sdf
    gpu = s2m.generate(sdf, s2m.AppState.from_args(resolution=96, bounds=2.0))
    assert gpu.info.resolution == 128
    ref = oracle.mesh(oracle.TORUS, prm, 128, 2.0, slice_lag=True)
    assert_bit_exact(gpu, ref, "torus 96->128 lag")
    assert int(gpu.cell_xyz[:, 2].min()) >= 1


def test_slice_lag_surface_at_bounds(lib):
    """A box larger than the domain: the surface crosses the bounds, the lag
    drops slice 0's neighbours and the invalid-quad count must match."""
    src = "use sdf3d::*;\nfn sdf3d(p: vec3f) -> f32 {\n  return sdf3d_sphere(p - vec3f(0.0, 0.0, -0.9), 0.6);\n}\n"
    sdf = s2m.Sdf3DShader.from_source(src).compile()
    gpu = s2m.generate(sdf, s2m.AppState(resolution=64, bounds=2.0, slice_lag=True))
    # same SDF as a tree program: sphere at (0, 0, -0.9), r = 0.6
    ref = oracle.mesh(oracle.TREE, [0, 0.0, 0.0, -0.9, 0.6], 64, 2.0, slice_lag=True)
    assert ref.invalid_quads > 0
    assert_bit_exact(gpu, ref, "sphere at bounds, lag")


@pytest.mark.parametrize("depth", [1, 2, 5, 13, 64])
def test_slab_depth_invariance(torus_sdf, depth):
    sdf, prm = torus_sdf
    gpu = run(sdf, 72, slab_depth=depth)
    assert_bit_exact(gpu, oracle.mesh(oracle.TORUS, prm, 72, 2.0), f"slab depth {depth}")


def test_exact_corner_mode_matches(torus_sdf):
    sdf, prm = torus_sdf
    a = run(sdf, 80)
    b = run(sdf, 80, exact_corners=True)
    assert b.info.candidate_cells >= a.info.candidate_cells
    assert_bit_exact(b, oracle.mesh(oracle.TORUS, prm, 80, 2.0), "exact corners")


def test_overflow_regrow(torus_sdf):
    """Tiny initial capacities: the library regrows to the exact totals and re-runs."""
    sdf, prm = torus_sdf
    gpu = run(sdf, 96, max_vertices=100, max_triangles=100)
    assert_bit_exact(gpu, oracle.mesh(oracle.TORUS, prm, 96, 2.0), "regrow")


def test_empty_and_full(lib):
    for body, what in (("return -1.0;", "all inside"), ("return 1.0;", "all outside"),
                       ("return sdf3d_sphere(p, 0.001);", "sphere below one cell")):
        src = "use sdf3d::*;\nfn sdf3d(p: vec3f) -> f32 {\n  " + body + "\n}\n"
        gpu = run(s2m.Sdf3DShader.from_source(src).compile(), 32)
        assert gpu.positions.shape[0] == 0, what
        assert gpu.triangle_indices.shape[0] == 0, what


def test_zero_level_grid(lib):
    """f == 0 on lattice planes: `> 0` sign tests and the t == 0 crossing rule (dualcontour.wgsl:120)."""
    for n, d in (((1.0, 0.0, 0.0), 0.0), ((0.0, 1.0, 0.0), 0.25), ((0.0, 0.0, -1.0), 0.0),
                 ((0.6, 0.0, 0.8), 0.1)):
        src = ("fn sdf3d(p: vec3f) -> f32 {\n  return dot(p, vec3f(%r, %r, %r)) - %r;\n}\n" % (*n, d))
        gpu = run(s2m.Sdf3DShader.from_source(src).compile(), 17)
        ref = oracle.mesh(oracle.TREE, [4, *n, d], 17, 2.0)
        assert ref.nverts > 0
        assert_bit_exact(gpu, ref, f"plane {n} {d}")


def test_csg64_128(lib):
    src, prm = workloads.csg64(seed=0)
    sdf = s2m.Sdf3DShader.from_source(src).compile()
    gpu = run(sdf, 128)
    ref = oracle.mesh(oracle.CSG, prm, 128, 2.0)
    assert ref.nverts > 1000
    assert_bit_exact(gpu, ref, "csg64 128")


@pytest.mark.parametrize("seed", range(8))
def test_random_trees(lib, seed):
    src, prog = workloads.random_tree(seed)
    N = [48, 64, 96, 40][seed % 4]
    gpu = run(s2m.Sdf3DShader.from_source(src).compile(), N)
    ref = oracle.mesh(oracle.TREE, prog, N, 2.0)
    assert_bit_exact(gpu, ref, f"tree {seed}")


def test_mandelbulb_ties(lib):
    """Transcendentals differ in the last bits between CUDA and the host libm:
    topology must agree outside tie cells (some corner |f| <= 1e-5)."""
    src, prm = workloads.mandelbulb(8.0, 8, 2.0, 0.003)
    sdf = s2m.Sdf3DShader.from_source(src, s2m.LANG_GLSL, "sdf").compile()
    N, B = 96, 2.5
    gpu = run(sdf, N, B)
    ref = oracle.mesh(oracle.MANDELBULB, prm, N, B)
    assert ref.nverts > 1000
    h = B / (N - 1)
    r = compare_with_ties(gpu, ref, oracle.MANDELBULB, prm, N, B, eps=1e-5, h=h)
    assert r["tri_diff_unexplained"] == 0, r
    assert r["vertex_only_one_side"] <= max(5, ref.nverts // 1000), r


def test_csg64_1024_full_size(lib, oracle_lib):
    """Full-size CSG (1024^3).  (1) The GPU's vertices of a window of slices
    equal the oracle's for the same window, bit for bit.  (2) The triangles
    are exactly the reference quad rule applied to the GPU's vertex list.
    (3) Every invalid quad (a hole of the reference rule) looks for a vertex
    that the oracle does not produce either."""
    from tests.parity import reference_quads
    src, prm = workloads.csg64(seed=0)
    sdf = s2m.Sdf3DShader.from_source(src).compile()
    N = 1024
    gpu = run(sdf, N)
    z = gpu.cell_xyz[:, 2]

    def window_matches(z0, z1):
        ref = oracle.mesh(oracle.CSG, prm, N, 2.0, z_begin=z0, z_end=z1, skip_quads=True)
        sel = (z >= z0) & (z < z1)
        assert int(sel.sum()) == ref.nverts
        assert np.array_equal(gpu.cell_xyz[sel], ref.cell)
        assert np.array_equal(gpu.signs[sel], ref.signs)
        assert np.array_equal(gpu.positions[sel].view(np.uint32), ref.pos.astype(np.float32).view(np.uint32))
        assert same_bits(gpu.normals[sel], ref.nrm).all()
        return ref

    assert window_matches(500, 503).nverts > 0
    tris, invalid, missing = reference_quads(gpu.cell_xyz, gpu.signs)
    assert invalid == gpu.invalid_quads
    assert np.array_equal(tris, gpu.triangle_indices)
    # keys sorted (z, y, x) like the reference's VertexList
    k = keys_of(gpu.cell_xyz)
    assert (np.diff(k.astype(np.int64)) > 0).all()
    for zz in sorted(set(int(v) for v in missing[:, 2]))[:4]:
        window_matches(max(0, zz - 1), min(N, zz + 2))


def test_custom_normal_function(lib, oracle_lib):
    """A user-defined sdf3d_normal is what the kernel calls (dualcontour.wgsl:170):
    positions still match the oracle bit for bit, normals are the custom
    central difference, normalised."""
    custom = ("use sdf3d::primitives;\n"
              "fn sdf3d_normal(p: vec3f, eps: f32) -> vec3f {\n"
              "  let h = vec3f(eps, 0.0, 0.0);\n"
              "  return vec3f(sdf3d(p + h.xyy) - sdf3d(p - h.xyy), sdf3d(p + h.yxy) - sdf3d(p - h.yxy),\n"
              "               sdf3d(p + h.yyx) - sdf3d(p - h.yyx));\n}\n"
              "fn sdf3d(p: vec3f) -> f32 { return sdf3d_sphere(p, 0.5); }\n")
    gpu = run(s2m.Sdf3DShader.from_source(custom).compile(), 48)
    ref = oracle.mesh(oracle.SPHERE, [0.5], 48, 2.0)
    assert np.array_equal(gpu.cell_xyz, ref.cell)
    assert np.array_equal(gpu.positions.view(np.uint32), ref.pos.astype(np.float32).view(np.uint32))
    radial = ref.pos / np.linalg.norm(ref.pos, axis=1, keepdims=True)
    assert (np.sum(gpu.normals * radial, axis=1) > 0.999).all()


@pytest.fixture(scope="module")
def csg64_seed1(lib):
    src, prm = workloads.csg64(seed=1)
    return s2m.Sdf3DShader.from_source(src).compile(), prm


@pytest.fixture(scope="module")
def csg64_seed1_full(lib):
    src, prm = workloads.csg64(seed=1)
    return s2m.Sdf3DShader.from_source(src).compile(prune=False), prm


@pytest.mark.parametrize("variant", range(s2m.EVAL_VARIANTS))
def test_eval_variants_identical(csg64_seed1, csg64_seed1_full, variant):
    """Every evaluation-kernel variant the autotuner may pick (5 to 7: tile
    pruned) gives the same bits.  The full-evaluation run-of-4 variants (3, 4)
    are compiled only into modules without pruning."""
    sdf, prm = csg64_seed1_full if variant in (3, 4) else csg64_seed1
    sdf.set_eval_variant(variant)
    gpu = run(sdf, 96)
    assert sdf.eval_variant()[0] == sdf.eval_variants()[variant][0]
    assert_bit_exact(gpu, oracle.mesh(oracle.CSG, prm, 96, 2.0), f"variant {variant}")


def test_autotuner_picks_a_variant(lib):
    src, _ = workloads.csg64(seed=0)
    sdf = s2m.Sdf3DShader.from_source(src).compile()
    assert sdf.eval_variant()[0] == "untuned"
    run(sdf, 512)  # large enough for the tuner to time (>= 2e6 points per trial)
    name, ns = sdf.eval_variant()
    # every variant of the module was timed; a pruned module holds no
    # full-evaluation run-of-4 variants (3, 4)
    assert name.startswith("s2m_eval") and all(x > 0 for v, x in enumerate(ns) if v not in (3, 4))
    assert ns[3] == 0 and ns[4] == 0


# ---------------------------------------------------------------------------
# Precision mode (S2M_JOB_QEF): lattice corners, QEF vertex, FP32 compensated
# sums, FP64 solve.  The oracle's binary32 build runs the same arithmetic, so
# correctly rounded SDFs match it bit for bit; the all-binary64 oracle is the
# accuracy yardstick: topology equal outside tie cells and every common vertex
# within QEF_TOL_CELLS cell sizes.
QEF_TOL_CELLS = 1e-3


@pytest.mark.parametrize("case", ["torus64", "torus128", "csg96", "tree2", "tree3", "tree7"])
def test_qef_bit_exact_with_oracle(lib, case):
    if case.startswith("torus"):
        src, prm = workloads.torus()
        kind, N = oracle.TORUS, int(case[5:])
    elif case == "csg96":
        src, prm = workloads.csg64(seed=0)
        kind, N = oracle.CSG, 96
    else:
        src, prm = workloads.random_tree(int(case[4:]))
        kind, N = oracle.TREE, 64
    gpu = run(s2m.Sdf3DShader.from_source(src).compile(), N, qef=True)
    ref = oracle.mesh(kind, prm, N, 2.0, qef=True)
    assert ref.nverts > 100
    assert_bit_exact(gpu, ref, f"qef {case}")


def test_qef_against_fp64_oracle(lib):
    src, prm = workloads.csg64(seed=0)
    N = 128
    gpu = run(s2m.Sdf3DShader.from_source(src).compile(), N, qef=True)
    ref = oracle.mesh(oracle.CSG, prm, N, 2.0, qef=True, precision=oracle.F64)
    h = 2.0 / (N - 1)
    r = compare_with_ties(gpu, ref, oracle.CSG, prm, N, 2.0, eps=1e-6, h=h)
    assert r["tri_diff_unexplained"] == 0, r
    assert r["max_pos_err_cells"] < QEF_TOL_CELLS, r


def test_qef_mandelbulb_vs_fp64(lib):
    src, prm = workloads.mandelbulb(8.0, 8, 2.0, 0.003)
    N, B = 96, 2.5
    gpu = run(s2m.Sdf3DShader.from_source(src, s2m.LANG_GLSL, "sdf").compile(), N, B, qef=True)
    ref = oracle.mesh(oracle.MANDELBULB, prm, N, B, qef=True, precision=oracle.F64)
    r = compare_with_ties(gpu, ref, oracle.MANDELBULB, prm, N, B, eps=1e-5, h=B / (N - 1))
    assert r["tri_diff_unexplained"] == 0, r
    assert r["vertex_only_one_side"] <= max(5, ref.nverts // 1000), r


def test_qef_1024_watertight(lib):
    """Precision mode closes the reference rule's holes: at 1024^3 the CSG mesh
    has no invalid quad and every edge is shared by exactly two triangles."""
    from tests.parity import reference_quads
    src, _ = workloads.csg64(seed=0)
    gpu = run(s2m.Sdf3DShader.from_source(src).compile(), 1024, qef=True)
    assert gpu.invalid_quads == 0
    tris, invalid, _ = reference_quads(gpu.cell_xyz, gpu.signs)
    assert invalid == 0 and np.array_equal(tris, gpu.triangle_indices)
    t = gpu.triangle_indices.astype(np.int64)
    e = np.concatenate([t[:, [0, 1]], t[:, [1, 2]], t[:, [2, 0]]])
    e.sort(axis=1)
    _, counts = np.unique(e[:, 0] * np.int64(1 << 32) + e[:, 1], return_counts=True)
    assert (counts == 2).all()


def test_graph_replay_identical(lib):
    """s2m_mesh_run_async replaying the captured CUDA graph gives the same bits."""
    src, prm = workloads.csg64(seed=2)
    sdf = s2m.Sdf3DShader.from_source(src).compile()
    dm = s2m.mesh_device(sdf, s2m.AppState(resolution=80, bounds=2.0))
    first = dm.to_host()
    dm.set_graph(True)
    for _ in range(3):
        dm.run_async()
        dm.sync()
    again = dm.to_host()
    dm.close()
    assert_bit_exact(again, oracle.mesh(oracle.CSG, prm, 80, 2.0), "graph replay")
    assert np.array_equal(first.triangle_indices, again.triangle_indices)


# Error of the binary32 reference rule against the same rule in binary64:
# topology equal outside tie cells (a corner within 1e-6 of zero), common
# vertices within REF_RULE_TOL_CELLS cell sizes.
REF_RULE_TOL_CELLS = 5e-4  # measured 8.6e-5 on these cases


@pytest.mark.parametrize("case", ["torus128", "csg128"])
def test_reference_rule_against_fp64_oracle(lib, case):
    if case == "torus128":
        src, prm = workloads.torus()
        kind = oracle.TORUS
    else:
        src, prm = workloads.csg64(seed=0)
        kind = oracle.CSG
    N = 128
    gpu = run(s2m.Sdf3DShader.from_source(src).compile(), N)
    ref = oracle.mesh(kind, prm, N, 2.0, precision=oracle.F64)
    r = compare_with_ties(gpu, ref, kind, prm, N, 2.0, eps=1e-6, h=2.0 / (N - 1))
    assert r["tri_diff_unexplained"] == 0, r
    assert r["max_pos_err_cells"] < REF_RULE_TOL_CELLS, r
