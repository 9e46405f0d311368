"""Tile-pruned lattice evaluation on the GPU.

The pruned variants evaluate, per tile of 8 x 8 x <= 8 lattice points, only
the operations that the tile pass did not prove irrelevant.  Their meshes
must be bit-identical to those of the full evaluation (every operation at
every point) and to the oracle: vertex cells, sign bits, positions, normals,
triangles and invalid-quad counts.
"""
from __future__ import annotations

import numpy as np
import pytest

import oracle
import sdf2mesh_gb300 as s2m
from sdf2mesh_gb300 import workloads
from tests.parity import assert_bit_exact
from tests.test_prune_host import EDGE, SMOOTH_OPS

pytestmark = pytest.mark.gpu

PRUNED = (5, 6, 7)  # s2m_evalp_b8, s2m_evalpl_b8, s2m_evalpl_b8v4 (undecided tiles listed)
PLAIN = 1        # s2m_eval_b3r4


def same_mesh(a, b, what):
    assert a.invalid_quads == b.invalid_quads, what
    assert np.array_equal(a.cells, b.cells), what
    assert np.array_equal(a.positions.view(np.uint32), b.positions.view(np.uint32)), what
    assert np.array_equal(a.normals.view(np.uint32), b.normals.view(np.uint32)), what
    assert np.array_equal(a.triangle_indices, b.triangle_indices), what


def pair(src, lang=s2m.LANG_WGSL, name="sdf"):
    sh = s2m.Sdf3DShader.from_source(src, lang, name)
    return sh.compile(), sh.compile(prune=False)


def mesh(sdf, N, variant, **kw):
    sdf.set_eval_variant(variant)
    m = s2m.mesh_device(sdf, s2m.AppState(resolution=N, **kw))
    try:
        return m.to_host(), m.eval_ops()
    finally:
        m.close()


@pytest.fixture(scope="module")
def csg64(lib):
    src, prm = workloads.csg64(seed=0)
    pruned, plain = pair(src)
    return pruned, plain, prm


def test_prune_info(csg64):
    pruned, plain, _ = csg64
    comb, words = pruned.prune_info()
    assert comb >= 64 and words == (2 * comb + 31) // 32
    assert plain.prune_info() == (0, 0)
    with pytest.raises(s2m.S2MError):
        plain.set_eval_variant(PRUNED[0])


@pytest.mark.parametrize("N", [33, 100, 256, 512])
def test_csg64_pruned_equals_full(csg64, N):
    pruned, plain, prm = csg64
    full, ops_full = mesh(plain, N, PLAIN)
    assert not ops_full["pruned"]
    for v in PRUNED:
        got, ops = mesh(pruned, N, v)
        same_mesh(got, full, f"csg64 N={N} variant {v}")
        assert ops["pruned"] and ops["points"] == ops_full["points"]
        assert 0 < ops["fp32_ops"] < ops_full["fp32_ops"]
    if N <= 100:
        assert_bit_exact(got, oracle.mesh(oracle.CSG, prm, N, 2.0), f"csg64 N={N} pruned vs oracle")


def test_csg64_1024_pruned_equals_full(csg64):
    """The headline job: bit-identical mesh, and the tile pass leaves a small
    fraction of the SDF's operations to evaluate."""
    pruned, plain, _ = csg64
    full, ops_full = mesh(plain, 1024, PLAIN)
    got, ops = mesh(pruned, 1024, PRUNED[0])
    same_mesh(got, full, "csg64 1024")
    assert ops["fp32_ops"] < 0.1 * ops_full["fp32_ops"]


@pytest.mark.parametrize("depth", [1, 3, 13])
def test_slab_depths(csg64, depth):
    """Tiles are cut per slab (tile depth <= 8, balanced): every slab depth
    gives the same mesh."""
    pruned, plain, _ = csg64
    full, _ = mesh(plain, 130, PLAIN)
    got, _ = mesh(pruned, 130, PRUNED[0], slab_depth=depth)
    same_mesh(got, full, f"slab depth {depth}")


@pytest.mark.parametrize("seed", range(8))
def test_random_trees_pruned(lib, seed):
    src, prog = workloads.random_tree(seed)
    pruned, plain = pair(src)
    assert pruned.prune_info()[1] > 0  # every straight-line SDF has the tile form
    N = [48, 64, 96, 40][seed % 4]
    got, _ = mesh(pruned, N, PRUNED[0])
    assert_bit_exact(got, oracle.mesh(oracle.TREE, prog, N, 2.0), f"tree {seed} pruned")
    full, _ = mesh(plain, 200, PLAIN)
    got, _ = mesh(pruned, 200, PRUNED[1])
    same_mesh(got, full, f"tree {seed} N=200")


@pytest.mark.parametrize("name,src,N", [("smooth", SMOOTH_OPS, 160), ("edge", EDGE, 64)])
def test_operators_and_edge_cases(lib, name, src, N):
    pruned, plain = pair(src)
    assert pruned.prune_info()[0] > 0
    full, _ = mesh(plain, N, PLAIN)
    for v in PRUNED:
        got, _ = mesh(pruned, N, v)
        same_mesh(got, full, f"{name} variant {v}")


def test_fmad_turns_pruning_off(lib):
    src, _ = workloads.csg64(seed=0)
    assert s2m.Sdf3DShader.from_source(src).compile(fmad=True).prune_info() == (0, 0)


@pytest.mark.parametrize("mode", ["qef", "exact_corners", "reference_cli"])
def test_job_modes_pruned_equals_full(csg64, mode):
    """Precision mode, exact off-lattice corners and the reference CLI's
    rounding and slice lag run the same lattice through the pruned kernels."""
    pruned, plain, _ = csg64
    kw = {"qef": dict(qef=True), "exact_corners": dict(exact_corners=True),
          "reference_cli": dict(reference_rounding=True, slice_lag=True)}[mode]
    N = 150
    full, _ = mesh(plain, N, PLAIN, **kw)
    for v in PRUNED:
        got, ops = mesh(pruned, N, v, **kw)
        assert ops["pruned"]
        same_mesh(got, full, f"{mode} variant {v}")


@pytest.mark.parametrize("kind", ["torus", "sphere"])
def test_tile_form_without_combinators(lib, kind):
    """No combinator to prune: only the decided tiles far from the surface
    skip evaluation, and the mesh is bit-identical."""
    src = getattr(workloads, kind)()[0]
    pruned, plain = pair(src)
    assert pruned.prune_info() == (0, 1)
    full, ops_full = mesh(plain, 200, PLAIN)
    for v in PRUNED:
        got, ops = mesh(pruned, 200, v)
        same_mesh(got, full, f"{kind} variant {v}")
        assert ops["fp32_ops"] < 0.5 * ops_full["fp32_ops"]
