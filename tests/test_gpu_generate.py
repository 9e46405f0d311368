"""One call to a host mesh (s2m_mesh_generate) in z parts.

A job split into parts along z (each later part also meshing the cell plane
below it, for its quads, and copying none of it) must give exactly the mesh of
the one-piece path: s2m_mesh_create + s2m_mesh_copy_to_host, itself
bit-identical to the oracle.  Positions, normals, triangle indices (with their
offsets across parts) and the invalid-quad count are compared bit for bit, in
both rules, with the slice lag, and for part boundaries that fall anywhere."""
from __future__ import annotations

import numpy as np
import pytest

import oracle
import sdf2mesh_gb300 as s2m
from sdf2mesh_gb300 import workloads
from tests.parity import assert_bit_exact

pytestmark = pytest.mark.gpu


def same(a, b, what):
    assert a.positions.shape == b.positions.shape, (what, a.positions.shape, b.positions.shape)
    assert np.array_equal(a.positions.view(np.uint32), b.positions.view(np.uint32)), what
    assert np.array_equal(a.normals.view(np.uint32), b.normals.view(np.uint32)), what
    assert np.array_equal(a.triangle_indices, b.triangle_indices), what
    assert a.invalid_quads == b.invalid_quads, what


@pytest.fixture(scope="module")
def csg(lib):
    src, prm = workloads.csg64(seed=0)
    return s2m.Sdf3DShader.from_source(src).compile(), prm


@pytest.mark.parametrize("N,parts,kw", [(96, 2, {}), (97, 3, {}), (128, 4, {"slice_lag": True}),
                                        (200, 2, {"qef": True}), (256, 5, {}), (512, 2, {}), (512, 0, {}),
                                        (160, 2, {"reference_rounding": True, "slice_lag": True})])
def test_parts_equal_one_piece(csg, N, parts, kw):
    sdf, _ = csg
    st = s2m.AppState(resolution=N, bounds=2.0, **kw)
    one = s2m.generate(sdf, st)  # also tunes the SDF's evaluation on its first job
    got = s2m.generate_host(sdf, st, parts=parts)
    if parts:
        assert got.info["parts"] == min(parts, max(1, (one.info.resolution - (1 if kw.get("slice_lag") else 0)) // 16))
    same(got, one, f"N={N} parts={parts} {kw}")


def test_parts_against_oracle(lib):
    src, prm = workloads.torus()
    sdf = s2m.Sdf3DShader.from_source(src).compile()
    s2m.generate(sdf, s2m.AppState(resolution=64, bounds=2.0))
    got = s2m.generate_host(sdf, s2m.AppState(resolution=120, bounds=2.0), parts=3)
    assert got.info["parts"] == 3
    ref = oracle.mesh(oracle.TORUS, prm, 120, 2.0)
    assert got.positions.shape[0] == ref.nverts
    assert np.array_equal(got.positions.view(np.uint32), np.asarray(ref.pos, np.float32).view(np.uint32))
    assert np.array_equal(got.normals.view(np.uint32), np.asarray(ref.nrm, np.float32).view(np.uint32))
    assert np.array_equal(got.triangle_indices, ref.tris)
    assert got.invalid_quads == ref.invalid_quads


def test_part_overflow_falls_back_to_one_piece(csg):
    """Capacities too small for a part: the call meshes the job again in one
    piece (which grows its buffers to the exact totals), with the same result."""
    sdf, _ = csg
    st = s2m.AppState(resolution=160, bounds=2.0, max_vertices=4096, max_triangles=8192)
    one = s2m.generate(sdf, s2m.AppState(resolution=160, bounds=2.0))
    got = s2m.generate_host(sdf, st, parts=2)
    same(got, one, "overflow fallback")
    assert got.info["parts"] == 1
