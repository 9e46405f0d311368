"""Known-answer tests of the CPU oracle (the checker of every GPU parity test).

The reference ships no golden meshes, so the oracle is pinned here by
analytic facts of the reference rule (dualcontour.wgsl:22-180,
mesh.rs:213-331): vertices of a sphere / torus lie within a cell of the true
surface, the mesh is a closed, consistently oriented 2-manifold with the
right Euler characteristic, the slice lag relabels slices, and the text
writers follow Rust's `{}` float Display (mesh.rs:8-141).
"""
from __future__ import annotations

import math
import os

import numpy as np
import pytest

import oracle


def edges_of(tris):
    t = np.asarray(tris, np.int64)
    e = np.concatenate([t[:, [0, 1]], t[:, [1, 2]], t[:, [2, 0]]])
    return e


def manifold_stats(m):
    e = edges_of(m.tris)
    und = np.sort(e, axis=1)
    code = und[:, 0] * (1 << 32) + und[:, 1]
    uniq, counts = np.unique(code, return_counts=True)
    # consistent orientation: each directed edge appears once
    dcode = e[:, 0] * (1 << 32) + e[:, 1]
    directed_unique = np.unique(dcode).size == dcode.size
    used = np.unique(np.asarray(m.tris).ravel()).size
    return {"E": uniq.size, "counts": counts, "oriented": directed_unique, "V_used": used, "F": len(m.tris)}


@pytest.mark.parametrize("N", [24, 33, 64])
def test_sphere_known_answers(oracle_lib, N):
    r = 0.6
    m = oracle.mesh(oracle.SPHERE, [r], N, 2.0)
    h = 2.0 / (N - 1)
    d = np.abs(np.linalg.norm(m.pos.astype(np.float64), axis=1) - r)
    assert d.max() < 0.5 * h
    s = manifold_stats(m)
    assert (s["counts"] == 2).all()
    assert s["oriented"]
    assert m.invalid_quads == 0
    # Euler characteristic of a sphere (every vertex is used by a triangle)
    assert s["V_used"] == m.nverts
    assert m.nverts - s["E"] + s["F"] == 2
    # unit normals pointing outward
    n = m.nrm.astype(np.float64)
    assert np.allclose(np.linalg.norm(n, axis=1), 1.0, atol=1e-6)
    radial = m.pos / np.linalg.norm(m.pos, axis=1, keepdims=True)
    assert (np.sum(n * radial, axis=1) > 0.99).all()


def test_torus_known_answers(oracle_lib):
    N, R, r = 128, 0.5, 0.2
    m = oracle.mesh(oracle.TORUS, [R, r], N, 2.0)
    h = 2.0 / (N - 1)
    p = m.pos.astype(np.float64)
    q = np.sqrt(p[:, 0] ** 2 + p[:, 2] ** 2) - R
    d = np.abs(np.sqrt(q ** 2 + p[:, 1] ** 2) - r)
    assert d.max() < 0.5 * h
    s = manifold_stats(m)
    assert (s["counts"] == 2).all() and s["oriented"]
    assert m.nverts - s["E"] + s["F"] == 0          # genus 1
    area = 4 * math.pi ** 2 * R * r
    assert 1.0 < m.nverts / (area / h ** 2) < 2.0   # one vertex per surface cell, roughly
    assert m.ntris == 2 * s["F"] // 2


def test_facet_orientation_outward(oracle_lib):
    """Triangles (q2, q1, q0), (q0, q3, q2) after Quad::swap (lib.rs:190-211):
    the STL facet normal (v2 - v0) x (v1 - v0) (lib.rs:181-185) points one way
    consistently; for a sphere, outward."""
    m = oracle.mesh(oracle.SPHERE, [0.5], 40, 2.0)
    p = m.pos.astype(np.float64)
    t = m.tris.astype(np.int64)
    a, b, c = p[t[:, 0]], p[t[:, 1]], p[t[:, 2]]
    n = np.cross(c - a, b - a)
    centre = (a + b + c) / 3
    s = np.sign(np.sum(n * centre, axis=1))
    assert abs(s.sum()) == len(s)


def test_slice_lag_relabels(oracle_lib):
    """main.rs:324-355: iteration z reads slice z - 1; the last slice never surfaces."""
    N = 40
    plain = oracle.mesh(oracle.TORUS, [0.5, 0.2], N, 2.0)
    lag = oracle.mesh(oracle.TORUS, [0.5, 0.2], N, 2.0, slice_lag=True)
    keep = plain.cell[:, 2] < N - 1
    assert lag.nverts == int(keep.sum())
    shifted = plain.cell[keep].copy()
    shifted[:, 2] += 1
    assert np.array_equal(lag.cell, shifted)
    assert np.array_equal(lag.pos, plain.pos[keep])


def test_f64_oracle_close_to_f32(oracle_lib):
    N = 64
    a = oracle.mesh(oracle.TORUS, [0.5, 0.2], N, 2.0)
    b = oracle.mesh(oracle.TORUS, [0.5, 0.2], N, 2.0, precision=oracle.F64)
    assert np.array_equal(a.cell, b.cell)
    h = 2.0 / (N - 1)
    assert np.abs(a.pos - b.pos).max() < 1e-4 * h


def test_cell_corners_match_rule(oracle_lib):
    """Corner coordinates mn = bmin + size * pos, mx = mn + size (dualcontour.wgsl:22-27)."""
    N, B = 10, 2.0
    c = oracle.cell_corners(oracle.TREE, [4, 1.0, 0.0, 0.0, 0.0], N, B, 3, 0, 0)
    size = np.float32(np.float32(1.0) - np.float32(-1.0)) / np.float32(N - 1)
    mn = np.float32(-1.0) + size * np.float32(3)
    mx = np.float32(mn + size)
    assert c[0] == float(mn) and c[1] == float(mx)


@pytest.mark.parametrize("v,s", [(0.5, "0.5"), (1.0, "1"), (-0.0, "-0"), (0.0, "0"), (1e-7, "0.0000001"),
                                 (123456789.0, "123456790"), (0.1, "0.1"), (1.0 / 3.0, "0.33333334"),
                                 (-2.5, "-2.5"), (1e20, "100000000000000000000"), (float("nan"), "NaN"),
                                 (float("inf"), "inf"), (float("-inf"), "-inf"), (3.4028235e38,
                                 "340282350000000000000000000000000000000"), (1.4e-45, "0." + "0" * 44 + "1")])
def test_rust_display_f32(oracle_lib, v, s):
    assert oracle.format_f32(v) == s


def test_stl_and_ply_text(oracle_lib, tmp_path):
    pos = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32)
    nrm = np.array([[0, 0, 1]] * 3, np.float32)
    tris = np.array([[0, 1, 2]], np.uint32)
    p = os.fspath(tmp_path / "t.stl")
    oracle.write_stl(pos, tris, p)
    assert open(p).read() == ("solid\nfacet normal 0 0 -1\n\touter loop\n\t\tvertex 0 0 0\n\t\tvertex 1 0 0\n"
                              "\t\tvertex 0 1 0\n\tendloop\nendfacet\nendsolid\n")
    q = os.fspath(tmp_path / "t.ply")
    oracle.write_ply(pos, nrm, tris, q)
    text = open(q).read().splitlines()
    assert text[:3] == ["ply", "format ascii 1.0", "comment written by rust-sdf"]
    assert "element vertex 3" in text and "element face 1" in text and "end_header" in text
    assert text[-1] == "3 0 1 2"
    assert text[-4] == "0 0 0 0 0 1"


@pytest.mark.parametrize("case", ["torus", "torus_lag", "sphere_at_bounds_lag", "tree3"])
def test_numpy_quad_rule_matches_oracle(oracle_lib, case):
    """tests.parity.reference_quads (used at full size on the GPU's vertex list)
    reproduces the oracle's triangles and invalid-quad count exactly."""
    from sdf2mesh_gb300 import workloads
    from tests.parity import reference_quads
    if case == "torus":
        m = oracle.mesh(oracle.TORUS, [0.5, 0.2], 64, 2.0)
    elif case == "torus_lag":
        m = oracle.mesh(oracle.TORUS, [0.5, 0.2], 64, 2.0, slice_lag=True)
    elif case == "sphere_at_bounds_lag":
        m = oracle.mesh(oracle.TREE, [0, 0.0, 0.0, -0.9, 0.6], 64, 2.0, slice_lag=True)
    else:
        m = oracle.mesh(oracle.TREE, workloads.random_tree(3)[1], 48, 2.0)
    tris, invalid, _ = reference_quads(m.cell, m.signs)
    assert invalid == m.invalid_quads
    assert np.array_equal(tris, m.tris)


@pytest.mark.parametrize("N", [32, 96])
def test_qef_precision_mode_known_answers(oracle_lib, N):
    """Precision mode: lattice corners (neighbours agree), QEF vertex with a
    binary64 solve.  Closed, oriented torus (genus 1), vertices within a cell
    of the analytic surface and no farther than the mass point's, binary32
    sums within 1e-3 cells of the all-binary64 rule."""
    R, r = 0.5, 0.2
    a = oracle.mesh(oracle.TORUS, [R, r], N, 2.0, qef=True)
    b = oracle.mesh(oracle.TORUS, [R, r], N, 2.0, qef=True, precision=oracle.F64)
    mp = oracle.mesh(oracle.TORUS, [R, r], N, 2.0)
    h = 2.0 / (N - 1)

    def dist(p):
        p = p.astype(np.float64)
        q = np.sqrt(p[:, 0] ** 2 + p[:, 2] ** 2) - R
        return np.abs(np.sqrt(q ** 2 + p[:, 1] ** 2) - r)

    assert dist(a.pos).max() < 0.25 * h
    assert dist(a.pos).max() <= dist(mp.pos).max() * 1.05
    s = manifold_stats(a)
    assert (s["counts"] == 2).all() and s["oriented"] and a.invalid_quads == 0
    assert a.nverts - s["E"] + s["F"] == 0
    assert np.array_equal(a.cell, b.cell)
    assert np.abs(a.pos - b.pos).max() < 1e-3 * h
