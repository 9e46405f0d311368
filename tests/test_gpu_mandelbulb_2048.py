"""The Mandelbulb at full size: power 8, 8 iterations, bailout 2, bounds 2.5,
2048^3 cells (the resolution above which the reference crashes,
README.md:131, main.rs:190), in the reference rule and in precision mode.

CUDA's transcendentals and the host libm differ in the last bits, and the
iteration amplifies those differences near the fractal's escape boundary.
So a cell whose reference corners include one that binary32 does not pin
down (within 1e-5 of zero, or more than 1e-5 from its binary64 value: a
"tie cell") may flip; everything else must match the oracle.  Positions are
held to the accuracy a binary32 implementation of the same rule can have:
the GPU's distance to the binary64 oracle must be no worse than the CPU
binary32 oracle's own distance to it (median, 99th percentile, maximum),
within a small slack.  At this size the oracle runs on windows of slices:
  (1) the GPU's vertices of a window of slices against the oracle's meshes of
      the same window (binary32 for topology, binary64 for accuracy);
  (2) the whole triangle list equals the reference quad rule
      (mesh.rs:267-331) applied to the GPU's sorted vertex list;
  (3) reference rule: the slices around every invalid quad (a hole of the
      rule) are compared too; precision mode: no invalid quad and no boundary
      edge (closed).
"""
from __future__ import annotations

import numpy as np
import pytest

import oracle
import sdf2mesh_gb300 as s2m
from sdf2mesh_gb300 import workloads
from tests.parity import compare_window_with_ties, keys_of, reference_quads_chunked

pytestmark = pytest.mark.gpu

N, B = 2048, 2.5
H = B / (N - 1)
TIE_EPS = 1e-5
WINDOW = (1023, 1026)  # cell slices through the middle of the bulb


@pytest.fixture(scope="module")
def mandel(lib):
    src, prm = workloads.mandelbulb(8.0, 8, 2.0, 0.003)
    return s2m.Sdf3DShader.from_source(src, s2m.LANG_GLSL, "sdf").compile(), prm


def window(gpu, z0, z1):
    z = gpu.cell_xyz[:, 2]
    sel = (z >= z0) & (z < z1)
    return s2m.TriangleMesh(gpu.positions[sel], gpu.normals[sel], np.zeros((0, 3), np.uint32), gpu.cells[sel])


def check_window(gpu, prm, z0, z1, **kw):
    ref = oracle.mesh(oracle.MANDELBULB, prm, N, B, z_begin=z0, z_end=z1, skip_quads=True, **kw)
    assert ref.nverts > 1000
    r = compare_window_with_ties(window(gpu, z0, z1), ref, oracle.MANDELBULB, prm, N, B, TIE_EPS, H)
    assert r["vertex_only_one_side"] <= max(5, r["vertices"] // 1000), r
    return r


def check_triangles(gpu):
    tris, invalid, missing = reference_quads_chunked(gpu.cell_xyz, gpu.signs)
    assert invalid == gpu.invalid_quads
    assert np.array_equal(tris, gpu.triangle_indices)
    k = keys_of(gpu.cell_xyz)
    assert (np.diff(k.astype(np.int64)) > 0).all(), "vertex list sorted (z, y, x) like the reference's VertexList"
    return missing


def accuracy(gpu, prm, z0, z1, qef):
    """Distances (in cells) of the GPU's and of the CPU binary32 oracle's
    vertices to the binary64 oracle's, over the vertex cells all three share."""
    g = window(gpu, z0, z1)
    r32 = oracle.mesh(oracle.MANDELBULB, prm, N, B, z_begin=z0, z_end=z1, skip_quads=True, qef=qef)
    r64 = oracle.mesh(oracle.MANDELBULB, prm, N, B, z_begin=z0, z_end=z1, skip_quads=True, qef=qef,
                      precision=oracle.F64)
    gk, k32, k64 = keys_of(g.cell_xyz), keys_of(r32.cell), keys_of(r64.cell)
    common = np.intersect1d(np.intersect1d(gk, k32), k64)
    p64 = np.asarray(r64.pos, np.float64)[np.searchsorted(k64, common)]
    e_gpu = np.abs(g.positions[np.searchsorted(gk, common)].astype(np.float64) - p64).max(axis=1) / H
    e_cpu = np.abs(np.asarray(r32.pos, np.float64)[np.searchsorted(k32, common)] - p64).max(axis=1) / H
    q = lambda e: {"p50": float(np.median(e)), "p99": float(np.quantile(e, 0.99)), "max": float(e.max())}
    out = {"vertices": int(common.size), "gpu_vs_fp64": q(e_gpu), "cpu_f32_vs_fp64": q(e_cpu)}
    print(f"mandelbulb 2048^3 {'precision' if qef else 'reference rule'} window {z0}..{z1}: {out}")
    return out


def check_accuracy(a, slack):
    g, c = a["gpu_vs_fp64"], a["cpu_f32_vs_fp64"]
    for k in ("p50", "p99", "max"):
        assert g[k] <= 2.0 * c[k] + slack[k], (k, a)


def test_mandelbulb_2048_reference_rule(mandel):
    sdf, prm = mandel
    gpu = s2m.generate(sdf, s2m.AppState(resolution=N, bounds=B))
    assert gpu.positions.shape[0] > 10 ** 6
    check_window(gpu, prm, *WINDOW)
    a = accuracy(gpu, prm, *WINDOW, qef=False)
    check_accuracy(a, {"p50": 1e-5, "p99": 1e-4, "max": 1e-2})
    missing = check_triangles(gpu)
    for zz in sorted(set(int(v) for v in missing[:, 2]))[:3]:
        check_window(gpu, prm, max(0, zz - 1), min(N, zz + 2))


def test_mandelbulb_2048_precision(mandel):
    sdf, prm = mandel
    gpu = s2m.generate(sdf, s2m.AppState(resolution=N, bounds=B, qef=True))
    assert gpu.positions.shape[0] > 10 ** 6
    check_window(gpu, prm, *WINDOW, qef=True)  # topology against the binary32 build of the same arithmetic
    a = accuracy(gpu, prm, *WINDOW, qef=True)
    check_accuracy(a, {"p50": 1e-5, "p99": 1e-3, "max": 5e-2})
    check_triangles(gpu)
    assert gpu.invalid_quads == 0
    t = gpu.triangle_indices.astype(np.int64)
    e = np.concatenate([t[:, [0, 1]], t[:, [1, 2]], t[:, [2, 0]]])
    e.sort(axis=1)
    ek = np.sort(e[:, 0] * np.int64(1 << 32) + e[:, 1])
    starts = np.flatnonzero(np.r_[True, ek[1:] != ek[:-1]])
    counts = np.diff(np.r_[starts, ek.size])
    # closed: no boundary edge.  A cell face with four sign-change edges (the
    # fractal has them) makes its mesh edge shared by four triangles, so the
    # count is even rather than exactly two.
    assert (counts % 2 == 0).all(), f"{int((counts % 2 != 0).sum())} boundary (odd-count) edges"
