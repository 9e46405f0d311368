"""Comparison of a GPU mesh with the CPU oracle's.

Bit-exact SDFs (only +, -, *, /, sqrt, min, max, abs, clamp: every operation
correctly rounded on both sides) must match exactly: the same vertices in
the same order with the same bits, the same triangles, the same invalid-quad
count.  SDFs with transcendental functions (Mandelbulb) may differ in the
last bits of an evaluation, so a cell whose corner values straddle zero by
less than a stated epsilon ("tie cell") may flip; everything else must match.
"""
from __future__ import annotations

import numpy as np

import oracle


def same_bits(a, b):
    """Elementwise: the same binary32 bits, or both NaN.  A NaN's sign and
    payload are the hardware's (0/0 in a normalised zero gradient gives
    0xFFC00000 on x86, 0x7FC00000 on Arm, 0x7FFFFFFF on the GPU); every text
    writer prints them all as NaN."""
    a = np.ascontiguousarray(a, np.float32)
    b = np.ascontiguousarray(b, np.float32)
    return (a.view(np.uint32) == b.view(np.uint32)) | (np.isnan(a) & np.isnan(b))


def assert_bit_exact(gpu, ref, what=""):
    assert gpu.positions.shape[0] == ref.nverts, f"{what}: vertices {gpu.positions.shape[0]} != {ref.nverts}"
    assert np.array_equal(gpu.cell_xyz, ref.cell), f"{what}: vertex cells differ"
    assert np.array_equal(gpu.signs, ref.signs), f"{what}: sign bits differ"
    bad = np.nonzero(~same_bits(gpu.positions, ref.pos).all(axis=1))[0]
    assert bad.size == 0, f"{what}: {bad.size} positions differ, first {bad[:5]}"
    badn = np.nonzero(~same_bits(gpu.normals, ref.nrm).all(axis=1))[0]
    assert badn.size == 0, f"{what}: {badn.size} normals differ, first {badn[:5]}"
    assert gpu.triangle_indices.shape == ref.tris.shape, f"{what}: triangles {gpu.triangle_indices.shape} != {ref.tris.shape}"
    assert np.array_equal(gpu.triangle_indices, ref.tris), f"{what}: triangle indices differ"
    assert gpu.invalid_quads == ref.invalid_quads, f"{what}: invalid quads {gpu.invalid_quads} != {ref.invalid_quads}"


def keys_of(cell_xyz):
    c = np.asarray(cell_xyz, np.uint64)
    return c[:, 0] | (c[:, 1] << np.uint64(16)) | (c[:, 2] << np.uint64(32))


def tie_cells(kind, params, resolution, bounds, keys, eps, slice_lag=False):
    """The subset of cell keys with a corner whose sign binary32 arithmetic
    does not determine: its reference value (binary32) is within eps of zero,
    or differs from the same corner evaluated in binary64 by more than eps.
    The second case is the chaotic one -- an iterated SDF (the Mandelbulb)
    near its escape boundary, where the last bits of each transcendental
    (CUDA's or the host libm's) move the value by far more than an ulp."""
    out = []
    for k in np.asarray(keys, np.uint64):
        x, y, z = int(k & 0xFFFF), int((k >> 16) & 0xFFFF), int((k >> 32) & 0xFFFF)
        if slice_lag:
            z -= 1
        c = oracle.cell_corners(kind, params, resolution, bounds, x, y, z)
        if np.min(np.abs(c)) <= eps:
            out.append(int(k))
            continue
        c64 = oracle.cell_corners(kind, params, resolution, bounds, x, y, z, precision=oracle.F64)
        if np.max(np.abs(c - c64)) > eps:
            out.append(int(k))
    return set(out)


def compare_with_ties(gpu, ref, kind, params, resolution, bounds, eps, h, pos_tol_cells=1e-5, slice_lag=False):
    """Topology equal outside tie cells; positions within pos_tol_cells * h.

    Returns a dict with the counts of tie cells and the max position error
    (in cells) over the common vertices."""
    gk = keys_of(gpu.cell_xyz)
    rk = keys_of(ref.cell)
    gset, rset = set(gk.tolist()), set(rk.tolist())
    only = (gset ^ rset)
    ties = tie_cells(kind, params, resolution, bounds, list(only), eps, slice_lag)
    assert only <= ties, f"{len(only - ties)} vertex cells differ outside tie cells, e.g. {sorted(only - ties)[:5]}"
    common = np.array(sorted(gset & rset), np.uint64)
    gi = np.searchsorted(gk, common)
    ri = np.searchsorted(rk, common)
    gs, rs = gpu.signs[gi], ref.signs[ri]
    sign_diff = set(common[gs != rs].tolist())
    sd_ties = tie_cells(kind, params, resolution, bounds, list(sign_diff), eps, slice_lag)
    assert sign_diff <= sd_ties, f"{len(sign_diff - sd_ties)} sign words differ outside tie cells"
    # positions of common vertices whose cell is not a tie
    err = np.abs(gpu.positions[gi].astype(np.float64) - ref.pos[ri].astype(np.float64)).max(axis=1) / h
    flips = ties | sd_ties
    near = np.array([int(k) not in flips for k in common.tolist()], bool)
    max_err = float(err[near].max()) if near.any() else 0.0
    # a vertex may move when a neighbouring corner flips within eps; count those
    moved = int((err[near] > pos_tol_cells).sum())
    # triangles as sets of key triples
    def tri_keys(keys, tris):
        t = keys[np.asarray(tris, np.int64)]
        return set(map(tuple, t.tolist()))
    gt, rt = tri_keys(gk, gpu.triangle_indices), tri_keys(rk, ref.tris)
    tdiff = gt ^ rt
    touching = {t for t in tdiff if any(v in flips or v in only for v in t)}
    return {"tie_cells": len(flips | only), "vertex_only_one_side": len(only), "max_pos_err_cells": max_err,
            "moved": moved, "tri_diff": len(tdiff), "tri_diff_unexplained": len(tdiff - touching)}


def reference_quads(cell_xyz, signs):
    """Vectorised restatement of VertexList::fetch_triangle_indices
    (mesh.rs:267-331, Quad::swap / make_triangles / is_valid lib.rs:190-211)
    over a sorted vertex list.  Returns (triangles (T, 3) uint32, invalid
    quad count, missing cells (M, 3) of the invalid quads)."""
    c = np.asarray(cell_xyz, np.int64)
    keys = c[:, 0] | (c[:, 1] << 16) | (c[:, 2] << 32)
    V = len(keys)
    s = np.asarray(signs, np.int64)
    b0, b1, b2, b3 = (s & 1) != 0, (s & 2) != 0, (s & 4) != 0, (s & 8) != 0
    x, y, z = c[:, 0], c[:, 1], c[:, 2]
    idx = np.arange(V, dtype=np.int64)
    NONE = np.int64(0xFFFFFFFF)

    def find(xx, yy, zz):
        k = xx | (yy << 16) | (zz << 32)
        pos = np.searchsorted(keys, k)
        ok = (pos < V) & (keys[np.minimum(pos, V - 1)] == k)
        return np.where(ok, pos, NONE)

    quads = np.full((V, 3, 4), NONE, np.int64)
    active = np.zeros((V, 3), bool)
    swap = np.zeros((V, 3), bool)
    m = (b0 != b3) & (y > 0) & (z > 0)
    quads[m, 0] = np.stack([find(x[m], y[m] - 1, z[m] - 1), find(x[m], y[m], z[m] - 1), idx[m],
                            find(x[m], y[m] - 1, z[m])], 1)
    active[:, 0], swap[:, 0] = m, b0
    m = (b1 != b3) & (x > 0) & (z > 0)
    quads[m, 1] = np.stack([find(x[m] - 1, y[m], z[m] - 1), find(x[m], y[m], z[m] - 1), idx[m],
                            find(x[m] - 1, y[m], z[m])], 1)
    active[:, 1], swap[:, 1] = m, ~b1
    m = (b2 != b3) & (x > 0) & (y > 0)
    quads[m, 2] = np.stack([find(x[m] - 1, y[m] - 1, z[m]), find(x[m], y[m] - 1, z[m]), idx[m],
                            find(x[m] - 1, y[m], z[m])], 1)
    active[:, 2], swap[:, 2] = m, b2
    quads = np.where(swap[..., None], quads[..., ::-1], quads)
    valid = active & (quads != NONE).all(-1)
    invalid = active & ~valid
    q = quads[valid]
    tris = np.stack([q[:, [2, 1, 0]], q[:, [0, 3, 2]]], 1).reshape(-1, 3).astype(np.uint32)
    # cells whose vertex an invalid quad looked for and did not find
    missing = []
    for vi, qi in zip(*np.nonzero(invalid)):
        xx, yy, zz = c[vi]
        cand = {0: [(xx, yy - 1, zz - 1), (xx, yy, zz - 1), (xx, yy - 1, zz)],
                1: [(xx - 1, yy, zz - 1), (xx, yy, zz - 1), (xx - 1, yy, zz)],
                2: [(xx - 1, yy - 1, zz), (xx, yy - 1, zz), (xx - 1, yy, zz)]}[int(qi)]
        for cc in cand:
            k = cc[0] | (cc[1] << 16) | (cc[2] << 32)
            p = np.searchsorted(keys, k)
            if not (p < V and keys[p] == k):
                missing.append(cc)
    return tris, int(invalid.sum()), np.array(missing, np.int64).reshape(-1, 3)


def reference_quads_chunked(cell_xyz, signs, chunk=1 << 21):
    """reference_quads over vertex chunks (same triangles in the same order),
    for vertex lists of tens of millions: the per-quad arrays stay chunk-sized.
    Returns (triangles, invalid quad count, missing cells)."""
    c = np.asarray(cell_xyz, np.int64)
    keys = c[:, 0] | (c[:, 1] << 16) | (c[:, 2] << 32)
    V = len(keys)
    s_all = np.asarray(signs, np.int64)
    NONE = np.int64(0xFFFFFFFF)

    def find(xx, yy, zz):
        k = xx | (yy << 16) | (zz << 32)
        pos = np.searchsorted(keys, k)
        ok = (pos < V) & (keys[np.minimum(pos, V - 1)] == k)
        return np.where(ok, pos, NONE)

    tris_out, invalid_total, missing = [], 0, []
    for a in range(0, V, chunk):
        b = min(V, a + chunk)
        x, y, z = c[a:b, 0], c[a:b, 1], c[a:b, 2]
        s = s_all[a:b]
        b0, b1, b2, b3 = (s & 1) != 0, (s & 2) != 0, (s & 4) != 0, (s & 8) != 0
        idx = np.arange(a, b, dtype=np.int64)
        n = b - a
        quads = np.full((n, 3, 4), NONE, np.int64)
        active = np.zeros((n, 3), bool)
        swap = np.zeros((n, 3), bool)
        m = (b0 != b3) & (y > 0) & (z > 0)
        quads[m, 0] = np.stack([find(x[m], y[m] - 1, z[m] - 1), find(x[m], y[m], z[m] - 1), idx[m],
                                find(x[m], y[m] - 1, z[m])], 1)
        active[:, 0], swap[:, 0] = m, b0
        m = (b1 != b3) & (x > 0) & (z > 0)
        quads[m, 1] = np.stack([find(x[m] - 1, y[m], z[m] - 1), find(x[m], y[m], z[m] - 1), idx[m],
                                find(x[m] - 1, y[m], z[m])], 1)
        active[:, 1], swap[:, 1] = m, ~b1
        m = (b2 != b3) & (x > 0) & (y > 0)
        quads[m, 2] = np.stack([find(x[m] - 1, y[m] - 1, z[m]), find(x[m], y[m] - 1, z[m]), idx[m],
                                find(x[m] - 1, y[m], z[m])], 1)
        active[:, 2], swap[:, 2] = m, b2
        quads = np.where(swap[..., None], quads[..., ::-1], quads)
        valid = active & (quads != NONE).all(-1)
        invalid = active & ~valid
        invalid_total += int(invalid.sum())
        q = quads[valid]
        tris_out.append(np.stack([q[:, [2, 1, 0]], q[:, [0, 3, 2]]], 1).reshape(-1, 3).astype(np.uint32))
        for vi, qi in zip(*np.nonzero(invalid)):
            xx, yy, zz = c[a + vi]
            cand = {0: [(xx, yy - 1, zz - 1), (xx, yy, zz - 1), (xx, yy - 1, zz)],
                    1: [(xx - 1, yy, zz - 1), (xx, yy, zz - 1), (xx - 1, yy, zz)],
                    2: [(xx - 1, yy - 1, zz), (xx, yy - 1, zz), (xx - 1, yy, zz)]}[int(qi)]
            for cc in cand:
                k = cc[0] | (cc[1] << 16) | (cc[2] << 32)
                p = np.searchsorted(keys, k)
                if not (p < V and keys[p] == k):
                    missing.append(cc)
    tris = np.concatenate(tris_out) if tris_out else np.zeros((0, 3), np.uint32)
    return tris, invalid_total, np.array(missing, np.int64).reshape(-1, 3)


def compare_window_with_ties(gsel, ref, kind, params, resolution, bounds, eps, h, slice_lag=False):
    """The GPU's vertices of a window of slices (a TriangleMesh-like object with
    cell_xyz, signs, positions) against the oracle's mesh of the same window:
    vertex cells and sign words equal outside tie cells (a reference corner
    with |f| <= eps).  Returns the counts and the largest position difference
    (in cells) of the common vertices that are not tie cells."""
    gk = keys_of(gsel.cell_xyz)
    rk = keys_of(ref.cell)
    gset, rset = set(gk.tolist()), set(rk.tolist())
    only = gset ^ rset
    ties = tie_cells(kind, params, resolution, bounds, list(only), eps, slice_lag)
    assert only <= ties, f"{len(only - ties)} vertex cells differ outside tie cells, e.g. {sorted(only - ties)[:5]}"
    common = np.array(sorted(gset & rset), np.uint64)
    gi = np.searchsorted(gk, common)
    ri = np.searchsorted(rk, common)
    sign_diff = set(common[gsel.signs[gi] != ref.signs[ri]].tolist())
    sd_ties = tie_cells(kind, params, resolution, bounds, list(sign_diff), eps, slice_lag)
    assert sign_diff <= sd_ties, f"{len(sign_diff - sd_ties)} sign words differ outside tie cells"
    err = np.abs(gsel.positions[gi].astype(np.float64) - np.asarray(ref.pos, np.float64)[ri]).max(axis=1) / h
    flips = ties | sd_ties
    near = np.array([int(k) not in flips for k in common.tolist()], bool)
    return {"vertices": len(common), "tie_cells": len(flips | only), "vertex_only_one_side": len(only),
            "max_pos_err_cells": float(err[near].max()) if near.any() else 0.0, "errs": err[near]}
