"""The no-allocation entry point, s2m_mesh_noalloc, for callers that may not
allocate device memory while they mesh (a fixed memory arena planned up
front, a hard memory quota, or a loop that must not be stalled by the
device-wide synchronisation of cudaMalloc / cudaFree).  Its pipeline scratch
is one fixed array inside the library; the caller allocates the outputs.

It is checked through the C ABI against the ordinary entry point
(s2m_mesh_create): the same vertices, normals, cell keys and triangles, bit
for bit, on two calls in a row (the second call reuses the scratch the
first one left behind).  This file is named so that pytest collects it last.
"""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

import sdf2mesh_gb300 as s2m
from sdf2mesh_gb300 import workloads

pytestmark = pytest.mark.gpu


def noalloc(lib, sdf, state, max_vertices, max_triangles):
    import torch
    dev = torch.device("cuda", torch.cuda.current_device())
    pos = torch.empty(3 * max_vertices, dtype=torch.float32, device=dev)
    nrm = torch.empty(3 * max_vertices, dtype=torch.float32, device=dev)
    cell = torch.empty(max_vertices, dtype=torch.int64, device=dev)
    tris = torch.empty(3 * max_triangles, dtype=torch.int32, device=dev)
    out = s2m.NoallocMesh(pos.data_ptr(), nrm.data_ptr(), cell.data_ptr(), tris.data_ptr(), max_vertices,
                          max_triangles)
    p = state.params()
    err = ctypes.create_string_buffer(1024)
    torch.cuda.synchronize()
    rc = lib.s2m_mesh_noalloc(sdf.handle, ctypes.byref(p), ctypes.byref(out), None, err, len(err))
    return rc, err.value.decode(), out, (pos, nrm, cell, tris)


def as_host(out, bufs):
    nv, nt = int(out.nverts), int(out.ntris)
    pos, nrm, cell, tris = bufs
    return (pos[: 3 * nv].cpu().numpy().reshape(nv, 3), nrm[: 3 * nv].cpu().numpy().reshape(nv, 3),
            cell[:nv].cpu().numpy().view(np.uint64), tris[: 3 * nt].cpu().numpy().view(np.uint32).reshape(nt, 3))


@pytest.mark.parametrize("which", ["torus", "csg64"])
def test_noalloc_matches_mesh_create_twice(lib, which):
    if which == "torus":
        src, _ = workloads.torus(0.5, 0.2)
        N = 160
    else:
        src, _ = workloads.csg64(seed=0)
        N = 256
    sdf = s2m.Sdf3DShader.from_source(src).compile()
    state = s2m.AppState(resolution=N, bounds=2.0)
    ref = s2m.generate(sdf, state)
    nv, nt = ref.positions.shape[0], ref.triangle_indices.shape[0]
    assert nv > 1000
    for call in range(2):
        rc, msg, out, bufs = noalloc(lib, sdf, state, nv + 100, nt + 100)
        assert rc == 0, msg
        assert (int(out.nverts), int(out.ntris), int(out.invalid_quads)) == (nv, nt, ref.invalid_quads)
        pos, nrm, cell, tris = as_host(out, bufs)
        assert np.array_equal(pos.view(np.uint32), ref.positions.view(np.uint32)), f"call {call}: positions"
        assert np.array_equal(nrm.view(np.uint32), ref.normals.view(np.uint32)), f"call {call}: normals"
        assert np.array_equal(cell, ref.cells), f"call {call}: cell keys"
        assert np.array_equal(tris, ref.triangle_indices), f"call {call}: triangles"


def test_noalloc_limits(lib):
    src, _ = workloads.torus(0.5, 0.2)
    sdf = s2m.Sdf3DShader.from_source(src).compile()
    # resolution beyond the limit: rejected before any device work
    rc, msg, _, _ = noalloc(lib, sdf, s2m.AppState(resolution=s2m.NOALLOC_MAX_RESOLUTION + 1), 16, 16)
    assert rc == 1 and "exceeds the no-allocation limit" in msg
    # outputs too small: an overflow status with the exact counts needed
    ref = s2m.generate(sdf, s2m.AppState(resolution=96))
    rc, msg, out, _ = noalloc(lib, sdf, s2m.AppState(resolution=96), 64, 64)
    assert rc == 8, msg
    assert int(out.nverts) == ref.positions.shape[0]
    # and a correct call right after the failed one
    rc, msg, out, bufs = noalloc(lib, sdf, s2m.AppState(resolution=96), ref.positions.shape[0],
                                 ref.triangle_indices.shape[0])
    assert rc == 0, msg
    assert np.array_equal(as_host(out, bufs)[3], ref.triangle_indices)
