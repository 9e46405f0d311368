"""Binary STL writer (s2m_write_stl_binary), byte for byte against a numpy
restatement of the format: 80-byte header, u32 count, then per facet the
normal (v2 - v0) x (v1 - v0) of lib.rs:181-185 in binary32, the three
vertices and a zero attribute word.  CPU only (host writer)."""
from __future__ import annotations

import os

import numpy as np
import pytest

import sdf2mesh_gb300 as s2m


def numpy_stl_binary(pos, tris):
    pos = np.asarray(pos, np.float32)
    t = np.asarray(tris, np.int64)
    v0, v1, v2 = pos[t[:, 0]], pos[t[:, 1]], pos[t[:, 2]]
    u = (v2 - v0).astype(np.float32)
    w = (v1 - v0).astype(np.float32)
    n = np.stack([u[:, 1] * w[:, 2] - u[:, 2] * w[:, 1],
                  u[:, 2] * w[:, 0] - u[:, 0] * w[:, 2],
                  u[:, 0] * w[:, 1] - u[:, 1] * w[:, 0]], 1).astype(np.float32)
    rec = np.zeros(len(t), dtype=np.dtype([("n", "<f4", 3), ("v", "<f4", (3, 3)), ("a", "<u2")]))
    rec["n"] = n
    rec["v"] = np.stack([v0, v1, v2], 1)
    return rec.tobytes()


@pytest.mark.parametrize("ntris", [0, 1, 1000, 200003])
def test_binary_stl_bytes(lib, tmp_path, ntris):
    rng = np.random.default_rng(ntris)
    nv = max(3, ntris // 2)
    pos = rng.standard_normal((nv, 3)).astype(np.float32)
    pos[0] = [0.0, -0.0, 1e-38]  # subnormal and signed zero pass through
    tris = rng.integers(0, nv, size=(ntris, 3)).astype(np.uint32)
    path = os.fspath(tmp_path / "m.stl")
    s2m.TriangleMesh(pos, pos, tris).write_stl_binary_to_file(path)
    data = open(path, "rb").read()
    assert len(data) == 84 + 50 * ntris
    assert not data[:5].startswith(b"solid")  # readers would take it for ASCII
    assert int.from_bytes(data[80:84], "little") == ntris
    assert data[84:] == numpy_stl_binary(pos, tris)


def test_binary_stl_bad_path(lib):
    with pytest.raises(s2m.S2MError):
        s2m.TriangleMesh(np.zeros((3, 3), np.float32), np.zeros((3, 3), np.float32),
                         np.zeros((1, 3), np.uint32)).write_stl_binary_to_file("/nonexistent/dir/m.stl")
