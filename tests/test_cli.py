"""The `sdf2mesh` CLI, drop-in for the reference binary (main.rs:95-137):
argument handling on the CPU, and a full run on the GPU whose STL must equal,
byte for byte, the oracle's mesh written by the oracle's STL writer."""
from __future__ import annotations

import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CLI = os.path.join(ROOT, "sdf2mesh_gb300", "_lib", "sdf2mesh")
TORUS = "use sdf3d::*;\n\nfn sdf3d(p: vec3f) -> f32 {\n    return sdf3d_torus(p, vec2(0.5, 0.2));\n}\n"


def run(*args):
    return subprocess.run([CLI, *args], capture_output=True, text=True, timeout=300)


def test_cli_help_and_errors(lib):
    assert os.path.exists(CLI)
    r = run("--help")
    assert r.returncode == 0 and "--resolution" in r.stderr
    r = run("-i", "x.sdf3d")
    assert r.returncode == 2 and "--mesh" in r.stderr
    r = run("-0", "out.stl", "-r", "abc", "-i", "x.sdf3d")
    assert r.returncode == 2
    r = run("-0", "out.stl", "--frobnicate")
    assert r.returncode == 2
    r = run("-0", "out.stl", "--shadertoy-id", "DldfR7")
    assert r.returncode == 1 and "network" in r.stderr
    r = run("-0", "out.stl", "-i", "/nonexistent/file.sdf3d")
    assert r.returncode == 1


@pytest.mark.gpu
@pytest.mark.parametrize("res,ext", [(100, "stl"), (64, "ply"), (64, "STL")])
def test_cli_matches_oracle_bytes(lib, oracle_lib, tmp_path, res, ext):
    import oracle
    src = tmp_path / "torus.sdf3d"
    src.write_text(TORUS)
    out = tmp_path / f"mesh.{ext}"
    wgsl = tmp_path / "debug.wgsl"
    r = run("--sdf", os.fspath(src), "--mesh", os.fspath(out), "--resolution", str(res), "--bounds", "2",
            "--debug-wgsl", os.fspath(wgsl))
    assert r.returncode == 0, r.stderr
    assert "fn sdf3d_torus(" in wgsl.read_text()
    N = 1 << (res - 1).bit_length() if res & (res - 1) else res
    ref = oracle.mesh(oracle.TORUS, [0.5, 0.2], N, 2.0, slice_lag=True)
    expect = tmp_path / f"oracle.{ext}"
    if ext.upper() == "STL":
        oracle.write_stl(ref.pos, ref.tris, os.fspath(expect))
    else:
        oracle.write_ply(ref.pos, ref.nrm, ref.tris, os.fspath(expect))
    assert out.read_bytes() == expect.read_bytes()


@pytest.mark.gpu
def test_cli_glsl(lib, tmp_path):
    from sdf2mesh_gb300 import workloads
    src, _ = workloads.mandelbulb(8.0, 5, 2.0, 0.003)
    f = tmp_path / "mb.frag"
    f.write_text(src)
    out = tmp_path / "mb.stl"
    r = run("--glsl", os.fspath(f), "--glsl-sdf", "sdf", "-0", os.fspath(out), "-r", "64", "-b", "2.5")
    assert r.returncode == 0, r.stderr
    text = out.read_text()
    assert text.startswith("solid\n") and text.endswith("endsolid\n") and text.count("endfacet") > 1000


@pytest.mark.gpu
def test_cli_binary_stl(lib, oracle_lib, tmp_path):
    """--binary-stl: the same facets as the ASCII file, in the binary form."""
    import oracle
    from tests.test_stl_binary import numpy_stl_binary
    src = tmp_path / "torus.sdf3d"
    src.write_text(TORUS)
    out = tmp_path / "mesh.stl"
    r = run("-i", os.fspath(src), "-0", os.fspath(out), "-r", "128", "--binary-stl")
    assert r.returncode == 0, r.stderr
    ref = oracle.mesh(oracle.TORUS, [0.5, 0.2], 128, 2.0, slice_lag=True)
    data = out.read_bytes()
    assert int.from_bytes(data[80:84], "little") == ref.ntris
    assert data[84:] == numpy_stl_binary(ref.pos, ref.tris)
