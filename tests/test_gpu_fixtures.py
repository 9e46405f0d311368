"""GPU meshes of the reference's own example inputs and of the frontend's
less common paths, through the C ABI, against the CPU oracle.

examples/martin_cube.sdf3d and examples/p_key.sdf3d (extracted into
tests/golden/reference_examples.json) exercise swizzle assignment, `const`
folding, `if`, `var`, compound assignment, the capsule, the cylinder and the
smooth operators.  Every operation they use is correctly rounded, so the
GPU mesh must equal the oracle's restatement of the same file bit for bit.
"""
from __future__ import annotations

import json
import os
import subprocess

import numpy as np
import pytest

import oracle
import sdf2mesh_gb300 as s2m
from tests.parity import assert_bit_exact

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
CLI = os.path.join(ROOT, "sdf2mesh_gb300", "_lib", "sdf2mesh")


def reference_example(name):
    with open(os.path.join(GOLDEN, "reference_examples.json")) as f:
        return json.load(f)["files"][name]


@pytest.mark.parametrize("name,kind,N,B", [("martin_cube.sdf3d", oracle.MARTIN_CUBE, 96, 3.0),
                                           ("martin_cube.sdf3d", oracle.MARTIN_CUBE, 161, 3.0),
                                           ("p_key.sdf3d", oracle.P_KEY, 128, 40.0)])
def test_reference_example_mesh(lib, name, kind, N, B):
    sdf = s2m.Sdf3DShader.from_source(reference_example(name)).compile()
    gpu = s2m.generate(sdf, s2m.AppState(resolution=N, bounds=B))
    ref = oracle.mesh(kind, [], N, B)
    assert ref.nverts > 1000
    assert_bit_exact(gpu, ref, f"{name} {N}")


def test_reference_example_cli_rounding_and_lag(lib):
    """The reference CLI's own settings on martin_cube: 100 -> 128, slice lag."""
    sdf = s2m.Sdf3DShader.from_source(reference_example("martin_cube.sdf3d")).compile()
    gpu = s2m.generate(sdf, s2m.AppState.from_args(resolution=100, bounds=3.0))
    assert gpu.info.resolution == 128
    assert_bit_exact(gpu, oracle.mesh(oracle.MARTIN_CUBE, [], 128, 3.0, slice_lag=True), "martin_cube lag")


@pytest.mark.parametrize("prune", [True, False])
def test_cylinder_mesh(lib, prune):
    """sdf3d_cylinder (sdf3d_primitives.wgsl:13-17) smooth-unioned with a box."""
    src = ("use sdf3d::*;\nuse sdf::op;\nfn sdf3d(p: vec3f) -> f32 {\n"
           "  return sdf_op_smooth_union(sdf3d_cylinder(p - vec3f(0.125, -0.25, 0.0625), 0.5, 0.375),\n"
           "                             sdf3d_box(p - vec3f(0.0, 0.5, 0.0), vec3f(0.5, 0.25, 0.75)), 0.0625);\n}\n")
    sdf = s2m.Sdf3DShader.from_source(src).compile(prune=prune)
    prog = [5, 0.125, -0.25, 0.0625, 0.5, 0.375, 1, 0.0, 0.5, 0.0, 0.5, 0.25, 0.75, 13, 0.0625]
    gpu = s2m.generate(sdf, s2m.AppState(resolution=90, bounds=2.0))
    assert_bit_exact(gpu, oracle.mesh(oracle.TREE, prog, 90, 2.0), f"cylinder prune={prune}")


def test_shadertoy_style_mesh(lib):
    """ShaderToy-style GLSL (shadertoy.rs:154-166), inputs constant zero: the
    sphere of radius 0.5 + 0.25 sin(0)."""
    code = ("float sdSphere(vec3 p, float r) { return length(p) - r; }\n"
            "float sdf(vec3 p) { return sdSphere(p, 0.5 + 0.25 * sin(iTime)) + 0.0 * iResolution.x; }\n"
            "void mainImage(out vec4 fragColor, in vec2 fragCoord) {\n"
            "  fragColor = vec4(sdf(vec3(fragCoord / iResolution.xy, 0.0)));\n}\n")
    sdf = s2m.Sdf3DShader.from_source(code, s2m.LANG_SHADERTOY, "sdf").compile()
    gpu = s2m.generate(sdf, s2m.AppState(resolution=72, bounds=2.0))
    assert_bit_exact(gpu, oracle.mesh(oracle.SPHERE, [0.5], 72, 2.0), "shadertoy sphere")


def test_cli_debug_cuda(lib, tmp_path):
    """--debug-cuda writes the lowered CUDA C that NVRTC compiled."""
    src = tmp_path / "mc.sdf3d"
    src.write_text(reference_example("martin_cube.sdf3d"))
    out = tmp_path / "mc.stl"
    dbg = tmp_path / "mc.cu"
    r = subprocess.run([CLI, "-i", os.fspath(src), "-0", os.fspath(out), "-r", "64", "-b", "3",
                        "--debug-cuda", os.fspath(dbg)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    cuda = dbg.read_text()
    assert "s2m_user_sdf" in cuda and "letter_r_arc" in cuda
    sdf = s2m.Sdf3DShader.from_source(reference_example("martin_cube.sdf3d")).compile()
    assert cuda == sdf.cuda_source
    text = out.read_text()
    assert text.startswith("solid\n") and text.endswith("endsolid\n")
    assert np.isfinite([float(t) for t in text.split() if t[:1].isdigit() or t[:1] == "-"]).all()
