"""The shader front end: `.sdf3d` preprocessing (shader.rs:44-67, 159-203),
WGSL / GLSL lowering to CUDA C, and the WGSL text helpers
(shadertoy.rs:248-352) -- all on the CPU.

The lowered CUDA C is also valid host C++ (s2m_prelude.cuh is
__host__ __device__); compiled with g++ -ffp-contract=off it must evaluate
every fixture SDF bit-for-bit like the oracle's hand restatement.
"""
from __future__ import annotations

import json
import os

import numpy as np
import pytest

import oracle
import sdf2mesh_gb300 as s2m
from sdf2mesh_gb300 import workloads
from tests.hostsdf import compile_host, eval_host

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
# A checkout of the reference sources, when one is at hand (S2M_REFERENCE_DIR);
# the tests that read its example files as text skip without it.
REF_EXAMPLES = os.path.join(os.environ.get("S2M_REFERENCE_DIR", ""), "examples")


def lower(src, lang=s2m.LANG_WGSL, name="sdf"):
    if lang == s2m.LANG_WGSL:
        src = s2m.Sdf3DShader.from_source(src).source
    return s2m.translate(src, lang, name)


def points(n=20000, seed=1, lo=-1.2, hi=1.2):
    rng = np.random.default_rng(seed)
    p = rng.uniform(lo, hi, size=(n, 3)).astype(np.float32).astype(np.float64)
    # include lattice coordinates of a 64^3 job exactly as the kernel forms them
    size = np.float32(np.float32(2.0) / np.float32(63))
    c = (np.float32(-1.0) + size * np.arange(64, dtype=np.float32)).astype(np.float64)
    g = np.stack(np.meshgrid(c[::7], c[::5], c[::3], indexing="ij"), -1).reshape(-1, 3)
    return np.concatenate([p, g])


def assert_same_bits(a, b):
    a32, b32 = a.astype(np.float32), b.astype(np.float32)
    same = (a32.view(np.uint32) == b32.view(np.uint32)) | (np.isnan(a32) & np.isnan(b32))
    assert same.all(), f"{(~same).sum()} of {len(a)} differ; first {np.nonzero(~same)[0][:5]}"


def test_torus_lowering_bit_exact(lib, oracle_lib):
    src, prm = workloads.torus()
    cuda, fp32, sfu = lower(src)
    assert (fp32, sfu) == (8.0, 2.0)
    p = points()
    assert_same_bits(eval_host(cuda, p), oracle.evaluate(oracle.TORUS, prm, p))


def test_csg64_lowering_bit_exact(lib, oracle_lib):
    src, prm = workloads.csg64(seed=0)
    cuda, fp32, sfu = lower(src)
    assert fp32 > 1000 and sfu > 64
    p = points(5000)
    assert_same_bits(eval_host(cuda, p), oracle.evaluate(oracle.CSG, prm, p))


@pytest.mark.parametrize("seed", range(12))
def test_random_tree_lowering_bit_exact(lib, oracle_lib, seed):
    src, prog = workloads.random_tree(seed)
    cuda, _, _ = lower(src)
    p = points(4000, seed=seed)
    assert_same_bits(eval_host(cuda, p), oracle.evaluate(oracle.TREE, prog, p))


def test_mandelbulb_glsl_lowering_bit_exact_on_host(lib, oracle_lib):
    """Same host libm on both sides: the GLSL lowering (swizzle-assign, for /
    continue, atan/asin/pow/log/sin/cos) matches the oracle's restatement."""
    src, prm = workloads.mandelbulb(8.0, 8, 2.0, 0.003)
    cuda, fp32, sfu = lower(src, s2m.LANG_GLSL, "sdf")
    assert sfu > 8 * 6
    p = points(5000, lo=-1.25, hi=1.25)
    assert_same_bits(eval_host(cuda, p), oracle.evaluate(oracle.MANDELBULB, prm, p))


def test_normal_is_tetrahedral_sum(lib):
    """sdf3d_normal (sdf3d_normal.wgsl:4-10): sum of v_i * f(p + v_i * eps), not normalised."""
    src, _ = workloads.sphere(0.5)
    cuda, _, _ = lower(src)
    L = compile_host(cuda)
    p = np.array([[0.3, -0.2, 0.7]], np.float32)
    out = np.zeros(3, np.float32)
    L.normal_points(1, p.ctypes.data, np.float32(1e-4), out.ctypes.data)
    f32 = np.float32
    eps = f32(1e-4)
    vs = [(1, -1, -1), (-1, -1, 1), (-1, 1, -1), (1, 1, 1)]
    acc = None
    for v in vs:
        v = np.array(v, np.float32)
        q = p[0] + v * eps
        d = f32(np.sqrt(f32(f32(f32(q[0] * q[0]) + f32(q[1] * q[1])) + f32(q[2] * q[2])))) - f32(0.5)
        term = v * f32(d)
        acc = term if acc is None else (acc + term).astype(np.float32)
    assert np.array_equal(out.view(np.uint32), acc.astype(np.float32).view(np.uint32))


def reference_example(name):
    """An example input the reference ships (examples/<name>), from the fixture
    tests/golden/make_golden.py extracted."""
    with open(os.path.join(GOLDEN, "reference_examples.json")) as f:
        return json.load(f)["files"][name]


@pytest.mark.skipif(not os.environ.get("S2M_REFERENCE_DIR") or not os.path.isdir(REF_EXAMPLES),
                    reason="no reference checkout (S2M_REFERENCE_DIR)")
def test_example_fixture_matches_checkout():
    for name in ("torus.sdf3d", "martin_cube.sdf3d", "p_key.sdf3d", "mandelmesh.frag"):
        assert open(os.path.join(REF_EXAMPLES, name)).read() == reference_example(name), name


@pytest.mark.parametrize("name,kind,B", [("torus.sdf3d", oracle.TORUS, 2.0),
                                         ("martin_cube.sdf3d", oracle.MARTIN_CUBE, 3.0),
                                         ("p_key.sdf3d", oracle.P_KEY, 40.0)])
def test_reference_examples_lower_bit_exact(lib, oracle_lib, name, kind, B):
    """The reference's example files (swizzle assignment, `const` folding in
    binary64, `if`, `var`, compound assignment, capsule, cylinder and the
    smooth operators) lower to code that evaluates bit for bit like the
    oracle's restatement of the same file."""
    sh = s2m.Sdf3DShader.from_source(reference_example(name))
    cuda, fp32, _ = s2m.translate(sh.source)
    assert fp32 > 0
    p = points(20000, lo=-B / 2, hi=B / 2)
    v = eval_host(cuda, p)
    assert (v < 0).any() and (v > 0).any(), "the surface crosses the box"
    prm = [0.5, 0.2] if kind == oracle.TORUS else []
    assert_same_bits(v, oracle.evaluate(kind, prm, p))


def test_reference_mandelmesh_glsl(lib, oracle_lib):
    """examples/mandelmesh.frag: 5 iterations, power 8, bailout 2, offset 0.003."""
    text = reference_example("mandelmesh.frag")
    cuda, _, _ = s2m.translate(text, s2m.LANG_GLSL, "sdf")
    p = points(3000, lo=-1.25, hi=1.25)
    ref = oracle.evaluate(oracle.MANDELBULB, [8.0, 5, 2.0, 0.003], p)
    assert_same_bits(eval_host(cuda, p), ref)


def test_cylinder_lowering_bit_exact(lib, oracle_lib):
    """sdf3d_cylinder (sdf3d_primitives.wgsl:13-17) against the oracle."""
    src = ("use sdf3d::*;\nfn sdf3d(p: vec3f) -> f32 {\n"
           "  return sdf3d_cylinder(p - vec3f(0.125, -0.25, 0.0625), 0.5, 0.375);\n}\n")
    cuda, _, _ = lower(src)
    p = points(20000)
    assert_same_bits(eval_host(cuda, p), oracle.evaluate(oracle.TREE, [5, 0.125, -0.25, 0.0625, 0.5, 0.375], p))


def test_csg64_fixture_reproduced():
    """The 1024^3 workload's source is checked in (tests/golden/csg64_seed0.sdf3d);
    the generator still writes exactly that text."""
    src, _ = workloads.csg64(seed=0)
    with open(os.path.join(GOLDEN, "csg64_seed0.sdf3d")) as f:
        assert f.read() == src


def test_glsl_missing_function(lib):
    with pytest.raises(s2m.S2MError) as e:
        s2m.translate("#version 450\nfloat other(vec3 p) { return p.x; }\nvoid main() {}\n", s2m.LANG_GLSL, "sdf")
    assert e.value.name == "MISSING_SDF"


def test_wgsl_missing_sdf3d(lib):
    with pytest.raises(s2m.S2MError) as e:
        s2m.translate("fn f(p: vec3f) -> f32 { return p.x; }\n")
    assert e.value.name == "MISSING_SDF"


def test_parse_error_names_line(lib):
    with pytest.raises(s2m.S2MError) as e:
        s2m.translate("fn sdf3d(p: vec3f) -> f32 {\n  let a = ;\n  return a;\n}\n")
    assert "line 2" in str(e.value)


def test_preprocess_use_and_include(lib, tmp_path):
    inc = tmp_path / "shapes.wgsl"
    inc.write_text("fn my_ball(p: vec3f) -> f32 { return sdf3d_sphere(p, 0.5); }\n")
    main = tmp_path / "m.sdf3d"
    main.write_text('use sdf3d::primitives;\nuse nothing::here;\ninclude "shapes.wgsl";\n'
                    'include "m.sdf3d";\nfn sdf3d(p: vec3f) -> f32 { return my_ball(p); }\n')
    sh = s2m.Sdf3DShader.from_path(os.fspath(main))
    assert "fn sdf3d_sphere(" in sh.source          # use sdf3d::primitives
    assert "nothing::here" not in sh.source         # unknown modules are dropped
    assert "fn my_ball(" in sh.source               # include, relative to the file
    assert sh.source.count("fn sdf3d(") == 1        # self-include ignored
    cuda, _, _ = s2m.translate(sh.source)
    v = eval_host(cuda, np.array([[0.5, 0.0, 0.0], [0.0, 0.0, 0.0]]))
    assert v[0] == 0.0 and v[1] == -0.5


def test_builtin_modules(lib):
    for use, fns in (("sdf3d::*", ["sdf3d_box", "sdf3d_torus", "sdf3d_normal"]),
                     ("sdf3d::normal", ["sdf3d_normal"]), ("sdf::op", ["sdf_op_smooth_union"]),
                     ("sdf::*", ["sdf_op_smooth_subtraction"])):
        sh = s2m.Sdf3DShader.from_source(f"use {use};\n")
        for fn in fns:
            assert f"fn {fn}(" in sh.source, (use, fn)


def test_golden_remove_function(lib):
    g = json.load(open(os.path.join(GOLDEN, "wgsl_surgery.json")))["remove_function"]
    w = g["input"]
    for step in g["steps"]:
        w = s2m.wgsl_remove_function(w, step["remove"])
        for c in step.get("contains", []):
            assert c in w
        for c in step.get("absent", []):
            assert c not in w
        if "trim_equals" in step:
            assert w.strip() == step["trim_equals"]


def test_golden_rename_function(lib):
    g = json.load(open(os.path.join(GOLDEN, "wgsl_surgery.json")))["rename_function"]
    out = s2m.wgsl_rename_function(g["input"], g["old"], g["new"])
    for c in g["contains"]:
        assert c in out


def test_text_helpers_errors(lib):
    with pytest.raises(s2m.S2MError):
        s2m.wgsl_remove_function("fn a() {}\n", "fn b(")
    assert s2m.wgsl_has_function("  fn sdf3d(p: vec3f) -> f32 {}", "sdf3d")
    assert not s2m.wgsl_has_function("fn sdf3dx(p: vec3f) -> f32 {}", "sdf3d")


def test_standard_normal_marker(lib):
    """The library normal (inserted by `use` or supplied) is marked so the
    kernels may loop over its four directions; a user-defined one is not."""
    src, _ = workloads.torus()
    assert "S2M_STD_NORMAL" in lower(src)[0]
    custom = ("use sdf3d::primitives;\n"
              "fn sdf3d_normal(p: vec3f, eps: f32) -> vec3f {\n"
              "  let h = vec3f(eps, 0.0, 0.0);\n"
              "  return vec3f(sdf3d(p + h.xyy) - sdf3d(p - h.xyy), sdf3d(p + h.yxy) - sdf3d(p - h.yxy),\n"
              "               sdf3d(p + h.yyx) - sdf3d(p - h.yyx));\n}\n"
              "fn sdf3d(p: vec3f) -> f32 { return sdf3d_sphere(p, 0.5); }\n")
    assert "S2M_STD_NORMAL" not in lower(custom)[0]


@pytest.mark.parametrize("seed", range(16))
def test_csg_program_from_source(lib, oracle_lib, seed):
    """The batching workload's .sdf3d sources convert to exactly the programs
    the oracle evaluates, and the program evaluates like the source."""
    src, prog = workloads.random_tree(seed)
    got = s2m.Sdf3DShader.from_source(src).csg_program()
    assert np.array_equal(got, np.asarray(prog, np.float32))


def test_csg_program_rejects_other_sources(lib):
    for src in (workloads.csg64()[0],
                "use sdf3d::*;\nfn sdf3d(p: vec3f) -> f32 { return sdf3d_sphere(p * 2.0, 0.5); }\n",
                "use sdf3d::*;\nfn sdf3d(p: vec3f) -> f32 { return sdf3d_sphere(p, p.x); }\n",
                "fn sdf3d_sphere(p: vec3f, r: f32) -> f32 { return length(p) - 2.0 * r; }\n"
                "fn sdf3d(p: vec3f) -> f32 { return sdf3d_sphere(p, 0.5); }\n"):
        with pytest.raises(s2m.S2MError) as e:
            s2m.Sdf3DShader.from_source(src).csg_program()
        assert e.value.name == "PARSE"
    prog = s2m.Sdf3DShader.from_source(
        "use sdf3d::*;\nuse sdf::op;\nfn sdf3d(p: vec3f) -> f32 {\n"
        "  return sdf_op_smooth_subtraction(sdf3d_box(p, vec3f(1.0)), max(sdf3d_torus(p - vec3(0.1, 0.0, 0.0), "
        "vec2(0.5, 0.1)), -sdf3d_capsule(p, vec3(-1.0), vec3(1.0), 0.2)), 0.05);\n}\n").csg_program()
    assert prog.tolist() == [1, 0, 0, 0, 1, 1, 1, 2, np.float32(0.1), 0, 0, 0.5, np.float32(0.1),
                             3, -1, -1, -1, 1, 1, 1, np.float32(0.2), 11, 15, np.float32(0.05)]


def test_shadertoy_style_file(lib, oracle_lib):
    """ShaderToy-style code (no version line, uniforms or main; shadertoy.rs:154-166):
    wrapped, inputs folded to zero, mainImage ignored."""
    code = ("float sdSphere(vec3 p, float r) { return length(p) - r; }\n"
            "float sdf(vec3 p) { return sdSphere(p, 0.5 + 0.25 * sin(iTime)) + 0.0 * iResolution.x; }\n"
            "void mainImage(out vec4 fragColor, in vec2 fragCoord) {\n"
            "  fragColor = vec4(sdf(vec3(fragCoord / iResolution.xy, 0.0)));\n}\n")
    cuda, _, _ = s2m.translate(code, s2m.LANG_SHADERTOY, "sdf")
    p = points(2000)
    assert_same_bits(eval_host(cuda, p), oracle.evaluate(oracle.SPHERE, [0.5], p))
    with pytest.raises(s2m.S2MError) as e:
        s2m.translate(code, s2m.LANG_SHADERTOY, "missing")
    assert e.value.name == "MISSING_SDF"



@pytest.mark.parametrize("which", ["torus", "csg64", "tree3", "tree9", "capsules"])
def test_run4_form_matches_per_point(lib, which):
    """s2m_user_sdf_run4 (x/y-only part once per run of 4 z values) equals
    s2m_user_sdf lane by lane, bit for bit; SDFs with loops have no run form."""
    from tests.hostsdf import eval_run4_host
    if which == "torus":
        src = workloads.torus()[0]
    elif which == "csg64":
        src = workloads.csg64(seed=3)[0]
    elif which == "capsules":
        src = ("use sdf3d::*;\nuse sdf::op;\nfn sdf3d(p: vec3f) -> f32 {\n"
               "  let q = abs(p) - vec3f(0.2);\n  var d = sdf3d_capsule(q, vec3f(0.0), vec3f(0.3, 0.1, 0.2), 0.1);\n"
               "  d = sdf_op_smooth_subtraction(d, sdf3d_box(p, vec3(0.5, 0.4, 0.3)) * 0.5, 0.05);\n"
               "  return mix(d, dot(p, vec3f(0.3, 0.4, -0.2)) / 2.0, 0.25);\n}\n")
    else:
        src = workloads.random_tree(int(which[4:]))[0]
    cuda, _, _ = lower(src)
    assert "S2M_HAS_RUN4" in cuda
    rng = np.random.default_rng(5)
    xy = rng.uniform(-1.2, 1.2, size=(500, 1, 2)).astype(np.float32).astype(np.float64)
    z = rng.uniform(-1.2, 1.2, size=(500, 4, 1)).astype(np.float32).astype(np.float64)
    pts = np.concatenate([np.broadcast_to(xy, (500, 4, 2)), z], axis=2).reshape(-1, 3)
    assert_same_bits(eval_run4_host(cuda, pts), eval_host(cuda, pts))
    mb = lower(workloads.mandelbulb()[0], s2m.LANG_GLSL, "sdf")[0]
    assert "S2M_HAS_RUN4" not in mb
