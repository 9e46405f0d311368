"""Tile pruning on the CPU: the frontend's generated tile function and pruned
point function, compiled for the host, against the full per-point function.
For every tile, each pruned value must be bit-identical to the full value:
the proof obligations of each pruning decision (interval bounds under
round-to-nearest, operand separation, signed zeros) are checked here on
lattice tiles of real jobs, including the tiles clipped at the lattice edge."""
import numpy as np
import pytest

import sdf2mesh_gb300 as s2m
from sdf2mesh_gb300 import workloads

from hostsdf import lattice_tiles, prune_host, prune_host_in


def lowered(src, lang=s2m.LANG_WGSL, name="sdf"):
    if lang == s2m.LANG_WGSL:
        src = s2m.Sdf3DShader.from_source(src).source
    return s2m.translate(src, lang, name)


def check(cu, N, bounds=2.0, tiles=None, seed=0, count=None):
    if count is not None:
        rng = np.random.default_rng(seed)
        nt = (N + 1 + 7) // 8
        tiles = [tuple(int(v) for v in rng.integers(0, nt, 3)) for _ in range(count)]
    boxes, pts, parents = lattice_tiles(N, bounds, tiles, with_parents=True)
    w, ops, full, pruned, full4, pruned4, root = prune_host(cu, boxes, pts)
    assert w > 0, "no pruning form"
    bad = full.view(np.uint32) != pruned.view(np.uint32)
    assert not bad.any(), f"{int(bad.sum())} pruned values differ, e.g. tile {np.argwhere(bad)[0]}"
    bad4 = full4.view(np.uint32) != pruned4.view(np.uint32)
    assert not bad4.any(), f"{int(bad4.sum())} run-of-4 pruned values differ, e.g. {np.argwhere(bad4)[0]}"
    # the interval of the SDF's value bounds every point of the tile (a
    # "decided" tile's points are never evaluated); NaN intervals are unknown
    known = np.isfinite(root).all(axis=1)
    fin = np.isfinite(full)
    assert ((full >= root[:, :1]) | ~fin | ~known[:, None]).all(), "value below its tile's interval"
    assert ((full <= root[:, 1:]) | ~fin | ~known[:, None]).all(), "value above its tile's interval"
    assert (fin | ~known[:, None]).all(), "a known interval must bound finite values"
    # two-level tile pass: the tile's bits from its coarse box's bits
    ops_in, pruned_in, root_in = prune_host_in(cu, parents, boxes, pts)
    known_in = np.isfinite(root_in).all(axis=1)
    assert ((full >= root_in[:, :1]) & (full <= root_in[:, 1:]) | ~known_in[:, None]).all()
    bad_in = full.view(np.uint32) != pruned_in.view(np.uint32)
    assert not bad_in.any(), f"{int(bad_in.sum())} values differ with two-level bits, e.g. {np.argwhere(bad_in)[0]}"
    assert (ops_in[:, 0] <= ops[:, 0] + 0.5).all()  # a coarse decision is never undone
    return ops


def test_csg64_every_tile_n48(lib):
    cu, fp, sfu = lowered(workloads.csg64()[0])
    ops = check(cu, 48)
    assert ops[:, 0].max() <= fp and ops[:, 1].max() <= sfu
    assert ops[:, 0].mean() < 0.5 * fp  # most tiles skip most spheres


@pytest.mark.parametrize("N", [256, 1024])
def test_csg64_random_tiles(lib, N):
    cu, fp, sfu = lowered(workloads.csg64()[0])
    ops = check(cu, N, count=400, seed=N)
    assert ops[:, 0].mean() < 0.1 * fp


@pytest.mark.parametrize("seed", range(8))
def test_random_trees(lib, seed):
    cu, _, _ = lowered(workloads.random_tree(seed)[0])
    if "S2M_HAS_PRUNE" not in cu:
        pytest.skip("tree without a combinator worth pruning")
    check(cu, 64, count=300, seed=seed)
    check(cu, 256, count=300, seed=seed + 100)


SMOOTH_OPS = """use sdf3d::primitives;
use sdf::op;
fn sdf3d(p: vec3f) -> f32 {
    let a = sdf3d_sphere(p - vec3f(0.3, 0.0, 0.0), 0.4);
    let b = sdf3d_box(p + vec3f(0.3, 0.1, 0.0), vec3f(0.5, 0.6, 0.4));
    let c = sdf3d_torus(p - vec3f(0.0, 0.2, 0.1), vec2f(0.4, 0.1));
    let u = sdf_op_smooth_union(a, b, 0.05);
    let i = sdf_op_smooth_intersection(u, c - 0.2, 0.03);
    return min(sdf_op_smooth_subtraction(sdf3d_sphere(p, 0.25), i, 0.04), max(c, -a));
}
"""


@pytest.mark.parametrize("N", [33, 128])
def test_smooth_operators_and_min_max(lib, N):
    cu, _, _ = lowered(SMOOTH_OPS)
    assert "S2M_HAS_PRUNE" in cu
    check(cu, N, count=500, seed=N)


# Operands that are exactly +-0 on whole planes of the lattice (p.x * 0.0,
# coordinates that are 0.0 at the centre), blend widths that are zero or
# negative, and a square root of a negative value (NaN): every decision must
# either be proven or not taken.
EDGE = """use sdf3d::primitives;
use sdf::op;
fn sdf3d(p: vec3f) -> f32 {
    let s = sdf3d_sphere(p, 0.5);
    let z0 = p.x * 0.0;
    let a = sdf_op_smooth_union(z0, sdf3d_sphere(p - vec3f(0.9, 0.9, 0.9), 0.1), 0.05);
    let b = sdf_op_smooth_union(s, sdf3d_box(p, vec3f(0.3, 0.3, 0.3)), 0.0);
    let c = sdf_op_smooth_intersection(-z0, sdf3d_sphere(p + vec3f(0.8, 0.0, 0.0), 0.1), -0.1);
    let d = min(sqrt(p.y), sdf3d_torus(p, vec2f(0.5, 0.2)));
    let e = max(p.z, -sdf3d_sphere(p - vec3f(0.0, 0.0, 0.7), 0.2));
    return min(min(a, b), min(min(c, d), e));
}
"""


@pytest.mark.parametrize("N", [16, 64])
def test_edge_cases(lib, N):
    cu, _, _ = lowered(EDGE)
    assert "S2M_HAS_PRUNE" in cu
    check(cu, N)  # every tile


# A decided smooth operator whose kept operand is +-0: the pruned code
# returns it through s2_canon (-0 -> +0), which must match the operator's own
# arithmetic at h = 1 or h = 0 bit for bit.  Each SDF returns the operator's
# value itself, so the sign of a zero reaches the comparison.  z0 is +0 for
# x >= 0 and -0 for x < 0; `far` is positive except near one corner.
_ZERO_PRE = """use sdf3d::primitives;
use sdf::op;
fn sdf3d(p: vec3f) -> f32 {
    let z0 = p.x * 0.0;
    let far = sdf3d_sphere(p - vec3f(0.9, 0.9, 0.9), 0.05);
    return %s;
}
"""
SIGNED_ZERO_KEEPS = [
    "sdf_op_smooth_union(z0, far, 0.05)",                       # keep a = +-0, b > 0
    "sdf_op_smooth_union(far, -z0, 0.05)",                      # keep b = -+0, a > 0
    "sdf_op_smooth_intersection(z0, -far - 1.0, 0.05)",         # keep a, b < 0
    "sdf_op_smooth_intersection(-far - 1.0, -z0, 0.05)",        # keep b, a < 0
    "sdf_op_smooth_subtraction(z0, -far - 1.0, 0.05)",          # keep -a
    "sdf_op_smooth_subtraction(far + 1.0, -z0, 0.05)",          # keep b
    "sdf_op_smooth_union(sdf_op_smooth_union(z0, far, 0.05), far + 0.5, 0.05)",  # canonical chain input
]


@pytest.mark.parametrize("expr", SIGNED_ZERO_KEEPS)
@pytest.mark.parametrize("N", [16, 33])
def test_smooth_keep_of_signed_zero(lib, expr, N):
    cu, fp, _ = lowered(_ZERO_PRE % expr)
    assert "S2M_HAS_PRUNE" in cu
    ops = check(cu, N)  # every tile, bitwise
    # the decision is taken somewhere (the operand that is not kept is pruned)
    assert ops[:, 0].min() < fp


def test_user_function_with_library_arithmetic_is_a_combinator(lib):
    """A user function whose body is sdf::op's smooth union arithmetic is
    recognised by its arithmetic, not its name."""
    src = """use sdf3d::primitives;
fn blend(a: f32, b: f32, k: f32) -> f32 {
    let h = clamp(0.5 + 0.5 * (b - a) / k, 0.0, 1.0);
    return mix(b, a, h) - k * h * (1.0 - h);
}
fn sdf3d(p: vec3f) -> f32 {
    return blend(sdf3d_sphere(p - vec3f(0.5, 0.0, 0.0), 0.3), sdf3d_sphere(p + vec3f(0.5, 0.0, 0.0), 0.3), 0.1);
}
"""
    cu, _, _ = lowered(src)
    assert "s2_op_smooth_union_call(" in cu
    check(cu, 64, count=200)


def test_tile_form_without_combinators_and_none_with_loops(lib):
    """A straight-line SDF without combinators still gets the tile form (its
    value interval decides the tiles far from the surface); one with loops
    gets none."""
    cu, _, _ = lowered(workloads.torus()[0])
    assert "S2M_HAS_PRUNE" in cu and "tile pruning: 0 combinators" in cu
    ops = check(cu, 48)
    assert (ops[:, 0] >= 0).all()
    cu, _, _ = lowered(workloads.mandelbulb()[0], s2m.LANG_GLSL, "sdf")
    assert "S2M_HAS_PRUNE" not in cu
