"""Seeded synthetic SDF workloads (sources plus parameter vectors).

The generators write `.sdf3d` WGSL / GLSL text for the library and, beside
it, the same numbers as a float32 vector in the layout the CPU oracle takes,
so both sides evaluate identical constants.  Literals are written with 17
significant digits of their float32 value, so the WGSL abstract-float
literal converts back to exactly that float32.

  torus()       sdf3d_torus(p, vec2(0.5, 0.2)), the plain small case (128^3)
  csg64()       rounded box minus a smooth union of 64 spheres, unioned with a
                torus (1024^3 throughput case)
  mandelbulb()  power-8 Mandelbulb distance estimate in GLSL (2048^3 case)
  random_tree() seeded CSG tree over sphere / box / torus / capsule (batching)
"""
from __future__ import annotations

import math

import numpy as np

MASK64 = (1 << 64) - 1


class SplitMix64:
    """splitmix64 (Steele, Lea, Flood 2014); u01() uses the top 53 bits."""

    def __init__(self, seed: int):
        self.state = seed & MASK64

    def next(self) -> int:
        self.state = (self.state + 0x9E3779B97F4A7C15) & MASK64
        z = self.state
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & MASK64
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & MASK64
        return z ^ (z >> 31)

    def u01(self) -> float:
        return (self.next() >> 11) * (1.0 / 9007199254740992.0)

    def uniform(self, lo: float, hi: float) -> float:
        return lo + (hi - lo) * self.u01()

    def randint(self, lo: int, hi: int) -> int:
        """Integer in [lo, hi]."""
        return lo + int(self.u01() * (hi - lo + 1))


def f32(v: float) -> float:
    return float(np.float32(v))


def lit(v: float) -> str:
    """WGSL / GLSL literal that parses back to exactly float32(v)."""
    s = repr(float(np.float32(v)))
    if "e" in s or "E" in s:
        s = "%.17e" % float(np.float32(v))
    elif "." not in s:
        s += ".0"
    return s


def torus(R: float = 0.5, r: float = 0.2):
    src = ("use sdf3d::*;\n\n"
           "fn sdf3d(p: vec3f) -> f32 {\n"
           f"    return sdf3d_torus(p, vec2({lit(R)}, {lit(r)}));\n"
           "}\n")
    return src, [f32(R), f32(r)]


def sphere(r: float = 0.5):
    src = ("use sdf3d::*;\n\n"
           "fn sdf3d(p: vec3f) -> f32 {\n"
           f"    return sdf3d_sphere(p, {lit(r)});\n"
           "}\n")
    return src, [f32(r)]


def csg64(seed: int = 0, n: int = 64, box_full: float = 1.3, box_round: float = 0.05,
          torus_R: float = 0.5, torus_r: float = 0.1, k: float = 0.02):
    """Rounded box (half-size 0.7, radius 0.05) minus a smooth union (k) of n
    spheres (centres U(-0.8, 0.8)^3, radii U(0.02, 0.10)), unioned with a
    torus (0.5, 0.1)."""
    rng = SplitMix64(seed)
    spheres = []
    for _ in range(n):
        c = [f32(rng.uniform(-0.8, 0.8)) for _ in range(3)]
        r = f32(rng.uniform(0.02, 0.10))
        spheres.append((c, r))
    lines = ["use sdf3d::*;", "use sdf::op;", "",
             f"// {n} seeded spheres (splitmix64 seed {seed}) blended with sdf_op_smooth_union",
             "fn spheres(p: vec3f) -> f32 {"]
    (c0, r0) = spheres[0]
    lines.append(f"    var d = sdf3d_sphere(p - vec3f({lit(c0[0])}, {lit(c0[1])}, {lit(c0[2])}), {lit(r0)});")
    for c, r in spheres[1:]:
        lines.append(f"    d = sdf_op_smooth_union(d, sdf3d_sphere(p - vec3f({lit(c[0])}, {lit(c[1])}, "
                     f"{lit(c[2])}), {lit(r)}), {lit(k)});")
    lines += ["    return d;", "}", "",
              "fn sdf3d(p: vec3f) -> f32 {",
              f"    let carved = max(sdf3d_box(p, vec3f({lit(box_full)})) - {lit(box_round)}, -spheres(p));",
              f"    return min(carved, sdf3d_torus(p, vec2f({lit(torus_R)}, {lit(torus_r)})));",
              "}", ""]
    params = [f32(box_full), f32(box_round), f32(torus_R), f32(torus_r), f32(k), float(n)]
    for c, r in spheres:
        params += [c[0], c[1], c[2], r]
    return "\n".join(lines), params


def mandelbulb(power: float = 8.0, iterations: int = 8, bailout: float = 2.0, offset: float = 0.003):
    """Power-N Mandelbulb distance estimate as a GLSL fragment shader with
    `float sdf(vec3)`; the point is swizzled to xzy first."""
    src = f"""#version 450 core
// Mandelbulb distance estimate: z -> z^{lit(power)} + c in spherical form,
// running derivative dr, estimate 0.5 * log(r) * r / dr.
const float POWER = {lit(power)};
const float BAILOUT = {lit(bailout)};

float sdf(vec3 p) {{
    p.xyz = p.xzy;
    vec3 z = p;
    float dr = 1.0;
    float r = 0.0;
    float theta = 0.0;
    float phi = 0.0;
    for (int i = 0; i < {int(iterations)}; ++i) {{
        r = length(z);
        if (r > BAILOUT) continue;
        theta = atan(z.y / z.x);
        phi = asin(z.z / r);
        dr = pow(r, POWER - 1.0) * dr * POWER + 1.0;
        r = pow(r, POWER);
        theta = theta * POWER;
        phi = phi * POWER;
        z = r * vec3(cos(theta) * cos(phi), sin(theta) * cos(phi), sin(phi)) + p;
    }}
    return 0.5 * log(r) * r / dr - {lit(offset)};
}}

void main() {{
}}
"""
    return src, [f32(power), float(iterations), f32(bailout), f32(offset)]


# ---------------------------------------------------------------------------
# Random CSG trees (batching / serving workloads)

_PRIMS = ("sphere", "box", "torus", "capsule")
_OPS = ("union", "subtract", "intersect", "smooth")


def random_tree(seed: int, depth: int | None = None):
    """A CSG tree of depth U{2..6} over sphere / box / torus / capsule with
    parameters U(0.05, 0.6) and offsets U(-0.5, 0.5)^3; operations union
    (min), subtract (max(a, -b)), intersect (max) and smooth union
    (k ~ U(0.01, 0.05)).  Returns (wgsl, oracle postfix program)."""
    rng = SplitMix64(0xC56 ^ (seed * 0x9E3779B97F4A7C15))
    if depth is None:
        depth = rng.randint(2, 6)
    prog: list[float] = []

    def leaf():
        kind = _PRIMS[rng.randint(0, 3)]
        off = [f32(rng.uniform(-0.5, 0.5)) for _ in range(3)]
        if kind == "sphere":
            r = f32(rng.uniform(0.05, 0.6))
            prog.extend([0.0, *off, r])
            return f"sdf3d_sphere(p - vec3f({lit(off[0])}, {lit(off[1])}, {lit(off[2])}), {lit(r)})"
        if kind == "box":
            b = [f32(rng.uniform(0.05, 0.6)) for _ in range(3)]
            prog.extend([1.0, *off, *b])
            return (f"sdf3d_box(p - vec3f({lit(off[0])}, {lit(off[1])}, {lit(off[2])}), "
                    f"vec3f({lit(b[0])}, {lit(b[1])}, {lit(b[2])}))")
        if kind == "torus":
            R = f32(rng.uniform(0.05, 0.6))
            r = f32(rng.uniform(0.05, 0.6) * 0.5)
            prog.extend([2.0, *off, R, r])
            return (f"sdf3d_torus(p - vec3f({lit(off[0])}, {lit(off[1])}, {lit(off[2])}), "
                    f"vec2f({lit(R)}, {lit(r)}))")
        a = off
        b = [f32(rng.uniform(-0.5, 0.5)) for _ in range(3)]
        r = f32(rng.uniform(0.05, 0.6) * 0.5)
        prog.extend([3.0, *a, *b, r])
        return (f"sdf3d_capsule(p, vec3f({lit(a[0])}, {lit(a[1])}, {lit(a[2])}), "
                f"vec3f({lit(b[0])}, {lit(b[1])}, {lit(b[2])}), {lit(r)})")

    def node(d):
        if d <= 1:
            return leaf()
        op = _OPS[rng.randint(0, 3)]
        left = node(d - 1)
        right = node(rng.randint(1, d - 1))
        if op == "union":
            prog.append(10.0)
            return f"min({left}, {right})"
        if op == "subtract":
            prog.append(11.0)
            return f"max({left}, -{right})"
        if op == "intersect":
            prog.append(12.0)
            return f"max({left}, {right})"
        k = f32(rng.uniform(0.01, 0.05))
        prog.extend([13.0, k])
        return f"sdf_op_smooth_union({left}, {right}, {lit(k)})"

    body = node(depth)
    src = ("use sdf3d::*;\nuse sdf::op;\n\n"
           f"// random CSG tree, seed {seed}, depth {depth}\n"
           "fn sdf3d(p: vec3f) -> f32 {\n"
           f"    return {body};\n"
           "}\n")
    return src, prog


def log_uniform_resolution(rng: SplitMix64, choices=(64, 96, 128, 192, 256, 384)) -> int:
    """A resolution drawn log-uniformly from a set (the batching workload)."""
    logs = [math.log(c) for c in choices]
    u = rng.uniform(logs[0], logs[-1])
    return min(choices, key=lambda c: abs(math.log(c) - u))
