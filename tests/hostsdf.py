"""Compile the frontend's lowered SDF code for the HOST (g++), to check the
frontend against the hand-written oracle SDFs on the CPU."""
from __future__ import annotations

import ctypes
import hashlib
import os
import subprocess
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PRELUDE = os.path.join(ROOT, "sdf2mesh_gb300", "csrc", "s2m_prelude.cuh")
_cache: dict[str, ctypes.CDLL] = {}


def compile_host(cuda_src: str) -> ctypes.CDLL:
    key = hashlib.sha1(cuda_src.encode()).hexdigest()
    if key in _cache:
        return _cache[key]
    d = tempfile.mkdtemp(prefix="s2m_host_")
    src = os.path.join(d, "sdf.cpp")
    with open(src, "w") as f:
        f.write(f'#include "{PRELUDE}"\n')
        f.write(cuda_src)
        f.write('\nextern "C" void eval_points(long n, const double* xyz, double* out) {\n'
                '  for (long i = 0; i < n; ++i)\n'
                '    out[i] = s2m_user_sdf((float)xyz[3*i], (float)xyz[3*i+1], (float)xyz[3*i+2]);\n}\n'
                'extern "C" void normal_points(long n, const float* xyz, float eps, float* out) {\n'
                '  for (long i = 0; i < n; ++i) { s2v3 r = s2m_user_normal(s2mk(xyz[3*i], xyz[3*i+1], xyz[3*i+2]), eps);\n'
                '    out[3*i] = r.x; out[3*i+1] = r.y; out[3*i+2] = r.z; }\n}\n'
                '#ifdef S2M_HAS_RUN4\n'
                'extern "C" int eval_run4(long n, const double* xyz, double* out) {\n'
                '  for (long i = 0; i < n; ++i) { s2x4 z, f;\n'
                '    for (int w = 0; w < 4; ++w) z.v[w] = (float)xyz[3*(4*i+w)+2];\n'
                '    s2m_user_sdf_run4((float)xyz[3*4*i], (float)xyz[3*4*i+1], z, f);\n'
                '    for (int w = 0; w < 4; ++w) out[4*i+w] = f.v[w]; }\n  return 1;\n}\n'
                '#else\nextern "C" int eval_run4(long, const double*, double*) { return 0; }\n#endif\n'
                '#ifdef S2M_HAS_PRUNE\n'
                'extern "C" int prune_tiles(long ntiles, const float* box, int npts, const float* pts, unsigned* bits,\n'
                '                           float* ops, float* full, float* pruned, float* full4, float* pruned4,\n'
                '                           float* rootb) {\n'
                '  for (long t = 0; t < ntiles; ++t) {\n'
                '    s2i X, Y, Z; X.lo = box[6*t]; X.hi = box[6*t+1]; Y.lo = box[6*t+2]; Y.hi = box[6*t+3];\n'
                '    Z.lo = box[6*t+4]; Z.hi = box[6*t+5];\n'
                '    unsigned m[S2M_PRUNE_WORDS]; float fp, sfu; s2i root;\n'
                '    s2m_user_sdf_tile(X, Y, Z, m, &fp, &sfu, &root);\n'
                '    rootb[2*t] = root.lo; rootb[2*t+1] = root.hi;\n'
                '    for (int w = 0; w < S2M_PRUNE_WORDS; ++w) bits[t * S2M_PRUNE_WORDS + w] = m[w];\n'
                '    ops[2*t] = fp; ops[2*t+1] = sfu;\n'
                '    for (int p = 0; p < npts; ++p) { const float* q = pts + 3 * (t * npts + p);\n'
                '      full[t * npts + p] = s2m_user_sdf(q[0], q[1], q[2]);\n'
                '      pruned[t * npts + p] = s2m_user_sdf_pruned(q[0], q[1], q[2], m); }\n'
                '    for (int p = 0; p + 3 < npts; p += 4) { const float* q = pts + 3 * (t * npts + p);\n'
                '      s2x4 z; for (int w = 0; w < 4; ++w) z.v[w] = q[3 * w + 2];\n'
                '      s2x4 f = s2m_user_sdf_pruned_run4(q[0], q[1], z, m);\n'
                '      for (int w = 0; w < 4; ++w) { full4[t * npts + p + w] = s2m_user_sdf(q[0], q[1], z.v[w]);\n'
                '        pruned4[t * npts + p + w] = f.v[w]; } }\n'
                '  }\n  return S2M_PRUNE_WORDS;\n}\n'
                'extern "C" void prune_tiles_in(long ntiles, const float* pbox, const float* box, int npts,\n'
                '                               const float* pts, float* ops, float* pruned, float* rootb) {\n'
                '  for (long t = 0; t < ntiles; ++t) {\n'
                '    s2i X, Y, Z; X.lo = pbox[6*t]; X.hi = pbox[6*t+1]; Y.lo = pbox[6*t+2]; Y.hi = pbox[6*t+3];\n'
                '    Z.lo = pbox[6*t+4]; Z.hi = pbox[6*t+5];\n'
                '    unsigned pm[S2M_PRUNE_WORDS], m[S2M_PRUNE_WORDS]; float fp, sfu; s2i root;\n'
                '    s2m_user_sdf_tile(X, Y, Z, pm, &fp, &sfu, &root);\n'
                '    X.lo = box[6*t]; X.hi = box[6*t+1]; Y.lo = box[6*t+2]; Y.hi = box[6*t+3]; Z.lo = box[6*t+4]; Z.hi = box[6*t+5];\n'
                '    s2m_user_sdf_tile_in(X, Y, Z, pm, m, &fp, &sfu, &root);\n'
                '    rootb[2*t] = root.lo; rootb[2*t+1] = root.hi;\n'
                '    ops[2*t] = fp; ops[2*t+1] = sfu;\n'
                '    for (int p = 0; p < npts; ++p) { const float* q = pts + 3 * (t * npts + p);\n'
                '      pruned[t * npts + p] = s2m_user_sdf_pruned(q[0], q[1], q[2], m); }\n'
                '  }\n}\n'
                '#else\nextern "C" int prune_tiles(long, const float*, int, const float*, unsigned*, float*, float*,\n'
                '                           float*, float*, float*, float*) { return 0; }\n#endif\n')
    so = os.path.join(d, "sdf.so")
    subprocess.run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math",
                    src, "-o", so], check=True, capture_output=True)
    L = ctypes.CDLL(so)
    L.eval_points.argtypes = [ctypes.c_long, ctypes.c_void_p, ctypes.c_void_p]
    L.normal_points.argtypes = [ctypes.c_long, ctypes.c_void_p, ctypes.c_float, ctypes.c_void_p]
    L.eval_run4.argtypes = [ctypes.c_long, ctypes.c_void_p, ctypes.c_void_p]
    L.prune_tiles.argtypes = [ctypes.c_long, ctypes.c_void_p, ctypes.c_int] + [ctypes.c_void_p] * 8
    if hasattr(L, "prune_tiles_in"):
        L.prune_tiles_in.argtypes = [ctypes.c_long, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int] + [ctypes.c_void_p] * 4
    _cache[key] = L
    return L


def eval_host(cuda_src: str, xyz: np.ndarray) -> np.ndarray:
    L = compile_host(cuda_src)
    pts = np.ascontiguousarray(np.asarray(xyz, np.float64).reshape(-1, 3))
    out = np.empty(len(pts), np.float64)
    L.eval_points(len(pts), pts.ctypes.data, out.ctypes.data)
    return out


def eval_run4_host(cuda_src: str, xyz: np.ndarray):
    """The run-of-4 form on runs of 4 points (rows 4i..4i+3 share x and y); None without one."""
    L = compile_host(cuda_src)
    pts = np.ascontiguousarray(np.asarray(xyz, np.float64).reshape(-1, 4, 3))
    out = np.empty(pts.shape[0] * 4, np.float64)
    if not L.eval_run4(pts.shape[0], pts.ctypes.data, out.ctypes.data):
        return None
    return out


def lattice_tiles(N: int, bounds: float, tiles=None, T: int = 8, with_parents: bool = False):
    """Tiles of T^3 lattice points (clipped at the lattice edge) of an N-cell
    job: their coordinate boxes (6 floats) and their points (padded to T^3
    by repeating), computed in binary32 as the kernels do: bmin + size * i
    with size = (B/2 - (-B/2)) / (N - 1), the reference's cell size."""
    P = N + 1
    half = np.float32(np.float32(bounds) * np.float32(0.5))
    bmin = np.float32(np.float32(0.0) - half)
    ext = np.float32(np.float32(0.0) + half) - bmin
    size = np.float32(ext / np.float32(N - 1))
    def coord(i):
        return (bmin + size * np.asarray(i, np.float32)).astype(np.float32)
    if tiles is None:
        nt = (P + T - 1) // T
        tiles = [(a, b, c) for a in range(nt) for b in range(nt) for c in range(nt)]
    boxes, pts, parents = [], [], []
    C = 4 * T  # coarse boxes of 4 x 4 tiles (the tile pass's first level)
    for (a, b, c) in tiles:
        ii = np.arange(a * T, min(a * T + T, P)); jj = np.arange(b * T, min(b * T + T, P))
        kk = np.arange(c * T, min(c * T + T, P))
        g = np.stack(np.meshgrid(coord(ii), coord(jj), coord(kk), indexing="ij"), -1).reshape(-1, 3)
        boxes.append([coord(ii[0]), coord(ii[-1]), coord(jj[0]), coord(jj[-1]), coord(kk[0]), coord(kk[-1])])
        pi0, pj0 = (a * T) // C * C, (b * T) // C * C
        parents.append([coord(pi0), coord(min(pi0 + C, P) - 1), coord(pj0), coord(min(pj0 + C, P) - 1),
                        coord(kk[0]), coord(kk[-1])])
        pts.append(np.resize(g, (T ** 3, 3)))
    if with_parents:
        return np.array(boxes, np.float32), np.array(pts, np.float32), np.array(parents, np.float32)
    return np.array(boxes, np.float32), np.array(pts, np.float32)


def prune_host(cuda_src: str, boxes: np.ndarray, pts: np.ndarray):
    """Run the tile function and the pruned point functions on the host:
    (words per tile or 0, ops per tile [fp, sfu], full values, pruned values,
    and the same for the run-of-4 form on groups of 4 consecutive points with
    the first one's x and y)."""
    L = compile_host(cuda_src)
    nt, npts = len(boxes), pts.shape[1]
    boxes = np.ascontiguousarray(boxes, np.float32)
    pts = np.ascontiguousarray(pts, np.float32)
    bits = np.zeros((nt, 64), np.uint32)
    ops = np.zeros((nt, 2), np.float32)
    full = np.zeros((nt, npts), np.float32)
    pruned = np.zeros((nt, npts), np.float32)
    full4 = np.zeros((nt, npts), np.float32)
    pruned4 = np.zeros((nt, npts), np.float32)
    root = np.zeros((nt, 2), np.float32)
    w = L.prune_tiles(nt, boxes.ctypes.data, npts, pts.ctypes.data, bits.ctypes.data, ops.ctypes.data,
                      full.ctypes.data, pruned.ctypes.data, full4.ctypes.data, pruned4.ctypes.data, root.ctypes.data)
    return w, ops, full, pruned, full4, pruned4, root


def prune_host_in(cuda_src: str, parents: np.ndarray, boxes: np.ndarray, pts: np.ndarray):
    """The two-level tile pass on the host: bits of each parent box, then the
    tile's bits from them (s2m_user_sdf_tile_in); (ops per tile, pruned values,
    the interval of the SDF's value over each tile)."""
    L = compile_host(cuda_src)
    nt, npts = len(boxes), pts.shape[1]
    parents = np.ascontiguousarray(parents, np.float32)
    boxes = np.ascontiguousarray(boxes, np.float32)
    pts = np.ascontiguousarray(pts, np.float32)
    ops = np.zeros((nt, 2), np.float32)
    pruned = np.zeros((nt, npts), np.float32)
    root = np.zeros((nt, 2), np.float32)
    L.prune_tiles_in(nt, parents.ctypes.data, boxes.ctypes.data, npts, pts.ctypes.data, ops.ctypes.data,
                     pruned.ctypes.data, root.ctypes.data)
    return ops, pruned, root
