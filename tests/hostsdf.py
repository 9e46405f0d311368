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
                '#else\nextern "C" int eval_run4(long, const double*, double*) { return 0; }\n#endif\n')
    so = os.path.join(d, "sdf.so")
    subprocess.run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math",
                    src, "-o", so], check=True, capture_output=True)
    L = ctypes.CDLL(so)
    L.eval_points.argtypes = [ctypes.c_long, ctypes.c_void_p, ctypes.c_void_p]
    L.normal_points.argtypes = [ctypes.c_long, ctypes.c_void_p, ctypes.c_float, ctypes.c_void_p]
    L.eval_run4.argtypes = [ctypes.c_long, ctypes.c_void_p, ctypes.c_void_p]
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
