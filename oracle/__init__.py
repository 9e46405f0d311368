"""ctypes binding of the CPU oracle (test infrastructure only).

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg use
this module, as the checker.  The product package never imports it.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libs2m_oracle.so")

SPHERE, TORUS, CSG, MANDELBULB, TREE, MARTIN_CUBE, P_KEY = 0, 1, 2, 3, 4, 5, 6
F32, F64 = 0, 1
FLAG_SLICE_LAG = 1
FLAG_QEF = 2

_lock = threading.Lock()
_lib = None


class _Params(ctypes.Structure):
    _fields_ = [
        ("resolution", ctypes.c_uint32),
        ("bounds", ctypes.c_float),
        ("eps", ctypes.c_float),
        ("flags", ctypes.c_uint32),
        ("z_begin", ctypes.c_int32),
        ("z_end", ctypes.c_int32),
        ("threads", ctypes.c_int32),
        ("skip_quads", ctypes.c_int32),
    ]


class _Mesh(ctypes.Structure):
    _fields_ = [
        ("nverts", ctypes.c_int64),
        ("ntris", ctypes.c_int64),
        ("invalid_quads", ctypes.c_int64),
        ("pos", ctypes.POINTER(ctypes.c_float)),
        ("nrm", ctypes.POINTER(ctypes.c_float)),
        ("pos64", ctypes.POINTER(ctypes.c_double)),
        ("nrm64", ctypes.POINTER(ctypes.c_double)),
        ("cell", ctypes.POINTER(ctypes.c_uint16)),
        ("signs", ctypes.POINTER(ctypes.c_uint8)),
        ("tris", ctypes.POINTER(ctypes.c_uint32)),
        ("seconds_cells", ctypes.c_double),
        ("seconds_quads", ctypes.c_double),
    ]


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (g++, OpenMP)."""
    src = os.path.join(HERE, "s2m_oracle.cpp")
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            L = ctypes.CDLL(LIB_PATH)
            fp = ctypes.POINTER(ctypes.c_float)
            dp = ctypes.POINTER(ctypes.c_double)
            L.oracle_mesh_run.argtypes = [ctypes.c_int, fp, ctypes.c_int, ctypes.c_int,
                                          ctypes.POINTER(_Params), ctypes.POINTER(_Mesh)]
            L.oracle_mesh_free.argtypes = [ctypes.POINTER(_Mesh)]
            L.oracle_eval.argtypes = [ctypes.c_int, fp, ctypes.c_int, ctypes.c_int, dp,
                                      ctypes.c_int64, dp]
            L.oracle_cell_corners.argtypes = [ctypes.c_int, fp, ctypes.c_int, ctypes.c_int,
                                              ctypes.c_uint32, ctypes.c_float, ctypes.c_int32,
                                              ctypes.c_int32, ctypes.c_int32, dp]
            L.oracle_write_stl.argtypes = [fp, ctypes.POINTER(ctypes.c_uint32), ctypes.c_int64,
                                           ctypes.c_char_p]
            L.oracle_write_ply.argtypes = [fp, fp, ctypes.c_int64, ctypes.POINTER(ctypes.c_uint32),
                                           ctypes.c_int64, ctypes.c_char_p]
            L.oracle_format_f32.argtypes = [ctypes.c_float, ctypes.c_char_p, ctypes.c_int]
            _lib = L
    return _lib


def _fparams(params):
    a = np.ascontiguousarray(np.asarray(params, dtype=np.float32))
    return a, a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


class OracleMesh:
    """Host copy of an oracle result (positions, normals, cell labels, signs, triangles)."""

    def __init__(self, m: _Mesh, precision: int):
        nv, nt = int(m.nverts), int(m.ntris)
        self.nverts, self.ntris, self.invalid_quads = nv, nt, int(m.invalid_quads)
        if precision == F64:
            self.pos = np.ctypeslib.as_array(m.pos64, (3 * nv + 1,))[: 3 * nv].reshape(nv, 3).copy()
            self.nrm = np.ctypeslib.as_array(m.nrm64, (3 * nv + 1,))[: 3 * nv].reshape(nv, 3).copy()
        else:
            self.pos = np.ctypeslib.as_array(m.pos, (3 * nv + 1,))[: 3 * nv].reshape(nv, 3).copy()
            self.nrm = np.ctypeslib.as_array(m.nrm, (3 * nv + 1,))[: 3 * nv].reshape(nv, 3).copy()
        self.cell = np.ctypeslib.as_array(m.cell, (3 * nv + 1,))[: 3 * nv].reshape(nv, 3).copy()
        self.signs = np.ctypeslib.as_array(m.signs, (nv + 1,))[:nv].copy()
        self.tris = np.ctypeslib.as_array(m.tris, (3 * nt + 1,))[: 3 * nt].reshape(nt, 3).copy()
        self.seconds_cells = float(m.seconds_cells)
        self.seconds_quads = float(m.seconds_quads)


def mesh(kind, params, resolution, bounds, *, eps=1e-4, slice_lag=False, precision=F32,
         z_begin=-1, z_end=-1, threads=0, skip_quads=False, qef=False) -> OracleMesh:
    L = lib()
    a, ap = _fparams(params)
    flags = (FLAG_SLICE_LAG if slice_lag else 0) | (FLAG_QEF if qef else 0)
    p = _Params(resolution, bounds, eps, flags, z_begin, z_end, threads, 1 if skip_quads else 0)
    m = _Mesh()
    rc = L.oracle_mesh_run(kind, ap, len(a), precision, ctypes.byref(p), ctypes.byref(m))
    if rc != 0:
        raise RuntimeError(f"oracle_mesh_run failed ({rc})")
    try:
        return OracleMesh(m, precision)
    finally:
        L.oracle_mesh_free(ctypes.byref(m))


def evaluate(kind, params, xyz, precision=F32) -> np.ndarray:
    L = lib()
    a, ap = _fparams(params)
    pts = np.ascontiguousarray(np.asarray(xyz, dtype=np.float64).reshape(-1, 3))
    out = np.empty(len(pts), dtype=np.float64)
    L.oracle_eval(kind, ap, len(a), precision, pts.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                  len(pts), out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
    return out


def cell_corners(kind, params, resolution, bounds, x, y, z, precision=F32) -> np.ndarray:
    L = lib()
    a, ap = _fparams(params)
    out = np.empty(8, dtype=np.float64)
    L.oracle_cell_corners(kind, ap, len(a), precision, resolution, bounds, x, y, z,
                          out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
    return out


def format_f32(v: float) -> str:
    buf = ctypes.create_string_buffer(64)
    n = lib().oracle_format_f32(v, buf, 64)
    return buf.value[:n].decode()


def write_stl(pos, tris, path):
    pos = np.ascontiguousarray(pos, dtype=np.float32)
    tris = np.ascontiguousarray(tris, dtype=np.uint32)
    rc = lib().oracle_write_stl(pos.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                                tris.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)),
                                len(tris), path.encode())
    if rc != 0:
        raise OSError(path)


def write_ply(pos, nrm, tris, path):
    pos = np.ascontiguousarray(pos, dtype=np.float32)
    nrm = np.ascontiguousarray(nrm, dtype=np.float32)
    tris = np.ascontiguousarray(tris, dtype=np.uint32)
    rc = lib().oracle_write_ply(pos.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                                nrm.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), len(pos),
                                tris.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)),
                                len(tris), path.encode())
    if rc != 0:
        raise OSError(path)
