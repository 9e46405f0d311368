"""sdf2mesh_gb300 -- SDF to triangle mesh by dual contouring on one GB300.

Python mirror of the reference's interface (WilstonOreo/sdf2mesh), over the C
ABI of libsdf2mesh_gb300.so (include/sdf2mesh.h):

  Sdf3DShader.from_path(path)                      src/shader.rs:44-67
  Sdf3DShader.from_glsl_fragment_shader(path, sdf) src/shader.rs:73-104
  Sdf3DShader.write_to_file(path)                  src/shader.rs:206-209 (--debug-wgsl)
  AppState.from_args(resolution, bounds)           src/bin/sdf2mesh/main.rs:139-175
  generate(shader, state) -> TriangleMesh          src/bin/sdf2mesh/main.rs:298-357
  TriangleMesh.write_to_file / write_stl_to_file / write_ply_to_file
                                                   src/mesh.rs:167-210

All meshing runs on the GPU through the library; there is no CPU path.  The
library must have been built (python -m sdf2mesh_gb300.build) and a CUDA
device must be present, otherwise these calls raise.
"""
from __future__ import annotations

import ctypes
import os
import threading
from dataclasses import dataclass, field

import numpy as np

__all__ = [
    "S2MError", "Sdf3DShader", "CompiledSdf", "AppState", "DeviceMesh", "TriangleMesh", "generate", "Batch", "Server",
    "load_library", "translate", "wgsl_remove_function", "wgsl_rename_function", "wgsl_has_function",
    "LANG_WGSL", "LANG_GLSL", "LANG_SHADERTOY", "JOB_POW2_ROUNDING", "JOB_SLICE_LAG", "JOB_EXACT_CORNERS", "JOB_QEF", "COMPILE_FMAD", "COMPILE_NO_PRUNE",
]

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libsdf2mesh_gb300.so")

LANG_WGSL, LANG_GLSL, LANG_SHADERTOY = 0, 1, 2
COMPILE_FMAD = 0x1
COMPILE_NO_PRUNE = 0x2
EVAL_VARIANTS = 8
JOB_POW2_ROUNDING, JOB_SLICE_LAG, JOB_EXACT_CORNERS, JOB_QEF = 0x1, 0x2, 0x4, 0x8

S2M_OK = 0
STATUS_NAMES = {0: "OK", 1: "INVALID", 2: "IO", 3: "PARSE", 4: "MISSING_SDF", 5: "NVRTC", 6: "CUDA",
                7: "OOM", 8: "OVERFLOW", 9: "TIMEOUT", 10: "NO_DEVICE"}


class S2MError(RuntimeError):
    def __init__(self, status: int, message: str):
        self.status = status
        self.name = STATUS_NAMES.get(status, str(status))
        super().__init__(f"[{self.name}] {message}")


class Params(ctypes.Structure):
    _fields_ = [
        ("resolution", ctypes.c_uint32), ("bounds", ctypes.c_float), ("eps", ctypes.c_float),
        ("flags", ctypes.c_uint32), ("slab_depth", ctypes.c_uint32), ("reserved", ctypes.c_uint32),
        ("max_vertices", ctypes.c_uint64), ("max_triangles", ctypes.c_uint64),
    ]


class MeshInfo(ctypes.Structure):
    _fields_ = [
        ("nverts", ctypes.c_uint64), ("ntris", ctypes.c_uint64), ("invalid_quads", ctypes.c_uint64),
        ("cells", ctypes.c_uint64), ("candidate_cells", ctypes.c_uint64), ("resolution", ctypes.c_uint32),
        ("slab_depth", ctypes.c_uint32), ("d_pos", ctypes.c_void_p), ("d_nrm", ctypes.c_void_p),
        ("d_cell", ctypes.c_void_p), ("d_tris", ctypes.c_void_p), ("kernel_launches", ctypes.c_uint64),
        ("host_setup_ms", ctypes.c_double), ("host_launch_ms", ctypes.c_double), ("host_wait_ms", ctypes.c_double),
        ("runs", ctypes.c_uint32), ("reserved", ctypes.c_uint32),
    ]


class HostMesh(ctypes.Structure):
    """s2m_host_mesh: the mesh in library-owned pinned host memory."""
    _fields_ = [("pos", ctypes.c_void_p), ("nrm", ctypes.c_void_p), ("tris", ctypes.c_void_p),
                ("nverts", ctypes.c_uint64), ("ntris", ctypes.c_uint64), ("invalid_quads", ctypes.c_uint64),
                ("resolution", ctypes.c_uint32), ("parts", ctypes.c_uint32), ("owner", ctypes.c_void_p)]


class NoallocMesh(ctypes.Structure):
    """s2m_noalloc_mesh: caller-owned device outputs and the counts written back."""
    _fields_ = [("pos", ctypes.c_void_p), ("nrm", ctypes.c_void_p), ("cell", ctypes.c_void_p),
                ("tris", ctypes.c_void_p), ("max_vertices", ctypes.c_uint64), ("max_triangles", ctypes.c_uint64),
                ("nverts", ctypes.c_uint64), ("ntris", ctypes.c_uint64), ("invalid_quads", ctypes.c_uint64),
                ("candidate_cells", ctypes.c_uint64), ("resolution", ctypes.c_uint32), ("reserved", ctypes.c_uint32)]


NOALLOC_SCRATCH_BYTES = 64 << 20
NOALLOC_MAX_RESOLUTION = 256

class ServerConfig(ctypes.Structure):
    _fields_ = [("memory_budget_bytes", ctypes.c_uint64), ("max_inflight", ctypes.c_uint32),
                ("max_batch_jobs", ctypes.c_uint32), ("keep_results", ctypes.c_uint32),
                ("sdf_workers", ctypes.c_uint32), ("flags", ctypes.c_uint32), ("reserved", ctypes.c_uint32)]


SERVER_INTERPRET_ONLY = 0x1


class ServerStats(ctypes.Structure):
    _fields_ = [("submitted", ctypes.c_uint64), ("completed", ctypes.c_uint64), ("failed", ctypes.c_uint64),
                ("batches", ctypes.c_uint64), ("peak_bytes", ctypes.c_uint64), ("p50_ms", ctypes.c_double),
                ("p99_ms", ctypes.c_double), ("mean_ms", ctypes.c_double), ("span_s", ctypes.c_double),
                ("meshes_per_s", ctypes.c_double), ("gvoxels_per_s", ctypes.c_double),
                ("ran_compiled", ctypes.c_uint64), ("ran_interpreted", ctypes.c_uint64),
                ("compiled_sources", ctypes.c_uint64), ("compiles_pending", ctypes.c_uint64)]


KERNEL_KINDS = ("eval_planes", "cells", "vertices", "vcompact", "rowscan", "quads")


class Profile(ctypes.Structure):
    _fields_ = [("ms", ctypes.c_double * 6), ("launches", ctypes.c_uint64 * 6), ("eval_points", ctypes.c_double),
                ("cells", ctypes.c_double)]


_lib = None
_lock = threading.Lock()


def load_library(path: str | None = None) -> ctypes.CDLL:
    """Load libsdf2mesh_gb300.so (built in-tree); raises if it is missing."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        p = path or LIB_PATH
        if not os.path.exists(p):
            raise S2MError(1, f"{p} is not built; run `python -m sdf2mesh_gb300.build`")
        L = ctypes.CDLL(p)
        c_char_pp = ctypes.POINTER(ctypes.c_char_p)
        vp, sz, u32, u64, i = ctypes.c_void_p, ctypes.c_size_t, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_int
        dp = ctypes.POINTER(ctypes.c_double)
        sigs = {
            "s2m_abi_version": ([], i),
            "s2m_status_string": ([i], ctypes.c_char_p),
            "s2m_free_string": ([vp], None),
            "s2m_preprocess_file": ([ctypes.c_char_p, ctypes.POINTER(vp), ctypes.c_char_p, sz], i),
            "s2m_preprocess_source": ([ctypes.c_char_p, ctypes.c_char_p, ctypes.POINTER(vp), ctypes.c_char_p,
                                       sz], i),
            "s2m_translate": ([ctypes.c_char_p, i, ctypes.c_char_p, ctypes.POINTER(vp), dp, dp,
                               ctypes.c_char_p, sz], i),
            "s2m_compile": ([ctypes.c_char_p, i, ctypes.c_char_p, u32, ctypes.POINTER(vp), ctypes.c_char_p, sz], i),
            "s2m_compile_file": ([ctypes.c_char_p, i, ctypes.c_char_p, u32, ctypes.POINTER(vp),
                                  ctypes.c_char_p, sz], i),
            "s2m_sdf_cuda_source": ([vp], ctypes.c_char_p),
            "s2m_sdf_compile_info": ([vp, dp, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)], i),
            "s2m_sdf_op_counts": ([vp, dp, dp], i),
            "s2m_sdf_run_op_counts": ([vp, dp, dp], i),
            "s2m_sdf_set_eval_variant": ([vp, i], i),
            "s2m_sdf_prune_info": ([vp, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)], i),
            "s2m_mesh_eval_ops": ([vp, dp, dp, dp], i),
            "s2m_sdf_free": ([vp], None),
            "s2m_sdf_eval_variant": ([vp, ctypes.c_char_p, sz, dp], i),
            "s2m_sdf_eval_variant_info": ([vp, i, ctypes.c_char_p, sz, ctypes.POINTER(ctypes.c_int),
                                           ctypes.POINTER(ctypes.c_int)], i),
            "s2m_wgsl_remove_function": ([ctypes.c_char_p, ctypes.c_char_p, ctypes.POINTER(vp)], i),
            "s2m_wgsl_rename_function": ([ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p,
                                          ctypes.POINTER(vp)], i),
            "s2m_wgsl_has_function": ([ctypes.c_char_p, ctypes.c_char_p], i),
            "s2m_mesh_create": ([vp, ctypes.POINTER(Params), vp, ctypes.POINTER(vp), ctypes.c_char_p, sz], i),
            "s2m_mesh_run_async": ([vp, vp], i),
            "s2m_mesh_sync": ([vp, vp, ctypes.c_char_p, sz], i),
            "s2m_mesh_get_info": ([vp, ctypes.POINTER(MeshInfo)], i),
            "s2m_mesh_footprint": ([vp, ctypes.POINTER(Params), ctypes.POINTER(u64)], i),
            "s2m_mesh_copy_to_host": ([vp, vp, vp, vp, vp, vp], i),
            "s2m_mesh_write": ([vp, ctypes.c_char_p, ctypes.c_char_p, sz], i),
            "s2m_mesh_free": ([vp], None),
            "s2m_write_stl": ([vp, vp, u64, ctypes.c_char_p], i),
            "s2m_write_stl_binary": ([vp, vp, u64, ctypes.c_char_p], i),
            "s2m_mesh_write_stl_binary": ([vp, ctypes.c_char_p, ctypes.c_char_p, sz], i),
            "s2m_write_ply": ([vp, vp, u64, vp, u64, ctypes.c_char_p], i),
            "s2m_measure_fp32_peak": ([dp, vp], i),
            "s2m_mesh_noalloc": ([vp, ctypes.POINTER(Params), ctypes.POINTER(NoallocMesh), vp, ctypes.c_char_p, sz],
                                 i),
            "s2m_mesh_set_profiling": ([vp, i], i),
            "s2m_mesh_set_graph": ([vp, i], i),
            "s2m_mesh_set_wait_limit": ([vp, ctypes.c_double], i),
            "s2m_batch_set_wait_limit": ([vp, ctypes.c_double, ctypes.c_double], i),
            "s2m_batch_set_pruning": ([vp, i], i),
            "s2m_mesh_generate": ([vp, ctypes.POINTER(Params), u32, vp, ctypes.POINTER(HostMesh), ctypes.c_char_p,
                                   sz], i),
            "s2m_host_mesh_free": ([ctypes.POINTER(HostMesh)], None),
            "s2m_batch_stage_profile": ([vp, dp, u32, dp], i),
            "s2m_measure_sfu_peak": ([dp, vp], i),
            "s2m_csg_from_source": ([ctypes.c_char_p, ctypes.POINTER(ctypes.c_float), u32, ctypes.POINTER(u32),
                                     ctypes.c_char_p, sz], i),
            "s2m_batch_create": ([ctypes.POINTER(vp), u64], i),
            "s2m_batch_add_csg": ([vp, ctypes.POINTER(ctypes.c_float), u32, ctypes.POINTER(Params),
                                   ctypes.POINTER(u32), ctypes.c_char_p, sz], i),
            "s2m_batch_job_footprint": ([vp, u32], u64),
            "s2m_batch_run": ([vp, vp, ctypes.c_char_p, sz], i),
            "s2m_batch_job_info": ([vp, u32, ctypes.POINTER(MeshInfo)], i),
            "s2m_batch_job_copy_to_host": ([vp, u32, vp, vp, vp, vp, vp], i),
            "s2m_batch_stats": ([vp, dp, ctypes.POINTER(u64), ctypes.POINTER(u32)], i),
            "s2m_batch_free": ([vp], None),
            "s2m_server_create": ([ctypes.POINTER(ServerConfig), ctypes.POINTER(vp), ctypes.c_char_p, sz], i),
            "s2m_server_submit_csg": ([vp, ctypes.POINTER(ctypes.c_float), u32, ctypes.POINTER(Params),
                                       ctypes.POINTER(u64), ctypes.c_char_p, sz], i),
            "s2m_server_submit_sdf": ([vp, vp, ctypes.POINTER(Params), ctypes.POINTER(u64), ctypes.c_char_p, sz], i),
            "s2m_server_submit_source": ([vp, ctypes.c_char_p, i, ctypes.c_char_p, ctypes.POINTER(Params),
                                          ctypes.POINTER(u64), ctypes.c_char_p, sz], i),
            "s2m_server_wait": ([vp, u64, ctypes.c_double, ctypes.POINTER(MeshInfo), ctypes.c_char_p, sz], i),
            "s2m_server_copy_to_host": ([vp, u64, vp, vp, vp, vp], i),
            "s2m_server_release": ([vp, u64], i),
            "s2m_server_drain": ([vp, ctypes.c_double], i),
            "s2m_server_get_stats": ([vp, ctypes.POINTER(ServerStats)], i),
            "s2m_server_reset_stats": ([vp], i),
            "s2m_server_free": ([vp], None),
            "s2m_mesh_get_profile": ([vp, ctypes.POINTER(Profile)], i),
            "s2m_mesh_reset_profile": ([vp], i),
        }
        for name, (args, res) in sigs.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = res
        del c_char_pp
        _lib = L
        return L


def _errbuf():
    return ctypes.create_string_buffer(8192)


def _check(rc: int, err=None, what: str = ""):
    if rc != S2M_OK:
        msg = err.value.decode(errors="replace") if err is not None else ""
        raise S2MError(rc, f"{what}: {msg}" if what else msg)


def _take_string(p: ctypes.c_void_p) -> str:
    if not p.value:
        return ""
    s = ctypes.string_at(p.value).decode()
    load_library().s2m_free_string(p)
    return s


# ---------------------------------------------------------------------------
# Shader front end


def translate(source: str, lang: int = LANG_WGSL, sdf_name: str = "sdf"):
    """Lower an SDF source to CUDA C (frontend only, no GPU). Returns (cuda, fp32_ops, sfu_ops)."""
    L = load_library()
    out = ctypes.c_void_p()
    fp, sfu = ctypes.c_double(), ctypes.c_double()
    err = _errbuf()
    rc = L.s2m_translate(source.encode(), lang, sdf_name.encode(), ctypes.byref(out), ctypes.byref(fp),
                         ctypes.byref(sfu), err, len(err))
    _check(rc, err, "translate")
    return _take_string(out), fp.value, sfu.value


def wgsl_remove_function(wgsl: str, function_name: str) -> str:
    out = ctypes.c_void_p()
    rc = load_library().s2m_wgsl_remove_function(wgsl.encode(), function_name.encode(), ctypes.byref(out))
    if rc != S2M_OK:
        raise S2MError(rc, f"Function {function_name} not found in shader")
    return _take_string(out)


def wgsl_rename_function(wgsl: str, old: str, new: str) -> str:
    out = ctypes.c_void_p()
    rc = load_library().s2m_wgsl_rename_function(wgsl.encode(), old.encode(), new.encode(), ctypes.byref(out))
    if rc != S2M_OK:
        raise S2MError(rc, f"Function `{old}` not found in shader")
    return _take_string(out)


def wgsl_has_function(wgsl: str, function_name: str) -> bool:
    return bool(load_library().s2m_wgsl_has_function(wgsl.encode(), function_name.encode()))


class CompiledSdf:
    """An SDF compiled for sm_103a (frontend -> CUDA C -> NVRTC)."""

    def __init__(self, handle: ctypes.c_void_p):
        self._h = handle

    @property
    def handle(self):
        return self._h

    @property
    def cuda_source(self) -> str:
        return load_library().s2m_sdf_cuda_source(self._h).decode()

    def compile_info(self) -> dict:
        """NVRTC wall seconds, programs, and programs read from the on-disk module cache."""
        sec, progs, hits = ctypes.c_double(), ctypes.c_int(), ctypes.c_int()
        _check(load_library().s2m_sdf_compile_info(self._h, ctypes.byref(sec), ctypes.byref(progs),
                                                   ctypes.byref(hits)), None, "compile info")
        return {"nvrtc_s": sec.value, "programs": progs.value, "cache_hits": hits.value}

    def run_op_counts(self):
        """Ops per point in runs of 4 sharing x and y, or None when the SDF has no run form."""
        fp, sfu = ctypes.c_double(), ctypes.c_double()
        rc = load_library().s2m_sdf_run_op_counts(self._h, ctypes.byref(fp), ctypes.byref(sfu))
        return (fp.value, sfu.value) if rc == 0 else None

    def op_counts(self):
        fp, sfu = ctypes.c_double(), ctypes.c_double()
        load_library().s2m_sdf_op_counts(self._h, ctypes.byref(fp), ctypes.byref(sfu))
        return fp.value, sfu.value

    def eval_variant(self):
        """(name, ns per lattice point of each variant) chosen by the autotuner; name is 'untuned' before the first job."""
        name = ctypes.create_string_buffer(64)
        ns = (ctypes.c_double * EVAL_VARIANTS)()
        load_library().s2m_sdf_eval_variant(self._h, name, 64, ns)
        return name.value.decode(), list(ns)

    def set_eval_variant(self, variant: int) -> None:
        """Use evaluation variant `variant` (0 .. EVAL_VARIANTS - 1) instead of tuning."""
        _check(load_library().s2m_sdf_set_eval_variant(self._h, variant), None, f"eval variant {variant}")

    def prune_info(self):
        """(combinators that can prune, activity words per tile); (0, 0) without tile pruning."""
        c, w = ctypes.c_int(), ctypes.c_int()
        load_library().s2m_sdf_prune_info(self._h, ctypes.byref(c), ctypes.byref(w))
        return c.value, w.value

    def eval_variants(self):
        """Per variant: (name, ns per point, registers, local bytes) as the autotuner measured them."""
        _, ns = self.eval_variant()
        out = []
        for v in range(len(ns)):
            name = ctypes.create_string_buffer(64)
            regs, loc = ctypes.c_int(), ctypes.c_int()
            load_library().s2m_sdf_eval_variant_info(self._h, v, name, 64, ctypes.byref(regs), ctypes.byref(loc))
            out.append((name.value.decode(), ns[v], regs.value, loc.value))
        return out

    def close(self):
        if self._h:
            load_library().s2m_sdf_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


@dataclass
class Sdf3DShader:
    """The SDF source: preprocessed WGSL (`.sdf3d`) or GLSL with a named function."""

    source: str = ""
    lang: int = LANG_WGSL
    sdf_name: str = "sdf"

    @classmethod
    def from_path(cls, path: str) -> "Sdf3DShader":
        """Read a .sdf3d file and expand its `use` / `include` lines (shader.rs:44-67)."""
        L = load_library()
        out = ctypes.c_void_p()
        err = _errbuf()
        _check(L.s2m_preprocess_file(os.fspath(path).encode(), ctypes.byref(out), err, len(err)), err, path)
        return cls(_take_string(out), LANG_WGSL, "sdf")

    @classmethod
    def from_source(cls, source: str, lang: int = LANG_WGSL, sdf_name: str = "sdf",
                    base_dir: str | None = None) -> "Sdf3DShader":
        """In-memory source; WGSL gets the same `use` / `include` expansion as a file."""
        if lang == LANG_WGSL:
            L = load_library()
            out = ctypes.c_void_p()
            err = _errbuf()
            _check(L.s2m_preprocess_source(source.encode(), (base_dir or "").encode(), ctypes.byref(out), err,
                                           len(err)), err, "preprocess")
            source = _take_string(out)
        return cls(source, lang, sdf_name)

    @classmethod
    def from_glsl_fragment_shader(cls, path: str, sdf: str = "sdf") -> "Sdf3DShader":
        with open(path) as f:
            return cls(f.read(), LANG_GLSL, sdf)

    def write_to_file(self, path: str) -> None:
        with open(path, "w") as f:
            f.write(self.source)

    def csg_program(self) -> np.ndarray:
        """The batch interpreter's CSG program of this source (raises for non-CSG sources)."""
        L = load_library()
        n = ctypes.c_uint32()
        err = _errbuf()
        _check(L.s2m_csg_from_source(self.source.encode(), None, 0, ctypes.byref(n), err, len(err)), err, "csg")
        prog = np.empty(n.value, np.float32)
        _check(L.s2m_csg_from_source(self.source.encode(), prog.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                                     n.value, ctypes.byref(n), err, len(err)), err, "csg")
        return prog

    def compile(self, fmad: bool = False, prune: bool = True) -> CompiledSdf:
        """NVRTC module for sm_103a.  fmad: FMA contraction (not bit-exact);
        prune=False: no tile pruning (every operation at every point)."""
        L = load_library()
        h = ctypes.c_void_p()
        err = _errbuf()
        flags = (COMPILE_FMAD if fmad else 0) | (0 if prune else COMPILE_NO_PRUNE)
        rc = L.s2m_compile(self.source.encode(), self.lang, self.sdf_name.encode(),
                           flags, ctypes.byref(h), err, len(err))
        _check(rc, err, "compile")
        return CompiledSdf(h)


@dataclass
class AppState:
    """Job parameters (main.rs:12-64, 139-175).

    `reference_rounding` rounds a non-power-of-two resolution up as the
    reference CLI does; `slice_lag` reproduces its read-before-submit lag.
    """

    resolution: int = 256
    bounds: float = 2.0
    eps: float = 1e-4
    reference_rounding: bool = False
    slice_lag: bool = False
    exact_corners: bool = False
    qef: bool = False
    slab_depth: int = 0
    max_vertices: int = 0
    max_triangles: int = 0

    @classmethod
    def from_args(cls, resolution: int | None = None, bounds: float | None = None, **kw) -> "AppState":
        """The reference CLI's defaults and quirks: N=256, B=2, pow2 rounding, slice lag."""
        kw.setdefault("reference_rounding", True)
        kw.setdefault("slice_lag", True)
        return cls(resolution if resolution is not None else 256, bounds if bounds is not None else 2.0, **kw)

    def params(self) -> Params:
        flags = ((JOB_POW2_ROUNDING if self.reference_rounding else 0) | (JOB_SLICE_LAG if self.slice_lag else 0)
                 | (JOB_EXACT_CORNERS if self.exact_corners else 0) | (JOB_QEF if self.qef else 0))
        return Params(self.resolution, self.bounds, self.eps, flags, self.slab_depth, 0, self.max_vertices,
                      self.max_triangles)


class DeviceMesh:
    """A mesh in device memory (owned by the library)."""

    def __init__(self, handle: ctypes.c_void_p, sdf: CompiledSdf):
        self._h = handle
        self._sdf = sdf  # keep the module alive

    @property
    def handle(self):
        return self._h

    def info(self) -> MeshInfo:
        mi = MeshInfo()
        load_library().s2m_mesh_get_info(self._h, ctypes.byref(mi))
        return mi

    def run_async(self, stream: int = 0) -> None:
        _check(load_library().s2m_mesh_run_async(self._h, ctypes.c_void_p(stream)), None, "run")

    def sync(self, stream: int = 0) -> None:
        err = _errbuf()
        _check(load_library().s2m_mesh_sync(self._h, ctypes.c_void_p(stream), err, len(err)), err, "sync")

    def set_graph(self, enable: bool = True) -> None:
        """Replay the pipeline as a CUDA graph in run_async."""
        _check(load_library().s2m_mesh_set_graph(self._h, 1 if enable else 0), None, "graph")

    def set_wait_limit(self, seconds: float) -> None:
        """Bound of each device-side wait of this mesh's runs (default 2 s)."""
        _check(load_library().s2m_mesh_set_wait_limit(self._h, float(seconds)), None, "wait limit")

    def set_profiling(self, enable: bool = True) -> None:
        """Record CUDA events around every kernel of later runs."""
        _check(load_library().s2m_mesh_set_profiling(self._h, 1 if enable else 0), None, "profiling")

    def profile(self) -> dict:
        """Accumulated per-kernel device time (ms) and launch counts."""
        pr = Profile()
        _check(load_library().s2m_mesh_get_profile(self._h, ctypes.byref(pr)), None, "profile")
        return {"ms": {k: pr.ms[i] for i, k in enumerate(KERNEL_KINDS)},
                "launches": {k: int(pr.launches[i]) for i, k in enumerate(KERNEL_KINDS)},
                "eval_points": pr.eval_points, "cells": pr.cells}

    def eval_ops(self) -> dict:
        """SDF operations the last run's lattice evaluation executed."""
        pts, fp, sfu = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        rc = load_library().s2m_mesh_eval_ops(self._h, ctypes.byref(pts), ctypes.byref(fp), ctypes.byref(sfu))
        return {"pruned": rc == 1, "points": pts.value, "fp32_ops": fp.value, "sfu_ops": sfu.value}

    def reset_profile(self) -> None:
        _check(load_library().s2m_mesh_reset_profile(self._h), None, "profile")

    def to_host(self, stream: int = 0) -> "TriangleMesh":
        mi = self.info()
        nv, nt = int(mi.nverts), int(mi.ntris)
        pos = np.empty((nv, 3), np.float32)
        nrm = np.empty((nv, 3), np.float32)
        cell = np.empty(nv, np.uint64)
        tris = np.empty((nt, 3), np.uint32)
        _check(load_library().s2m_mesh_copy_to_host(self._h, pos.ctypes.data, nrm.ctypes.data, cell.ctypes.data,
                                                     tris.ctypes.data, ctypes.c_void_p(stream)), None, "copy")
        return TriangleMesh(pos, nrm, tris, cell, int(mi.invalid_quads), mi)

    def write_to_file(self, path: str) -> None:
        err = _errbuf()
        _check(load_library().s2m_mesh_write(self._h, os.fspath(path).encode(), err, len(err)), err, "write")

    def close(self):
        if self._h:
            load_library().s2m_mesh_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


@dataclass
class TriangleMesh:
    """Host mesh: vertices (positions + normals) and triangle indices (mesh.rs:143-211)."""

    positions: np.ndarray
    normals: np.ndarray
    triangle_indices: np.ndarray
    cells: np.ndarray = field(default_factory=lambda: np.empty(0, np.uint64))
    invalid_quads: int = 0
    info: object = None

    @property
    def cell_xyz(self) -> np.ndarray:
        """Cell labels (x, y, z) of each vertex (mesh.rs:213-227)."""
        c = self.cells.astype(np.uint64)
        return np.stack([c & 0xFFFF, (c >> 16) & 0xFFFF, (c >> 32) & 0xFFFF], axis=1).astype(np.uint16)

    @property
    def signs(self) -> np.ndarray:
        return ((self.cells >> np.uint64(48)) & np.uint64(0xF)).astype(np.uint8)

    def write_stl_to_file(self, path: str) -> None:
        pos = np.ascontiguousarray(self.positions, np.float32)
        tris = np.ascontiguousarray(self.triangle_indices, np.uint32)
        _check(load_library().s2m_write_stl(pos.ctypes.data, tris.ctypes.data, len(tris), os.fspath(path).encode()),
               None, f"write {path}")

    def write_stl_binary_to_file(self, path: str) -> None:
        """Binary STL: same facets and normals as the ASCII writer, 50 bytes each."""
        pos = np.ascontiguousarray(self.positions, np.float32)
        tris = np.ascontiguousarray(self.triangle_indices, np.uint32)
        _check(load_library().s2m_write_stl_binary(pos.ctypes.data, tris.ctypes.data, len(tris),
                                                   os.fspath(path).encode()), None, f"write {path}")

    def write_ply_to_file(self, path: str) -> None:
        pos = np.ascontiguousarray(self.positions, np.float32)
        nrm = np.ascontiguousarray(self.normals, np.float32)
        tris = np.ascontiguousarray(self.triangle_indices, np.uint32)
        _check(load_library().s2m_write_ply(pos.ctypes.data, nrm.ctypes.data, len(pos), tris.ctypes.data,
                                            len(tris), os.fspath(path).encode()), None, f"write {path}")

    def write_to_file(self, path: str) -> None:
        ext = os.path.splitext(os.fspath(path))[1][1:].upper()
        if ext == "STL":
            self.write_stl_to_file(path)
        elif ext == "PLY":
            self.write_ply_to_file(path)
        else:
            raise S2MError(1, f"Unknown file extension: {ext}")


class Batch:
    """Many CSG jobs meshed in one persistent launch (s2m_batch_*).

    A job is a CSG program: a postfix list of floats, opcodes S2M_CSG_* each
    followed by its operands (see include/sdf2mesh.h); `workloads.random_tree`
    returns one beside the equivalent .sdf3d source."""

    def __init__(self, memory_budget_bytes: int = 0):
        self._h = ctypes.c_void_p()
        _check(load_library().s2m_batch_create(ctypes.byref(self._h), memory_budget_bytes), None, "batch")
        self.njobs = 0

    def add_csg(self, program, state: AppState) -> int:
        prog = np.ascontiguousarray(np.asarray(program, np.float32))
        p = state.params()
        jid = ctypes.c_uint32()
        err = _errbuf()
        rc = load_library().s2m_batch_add_csg(self._h, prog.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                                              len(prog), ctypes.byref(p), ctypes.byref(jid), err, len(err))
        _check(rc, err, "batch add")
        self.njobs += 1
        return int(jid.value)

    def footprint(self, job: int) -> int:
        return int(load_library().s2m_batch_job_footprint(self._h, job))

    def set_wait_limit(self, stage_seconds: float, lookback_seconds: float = 2.0) -> None:
        """Bounds of the persistent kernel's device waits (defaults 30 s and 2 s)."""
        _check(load_library().s2m_batch_set_wait_limit(self._h, float(stage_seconds), float(lookback_seconds)),
               None, "wait limit")

    BATCH_STAGES = ("tiles", "lattice", "cell_bits", "cell_slots", "candidates", "vertices", "vcompact", "rowscan",
                    "quads")

    def stage_profile(self) -> dict:
        """Block time (ms, summed over blocks) of the last run per stage, and the
        block time spent waiting for a job's previous stage."""
        n = len(self.BATCH_STAGES)
        busy = (ctypes.c_double * n)()
        wait = ctypes.c_double()
        _check(load_library().s2m_batch_stage_profile(self._h, busy, n, ctypes.byref(wait)), None, "profile")
        out = {k: float(busy[i]) for i, k in enumerate(self.BATCH_STAGES)}
        out["waiting"] = float(wait.value)
        return out

    def set_pruning(self, enabled: bool) -> None:
        """Tile pruning of the programs (default on) for jobs not run yet; the
        meshes are bit-identical either way."""
        _check(load_library().s2m_batch_set_pruning(self._h, int(bool(enabled))), None, "pruning")

    def run(self, stream: int = 0) -> None:
        err = _errbuf()
        _check(load_library().s2m_batch_run(self._h, ctypes.c_void_p(stream), err, len(err)), err, "batch run")

    def info(self, job: int) -> MeshInfo:
        mi = MeshInfo()
        _check(load_library().s2m_batch_job_info(self._h, job, ctypes.byref(mi)), None, "batch info")
        return mi

    def mesh(self, job: int, stream: int = 0) -> "TriangleMesh":
        mi = self.info(job)
        nv, nt = int(mi.nverts), int(mi.ntris)
        pos = np.empty((nv, 3), np.float32)
        nrm = np.empty((nv, 3), np.float32)
        cell = np.empty(nv, np.uint64)
        tris = np.empty((nt, 3), np.uint32)
        _check(load_library().s2m_batch_job_copy_to_host(self._h, job, pos.ctypes.data, nrm.ctypes.data,
                                                          cell.ctypes.data, tris.ctypes.data,
                                                          ctypes.c_void_p(stream)), None, "batch copy")
        return TriangleMesh(pos, nrm, tris, cell, int(mi.invalid_quads), mi)

    def stats(self):
        ms, launches, n = ctypes.c_double(), ctypes.c_uint64(), ctypes.c_uint32()
        load_library().s2m_batch_stats(self._h, ctypes.byref(ms), ctypes.byref(launches), ctypes.byref(n))
        return ms.value, int(launches.value), int(n.value)

    def close(self):
        if self._h:
            load_library().s2m_batch_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """Continuous-batching request loop (s2m_server_*): submit CSG programs or
    compiled SDFs from any thread; results complete asynchronously."""

    def __init__(self, memory_budget_bytes: int = 0, max_inflight: int = 2, max_batch_jobs: int = 1024,
                 keep_results: bool = True, sdf_workers: int = 4, interpret_only: bool = False):
        cfg = ServerConfig(memory_budget_bytes, max_inflight, max_batch_jobs, 1 if keep_results else 0, sdf_workers,
                           SERVER_INTERPRET_ONLY if interpret_only else 0, 0)
        self._h = ctypes.c_void_p()
        err = _errbuf()
        _check(load_library().s2m_server_create(ctypes.byref(cfg), ctypes.byref(self._h), err, len(err)), err,
               "server")
        self._keep = []

    def submit_csg(self, program, state: AppState) -> int:
        prog = np.ascontiguousarray(np.asarray(program, np.float32))
        p = state.params()
        rid = ctypes.c_uint64()
        err = _errbuf()
        _check(load_library().s2m_server_submit_csg(self._h, prog.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                                                     len(prog), ctypes.byref(p), ctypes.byref(rid), err, len(err)),
               err, "submit")
        return int(rid.value)

    def submit_sdf(self, sdf: "CompiledSdf", state: AppState) -> int:
        self._keep.append(sdf)
        p = state.params()
        rid = ctypes.c_uint64()
        err = _errbuf()
        _check(load_library().s2m_server_submit_sdf(self._h, sdf.handle, ctypes.byref(p), ctypes.byref(rid), err,
                                                     len(err)), err, "submit")
        return int(rid.value)

    def submit_source(self, source: str, state: AppState, lang: int = LANG_WGSL, sdf_name: str = "sdf") -> int:
        """Submit .sdf3d / GLSL text: CSG expressions run on the interpreter, others compile once (cached)."""
        p = state.params()
        rid = ctypes.c_uint64()
        err = _errbuf()
        _check(load_library().s2m_server_submit_source(self._h, source.encode(), lang, sdf_name.encode(),
                                                        ctypes.byref(p), ctypes.byref(rid), err, len(err)),
               err, "submit")
        return int(rid.value)

    def wait(self, request: int, timeout_s: float = 600.0) -> MeshInfo:
        mi = MeshInfo()
        err = _errbuf()
        _check(load_library().s2m_server_wait(self._h, request, timeout_s, ctypes.byref(mi), err, len(err)), err,
               f"request {request}")
        return mi

    def mesh(self, request: int) -> "TriangleMesh":
        mi = self.wait(request)
        nv, nt = int(mi.nverts), int(mi.ntris)
        pos = np.empty((nv, 3), np.float32)
        nrm = np.empty((nv, 3), np.float32)
        cell = np.empty(nv, np.uint64)
        tris = np.empty((nt, 3), np.uint32)
        _check(load_library().s2m_server_copy_to_host(self._h, request, pos.ctypes.data, nrm.ctypes.data,
                                                       cell.ctypes.data, tris.ctypes.data), None, "copy")
        return TriangleMesh(pos, nrm, tris, cell, int(mi.invalid_quads), mi)

    def release(self, request: int) -> None:
        load_library().s2m_server_release(self._h, request)

    def drain(self, timeout_s: float = 3600.0) -> None:
        _check(load_library().s2m_server_drain(self._h, timeout_s), None, "drain")

    def stats(self) -> dict:
        st = ServerStats()
        load_library().s2m_server_get_stats(self._h, ctypes.byref(st))
        return {k: getattr(st, k) for k, _ in ServerStats._fields_}

    def reset_stats(self) -> None:
        """A new measurement window (after drain); compiled sources stay cached."""
        _check(load_library().s2m_server_reset_stats(self._h), None, "reset stats")

    def close(self):
        if self._h:
            load_library().s2m_server_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def mesh_device(sdf, state: AppState, stream: int = 0) -> DeviceMesh:
    """Run the whole pipeline on the GPU; the mesh stays in device memory."""
    compiled = sdf.compile() if isinstance(sdf, Sdf3DShader) else sdf
    L = load_library()
    p = state.params()
    h = ctypes.c_void_p()
    err = _errbuf()
    rc = L.s2m_mesh_create(compiled.handle, ctypes.byref(p), ctypes.c_void_p(stream), ctypes.byref(h), err, len(err))
    _check(rc, err, "mesh")
    return DeviceMesh(h, compiled)


def mesh_footprint(sdf, state: AppState) -> int:
    """Device bytes s2m_mesh_create allocates for this job (its first attempt)."""
    compiled = sdf.compile() if isinstance(sdf, Sdf3DShader) else sdf
    p = state.params()
    b = ctypes.c_uint64()
    _check(load_library().s2m_mesh_footprint(compiled.handle, ctypes.byref(p), ctypes.byref(b)), None, "footprint")
    return int(b.value)


def generate(sdf, state: AppState | None = None, stream: int = 0) -> TriangleMesh:
    """Shader (or compiled SDF) + job parameters -> host TriangleMesh."""
    dm = mesh_device(sdf, state or AppState(), stream)
    try:
        return dm.to_host(stream)
    finally:
        dm.close()


def generate_host(sdf, state: AppState | None = None, parts: int = 0, stream: int = 0) -> TriangleMesh:
    """One call to a host mesh (s2m_mesh_generate): positions, normals and
    triangle indices, the same bits as `generate`; a large job runs as z parts
    whose copies to host memory overlap the next part's kernels (parts=0: the
    library's choice).  `info` holds the parts it ran as."""
    if isinstance(sdf, Sdf3DShader):
        sdf = sdf.compile()
    st = state or AppState()
    p = st.params()
    hm = HostMesh()
    err = _errbuf()
    L = load_library()
    _check(L.s2m_mesh_generate(sdf.handle, ctypes.byref(p), int(parts), ctypes.c_void_p(stream), ctypes.byref(hm),
                               err, len(err)), err, "generate")
    try:
        nv, nt = int(hm.nverts), int(hm.ntris)
        fp = ctypes.POINTER(ctypes.c_float)
        pos = np.ctypeslib.as_array(ctypes.cast(hm.pos, fp), (max(nv, 1) * 3,))[:nv * 3].reshape(nv, 3).copy()
        nrm = np.ctypeslib.as_array(ctypes.cast(hm.nrm, fp), (max(nv, 1) * 3,))[:nv * 3].reshape(nv, 3).copy()
        tris = np.ctypeslib.as_array(ctypes.cast(hm.tris, ctypes.POINTER(ctypes.c_uint32)),
                                     (max(nt, 1) * 3,))[:nt * 3].reshape(nt, 3).copy()
        info = {"parts": int(hm.parts), "resolution": int(hm.resolution)}
        return TriangleMesh(pos, nrm, tris, invalid_quads=int(hm.invalid_quads), info=info)
    finally:
        L.s2m_host_mesh_free(ctypes.byref(hm))


def measure_sfu_peak(stream: int = 0) -> float:
    """Measured SFU (MUFU) issue rate of the current GPU, Gop/s."""
    g = ctypes.c_double()
    _check(load_library().s2m_measure_sfu_peak(ctypes.byref(g), ctypes.c_void_p(stream)), None, "sfu probe")
    return g.value


def measure_fp32_peak(stream: int = 0) -> float:
    """Measured FP32 add/mul issue rate of the current GPU, Gop/s."""
    g = ctypes.c_double()
    _check(load_library().s2m_measure_fp32_peak(ctypes.byref(g), ctypes.c_void_p(stream)), None, "fp32 probe")
    return g.value
