"""Admission footprint against real device use.

s2m_mesh_footprint (and the server's admission, which sums the same buffer
plan) must cover what s2m_mesh_create actually takes from the stream-ordered
pool: the pool's used-memory counter is read through the CUDA runtime before
and after a create, for an SDF with a tile form (deep slabs, tile records,
vertex sort buffers) and one without (loops: L2-sized ring)."""
from __future__ import annotations

import ctypes
import os

import pytest

import sdf2mesh_gb300 as s2m
from sdf2mesh_gb300 import workloads

pytestmark = pytest.mark.gpu

CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
USED_MEM_CURRENT = 7  # cudaMemPoolAttrUsedMemCurrent


def pool_used():
    rt = ctypes.CDLL(os.path.join(CUDA_HOME, "lib64", "libcudart.so"))
    dev = ctypes.c_int()
    assert rt.cudaGetDevice(ctypes.byref(dev)) == 0
    pool = ctypes.c_void_p()
    assert rt.cudaDeviceGetDefaultMemPool(ctypes.byref(pool), dev) == 0
    v = ctypes.c_uint64()
    assert rt.cudaMemPoolGetAttribute(pool, USED_MEM_CURRENT, ctypes.byref(v)) == 0
    return v.value


@pytest.mark.parametrize("case", ["csg_pruned_512", "csg_rounded_300", "mandelbulb_160", "torus_capacities"])
def test_footprint_covers_pool_use(lib, case):
    if case.startswith("csg"):
        src, _ = workloads.csg64(seed=0)
        sdf = s2m.Sdf3DShader.from_source(src).compile()
        state = (s2m.AppState(resolution=512, bounds=2.0) if case == "csg_pruned_512"
                 else s2m.AppState(resolution=300, bounds=2.0, reference_rounding=True))
    elif case == "mandelbulb_160":
        src, _ = workloads.mandelbulb(8.0, 8, 2.0, 0.003)
        sdf = s2m.Sdf3DShader.from_source(src, s2m.LANG_GLSL, "sdf").compile()
        # explicit capacities: a fractal surface may outgrow the automatic ones, and a
        # re-run holds more than the first attempt's plan
        state = s2m.AppState(resolution=160, bounds=2.5, max_vertices=1 << 21, max_triangles=1 << 23)
    else:
        src, _ = workloads.torus()
        sdf = s2m.Sdf3DShader.from_source(src).compile()
        state = s2m.AppState(resolution=200, bounds=2.0, max_vertices=1 << 20, max_triangles=3 << 20)
    s2m.generate(sdf, s2m.AppState(resolution=32, bounds=2.0))  # library and pool initialised
    fp = s2m.mesh_footprint(sdf, state)
    used0 = pool_used()
    dm = s2m.mesh_device(sdf, state)
    used = pool_used() - used0
    info = dm.info()
    dm.close()
    if case == "csg_rounded_300":
        assert info.resolution == 512
    # the plan is what was allocated (the pool may round each allocation up)
    assert fp <= used + (1 << 20) and used <= fp + (64 << 20), (fp, used)
