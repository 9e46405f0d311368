"""The C-ABI library loads on any machine and exports every symbol that
include/sdf2mesh.h declares; the device-free entry points work without a GPU."""
from __future__ import annotations

import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    text = open(os.path.join(ROOT, "include", "sdf2mesh.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_ ]*?\**\s*\b(s2m_[a-z0-9_]+)\s*\(", text, flags=re.M)
    return sorted(set(names))


def test_header_declares_entry_points():
    names = declared_functions()
    for must in ("s2m_compile", "s2m_mesh_create", "s2m_mesh_copy_to_host", "s2m_write_stl", "s2m_mesh_free",
                 "s2m_preprocess_file", "s2m_translate"):
        assert must in names


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_abi_version_and_status(lib):
    assert lib.s2m_abi_version() == 2
    assert lib.s2m_status_string(0) == b"ok"
    assert lib.s2m_status_string(5) == b"NVRTC compile error"


def test_invalid_arguments_return_status(lib):
    err = ctypes.create_string_buffer(256)
    out = ctypes.c_void_p()
    assert lib.s2m_compile(None, 0, None, 0, ctypes.byref(out), err, 256) == 1
    assert lib.s2m_mesh_create(None, None, None, ctypes.byref(out), err, 256) == 1
    assert lib.s2m_mesh_get_info(None, None) == 1


def test_parse_error_is_a_status_not_an_abort(lib):
    import sdf2mesh_gb300 as s2m
    with pytest.raises(s2m.S2MError) as e:
        s2m.translate("fn sdf3d(p: vec3f) -> f32 { return p.x +; }")
    assert e.value.name == "PARSE"
    with pytest.raises(s2m.S2MError) as e:
        s2m.translate("fn other(p: vec3f) -> f32 { return p.x; }")
    assert e.value.name in ("MISSING_SDF", "PARSE")


@pytest.mark.parametrize("which", ["sphere", "csg64", "mandelbulb", "tree"])
def test_compile_without_device_fails_loudly(lib, which):
    """No CPU fallback: with no CUDA device the device module still compiles
    (NVRTC needs no GPU) and then loading it fails with a status."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    import sdf2mesh_gb300 as s2m
    from sdf2mesh_gb300 import workloads
    if which == "sphere":
        sh = s2m.Sdf3DShader.from_source("use sdf3d::*;\nfn sdf3d(p: vec3f) -> f32 { return sdf3d_sphere(p, 0.5); }\n")
    elif which == "csg64":
        sh = s2m.Sdf3DShader.from_source(workloads.csg64()[0])
    elif which == "tree":
        sh = s2m.Sdf3DShader.from_source(workloads.random_tree(5)[0])
    else:
        sh = s2m.Sdf3DShader.from_source(workloads.mandelbulb()[0], s2m.LANG_GLSL, "sdf")
    with pytest.raises(s2m.S2MError) as e:
        sh.compile()
    assert e.value.name in ("NO_DEVICE", "CUDA"), str(e.value)
