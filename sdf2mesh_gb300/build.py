"""Build libsdf2mesh_gb300.so and the sdf2mesh CLI in-tree (sdf2mesh_gb300/_lib/).

nvcc compiles the runtime and its SDF-independent kernels for sm_103a; the
per-SDF kernels are compiled later, at run time, by NVRTC for sm_103a.  The
device sources NVRTC needs are embedded into the library as string literals.
Run: python -m sdf2mesh_gb300.build  (or import and call build()).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIB_DIR = os.path.join(HERE, "_lib")
OBJ_DIR = os.path.join(LIB_DIR, "obj")
REPO = os.path.dirname(HERE)
INCLUDE = os.path.join(REPO, "include")
LIB_NAME = "libsdf2mesh_gb300.so"
LIB_PATH = os.path.join(LIB_DIR, LIB_NAME)
CLI_PATH = os.path.join(LIB_DIR, "sdf2mesh")

CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
HOST_FLAGS = ["-O3", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", "-Wextra"]

EMBEDDED = [
    ("kS2mDeviceH", "s2m_device.h"),
    ("kS2mLookbackCuh", "s2m_lookback.cuh"),
    ("kS2mPreludeCuh", "s2m_prelude.cuh"),
    ("kS2mDcCoreCuh", "s2m_dc_core.cuh"),
    ("kS2mDcKernelsCuh", "s2m_dc_kernels.cuh"),
]
SOURCES = ["runtime.cu", "batch.cu", "frontend.cpp", "frontend_lib.cpp", "prune.cpp", "mesh_io.cpp"]
HEADERS = ["frontend.h", "prune.h", "mesh_io.h", "static_kernels.cuh", "s2m_device.h", "s2m_lookback.cuh",
           "s2m_prelude.cuh", "s2m_dc_core.cuh", "s2m_dc_kernels.cuh", "s2m_workers.cuh", "s2m_csg.cuh"]


def _mtime(p):
    return os.path.getmtime(p) if os.path.exists(p) else -1.0


def _write_embedded():
    out = os.path.join(OBJ_DIR, "s2m_embedded.inc")
    text = ["// generated by sdf2mesh_gb300/build.py from the device sources\n"]
    for var, fname in EMBEDDED:
        with open(os.path.join(CSRC, fname)) as f:
            body = f.read()
        assert ")S2MSRC\"" not in body
        text.append(f'static const char *{var} = R"S2MSRC({body}\n)S2MSRC";\n')
    data = "".join(text)
    if not os.path.exists(out) or open(out).read() != data:
        with open(out, "w") as f:
            f.write(data)
    return out


def _compile(src):
    path = os.path.join(CSRC, src)
    obj = os.path.join(OBJ_DIR, src + ".o")
    deps = [path] + [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(INCLUDE, "sdf2mesh.h"),
                                                                os.path.join(OBJ_DIR, "s2m_embedded.inc")]
    if _mtime(obj) >= max(_mtime(d) for d in deps):
        return obj
    if src.endswith(".cu"):
        cmd = [NVCC, *ARCH, "-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
               "-I", OBJ_DIR, "-I", INCLUDE, "-c", path, "-o", obj]
    else:
        cmd = ["g++", *HOST_FLAGS, "-I", INCLUDE, "-I", f"{CUDA_HOME}/include", "-c", path, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return obj


def build(verbose: bool = False) -> str:
    """Compile every source (in parallel) and link the library and the CLI."""
    os.makedirs(OBJ_DIR, exist_ok=True)
    _write_embedded()
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(_compile, SOURCES))
    if _mtime(LIB_PATH) < max(_mtime(o) for o in objs):
        cmd = [NVCC, *ARCH, "-shared", "-o", LIB_PATH, *objs, "-lnvrtc",
               "-Xlinker", f"-rpath,{CUDA_HOME}/lib64", "-L", f"{CUDA_HOME}/lib64"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    cli_src = os.path.join(CSRC, "cli.cpp")
    if os.path.exists(cli_src) and _mtime(CLI_PATH) < max(_mtime(cli_src), _mtime(LIB_PATH)):
        cmd = ["g++", *HOST_FLAGS, "-I", INCLUDE, cli_src, "-o", CLI_PATH, "-L", LIB_DIR,
               "-lsdf2mesh_gb300", "-Wl,-rpath,$ORIGIN", "-Wl,-rpath," + LIB_DIR]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"cli link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    if verbose:
        print(LIB_PATH)
    return LIB_PATH


def clean():
    shutil.rmtree(LIB_DIR, ignore_errors=True)


if __name__ == "__main__":
    if "--clean" in sys.argv:
        clean()
    build(verbose=True)
