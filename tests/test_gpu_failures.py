"""Failure detection without a GPU fault.

The reference panics when a device step fails (main.rs:184, 196,
texture.rs:110).  Here every device wait is bounded and reports a status:

  * the look-back of the ordered scans: a test hook (S2M_TEST_HOLD=1) keeps
    tile 0 of the row-start scan from publishing its prefix -- a flag that
    nothing sets -- so every later tile's wait runs out after the mesh's
    wait limit; the run returns S2M_E_TIMEOUT and the next run on the same
    handle is bit-exact again;
  * the persistent batch kernel's stage waits (S2M_TEST_HOLD=2: job 0's row
    scan never counts as done), S2M_E_TIMEOUT from s2m_batch_run;
  * a device allocation that fails (host hook S2M_TEST_FAIL_ALLOC=k fails the
    k-th allocation of the process): S2M_E_OOM, nothing left allocated, and
    the next job in the same process succeeds.

Only waiting is affected; every write stays bounds-checked, so nothing
faults and the context stays usable.
"""
from __future__ import annotations

import json
import os
import subprocess
import sys

import pytest

import oracle
import sdf2mesh_gb300 as s2m
from sdf2mesh_gb300 import workloads
from tests.parity import assert_bit_exact

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_lookback_wait_runs_out(lib, monkeypatch):
    src, prm = workloads.csg64(seed=0)
    sdf = s2m.Sdf3DShader.from_source(src).compile()
    dm = s2m.mesh_device(sdf, s2m.AppState(resolution=128, bounds=2.0))
    ref = oracle.mesh(oracle.CSG, prm, 128, 2.0)
    assert_bit_exact(dm.to_host(), ref, "before")
    dm.set_wait_limit(0.005)
    monkeypatch.setenv("S2M_TEST_HOLD", "1")
    dm.run_async()
    with pytest.raises(s2m.S2MError) as e:
        dm.sync()
    assert e.value.name == "TIMEOUT", str(e.value)
    monkeypatch.delenv("S2M_TEST_HOLD")
    dm.set_wait_limit(2.0)
    dm.run_async()
    dm.sync()
    assert_bit_exact(dm.to_host(), ref, "after the timed-out run")
    dm.close()


def test_batch_stage_wait_runs_out(lib, monkeypatch):
    jobs = [workloads.random_tree(s) for s in (1, 2, 3)]
    b = s2m.Batch()
    for _, prog in jobs:
        b.add_csg(prog, s2m.AppState(resolution=64, bounds=2.0))
    b.set_wait_limit(0.01, 0.01)
    monkeypatch.setenv("S2M_TEST_HOLD", "2")
    with pytest.raises(s2m.S2MError) as e:
        b.run()
    assert e.value.name == "TIMEOUT", str(e.value)
    b.close()
    monkeypatch.delenv("S2M_TEST_HOLD")
    b = s2m.Batch()
    for _, prog in jobs:
        b.add_csg(prog, s2m.AppState(resolution=64, bounds=2.0))
    b.run()
    for k, (_, prog) in enumerate(jobs):
        assert_bit_exact(b.mesh(k), oracle.mesh(oracle.TREE, prog, 64, 2.0), f"batch job {k} after timeout")
    b.close()


CHILD = r"""
import ctypes, json, os, sys
sys.path.insert(0, os.environ["S2M_ROOT"])
import numpy as np
import oracle, sdf2mesh_gb300 as s2m
from sdf2mesh_gb300 import workloads
from tests.test_gpu_footprint import pool_used
rt = ctypes.CDLL(os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "lib64", "libcudart.so"))
src, prm = workloads.torus()
sdf = s2m.Sdf3DShader.from_source(src).compile()
rt.cudaDeviceSynchronize()
used0 = pool_used()
out = {}
try:
    s2m.mesh_device(sdf, s2m.AppState(resolution=96, bounds=2.0))
    out["first"] = "ok"
except s2m.S2MError as e:
    out["first"] = e.name
rt.cudaDeviceSynchronize()
out["leaked"] = pool_used() - used0
g = s2m.generate(sdf, s2m.AppState(resolution=96, bounds=2.0))
ref = oracle.mesh(oracle.TORUS, prm, 96, 2.0)
out["second_exact"] = bool(np.array_equal(g.positions.view(np.uint32), ref.pos.astype(np.float32).view(np.uint32))
                           and np.array_equal(g.triangle_indices, ref.tris))
print(json.dumps(out))
"""


@pytest.mark.parametrize("k", [3, 9, 15])
def test_allocation_failure_reports_oom(lib, oracle_lib, k):
    env = dict(os.environ, S2M_TEST_FAIL_ALLOC=str(k), S2M_ROOT=ROOT)
    r = subprocess.run([sys.executable, "-c", CHILD], env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    out = json.loads(r.stdout.strip().splitlines()[-1])
    assert out["first"] == "OOM", out
    assert out["leaked"] == 0, out
    assert out["second_exact"], out
