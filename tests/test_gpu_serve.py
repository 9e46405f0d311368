"""Serving: continuous batching (s2m_server_*).

Requests submitted from several threads while others run on the GPU; each
result must be the same alone and in the mix (bit for bit: the same rule and
arithmetic run whatever the batch), admission must hold the memory budget."""
from __future__ import annotations

import threading
import time

import numpy as np
import pytest

import sdf2mesh_gb300 as s2m
from sdf2mesh_gb300 import workloads
from tests.parity import assert_bit_exact
from tests.test_gpu_batch import per_job_as_oracle

pytestmark = pytest.mark.gpu


def test_results_same_alone_and_in_the_mix(lib):
    rng = workloads.SplitMix64(11)
    specs = []
    for seed in range(40):
        _, prog = workloads.random_tree(seed)
        N = workloads.log_uniform_resolution(rng, (32, 48, 64, 96, 128))
        specs.append(("csg", prog, s2m.AppState(resolution=N, bounds=2.0, qef=(seed % 5 == 0))))
    src, _ = workloads.mandelbulb(8.0, 6, 2.0, 0.003)
    mb = s2m.Sdf3DShader.from_source(src, s2m.LANG_GLSL, "sdf").compile()
    for N in (48, 64, 80):
        specs.append(("sdf", mb, s2m.AppState(resolution=N, bounds=2.5)))
    server = s2m.Server(memory_budget_bytes=2 << 30, max_inflight=2, max_batch_jobs=16)
    ids = [None] * len(specs)

    def submit(part):
        for i in part:
            kind, obj, st = specs[i]
            ids[i] = server.submit_csg(obj, st) if kind == "csg" else server.submit_sdf(obj, st)
            time.sleep(0.002 * (i % 3))

    threads = [threading.Thread(target=submit, args=(range(k, len(specs), 3),)) for k in range(3)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    server.drain(600)
    st = server.stats()
    assert st["completed"] == len(specs) and st["failed"] == 0
    assert st["batches"] >= 2 and st["p99_ms"] >= st["p50_ms"] > 0
    for i, (kind, obj, state) in enumerate(specs):
        got = server.mesh(ids[i])
        if kind == "csg":
            b = s2m.Batch()
            j = b.add_csg(obj, state)
            b.run()
            alone = b.mesh(j)
        else:
            alone = s2m.generate(obj, state)
        assert_bit_exact(got, per_job_as_oracle(alone), f"request {i} ({kind})")
    server.close()


def test_admission_under_budget(lib):
    budget = 192 << 20
    server = s2m.Server(memory_budget_bytes=budget, max_inflight=2, keep_results=False)
    reqs = []
    for seed in range(24):
        _, prog = workloads.random_tree(seed)
        reqs.append(server.submit_csg(prog, s2m.AppState(resolution=128, bounds=2.0)))
    server.drain(600)
    st = server.stats()
    assert st["completed"] == 24 and st["failed"] == 0
    assert 0 < st["peak_bytes"] <= budget
    assert st["batches"] >= 3  # the budget forces several launches
    # a request larger than the whole budget is refused, not queued forever
    _, prog = workloads.random_tree(1)
    rid = server.submit_csg(prog, s2m.AppState(resolution=1024, bounds=2.0))
    with pytest.raises(s2m.S2MError) as e:
        server.wait(rid, 60)
    assert e.value.name == "OOM"
    server.close()


def test_server_overflow_requeue(lib):
    """Requests whose guessed buffers overflow are re-queued with the exact sizes."""
    _, prog = workloads.random_tree(2)
    server = s2m.Server()
    rid = server.submit_csg(prog, s2m.AppState(resolution=96, bounds=2.0, max_vertices=64, max_triangles=64))
    got = server.mesh(rid)
    b = s2m.Batch()
    j = b.add_csg(prog, s2m.AppState(resolution=96, bounds=2.0))
    b.run()
    assert_bit_exact(got, per_job_as_oracle(b.mesh(j)), "requeued request")
    server.close()


def test_submit_source_routes_and_matches(lib):
    """Requests as source text: CSG-shaped .sdf3d runs on the interpreter,
    GLSL compiles once (cached) -- each result equals the per-job pipeline's
    mesh of the same source."""
    server = s2m.Server()
    reqs = []
    for seed in (2, 3, 7):
        src, _ = workloads.random_tree(seed)
        st = s2m.AppState(resolution=64, bounds=2.0)
        reqs.append((server.submit_source(src, st), src, s2m.LANG_WGSL, st))
    mb, _ = workloads.mandelbulb(8.0, 5, 2.0, 0.003)
    for N in (40, 56):
        st = s2m.AppState(resolution=N, bounds=2.5)
        reqs.append((server.submit_source(mb, st, s2m.LANG_GLSL, "sdf"), mb, s2m.LANG_GLSL, st))
    server.drain(600)
    for rid, src, lang, st in reqs:
        got = server.mesh(rid)
        alone = s2m.generate(s2m.Sdf3DShader.from_source(src, lang, "sdf").compile(), st)
        assert_bit_exact(got, per_job_as_oracle(alone), f"request {rid}")
    server.close()


def test_source_tiering_interpreter_then_compiled(lib):
    """A CSG source runs on the interpreter until its background compile is
    done, then on its compiled module; both give the same mesh, bit for bit
    (the interpreter's arithmetic is the library functions')."""
    server = s2m.Server(sdf_workers=3)
    srcs = [workloads.random_tree(seed)[0] for seed in (4, 5, 6)]
    st = s2m.AppState(resolution=72, bounds=2.0)
    first = [server.submit_source(src, st) for src in srcs]
    server.drain(600)
    t0 = time.time()
    while server.stats()["compiles_pending"] and time.time() - t0 < 600:
        time.sleep(0.05)
    stats = server.stats()
    assert stats["compiled_sources"] >= len(srcs) and stats["ran_interpreted"] >= len(srcs)
    server.reset_stats()
    second = [server.submit_source(src, st) for src in srcs]
    server.drain(600)
    assert server.stats()["ran_compiled"] == len(srcs)
    for a, b in zip(first, second):
        assert_bit_exact(server.mesh(b), per_job_as_oracle(server.mesh(a)), f"request {a} vs {b}")
    server.close()
    only = s2m.Server(interpret_only=True)
    rid = only.submit_source(srcs[0], st)
    only.drain(600)
    assert only.stats()["ran_interpreted"] == 1 and only.stats()["compiles_pending"] == 0
    assert_bit_exact(only.mesh(rid), per_job_as_oracle(server_mesh_alone(srcs[0], st)), "interpret only")
    only.close()


def server_mesh_alone(src, st):
    return s2m.generate(s2m.Sdf3DShader.from_source(src).compile(), st)
