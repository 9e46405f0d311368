"""Batching: many CSG jobs in one persistent launch (s2m_batch_*).

Each job of a mixed batch (different SDFs, resolutions, bounds, rules) must
equal, bit for bit, the oracle's mesh of the same SDF, and the per-job
compiled pipeline's mesh of the equivalent .sdf3d source."""
from __future__ import annotations

import numpy as np
import pytest

import oracle
import sdf2mesh_gb300 as s2m
from sdf2mesh_gb300 import workloads
from tests.parity import assert_bit_exact

pytestmark = pytest.mark.gpu


def test_batch_matches_oracle_and_per_job(lib):
    jobs = []
    b = s2m.Batch()
    res = [48, 64, 96, 40, 72, 33, 128, 64]
    for seed in range(8):
        src, prog = workloads.random_tree(seed)
        st = s2m.AppState(resolution=res[seed], bounds=2.0, qef=(seed % 3 == 2), slice_lag=(seed == 4))
        jobs.append((b.add_csg(prog, st), src, prog, st))
    b.run()
    ms, launches, n = b.stats()
    assert n == 8 and launches >= 1 and ms > 0
    for jid, src, prog, st in jobs:
        got = b.mesh(jid)
        ref = oracle.mesh(oracle.TREE, prog, st.resolution, st.bounds, qef=st.qef, slice_lag=st.slice_lag)
        assert_bit_exact(got, ref, f"batch job {jid} vs oracle")
        per_job = s2m.generate(s2m.Sdf3DShader.from_source(src).compile(), st)
        assert_bit_exact(got, per_job_as_oracle(per_job), f"batch job {jid} vs per-job pipeline")


def per_job_as_oracle(m):
    class R:
        pass
    r = R()
    r.nverts = m.positions.shape[0]
    r.cell = m.cell_xyz
    r.signs = m.signs
    r.pos = m.positions
    r.nrm = m.normals
    r.tris = m.triangle_indices
    r.invalid_quads = m.invalid_quads
    return r


def test_batch_all_opcodes(lib):
    """Every opcode, including smooth intersection / subtraction and planes."""
    prog = [0, 0.1, 0.0, 0.0, 0.5,          # sphere
            1, -0.2, 0.1, 0.0, 0.6, 0.4, 0.5,  # box
            14, 0.05,                       # smooth intersection
            2, 0.0, 0.2, 0.0, 0.4, 0.1,     # torus
            13, 0.03,                       # smooth union
            3, -0.5, -0.5, 0.0, 0.5, 0.5, 0.2, 0.1,  # capsule
            15, 0.04,                       # smooth subtraction
            4, 0.0, 0.0, 1.0, 0.6,          # plane z = 0.6
            12]                             # intersect
    b = s2m.Batch()
    j = b.add_csg(prog, s2m.AppState(resolution=80, bounds=2.0))
    b.run()
    ref = oracle.mesh(oracle.TREE, prog, 80, 2.0)
    assert ref.nverts > 100
    assert_bit_exact(b.mesh(j), ref, "all opcodes")


def test_batch_overflow_rerun_and_budget(lib):
    """Tiny capacities force the re-run path; a small budget splits the batch
    into waves; results are unchanged."""
    b = s2m.Batch(memory_budget_bytes=64 << 20)
    specs = []
    for seed in (1, 2, 7, 9):
        src, prog = workloads.random_tree(seed)
        st = s2m.AppState(resolution=96, bounds=2.0, max_vertices=64, max_triangles=64)
        specs.append((b.add_csg(prog, st), prog))
    b.run()
    for jid, prog in specs:
        assert_bit_exact(b.mesh(jid), oracle.mesh(oracle.TREE, prog, 96, 2.0), f"job {jid}")


def test_batch_rejects_bad_programs(lib):
    b = s2m.Batch()
    st = s2m.AppState(resolution=16)
    for bad in ([10], [0, 0, 0, 0], [0, 0, 0, 0, 0.5, 0, 0, 0, 0, 0.5], [99, 1, 2], [0, 0, 0, 0, float("nan")]):
        with pytest.raises(s2m.S2MError) as e:
            b.add_csg(bad, st)
        assert e.value.name == "INVALID"
    assert b.njobs == 0


def test_batch_256_random_trees(lib):
    """The batching workload: 256 seeded trees, resolutions log-uniform over
    {64, 96, 128, 192, 256, 384}, one persistent launch; a sample of jobs is
    checked against the oracle bit for bit."""
    rng = workloads.SplitMix64(4)
    b = s2m.Batch()
    specs = []
    for seed in range(256):
        _, prog = workloads.random_tree(seed)
        N = workloads.log_uniform_resolution(rng)
        specs.append((b.add_csg(prog, s2m.AppState(resolution=N, bounds=2.0)), prog, N))
    b.run()
    ms, launches, n = b.stats()
    assert n == 256
    for jid, prog, N in specs[::37]:
        if N > 200:
            continue
        assert_bit_exact(b.mesh(jid), oracle.mesh(oracle.TREE, prog, N, 2.0), f"job {jid} N={N}")


def test_batch_pruning_on_and_off_identical(lib):
    """Tile pruning (the interval pass per 8^3 tile, decided tiles stored as
    +-inf, pruned programs elsewhere) changes no bit: the same jobs with pruning
    off, and the oracle, in both rules, with the slice lag, every smooth
    operator, and tiles at the lattice's ragged far faces (N + 1 not a
    multiple of 8)."""
    specs = []
    for seed in range(20):
        _, prog = workloads.random_tree(seed + 40)
        prog = list(prog)
        i = 0
        while i < len(prog):  # turn some smooth unions into the other smooth operators
            op = int(prog[i])
            if op == 13 and seed % 3:
                prog[i] = 13.0 + seed % 3
            i += 1 + {0: 4, 1: 6, 2: 5, 3: 7, 4: 4, 10: 0, 11: 0, 12: 0, 13: 1, 14: 1, 15: 1}[op]
        N = [37, 64, 71, 96, 50][seed % 5]
        st = s2m.AppState(resolution=N, bounds=2.0, qef=(seed % 4 == 1), slice_lag=(seed % 5 == 3))
        specs.append((prog, st))
    meshes = {}
    for prune in (True, False):
        b = s2m.Batch()
        b.set_pruning(prune)
        ids = [b.add_csg(prog, st) for prog, st in specs]
        b.run()
        meshes[prune] = [b.mesh(j) for j in ids]
        b.close()
    assert sum(m.positions.shape[0] > 0 for m in meshes[True]) >= 12  # 7 of these trees are empty in the bounds
    for k, (prog, st) in enumerate(specs):
        on, off = meshes[True][k], meshes[False][k]
        for name in ("positions", "normals", "triangle_indices", "cells"):
            a, c = getattr(on, name), getattr(off, name)
            assert a.shape == c.shape and np.array_equal(a.view(np.uint8), c.view(np.uint8)), (k, name)
        if k % 4 == 0:
            ref = oracle.mesh(oracle.TREE, prog, st.resolution, st.bounds, qef=st.qef, slice_lag=st.slice_lag)
            assert_bit_exact(on, ref, f"pruned batch job {k} vs oracle")
