"""Tile pruning of the batch engine's CSG interpreter (s2m_csg.cuh), on the CPU.

For random CSG programs (the batch workload's trees, with every smooth
operator) and tiles of 8 x 8 x 8 lattice points:

- s2c_tile's root interval bounds the program's binary32 value at every
  point of the tile;
- the pruned interpreter (nodes coded 0 skipped, combinators coded 2 / 3
  returning the operand they keep) gives the same bits as the full one at
  every point, so a tile the batch engine evaluates pruned stores exactly
  what the full evaluation would;
- decisions happen: some combinators are decided on most programs, so the
  pruned path is exercised, not just the all-ones code.

The header is compiled by the host compiler without FMA contraction, which
gives the same round-to-nearest operations as the device's explicitly rounded
ones (the device build of the same header is checked bit for bit against the
CPU oracle by the GPU batch tests)."""
from __future__ import annotations

import ctypes
import os
import subprocess
import tempfile

import numpy as np
import pytest

from sdf2mesh_gb300 import workloads

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def lib():
    d = tempfile.mkdtemp(prefix="s2m_csgprune_")
    so = os.path.join(d, "csgprune.so")
    subprocess.run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math",
                    "-I", os.path.join(HERE, "..", "include"), os.path.join(HERE, "csg_prune_host.cpp"), "-o", so],
                   check=True, capture_output=True)
    L = ctypes.CDLL(so)
    L.csg_tile.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    L.csg_tile.restype = ctypes.c_int
    L.csg_eval4.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
                            ctypes.c_void_p]
    return L


def ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


SMOOTH = (13.0, 14.0, 15.0)


def program(seed):
    """random_tree's program with its smooth unions turned into each of the three
    smooth operators (their k kept)."""
    _, prog = workloads.random_tree(seed)
    prog = list(prog)
    rng = np.random.default_rng(seed)
    i = 0
    operands = {0: 4, 1: 6, 2: 5, 3: 7, 4: 4, 10: 0, 11: 0, 12: 0, 13: 1, 14: 1, 15: 1}
    while i < len(prog):
        op = int(prog[i])
        if op == 13:
            prog[i] = SMOOTH[rng.integers(0, 3)]
        i += 1 + operands[op]
    return np.asarray(prog, np.float32)


def coords(bmin, size, idx):
    """s2_coord: bmin + size * i, each operation rounded in binary32."""
    return (np.float32(bmin) + np.float32(size) * idx.astype(np.float32)).astype(np.float32)


def tile_points(bmin, size, i0, j0, k0):
    xs = coords(bmin, size, np.arange(i0, i0 + 8))
    ys = coords(bmin, size, np.arange(j0, j0 + 8))
    zs = coords(bmin, size, np.arange(k0, k0 + 8))
    runs = []
    for zr in range(2):
        for y in ys:
            for x in xs:
                runs.append([x, y, *zs[4 * zr:4 * zr + 4]])
    box = np.array([xs[0], xs[-1], ys[0], ys[-1], zs[0], zs[-1]], np.float32)
    return np.asarray(runs, np.float32), box


def evaluate(L, prog, runs, codes):
    out = np.empty(4 * len(runs), np.float32)
    L.csg_eval4(ptr(prog), len(prog), ptr(runs), len(runs), ptr(codes) if codes is not None else None, ptr(out))
    return out


@pytest.mark.parametrize("seed", range(24))
def test_pruned_equals_full_and_root_bounds(lib, seed):
    prog = program(seed)
    rng = np.random.default_rng(1000 + seed)
    N = int(rng.choice([64, 96, 128, 192]))
    B = 2.0
    size = np.float32(np.float32(2 * B) / np.float32(N))
    bmin = np.float32(-B)
    for _ in range(40):
        i0, j0, k0 = (int(v) for v in rng.integers(0, N - 7, 3))
        runs, box = tile_points(bmin, size, i0, j0, k0)
        codes = np.zeros(16, np.uint32)
        root = np.zeros(2, np.float32)
        ok = lib.csg_tile(ptr(prog), len(prog), ptr(box), ptr(codes), ptr(root))
        assert ok == 1
        full = evaluate(lib, prog, runs, None)
        pruned = evaluate(lib, prog, runs, codes)
        assert np.array_equal(full.view(np.uint32), pruned.view(np.uint32)), (seed, i0, j0, k0)
        if np.isfinite(root).all():
            assert (full >= root[0]).all() and (full <= root[1]).all(), (seed, root, full.min(), full.max())


def node_codes(codes):
    return ((codes[:, None] >> (2 * np.arange(16, dtype=np.uint32))[None, :]) & 3).reshape(-1)


def test_decisions_happen(lib):
    """Across the batch workload's trees, most tiles decide some combinator
    and skip the nodes of an operand."""
    tiles = decided = skipped = 0
    for seed in range(64):
        prog = program(seed)
        rng = np.random.default_rng(5000 + seed)
        N = 128
        size = np.float32(np.float32(4.0) / np.float32(N))
        for _ in range(16):
            i0, j0, k0 = (int(v) for v in rng.integers(0, N - 7, 3))
            _, box = tile_points(np.float32(-2.0), size, i0, j0, k0)
            codes = np.zeros(16, np.uint32)
            root = np.zeros(2, np.float32)
            lib.csg_tile(ptr(prog), len(prog), ptr(box), ptr(codes), ptr(root))
            c = node_codes(codes)
            tiles += 1
            decided += bool(((c == 2) | (c == 3)).any())
            skipped += bool((c == 0).any())
    assert decided > tiles // 4 and skipped > tiles // 4, (tiles, decided, skipped)


def test_skipped_operands_and_signed_zero(lib):
    """Hand-made cases: a union whose second operand is far away (code 2, its
    nodes skipped), a subtraction whose subtrahend wins (code 3: negated), and a
    smooth subtraction decided for its first operand (canon(-a)), on tiles that
    include points where a value is exactly zero."""
    far = [0.0, 5.0, 5.0, 5.0, 0.5]           # sphere far from the tile
    unit = [0.0, 0.0, 0.0, 0.0, 0.5]          # sphere at the origin, r = 0.5
    small = [1.0, 0.0, 0.0, 0.0, 0.25, 0.25, 0.25]
    cases = [
        unit + far + [10.0],                  # min(a, far): keeps a
        far + unit + [10.0],                  # min(far, a): keeps b
        unit + [0.0, 0.0, 0.0, 0.0, 3.0] + [11.0],   # max(a, -big): -big wins inside
        unit + far + [15.0, 0.02],            # smooth subtraction
        small + unit + [14.0, 0.03],
        [4.0, 0.0, 0.0, 1.0, 0.25] + unit + [13.0, 0.05],  # plane z = 0.25 (exact zeros on the lattice)
    ]
    size = np.float32(0.0625)
    bmin = np.float32(-1.0)
    for prog in cases:
        prog = np.asarray(prog, np.float32)
        for i0 in range(0, 26, 5):
            for k0 in range(0, 26, 7):
                runs, box = tile_points(bmin, size, i0, 12, k0)
                codes = np.zeros(16, np.uint32)
                root = np.zeros(2, np.float32)
                assert lib.csg_tile(ptr(prog), len(prog), ptr(box), ptr(codes), ptr(root)) == 1
                full = evaluate(lib, prog, runs, None)
                pruned = evaluate(lib, prog, runs, codes)
                assert np.array_equal(full.view(np.uint32), pruned.view(np.uint32)), (prog, i0, k0, codes[0])
