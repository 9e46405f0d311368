"""Index arithmetic on the CPU (no GPU), restated from the kernels' formulas:

- the batch engine's tile pass and evaluation (batch.cu: s2b_stage_tiles,
  s2b_stage_eval): every lattice point of a job is written by exactly one
  thread, each item's warps see one tile each (so a warp takes one path
  through the pruned program), and every tile record that the evaluation
  reads was written by the tile pass;
- the classification's candidate slots (static_kernels.cuh: s2m_cells_mark
  adds its tile counts to per-plane counts and scans those; s2m_cells_emit
  adds the counts of the plane's earlier tiles): each tile's first slot
  equals the exclusive scan of all tile counts in (z, y, x) order, so the
  candidate list is the same as with a scan over every tile."""
import os
import re

import numpy as np
import pytest

CSRC = os.path.join(os.path.dirname(__file__), "..", "sdf2mesh_gb300", "csrc")


def const(name, hdr):
    m = re.search(r"#define\s+%s\s+(\d+)" % name, open(os.path.join(CSRC, hdr)).read())
    assert m, name
    return int(m.group(1))


TILE = const("S2_B_TILE", "batch.cu")
TILES_ITEM = const("S2_B_TILES_ITEM", "batch.cu")
EVAL_TILES = const("S2_B_EVAL_TILES", "batch.cu")
RUN = const("S2_B_EVAL_RUN", "batch.cu")


def eval_tile_points(x0, y0, z0, P, decided):
    """Points one warp writes for the tile at (x0, y0, z0): the decided path's
    float4 stores of a whole tile (or its guarded scalar stores at the far
    faces), or the 128 runs of 4 planes of the evaluation path."""
    pts = []
    if decided:
        if x0 + TILE <= P and y0 + TILE <= P and z0 + TILE <= P:
            for k in range(4):
                for lane in range(32):
                    u = k * 32 + lane
                    h, y, z = u & 1, (u >> 1) & 7, u >> 4
                    assert (x0 + 4 * h) % 4 == 0  # 16-byte aligned float4 (row starts are 32-point multiples)
                    pts += [(z0 + z, y0 + y, x0 + 4 * h + i) for i in range(4)]
        else:
            for u in range(TILE ** 3):
                x, y, z = x0 + (u & 7), y0 + ((u >> 3) & 7), z0 + (u >> 6)
                if x < P and y < P and z < P:
                    pts.append((z, y, x))
        return pts
    for k in range(4):
        for lane in range(32):
            lr = k * 32 + lane
            x, y, k0 = x0 + (lr & 7), y0 + ((lr >> 3) & 7), z0 + RUN * (lr >> 6)
            if x >= P or y >= P or k0 >= P:
                continue
            pts += [(k0 + w, y, x) for w in range(RUN) if k0 + w < P]
    return pts


@pytest.mark.parametrize("N", [2, 7, 8, 31, 40, 63, 64, 65, 100])
def test_batch_eval_covers_lattice_once(N):
    P = N + 1
    nt = (P + TILE - 1) // TILE
    ntiles = nt ** 3
    # tile pass: items * 256 threads, thread t < ntiles writes record t
    tile_items = (ntiles + TILES_ITEM - 1) // TILES_ITEM
    written = np.zeros(ntiles, int)
    for item in range(tile_items):
        t = item * TILES_ITEM + np.arange(256)
        written[t[t < ntiles]] += 1
    assert (written == 1).all()
    # evaluation: warp w of item i takes tiles i * EVAL_TILES + q * 8 + w
    items = (ntiles + EVAL_TILES - 1) // EVAL_TILES
    seen = np.zeros(ntiles, int)
    rng = np.random.default_rng(N)
    count = np.zeros((P, P, P), int)
    for item in range(items):
        for q in range(EVAL_TILES // 8):
            for w in range(8):
                t = item * EVAL_TILES + q * 8 + w
                if t >= ntiles:
                    continue
                seen[t] += 1
                tx, r = t % nt, t // nt
                ty, tz = r % nt, r // nt
                for z, y, x in eval_tile_points(TILE * tx, TILE * ty, TILE * tz, P, bool(rng.integers(0, 2))):
                    count[z, y, x] += 1
    assert (seen == 1).all()
    assert (count == 1).all(), (N, np.argwhere(count != 1)[:5])


@pytest.mark.parametrize("N", [4, 8, 12, 64, 96])
def test_cell_groups_lie_in_one_tile(N):
    """Classification skips a group of 4 cells by the flag of one tile: with N a
    multiple of 4 the group is 4 cells of one row from x a multiple of 4, and the
    tile's box (one point past its points) holds all their corners."""
    CPT = const("S2_CELL_CPT", "s2m_device.h")
    ncells = N ** 3
    for c in range(0, ncells - 3, 4):
        z, rem = divmod(c, N * N)
        y, x = divmod(rem, N)
        assert x % 4 == 0 and x + 3 < N
        assert (x >> 3) == ((x + 3) >> 3)
        lo, hi = TILE * (x >> 3), TILE * (x >> 3) + TILE  # box points lo .. hi
        assert lo <= x and x + 3 + 1 <= hi
    assert CPT % 4 == 0


@pytest.mark.parametrize("N,planes", [(33, 5), (64, 9), (100, 3), (1024, 2)])
def test_emit_slots_equal_full_scan(N, planes):
    CW = const("S2_CW_BLOCK", "s2m_device.h")
    WN = (N + 31) // 32
    nbp = (N * WN + CW - 1) // CW
    rng = np.random.default_rng(N)
    cnt = rng.integers(0, 50, (planes, nbp)) * (rng.random((planes, nbp)) < 0.6)
    base = 12345
    full = base + np.concatenate([[0], np.cumsum(cnt.reshape(-1))[:-1]]).reshape(planes, nbp)
    plane_cnt = cnt.sum(1)
    plane_off = base + np.concatenate([[0], np.cumsum(plane_cnt)[:-1]])
    for dz in range(planes):
        for bx in range(nbp):
            first = plane_off[dz] + cnt[dz, :bx].sum()
            assert first == full[dz, bx]
    assert base + plane_cnt.sum() == base + cnt.sum()
