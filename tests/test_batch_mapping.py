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
    # evaluation
    items = (ntiles + EVAL_TILES - 1) // EVAL_TILES
    count = np.zeros((P, P, P), int)
    for item in range(items):
        for r in range(EVAL_TILES * 128 // 256):
            u = r * 256 + np.arange(256)
            t = item * EVAL_TILES + (u >> 7)
            for w in range(8):  # one tile per warp
                assert len(set(t[32 * w:32 * w + 32].tolist())) == 1
            ok = t < ntiles
            u, t = u[ok], t[ok]
            lr = u & 127
            tx, q = t % nt, t // nt
            ty, tz = q % nt, q // nt
            x = TILE * tx + (lr & 7)
            y = TILE * ty + ((lr >> 3) & 7)
            k0 = TILE * tz + RUN * (lr >> 6)
            inb = (x < P) & (y < P) & (k0 < P)
            for w in range(RUN):
                sel = inb & (k0 + w < P)
                np.add.at(count, (k0[sel] + w, y[sel], x[sel]), 1)
            assert (t[inb] < ntiles).all()
    assert (count == 1).all(), (N, np.argwhere(count != 1)[:5])


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
