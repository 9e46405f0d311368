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


def mark_local_word(WN, warp, lane):
    """s2m_cells_mark's tile-local word of (warp, lane)."""
    if 4 <= WN <= 256 and WN & (WN - 1) == 0:
        R = 256 // WN
        wr = min(8, R)
        ww = 32 // wr
        nwg = WN // ww
        band, wg = warp // nwg, warp % nwg
        return (band * wr + lane // ww) * WN + wg * ww + lane % ww
    return warp * 32 + lane


@pytest.mark.parametrize("N", [1, 31, 64, 96, 97, 128, 200, 512, 1000, 1024, 2048, 4096, 8192])
def test_mark_warp_rectangles(N):
    """Each tile's 256 words are taken once; with WN a power of two from 4 on, a
    warp's words lie in at most 8 rows of one pruning tile row (rows 8k .. 8k +
    7 of the lattice) and 32 / (its rows) consecutive words of each."""
    WN = (N + 31) // 32
    loc = np.array([[mark_local_word(WN, k, l) for l in range(32)] for k in range(8)])
    assert sorted(loc.reshape(-1)) == list(range(256))
    if 4 <= WN <= 256 and WN & (WN - 1) == 0:
        R = 256 // WN
        for b in range(3):  # tiles start at row b * R
            rows = (b * 256 + loc) // WN
            for k in range(8):
                assert len(set(rows[k] // 8)) == 1, (N, b, k)
                assert len(set(rows[k])) == min(8, R)


def slab_planes(zb, s, D, nzc):
    """s2_slab_planes: the first lattice plane and plane count of slab s."""
    zc0 = zb + s * D
    zc1 = min(zb + nzc, zc0 + D)
    k0 = zb if s == 0 else zc0 + 1
    return zc0, zc1, k0, zc1 - k0 + 1


@pytest.mark.parametrize("N,D,zb,nzc", [(64, 64, 0, 64), (100, 37, 0, 100), (33, 10, 5, 20), (1024, 512, 0, 1024)])
def test_mark_tiles_cover_each_cell_once(N, D, zb, nzc):
    """s2m_cells_mark_tiles: the warp of tile (tx, ty, tz) writes, lane by lane
    (row r = lane % 8, cell plane kb - 1 + lane / 8 + 4 j), the byte of cells
    8 tx .. 8 tx + 7 of each row and plane it covers; over all tiles of a slab
    every cell of the slab is written exactly once, by the tile of its point
    (x, y, z + 1) (s2_cell_prune_tile), and reads point planes of the slab's
    ring only."""
    P = N + 1
    ntx = (P + 7) // 8
    nslabs = (nzc + D - 1) // D
    rows = range(N) if N <= 100 else range(0, N, 61)  # a sample of rows at 1024
    for s in range(nslabs):
        zc0, zc1, k0, nk = slab_planes(zb, s, D, nzc)
        parts = (nk + 7) // 8
        tzs = (nk + parts - 1) // parts
        nzt = (nk + tzs - 1) // tzs
        seen = {}
        for tz in range(nzt):
            kb = k0 + tz * tzs
            ke = min(kb + tzs, k0 + nk) - 1
            for ty in range(ntx):
                for tx in range(ntx):
                    if 8 * tx >= N:
                        continue
                    for lane in range(32):
                        r, pz = lane & 7, lane >> 3
                        y = 8 * ty + r
                        if y not in rows:
                            continue
                        for zbb in range(kb - 1, ke, 4):
                            zc = zbb + pz
                            if zc <= ke - 1 and zc0 <= zc < zc1 and y < N:
                                assert zc0 <= zc and zc + 1 <= zc1  # point planes read: zc, zc + 1
                                key = (zc, y, tx)
                                assert key not in seen, key
                                seen[key] = (tx, ty, tz)
        for zc in range(zc0, zc1):
            for y in rows:
                for x in range(0, N, 8):
                    tz = (zc + 1 - k0) // tzs  # s2_cell_prune_tile
                    assert seen.get((zc, y, x // 8)) == (x // 8, y // 8, tz), (s, zc, y, x)
        assert len(seen) == (zc1 - zc0) * len(rows) * ((N + 7) // 8)


@pytest.mark.parametrize("N,zc0,zc1,kb,ke", [(64, 0, 64, 0, 7), (64, 9, 30, 10, 17), (100, 0, 100, 96, 100),
                                             (37, 5, 12, 6, 12)])
def test_mark_tiles_rows_from_neighbour_lanes(N, zc0, zc1, kb, ke):
    """s2m_cells_mark_tiles loads, in lane (r, pz), point row min(y, N) of plane
    K0 = clamp(zc) (A), plus row min(y + 1, N) in lanes r = 7 (C), plane K1 =
    clamp(zc + 1) in lanes pz = 3 (B), both in lane (7, 3) (D); the row above
    comes from lane + 1 for r < 7 and the plane above's terms from lane + 8
    for pz < 3.  For every active lane the rows it combines are exactly
    (zc, y), (zc, y + 1), (zc + 1, y), (zc + 1, y + 1)."""
    last = zc1
    for ty in range((N + 7) // 8 + 1):
        for zb in range(kb - 1, ke, 4):
            A, B, C, D, act, need = {}, {}, {}, {}, {}, {}
            for lane in range(32):
                r, pz = lane & 7, lane >> 3
                y = 8 * ty + r
                zc = zb + pz
                K0, K1 = min(max(zc, zc0), last), min(max(zc + 1, zc0), last)
                ya, yc = min(y, N), min(y + 1, N)
                A[lane] = (K0, ya)
                C[lane] = (K0, yc) if r == 7 else A[lane]
                B[lane] = (K1, ya) if pz == 3 else A[lane]
                D[lane] = (K1, yc) if (r == 7 and pz == 3) else A[lane]
                act[lane] = zc <= ke - 1 and zc0 <= zc < zc1 and y < N
                need[lane] = {(zc, y), (zc, y + 1), (zc + 1, y), (zc + 1, y + 1)}
            for lane in range(32):
                if not act[lane]:
                    continue
                r, pz = lane & 7, lane >> 3
                up = lane + 1 if r < 7 else lane
                rowc0 = A[up] if r < 7 else C[lane]
                rowc1 = B[up] if r < 7 else D[lane]
                # plane zc's terms: rows A, rowc0; plane zc + 1's: from lane + 8 (its A and its rowc0) or B, rowc1
                if pz < 3:
                    n8 = lane + 8
                    up8 = n8 + 1 if r < 7 else n8
                    t1 = {A[n8], A[up8] if r < 7 else C[n8]}
                else:
                    t1 = {B[lane], rowc1}
                assert {A[lane], rowc0} | t1 == need[lane], (lane, ty, zb)
                for K, yy in need[lane]:
                    assert zc0 <= K <= last and yy <= N


@pytest.mark.parametrize("nk,zc0_first", [(513, True), (512, False), (9, False), (3, True), (100, False)])
def test_mark_tiles_layers_and_slots(nk, zc0_first):
    """s2m_cells_mark_tiles forms a point plane's tile layer and ring slot
    without dividing: K in kb - 1 .. ke of tile layer tz lies in layer tz when
    K >= kb, tz - 1 below (none before the slab's first plane tk0), and the
    slab's planes zc0 .. last take consecutive ring slots from zc0 % ring."""
    parts = (nk + 7) // 8
    tzs = (nk + parts - 1) // parts
    nzt = (nk + tzs - 1) // tzs
    for ring in (nk + 1, nk + 5, 2 * nk + 3):
        for tk0 in (0, 7, 1000):
            zc0 = tk0 if zc0_first else tk0 - 1
            last = tk0 + nk - 1
            slot0 = zc0 % ring
            for K in range(zc0, last + 1):
                s = slot0 + (K - zc0)
                assert (s - ring if s >= ring else s) == K % ring
            for tz in range(nzt):
                kb = tk0 + tz * tzs
                ke = min(kb + tzs, tk0 + nk) - 1
                for K in range(max(kb - 1, zc0), ke + 1):
                    lay = -1 if K < tk0 else (tz if K >= kb else tz - 1)
                    assert lay == (-1 if K < tk0 else (K - tk0) // tzs), (K, tz)
