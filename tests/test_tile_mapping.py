"""Index arithmetic of the tile pass on the CPU (no GPU): the thread-to-tile
mapping of s2m_tiles, the coarse boxes of s2m_tiles_coarse, the tile layers of
s2m_fill_decided and the per-cell tile of s2_cell_prune_tile
(s2m_dc_kernels.cuh, static_kernels.cuh, s2m_dc_core.cuh), restated from the
kernels' formulas with the constants read from s2m_device.h.  Every tile of
every slab must be taken by exactly one thread; each tile's box must lie in
its coarse box; the fill's layers must cover each plane of a slab once; and
each cell's tile must cover the cell's 8 corners.  A tile record that no
thread wrote would keep another job's bits, which a GPU comparison could
miss when both jobs are alike."""
import os
import re

import pytest

HDR = os.path.join(os.path.dirname(__file__), "..", "sdf2mesh_gb300", "csrc", "s2m_device.h")


def const(name):
    m = re.search(r"#define\s+%s\s+(\d+)" % name, open(HDR).read())
    assert m, name
    return int(m.group(1))


XY, ZMAX, CO, COZ = const("S2_PT_XY"), const("S2_PT_ZMAX"), const("S2_PT_COARSE"), const("S2_PT_COARSE_Z")


def slab_planes(s, D, nzc):
    zc0 = s * D
    zc1 = min(nzc, zc0 + D)
    k0 = 0 if s == 0 else zc0 + 1
    return k0, zc1 - k0 + 1


def tile_depth(nk):
    parts = (nk + ZMAX - 1) // ZMAX
    return (nk + parts - 1) // parts


def slab_geometry(P, D, nzc):
    """Per slab: (k0, nk, tzs, nzt, tiles, coarse boxes), as prune_layout counts them."""
    ntx = (P + XY - 1) // XY
    ncx = (ntx + CO - 1) // CO
    out = []
    for s in range((nzc + D - 1) // D):
        k0, nk = slab_planes(s, D, nzc)
        tzs = tile_depth(nk)
        nzt = (nk + tzs - 1) // tzs
        out.append((k0, nk, tzs, nzt, ntx * ntx * nzt, ncx * ncx * ((nzt + COZ - 1) // COZ)))
    return out


def tiles_threads(P, geo):
    """(slab, t) -> the coarse box it took its parent bits from, for every live thread of s2m_tiles."""
    ntx = (P + XY - 1) // XY
    ncx = (ntx + CO - 1) // CO
    per_box = CO * CO * COZ
    taken = {}
    for s, (k0, nk, tzs, nzt, nt, nc) in enumerate(geo):
        for q in range(nc * per_box):
            lc, sub = divmod(q, per_box)
            cx, r = lc % ncx, lc // ncx
            tx = cx * CO + (sub & 3)
            ty = (r % ncx) * CO + ((sub >> 2) & 3)
            tz = (r // ncx) * COZ + (sub >> 4)
            if tx < ntx and ty < ntx and tz < nzt:
                key = (s, (tz * ntx + ty) * ntx + tx)
                assert key not in taken, f"tile {key} taken twice"
                taken[key] = (lc, cx, r % ncx, r // ncx)
    return taken


@pytest.mark.parametrize("N,D", [(16, 16), (37, 5), (64, 9), (100, 33), (129, 128), (200, 7)])
def test_every_tile_once_inside_its_coarse_box(N, D):
    P, nzc = N + 1, N
    geo = slab_geometry(P, D, nzc)
    taken = tiles_threads(P, geo)
    ntx = (P + XY - 1) // XY
    assert len(taken) == sum(g[4] for g in geo)
    for (s, t), (lc, cx, cy, cz) in taken.items():
        k0, nk, tzs, nzt, _, _ = geo[s]
        tx, ty, tz = t % ntx, (t // ntx) % ntx, t // (ntx * ntx)
        # tile box (lattice indices, before the margin) within the coarse box
        ti0, ti1 = tx * XY, min(tx * XY + XY, P) - 1
        tj0, tj1 = ty * XY, min(ty * XY + XY, P) - 1
        tkb, tke = k0 + tz * tzs, min(k0 + tz * tzs + tzs, k0 + nk) - 1
        span = XY * CO
        ci0, ci1 = cx * span, min(cx * span + span, P) - 1
        cj0, cj1 = cy * span, min(cy * span + span, P) - 1
        ckb = k0 + cz * COZ * tzs
        cke = min(ckb + COZ * tzs, k0 + nk) - 1
        assert ci0 <= ti0 and ti1 + 1 <= ci1 + 1 and cj0 <= tj0 and tj1 + 1 <= cj1 + 1
        assert ckb <= tkb and max(tkb, tke) <= max(ckb, cke) and tkb <= tke


@pytest.mark.parametrize("N,D", [(16, 16), (37, 5), (100, 33), (200, 7)])
def test_fill_layers_cover_each_plane_once(N, D):
    geo = slab_geometry(N + 1, D, N)
    for k0, nk, tzs, nzt, _, _ in geo:
        planes = []
        for layer in range(nzt):
            kb = k0 + layer * tzs
            ke = min(kb + tzs, k0 + nk)
            assert kb < ke, "empty layer"
            planes += list(range(kb, ke))
        assert planes == list(range(k0, k0 + nk))


@pytest.mark.parametrize("N,D", [(16, 16), (37, 5), (100, 33)])
def test_cell_tile_covers_the_cell(N, D):
    """s2_cell_prune_tile: the tile whose widened box (one point further in
    +x, +y and -z) holds all 8 corners of cell (x, y, z)."""
    P, nzc = N + 1, N
    geo = slab_geometry(P, D, nzc)
    base = [0]
    for g in geo:
        base.append(base[-1] + g[4])
    ntx = (P + XY - 1) // XY
    for z in range(nzc):
        s = z // D
        k0, nk, tzs, nzt, _, _ = geo[s]
        tz = (z + 1 - k0) // tzs
        assert 0 <= tz < nzt
        kb, ke = k0 + tz * tzs, min(k0 + tz * tzs + tzs, k0 + nk) - 1
        assert kb - 1 <= z and z + 1 <= max(kb, ke)  # planes z, z + 1 in the box's z range
        for y in range(0, N, 7):
            for x in range(0, N, 5):
                t = (tz * ntx + y // XY) * ntx + x // XY
                assert base[s] + t < base[s + 1]
                i0 = (x // XY) * XY
                j0 = (y // XY) * XY
                assert i0 <= x and x + 1 <= min(i0 + XY, P) - 1 + 1
                assert j0 <= y and y + 1 <= min(j0 + XY, P) - 1 + 1
