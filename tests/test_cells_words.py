"""Classification words on the CPU: the bitwise formulas of s2m_cells_mark
(static_kernels.cuh), restated in numpy, against the per-cell rule of
s2_classify_values (s2m_dc_core.cuh; dualcontour.wgsl's sign test plus the
reference rule's near-zero test of off-lattice corners).

The kernel forms 32 cells along x per word from the sign and near-zero bits
of the 4 point rows around them (a corner at x + 1 is the row's word shifted
right by one point), and computes per point plane the AND / OR of its corner
words and the near-zero terms of a cell's bottom (corners 1-3) and top
(corners 4-7) planes.  These tests check that decomposition on random
lattices with NaN, +-0 and values at the guard, random off-lattice columns,
rows and planes, N both a multiple of 32 and not, and every job mode."""
import numpy as np
import pytest

M32 = np.uint64(0xFFFFFFFF)


def pack_rows(bits):
    """bool [..., P] -> uint32 words [..., WP], bit x % 32 of word x // 32."""
    P = bits.shape[-1]
    WP = (P + 31) // 32
    pad = np.zeros(bits.shape[:-1] + (WP * 32,), bool)
    pad[..., :P] = bits
    w = pad.reshape(bits.shape[:-1] + (WP, 32)).astype(np.uint64)
    return (w << np.arange(32, dtype=np.uint64)).sum(-1).astype(np.uint64)


def funnel1(lo, hi):
    """__funnelshift_r(lo, hi, 1)."""
    return ((lo >> np.uint64(1)) | ((hi & np.uint64(1)) << np.uint64(31))) & M32


def words_rule(V, guard, offx, offy, offz, qef=False, exact=False):
    """Candidate words [nz, N, WN] as s2m_cells_mark forms them."""
    nzp, P, _ = V.shape
    N = P - 1
    WN, WP = (N + 31) // 32, (P + 31) // 32
    pos = pack_rows(V > 0)
    near = pack_rows(~(np.abs(V) >= guard))
    nxt = lambda a: np.concatenate([a[..., 1:], np.zeros(a.shape[:-1] + (1,), np.uint64)], -1)
    ox = pack_rows(offx[1:])[:WN] if not qef else np.zeros(WN, np.uint64)  # bit x: off(x + 1)
    oy = np.where(offy[1:] & (not qef), M32, np.uint64(0))                 # row y: off(y + 1)
    oz = np.where(offz & (not qef), M32, np.uint64(0))                     # plane p: off(p)
    out = np.zeros((nzp - 1, N, WN), np.uint64)
    for y in range(N):
        andp, orp, tb, tt = [], [], [], []
        for p in range(nzp):
            p0, p1 = pos[p, y, :WN], pos[p, y + 1, :WN]
            p0s, p1s = funnel1(p0, nxt(pos[p, y])[:WN]), funnel1(p1, nxt(pos[p, y + 1])[:WN])
            andp.append(p0 & p0s & p1 & p1s)
            orp.append(p0 | p0s | p1 | p1s)
            n0, n1 = near[p, y, :WN], near[p, y + 1, :WN]
            n0s, n1s = funnel1(n0, nxt(near[p, y])[:WN]), funnel1(n1, nxt(near[p, y + 1])[:WN])
            tb.append((n0s & ox) | (n1 & oy[y]) | (n1s & (ox | oy[y])))
            tt.append((n0 & oz[p]) | (n0s & (ox | oz[p])) | (n1 & (oy[y] | oz[p])) | (n1s & (ox | oy[y] | oz[p])))
        for z in range(nzp - 1):
            c = (orp[z] | orp[z + 1]) & ~(andp[z] & andp[z + 1]) & M32
            if not qef:
                c |= (ox | oy[y] | oz[z + 1]) if exact else (tb[z] | tt[z + 1])
            if N % 32:
                c[WN - 1] &= np.uint64((1 << (N % 32)) - 1)
            out[z, y] = c
    return out


def cells_rule(V, guard, offx, offy, offz, qef=False, exact=False):
    """bool [nz, N, N] by s2_classify_values, cell by cell."""
    nzp, P, _ = V.shape
    N = P - 1
    out = np.zeros((nzp - 1, N, N), bool)
    for z in range(nzp - 1):
        for y in range(N):
            for x in range(N):
                v = [V[z + (k >> 2), y + ((k >> 1) & 1), x + (k & 1)] for k in range(8)]
                pos = sum((1 << k) for k in range(8) if v[k] > 0)
                if pos not in (0, 255):
                    out[z, y, x] = True
                    continue
                if qef:
                    continue
                o = [((k & 1) and offx[x + 1]) or ((k & 2) and offy[y + 1]) or ((k & 4) and offz[z + 1])
                     for k in range(8)]
                if not any(o[1:]):
                    continue
                if exact:
                    out[z, y, x] = True
                    continue
                out[z, y, x] = any(o[k] and not (abs(v[k]) >= guard) for k in range(1, 8))
    return out


def unpack(words, N):
    bits = ((words[..., None] >> np.arange(32, dtype=np.uint64)) & np.uint64(1)).astype(bool)
    return bits.reshape(words.shape[:-1] + (-1,))[..., :N]


@pytest.mark.parametrize("N", [37, 64])
@pytest.mark.parametrize("mode", ["reference", "qef", "exact"])
def test_mark_words_match_the_cell_rule(N, mode):
    rng = np.random.default_rng(N + len(mode))
    guard = np.float32(0.05)
    nz = 5
    V = rng.normal(0.0, 0.1, (nz + 1, N + 1, N + 1)).astype(np.float32)
    flat = V.reshape(-1)
    special = rng.choice(flat.size, size=flat.size // 10, replace=False)
    flat[special[0::4]] = np.float32("nan")
    flat[special[1::4]] = np.float32(0.0)
    flat[special[2::4]] = np.float32(-0.0)
    flat[special[3::4]] = np.float32(guard) * rng.choice([-1, 1], special[3::4].size)
    offx = rng.random(N + 1) < 0.3
    offy = rng.random(N + 1) < 0.3
    offz = rng.random(nz + 1) < 0.4
    kw = dict(qef=mode == "qef", exact=mode == "exact")
    got = unpack(words_rule(V, guard, offx, offy, offz, **kw), N)
    want = cells_rule(V, guard, offx, offy, offz, **kw)
    assert got.shape == want.shape
    bad = np.argwhere(got != want)
    assert bad.size == 0, f"{len(bad)} cells differ, first (z, y, x) = {tuple(bad[0])}"
    assert want.any() and not want.all()


def tile_skip_words(V, guard, k0, zc0, tzs, N):
    """Positions (cell plane dz, row y, word w) that s2m_cells_mark skips: every
    tile 4w .. 4w + 3 of tile row y // 8, in the layer (zc0 + dz + 1 - k0) //
    tzs of the cell's upper plane, is decided.  A tile's flag is restated from
    the values themselves (s2m_tiles proves it by interval arithmetic over a
    box that holds these points): points 8 tx .. 8 tx + 8 along x and y, planes
    kb - 1 .. kb + tzs - 1 (kb = k0 + layer * tzs) along z, all >= guard or all
    <= -guard.  Tiles past the last one count as decided (they cover no cell)."""
    nzp, P, _ = V.shape
    WN = (N + 31) // 32
    ntx = (P + 7) // 8
    last = zc0 + nzp - 1  # last lattice plane held in V (V[0] is plane zc0)
    nzt = (last - k0) // tzs + 1

    def decided(tx, ty, tz):
        if tx >= ntx:
            return True
        kb = k0 + tz * tzs
        z0, z1 = max(kb - 1, zc0), min(kb + tzs - 1, last)
        box = V[z0 - zc0:z1 - zc0 + 1, 8 * ty:8 * ty + 9, 8 * tx:8 * tx + 9]
        return bool((box >= guard).all() or (box <= -guard).all())

    flags = {(tx, ty, tz): decided(tx, ty, tz) for tx in range(4 * WN) for ty in range(ntx) for tz in range(nzt)}
    skip = np.zeros((nzp - 1, N, WN), bool)
    for dz in range(nzp - 1):
        layer = (zc0 + dz + 1 - k0) // tzs
        for y in range(N):
            for w in range(WN):
                skip[dz, y, w] = all(flags[(4 * w + b, y >> 3, layer)] for b in range(4))
    return skip


@pytest.mark.parametrize("N,first_slab", [(96, True), (130, False), (64, False)])
@pytest.mark.parametrize("mode", ["reference", "qef"])
def test_mark_tile_skip_drops_no_candidate(N, first_slab, mode):
    """Words that the mark skips by decided tiles hold no candidate: each cell's
    corners lie in the box of the tile of its point (x, y, z + 1)."""
    rng = np.random.default_rng(7 * N + first_slab)
    guard = np.float32(0.02)
    nz = 13  # cell planes of the slab
    zc0 = 0 if first_slab else 9
    k0 = zc0 if first_slab else zc0 + 1  # the first slab's planes start at its first cell plane
    nk = zc0 + nz - k0 + 1
    tzs = (nk + (nk + 7) // 8 - 1) // ((nk + 7) // 8)
    P = N + 1
    z, y, x = np.meshgrid(np.arange(zc0, zc0 + nz + 1), np.arange(P), np.arange(P), indexing="ij")
    # a union of spheres and a box whose faces cross between the last point of
    # one tile and the first of the next (x, y: 8 t + 7.5; z: half a plane
    # below a tile layer's first plane), where a cell's tile is easy to get
    # wrong by one
    d = np.full(x.shape, np.inf)
    for _ in range(4):
        c = rng.uniform([0, 0, zc0], [N, N, zc0 + nz])
        d = np.minimum(d, np.sqrt((x - c[0]) ** 2 + (y - c[1]) ** 2 + (z - c[2]) ** 2) - rng.uniform(3, 10))
    bx = (8 * 1 + 7.5, 8 * 4 + 7.5)
    bz = (k0 + tzs - 0.5, zc0 + nz + 5)
    d = np.minimum(d, np.maximum.reduce([bx[0] - x, x - bx[1], bx[0] - y, y - bx[1], bz[0] - z, z - bz[1]]))
    V = (0.05 * d + rng.normal(0, 0.002, d.shape)).astype(np.float32)  # +-0.5 cells: beyond the guard
    offx = rng.random(N + 1) < 0.3
    offy = rng.random(N + 1) < 0.3
    offz = rng.random(nz + 1) < 0.4
    words = words_rule(V, guard, offx, offy, offz, qef=mode == "qef")
    skip = tile_skip_words(V, guard, k0, zc0, tzs, N)
    assert skip.mean() > 0.05 and not skip.all(), skip.mean()  # the skip happens, and not everywhere
    assert (words[skip] == 0).all()
    assert (words != 0).any()


def decided_bytes(f, fn, pos_lo, pos_hi, near_lo, near_hi):
    """s2_decided_bytes (static_kernels.cuh), on uint64 arrays holding 32-bit words."""
    m = np.uint64(0x01010101)
    dm = ((f & m) * np.uint64(0xFF)) & M32
    pm = (((f >> np.uint64(1)) & f & m) * np.uint64(0xFF)) & M32
    dmn, pmn = fn & np.uint64(1), (fn >> np.uint64(1)) & fn & np.uint64(1)
    return ((pos_lo & ~dm & M32) | pm, (pos_hi & ~dmn & M32) | pmn, near_lo & ~dm & M32, near_hi & ~dmn & M32)


def test_decided_bytes_follow_the_tile_flags():
    """A point row's 32 points lie in tiles 4w .. 4w + 3 (byte b of the word:
    points 8b .. 8b + 7 of tile 4w + b) and its next point in tile 4w + 4: the
    words with decided bytes replaced equal the bits of a lattice whose decided
    tiles hold their sign everywhere and no near-zero point, with garbage in the
    decided bytes before."""
    rng = np.random.default_rng(3)
    P = 200
    ntx = (P + 7) // 8
    WP = (P + 31) // 32
    rows = 64
    flag = rng.integers(0, 4, (rows, 4 * WP + 4)) * (rng.random((rows, 4 * WP + 4)) < 0.7)
    flag[:, ntx:] = 1  # past the last tile: decided, no sign
    pos = rng.random((rows, 32 * WP)) < 0.5
    near = rng.random((rows, 32 * WP)) < 0.3
    tile = np.arange(32 * WP) // 8
    dec = (flag[:, tile] & 1).astype(bool)
    want_pos = np.where(dec, (flag[:, tile] & 2).astype(bool), pos)  # a positive flag without decided: ignored
    want_near = np.where(dec, False, near)
    garbage_pos = np.where(dec, rng.random(pos.shape) < 0.5, pos)
    garbage_near = np.where(dec, rng.random(pos.shape) < 0.5, near)
    gp, gn = pack_rows(garbage_pos), pack_rows(garbage_near)
    wp, wn = pack_rows(want_pos), pack_rows(want_near)
    fw = np.zeros((rows, WP + 1), np.uint64)
    for w in range(WP + 1):
        for b in range(4):
            fw[:, w] |= flag[:, 4 * w + b].astype(np.uint64) << np.uint64(8 * b)
    for w in range(WP - 1):
        lo_p, hi_p, lo_n, hi_n = decided_bytes(fw[:, w], fw[:, w + 1], gp[:, w], gp[:, w + 1], gn[:, w], gn[:, w + 1])
        assert (lo_p == wp[:, w]).all() and (lo_n == wn[:, w]).all()
        assert ((hi_p & np.uint64(1)) == (wp[:, w + 1] & np.uint64(1))).all()
        assert ((hi_n & np.uint64(1)) == (wn[:, w + 1] & np.uint64(1))).all()
