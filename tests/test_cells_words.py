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


# ---------------------------------------------------------------------------
# Decided-tile map (s2m_tile_map, s2_map_bits, s2_map_points): with tile
# pruning, nothing writes the point-bit words of decided tiles; the mark
# kernel takes those points' bits from the map (sign from the tile's flag,
# near-zero 0) and the rest from the words.  Restated here over random tile
# flags and random stale bytes where decided tiles' bits would be.

def map_rows(flags, ntx):
    """s2m_tile_map: flags [rows, ntx] (bit 0 decided, bit 1 positive) -> words [rows, wt]."""
    rows = flags.shape[0]
    wt = (ntx + 15) // 16
    out = np.zeros((rows, wt), np.uint64)
    for tx in range(ntx):
        f = flags[:, tx].astype(np.uint64)
        bits = np.where(f & 1, np.uint64(1) | np.where(f & 2, np.uint64(2), np.uint64(0)), np.uint64(0))
        out[:, tx // 16] |= bits << np.uint64(2 * (tx % 16))
    return out


def map_bits(mrow, w, more):
    """s2_map_bits on one map row: 10 bits of tiles 4w .. 4w + 4."""
    lo = int(mrow[w >> 2])
    hi = int(mrow[(w >> 2) + 1]) if (w & 3) == 3 and more else 0
    return (((hi << 32) | lo) >> (8 * (w & 3))) & 0x3FF


def map_points(e, sel):
    """s2_map_points: the kernel's nibble spread, in 32-bit arithmetic."""
    x = (e >> sel) & 0x55
    nib = (x & 1) | ((x >> 1) & 2) | ((x >> 2) & 4) | ((x >> 3) & 8)
    return ((((nib * 0x00204081) & 0xFFFFFFFF) & 0x01010101) * 0xFF) & 0xFFFFFFFF


@pytest.mark.parametrize("P", [33, 64, 129, 200])
def test_tile_map_restores_decided_bits(P):
    rng = np.random.default_rng(P)
    ntx = (P + 7) // 8
    WP = (P + 31) // 32
    nrows_y = P
    flags = rng.integers(0, 4, size=(ntx, ntx))          # one tile layer: [ty, tx]
    flags[rng.random(flags.shape) < 0.3] = 0             # undecided
    truth_pos = rng.random((nrows_y, P)) < 0.5
    truth_near = rng.random((nrows_y, P)) < 0.2
    dec_pt = np.zeros((nrows_y, P), bool)
    for y in range(nrows_y):
        for x in range(P):
            f = flags[y // 8, x // 8]
            if f & 1:
                dec_pt[y, x] = True
                truth_pos[y, x] = bool(f & 2)
                truth_near[y, x] = False
    # memory: true bits where undecided, random stale bits where decided
    mem_pos = np.where(dec_pt, rng.random(dec_pt.shape) < 0.5, truth_pos)
    mem_near = np.where(dec_pt, rng.random(dec_pt.shape) < 0.5, truth_near)
    pos_w, near_w = pack_rows(mem_pos), pack_rows(mem_near)
    want_pos, want_near = pack_rows(truth_pos), pack_rows(truth_near)
    mp = map_rows(flags, ntx)
    for y in range(nrows_y):
        for w in range(WP):
            more = w + 1 < WP
            e = map_bits(mp[y >> 3], w, more)
            dec, posd = map_points(e, 0), map_points(e, 1)
            decn, posn = (e >> 8) & 1, (e >> 9) & 1
            got_pos = ((0 if dec == 0xFFFFFFFF else int(pos_w[y, w]) & ~dec) | posd) & 0xFFFFFFFF
            got_near = 0 if dec == 0xFFFFFFFF else int(near_w[y, w]) & ~dec & 0xFFFFFFFF
            valid = (1 << min(32, P - 32 * w)) - 1  # points past the lattice edge are never used
            assert got_pos & valid == int(want_pos[y, w]) & valid, (y, w)
            assert got_near & valid == int(want_near[y, w]) & valid, (y, w)
            if more:  # only bit 0 of the next word is used (the funnel shift)
                nxt_pos = (1 if posn else 0) if decn else int(pos_w[y, w + 1])
                nxt_near = 0 if decn else int(near_w[y, w + 1])
                assert nxt_pos & 1 == int(want_pos[y, w + 1]) & 1, (y, w)
                assert nxt_near & 1 == int(want_near[y, w + 1]) & 1, (y, w)
