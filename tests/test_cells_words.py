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
