"""The interval rules of the smooth operators (s2m_prelude.cuh), checked
directly on the CPU: for random operand and blend-width intervals, and for
many points inside them, the binary32 point value of
sdf_op_smooth_union / intersection / subtraction

- lies in the interval that s2i_smooth_*_sel returns when it keeps both
  operands (the monotone corner bound plus its slack), and
- equals, bit for bit, s2_canon of the operand that it keeps when it decides
  (h = 1 or h = +0 at every point: x + (+0), -0 becoming +0).

Operand intervals include ones that contain 0 or end exactly at +-0, and
points include both zeros, so the signed-zero cases of the decisions are
exercised."""
import ctypes
import os
import subprocess
import tempfile

import numpy as np
import pytest

from hostsdf import PRELUDE

DRIVER = r'''
extern "C" void sel(int kind, long n, const float* iv, float* out, int* d) {
  for (long i = 0; i < n; ++i) {
    s2i a, b, k; a.lo = iv[6*i]; a.hi = iv[6*i+1]; b.lo = iv[6*i+2]; b.hi = iv[6*i+3]; k.lo = iv[6*i+4]; k.hi = iv[6*i+5];
    s2i r = kind == 0 ? s2i_smooth_union_sel(a, b, k, &d[i]) : kind == 1 ? s2i_smooth_intersection_sel(a, b, k, &d[i])
                      : s2i_smooth_subtraction_sel(a, b, k, &d[i]);
    out[2*i] = r.lo; out[2*i+1] = r.hi;
  }
}
extern "C" void point(int kind, long n, const float* abk, float* out, float* canon_kept) {
  for (long i = 0; i < n; ++i) {
    float a = abk[3*i], b = abk[3*i+1], k = abk[3*i+2];
    out[i] = kind == 0 ? s2_op_smooth_union(a, b, k) : kind == 1 ? s2_op_smooth_intersection(a, b, k)
                       : s2_op_smooth_subtraction(a, b, k);
    canon_kept[2*i] = s2_canon(kind == 2 ? -a : a);
    canon_kept[2*i+1] = s2_canon(b);
  }
}
'''


@pytest.fixture(scope="module")
def lib():
    d = tempfile.mkdtemp(prefix="s2m_smooth_")
    src = os.path.join(d, "smooth.cpp")
    with open(src, "w") as f:
        f.write(f'#include "{PRELUDE}"\n' + DRIVER)
    so = os.path.join(d, "smooth.so")
    subprocess.run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math", src, "-o", so],
                   check=True, capture_output=True)
    L = ctypes.CDLL(so)
    L.sel.argtypes = [ctypes.c_int, ctypes.c_long, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    L.point.argtypes = [ctypes.c_int, ctypes.c_long, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    return L


def random_intervals(rng, n):
    c = rng.normal(0, 0.1, (n, 2)).astype(np.float32)
    w = (rng.random((n, 2)) ** 3 * 0.2).astype(np.float32)
    lo, hi = c - w, c + w
    # some intervals end exactly at +-0 or contain 0
    z = rng.random((n, 2))
    lo[z < 0.1] = np.float32(0.0)
    hi[(z >= 0.1) & (z < 0.2)] = np.float32(-0.0)
    lo = np.minimum(lo, hi)
    k = (0.005 + rng.random(n) * 0.05).astype(np.float32)
    return np.stack([lo[:, 0], hi[:, 0], lo[:, 1], hi[:, 1], k, k], 1).astype(np.float32)


@pytest.mark.parametrize("kind", [0, 1, 2], ids=["union", "intersection", "subtraction"])
def test_smooth_intervals_and_decisions(lib, kind):
    rng = np.random.default_rng(kind + 7)
    n, m = 4000, 24
    iv = np.ascontiguousarray(random_intervals(rng, n))
    out = np.zeros((n, 2), np.float32)
    dec = np.zeros(n, np.int32)
    lib.sel(kind, n, iv.ctypes.data, out.ctypes.data, dec.ctypes.data)
    # points: both ends, both zeros where inside, and random interior values
    t = rng.random((n, m, 2)).astype(np.float32)
    a = iv[:, 0:1] + (iv[:, 1:2] - iv[:, 0:1]) * t[..., 0]
    b = iv[:, 2:3] + (iv[:, 3:4] - iv[:, 2:3]) * t[..., 1]
    a[:, 0], a[:, 1], b[:, 2], b[:, 3] = iv[:, 0], iv[:, 1], iv[:, 2], iv[:, 3]
    for col, val in ((4, 0.0), (5, -0.0)):
        ina = (iv[:, 0] <= 0) & (iv[:, 1] >= 0)
        inb = (iv[:, 2] <= 0) & (iv[:, 3] >= 0)
        a[ina, col] = np.float32(val)
        b[inb, col + 2] = np.float32(val)
    a = np.clip(a, iv[:, 0:1], iv[:, 1:2])
    b = np.clip(b, iv[:, 2:3], iv[:, 3:4])
    abk = np.ascontiguousarray(np.stack([a, b, np.repeat(iv[:, 4:5], m, 1)], -1).reshape(-1, 3))
    val = np.zeros(n * m, np.float32)
    kept = np.zeros((n * m, 2), np.float32)
    lib.point(kind, n * m, abk.ctypes.data, val.ctypes.data, kept.ctypes.data)
    val, kept = val.reshape(n, m), kept.reshape(n, m, 2)
    known = np.isfinite(out).all(1)
    both = known & (dec == 0)
    assert ((val >= out[:, :1]) & (val <= out[:, 1:]))[both].all(), "a point value outside its interval"
    for dval, col in ((1, 0), (2, 1)):
        sel = dec == dval
        assert (val[sel].view(np.uint32) == kept[sel, :, col].view(np.uint32)).all(), \
            f"decision {dval} does not reproduce the operator bit for bit"
    # the rules decide often, including where the kept operand may be zero
    assert (dec == 1).sum() > n // 20 and (dec == 2).sum() > n // 20
    zero_kept = ((dec == 1) & (iv[:, 0] <= 0) & (iv[:, 1] >= 0)) | ((dec == 2) & (iv[:, 2] <= 0) & (iv[:, 3] >= 0))
    assert zero_kept.any()
