"""The double-float arithmetic of the P / P^T applies, restated in numpy on
the CPU (float32 operations round like the GPU's FP32 pipe with FMA
contraction off; TwoProduct's FMA is exact in float64 here because a
product of two floats has at most 48 bits):

* the error of the entry-by-entry (hi, lo) accumulation, renormalised every
  four entries, on the reference's own order-3 Gauss-Lobatto prolongation
  (tests/golden/brick_o3.npz) for P and P^T rows, against exact sums: within
  the 1e-13 bar relative to max(1, |y|) (observed about 1e-14 for P rows and
  6e-14 for the up to ~600-entry P^T rows);
* the integer assembly of sh + sl as a double (df_value) against the sum
  the FPU forms.

The device kernels themselves are checked against the oracle at 1e-13 in
tests/test_gpu_parity.py."""
import math

import numpy as np

from tests import pipeline

f32 = np.float32


def split(a):
    """hi = a rounded to float, lo = (a - hi) rounded to float."""
    h = a.astype(f32)
    return h, (a - h.astype(np.float64)).astype(f32)


def fma32(a, b, c):
    # float32 FMA: the exact product in float64, one rounding after the add
    # (double rounding through float64 is harmless at this tolerance)
    return (a.astype(np.float64) * b.astype(np.float64) + c.astype(np.float64)).astype(f32)


def df_rows(wh, wl, xh, xl, mask):
    """Accumulate rows entry by entry (columns of the padded arrays) the way
    df_fma / df_renorm do; masked entries add an exact zero."""
    n, L = wh.shape
    sh = np.zeros(n, f32)
    sl = np.zeros(n, f32)
    for k in range(L):
        a, b = np.where(mask[:, k], wh[:, k], 0), np.where(mask[:, k], wl[:, k], 0)
        c, d = np.where(mask[:, k], xh[:, k], 0), np.where(mask[:, k], xl[:, k], 0)
        a, b, c, d = (v.astype(f32) for v in (a, b, c, d))
        p = (a * c).astype(f32)
        e = fma32(a, c, -p)
        cr = fma32(a, d, fma32(b, c, e))
        t = (sh + p).astype(f32)
        bp = (t - sh).astype(f32)
        err = ((sh - (t - bp)) + (p - bp)).astype(f32)
        sl = (sl + (err + cr)).astype(f32)
        sh = t
        if k % 4 == 3:
            t = (sh + sl).astype(f32)
            sl = (sl - (t - sh)).astype(f32)
            sh = t
    t = (sh + sl).astype(f32)
    sl = (sl - (t - sh)).astype(f32)
    return t, sl


def _padded(rp, cols, vals, x):
    lens = np.diff(rp)
    L = int(lens.max())
    n = len(lens)
    idx = rp[:-1, None] + np.arange(L)[None, :]
    mask = np.arange(L)[None, :] < lens[:, None]
    idx = np.where(mask, idx, 0)
    return vals[idx], x[cols[idx]], mask


def test_double_float_accumulation_error_on_reference_prolongation():
    g = pipeline.load_golden("brick_o3")
    rp, cols, vals = g["levels"][0]["P"]
    keep = np.abs(vals) >= 2.0 ** -49
    # the apply copy: entries with |w| >= 2^-49, in row order
    kr = np.repeat(np.arange(len(rp) - 1), np.diff(rp))[keep]
    rp_a = np.concatenate([[0], np.cumsum(np.bincount(kr, minlength=len(rp) - 1))])
    c_a, v_a = cols[keep], vals[keep]
    rng = np.random.default_rng(4)
    ncols = int(cols.max()) + 1
    # P rows
    x = rng.standard_normal(ncols)
    W, X, M = _padded(rp_a, c_a, v_a, x)
    wh, wl = split(W)
    xh, xl = split(X)
    sh, sl = df_rows(wh, wl, xh, xl, M)
    y = sh.astype(np.float64) + sl.astype(np.float64)
    exact = np.array([math.fsum(W[i, M[i]] * X[i, M[i]]) for i in range(len(y))])
    err_p = np.abs(y - exact) / np.maximum(1.0, np.abs(exact))
    assert err_p.max() < 1e-13, err_p.max()
    # P^T rows: the transpose of the apply copy (rows ascending per column)
    order = np.lexsort((kr, c_a))
    t_rows, t_vals = kr[order], v_a[order]
    t_rp = np.concatenate([[0], np.cumsum(np.bincount(c_a, minlength=ncols))])
    xf = rng.standard_normal(len(rp) - 1)
    W, X, M = _padded(t_rp, t_rows, t_vals, xf)
    assert M.shape[1] > 100  # long transpose rows
    wh, wl = split(W)
    xh, xl = split(X)
    sh, sl = df_rows(wh, wl, xh, xl, M)
    y = sh.astype(np.float64) + sl.astype(np.float64)
    exact = np.array([math.fsum(W[i, M[i]] * X[i, M[i]]) for i in range(len(y))])
    err_t = np.abs(y - exact) / np.maximum(1.0, np.abs(exact))
    assert err_t.max() < 1e-13, err_t.max()


def df_value(sh, sl):
    """df_value's integer assembly of sh + sl as a double (normal sh)."""
    bh = sh.view(np.uint32).astype(np.uint64)
    bl = sl.view(np.uint32).astype(np.uint64)
    eh = ((bh >> 23) & 0xFF).astype(np.int64)
    el = ((bl >> 23) & 0xFF).astype(np.int64)
    hd = ((bh & 0x80000000) << 32) | ((eh.astype(np.uint64) + 896) << 52) | ((bh & 0x7FFFFF) << 29)
    g = eh - el
    neg = ((bh ^ bl) >> 31) != 0
    pow2 = (bh & 0x7FFFFF) == 0
    sft = np.where(neg & pow2, 30, 29) - g
    ml = (bl & 0x7FFFFF) | 0x800000
    d = np.zeros_like(ml)
    left = sft >= 0
    d[left] = ml[left] << sft[left].astype(np.uint64)
    right = (sft < 0) & (sft > -26)
    r = (-sft[right]).astype(np.uint64)
    d[right] = (ml[right] + (np.uint64(1) << (r - np.uint64(1)))) >> r
    out = np.where(neg, hd - d, hd + d)
    out = np.where(el == 0, hd, out)
    return out.view(np.float64)


def test_integer_double_assembly():
    rng = np.random.default_rng(7)
    n = 1_000_000
    v = rng.uniform(-1, 1, n) * np.ldexp(1.0, rng.integers(-40, 40, n))
    # powers of two with tails of both signs
    k = n // 5
    v[:k] = np.ldexp(1.0, rng.integers(-30, 30, k)) * (1 + rng.choice([-1e-9, 1e-9], k))
    sh = v.astype(f32)
    sl = (v - sh.astype(np.float64)).astype(f32)
    t = (sh + sl).astype(f32)
    sl = (sl - (t - sh)).astype(f32)
    sh = t
    ok = sh != 0
    exact = sh[ok].astype(np.float64) + sl[ok].astype(np.float64)
    assert np.array_equal(df_value(sh[ok], sl[ok]), exact)
    # tails far below sh: within one ulp of the FPU's sum
    sh2 = (rng.uniform(0.5, 1.0, n) * np.ldexp(1.0, rng.integers(-20, 20, n))).astype(f32)
    sl2 = (rng.uniform(-1, 1, n) * np.abs(sh2.astype(np.float64)) *
           np.ldexp(1.0, -rng.integers(24, 64, n))).astype(f32)
    ref = sh2.astype(np.float64) + sl2.astype(np.float64)
    got = df_value(sh2, sl2)
    assert (np.abs(got - ref) <= np.spacing(np.abs(ref))).all()
