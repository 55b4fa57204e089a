"""The double-float multiply-add of the mixed form's mat-vec, emulated in IEEE
float32 on the host (numpy float32 operations round to nearest like the
device's __fadd_rn / __fmul_rn; an FMA is the float64 value of the exact
product plus the addend rounded once to float32, exact at these widths).

df_mac(acc, a, b): p = fl(a.hi b.hi), pe = fma(a.hi, b.hi, -p) (exact),
pe = fma(a.hi, b.lo, pe), pe = fma(a.lo, b.hi, pe), (s, e) = TwoSum(acc.hi, p),
acc = (s, acc.lo + (e + pe)); after a row, one Fast2Sum normalisation.

Checked: the mat-vec's 16-term sums (one thread's share of a 32 x 32 tile)
stay within a few units of 2^-46 of sum |x y| on random rows of mixed
magnitudes, the figure the fixed-grid alternative was measured against."""
from fractions import Fraction

import numpy as np

f32 = np.float32


def _fma(a, b, c):
    return (a.astype(np.float64) * b.astype(np.float64) + c.astype(np.float64)).astype(f32)


def _two_sum(a, b):
    s = (a + b).astype(f32)
    bb = (s - a).astype(f32)
    e = ((a - (s - bb).astype(f32)).astype(f32) + (b - bb).astype(f32)).astype(f32)
    return s, e


def _fast_two_sum(a, b):
    s = (a + b).astype(f32)
    e = (b - (s - a).astype(f32)).astype(f32)
    return s, e


def _df(x):
    hi = x.astype(f32)
    lo = (x - hi.astype(np.float64)).astype(f32)
    return hi, lo


def _df_dot(xh, xl, yh, yl):
    hi = np.zeros(xh.shape[0], f32)
    lo = np.zeros(xh.shape[0], f32)
    for k in range(xh.shape[1]):
        p = (xh[:, k] * yh[:, k]).astype(f32)
        pe = _fma(xh[:, k], yh[:, k], -p)
        pe = _fma(xh[:, k], yl[:, k], pe)
        pe = _fma(xl[:, k], yh[:, k], pe)
        s, e = _two_sum(hi, p)
        hi = s
        lo = (lo + (e + pe).astype(f32)).astype(f32)
    return _fast_two_sum(hi, lo)


def test_df_multiply_add_accuracy_over_a_tile_row():
    rng = np.random.default_rng(12)
    worst = 0.0
    for spread in (0, 2, 6):
        scale = 10.0 ** rng.uniform(-8, 8, (300, 1))
        x = rng.standard_normal((300, 16)) * scale * 10.0 ** rng.uniform(-spread, 0, (300, 16))
        y = rng.standard_normal((300, 16)) * 10.0 ** rng.uniform(-spread, 0, (300, 16))
        (xh, xl), (yh, yl) = _df(x), _df(y)
        hi, lo = _df_dot(xh, xl, yh, yl)
        for r in range(300):
            exact = sum((Fraction(float(xh[r, k])) + Fraction(float(xl[r, k]))) *
                        (Fraction(float(yh[r, k])) + Fraction(float(yl[r, k]))) for k in range(16))
            mag = sum(abs(float(xh[r, k]) * float(yh[r, k])) for k in range(16))
            got = Fraction(float(hi[r])) + Fraction(float(lo[r]))
            worst = max(worst, abs(float(got - exact)) / mag)
    assert worst < 4 * 2.0 ** -46, worst


def test_two_sum_is_exact_and_fast_two_sum_normalises():
    rng = np.random.default_rng(13)
    a = (rng.standard_normal(20000) * 10.0 ** rng.uniform(-10, 10, 20000)).astype(f32)
    b = (rng.standard_normal(20000) * 10.0 ** rng.uniform(-10, 10, 20000)).astype(f32)
    s, e = _two_sum(a, b)
    assert np.all(s.astype(np.float64) + e.astype(np.float64) == a.astype(np.float64) + b.astype(np.float64))
    big = np.where(np.abs(a) >= np.abs(b), a, b)
    small = np.where(np.abs(a) >= np.abs(b), b, a)
    s2, e2 = _fast_two_sum(big, small)
    assert np.all(s2 == s) and np.all(e2 == e)
    assert np.all(np.abs(e2) <= np.spacing(np.abs(s2)) / 2)
