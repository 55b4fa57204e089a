"""The bf16 slicing of the tensor-core products, emulated in IEEE float32 on the
host (numpy float32 arithmetic rounds to nearest, like the device's __fadd_rn /
__fmul_rn).  The long-K kernel cuts a double-float value (hi, lo) scaled by its
row exponent into 7 digits on fixed grids 2^-8(s+1): it rounds with the
constant 1.5 * 2^(23-8(s+1)) and keeps the residual pair with Fast2Sum.  These
tests check that this gives the same digits as the per-element TwoSum form
(scale by 256, rint, TwoSum), that the digits fit bf16 exactly, that they
reconstruct the value to 2^-56 of the row scale, and that K = 64 slice
products sum below 2^24 (exact FP32 accumulation)."""
import numpy as np

f32 = np.float32


def _two_sum(a, b):
    s = (a + b).astype(f32)
    bb = (s - a).astype(f32)
    e = ((a - (s - bb).astype(f32)).astype(f32) + (b - bb).astype(f32)).astype(f32)
    return s, e


def _fast_two_sum(a, b):
    s = (a + b).astype(f32)
    e = (b - (s - a).astype(f32)).astype(f32)
    return s, e


def _rows(rng, nrows=400, k=64):
    scale = 10.0 ** rng.uniform(-30, 30, (nrows, 1))
    x = rng.standard_normal((nrows, k)) * scale * 10.0 ** rng.uniform(-9, 0, (nrows, k))
    x[rng.random((nrows, k)) < 0.1] = 0.0
    hi = x.astype(f32)
    lo = (x - hi.astype(np.float64)).astype(f32)
    amax = np.abs(hi).max(axis=1)
    _, E = np.frexp(amax)
    E = np.where(amax > 0, E, 0).astype(np.int64)[:, None]
    return x, hi, lo, E


def _digits_twosum(hi, lo, E):
    th = np.ldexp(hi, -E).astype(f32)
    tl = np.ldexp(lo, -E).astype(f32)
    out = []
    for _ in range(7):
        th = (th * f32(256)).astype(f32)
        tl = (tl * f32(256)).astype(f32)
        m = np.rint(th).astype(f32)
        th, tl = _two_sum((th - m).astype(f32), tl)
        out.append(m)
    return np.stack(out)


def _digits_fixed_grid(hi, lo, E):
    # rows whose largest magnitude is subnormal (E <= -128) scale in two exact
    # steps, 2^100 first: 2^-E alone overflows float32
    e1 = np.where(E < -100, 100, 0)
    pre = np.ldexp(np.ones_like(E, dtype=np.float64), e1).astype(f32)
    sc = np.ldexp(np.ones_like(E, dtype=np.float64), -E - e1).astype(f32)
    th = ((hi * pre).astype(f32) * sc).astype(f32)
    tl = ((lo * pre).astype(f32) * sc).astype(f32)
    out = []
    for s in range(7):
        mag = f32(1.5 * 2.0 ** (15 - 8 * s))
        up = f32(2.0 ** (8 * (s + 1)))
        m = ((th + mag).astype(f32) - mag).astype(f32)
        th, tl = _fast_two_sum((th - m).astype(f32), tl)
        out.append((m * up).astype(f32))
    return np.stack(out)


def test_fixed_grid_digits_equal_twosum_digits():
    rng = np.random.default_rng(5)
    _, hi, lo, E = _rows(rng)
    np.testing.assert_array_equal(_digits_fixed_grid(hi, lo, E), _digits_twosum(hi, lo, E))


def test_digits_are_bf16_integers_and_reconstruct():
    rng = np.random.default_rng(6)
    x, hi, lo, E = _rows(rng)
    d = _digits_fixed_grid(hi, lo, E).astype(np.float64)   # (7, rows, K)
    assert np.all(d == np.rint(d))
    assert np.abs(d[0]).max() <= 256 and np.abs(d[1:]).max() <= 129
    # bf16 keeps 8 significant bits: every |m| <= 256 is exact
    bf = (d.astype(f32).view(np.uint32) & np.uint32(0xFFFF0000)).view(f32)
    np.testing.assert_array_equal(bf.astype(np.float64), d)
    w = 2.0 ** (-8.0 * (np.arange(7) + 1))
    rec = np.einsum("s,srk->rk", w, d)
    target = np.ldexp(hi.astype(np.float64) + lo.astype(np.float64), -E)
    assert np.abs(rec - target).max() <= 2.0 ** -56


def test_slice_products_accumulate_exactly_in_fp32():
    # 64 products of digits: at most 64 * 256 * 256 = 2^22 < 2^24
    rng = np.random.default_rng(7)
    _, hi, lo, E = _rows(rng, nrows=64)
    d = _digits_fixed_grid(hi, lo, E)
    for s in range(7):
        for t in range(7 - s):
            p = d[s][:, None, :].astype(np.float64) * d[t][None, :, :].astype(np.float64)
            assert np.abs(p).sum(axis=2).max() < 2.0 ** 24


def test_subnormal_rows_slice_finite_and_exact():
    """Rows whose largest value is below the float32 normal range (the far
    tail of a localised eigenvector): the two-step scale keeps every digit
    finite and equal to the per-element TwoSum digits (which scale with
    ldexp), and the digits reconstruct the row."""
    rng = np.random.default_rng(8)
    x = rng.standard_normal((200, 64)) * 10.0 ** rng.uniform(-43, -40, (200, 1))
    hi = x.astype(f32)
    lo = np.zeros_like(hi)
    amax = np.abs(hi).max(axis=1)
    assert np.all(amax < np.finfo(f32).tiny)
    _, E = np.frexp(amax.astype(np.float64))
    E = np.where(amax > 0, E, 0).astype(np.int64)[:, None]
    assert E.min() < -127
    d = _digits_fixed_grid(hi, lo, E)
    assert np.all(np.isfinite(d))
    np.testing.assert_array_equal(d, _digits_twosum(hi, lo, E))
    w = 2.0 ** (-8.0 * (np.arange(7) + 1))
    rec = np.einsum("s,srk->rk", w, d.astype(np.float64))
    np.testing.assert_array_equal(rec, np.ldexp(hi.astype(np.float64), -E))
