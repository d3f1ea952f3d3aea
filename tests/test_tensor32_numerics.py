"""The complex64 tensor-core pass's arithmetic (tensor32.cu), emulated on the
CPU: every FP32 operand value is split into three BF16 values (h = bf16(x),
m = bf16(x - h), l = bf16(x - h - m), round to nearest even), and the six
slice products that reach 2^-16 of the leading one are summed.  Checks that
the slices are BF16 values, that the remainders are exact in FP32, that the
split reproduces x to 2^-24 of |x|, and that the six products reproduce the
exact product of the FP32 operands to within the FP32 accumulation level."""
import numpy as np


def bf16_rn(x):
    """x (float32 array) rounded to the nearest BF16 value, ties to even, as float32."""
    u = np.asarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32)


def split3(x):
    x = np.asarray(x, dtype=np.float32)
    h = bf16_rn(x)
    r = (x - h).astype(np.float32)
    m = bf16_rn(r)
    s = (r - m).astype(np.float32)
    l = bf16_rn(s)
    return h, m, l, r, s


def random_f32(rng, n):
    # magnitudes over a wide exponent range, both signs
    return (rng.standard_normal(n) * 2.0 ** rng.integers(-40, 20, n)).astype(np.float32)


def test_split_slices_are_bf16_and_remainders_exact():
    rng = np.random.default_rng(1)
    x = random_f32(rng, 200000)
    h, m, l, r, s = split3(x)
    for v in (h, m, l):
        assert np.all((v.view(np.uint32) & 0xFFFF) == 0)  # BF16: the low 16 bits are zero
    # the FP32 remainders equal the exact (float64) differences
    assert np.array_equal(r.astype(np.float64), x.astype(np.float64) - h.astype(np.float64))
    assert np.array_equal(s.astype(np.float64), r.astype(np.float64) - m.astype(np.float64))
    # the split reproduces x to 2^-24 of |x|
    rec = h.astype(np.float64) + m.astype(np.float64) + l.astype(np.float64)
    err = np.abs(rec - x.astype(np.float64))
    assert np.all(err <= np.abs(x.astype(np.float64)) * 2.0 ** -24)


def test_six_products_reach_fp32_accuracy():
    """A row of W (R = 32 reals) times a column x: the six kept slice pairs
    (l,h) (m,m) (h,l) (m,h) (h,m) (h,h) against the exact product of the FP32
    operands, relative to |W|_1 max|x|: below 2^-23 (the three dropped pairs
    are below 2^-24 of the leading one, the split errors below 2^-24)."""
    rng = np.random.default_rng(2)
    R = 32
    worst = 0.0
    for _ in range(2000):
        w = (rng.standard_normal(R) * 2.0 ** rng.integers(-3, 1)).astype(np.float32)
        x = random_f32(rng, R)
        wh, wm, wl, _, _ = split3(w)
        xh, xm, xl, _, _ = split3(x)
        W = [wh.astype(np.float64), wm.astype(np.float64), wl.astype(np.float64)]
        X = [xh.astype(np.float64), xm.astype(np.float64), xl.astype(np.float64)]
        kept = [(2, 0), (1, 1), (0, 2), (1, 0), (0, 1), (0, 0)]  # (x slice, W slice)
        approx = sum(float(np.dot(X[i], W[j])) for i, j in kept)
        exact = float(np.dot(x.astype(np.float64), w.astype(np.float64)))
        scale = float(np.abs(w.astype(np.float64)).sum() * np.abs(x.astype(np.float64)).max())
        worst = max(worst, abs(approx - exact) / scale)
    assert worst <= 2.0 ** -23, worst


def test_host_and_device_roundings_agree_on_ties():
    """Ties round to even, as __floats2bfloat162_rn and the host's bf16_round do."""
    # 1 + 2^-8 is halfway between BF16 neighbours 1 and 1 + 2^-7: rounds to 1 (even)
    # 1 + 3 * 2^-8 is halfway between 1 + 2^-7 and 1 + 2^-6: rounds to 1 + 2^-6 (even)
    x = np.array([1 + 2.0 ** -8, 1 + 3 * 2.0 ** -8, -(1 + 2.0 ** -8)], dtype=np.float32)
    assert list(bf16_rn(x)) == [1.0, 1 + 2.0 ** -6, -1.0]
