"""The arithmetic of the FP64-width tensor-core pass (tensor64.cu), emulated
bit for bit on the CPU with Python integers: FP64 bits aligned to a column
grid, 7 balanced base-256 digits, exact order sums (checked below 2^22, the
bound the kernel's integer extraction needs), 64-bit combination of the
orders, the bra columns' magnitude keys and alignment, and the final rounding
to FP64 (one correctly rounded conversion).  Checked against exact rational arithmetic on random unitaries and
density-matrix blocks with columns of very different sizes (bounds in the
test's docstring)."""
import struct
from fractions import Fraction

import numpy as np
import pytest

SLICES, ORDERS = 7, 8
BIAS = 0x0080808080808080
MASK64 = (1 << 64) - 1


def f64_bits(x):
    return struct.unpack("<Q", struct.pack("<d", x))[0]


def bits_f64(b):
    return struct.unpack("<d", struct.pack("<Q", b & MASK64))[0]


def f32(x):
    return struct.unpack("<f", struct.pack("<f", x))[0]


def f32_bits(x):
    return struct.unpack("<I", struct.pack("<f", x))[0]


def digits(t):
    """plan.cpp tc64_digits / tensor64.cu digits_of: balanced base-256 digits."""
    u = (t + BIAS) & MASK64
    d = [((u >> (8 * (6 - j))) & 0xFF) - 128 for j in range(1, 7)]
    top = (u >> 48) - 128
    out = [top] + d
    assert sum(v * 256 ** (6 - j) for j, v in enumerate(out)) == t
    assert all(abs(v) <= 128 for v in out)
    return out


def host_row(w):
    """build_tc64_k: w = t 2^ew, |t| <= 2^55, as digits."""
    mx = max(abs(v) for v in w)
    if mx == 0:
        return 0, [[0] * SLICES for _ in w]
    e = int(np.frexp(mx)[1])
    ts = [int(np.rint(np.ldexp(v, 55 - e))) for v in w]
    assert all(abs(t) <= 2 ** 55 for t in ts)
    return e - 55, [digits(t) for t in ts]


def column_digits_fp64(xs):
    """tensor64.cu digits_fp64 on one column: returns (Ec, digit lists)."""
    bits = [f64_bits(x) for x in xs]
    ecm = max(max((b >> 32) & 0x7FF00000 for b in bits), 64 << 20)
    out = []
    for b in bits:
        hi, lo = b >> 32, b & 0xFFFFFFFF
        d = (ecm - (hi & 0x7FF00000)) >> 20
        mant = (((hi & 0xFFFFF) | 0x100000) << 32) | lo
        v = (mant << 2) >> d if d < 64 else 0
        assert v < 2 ** 55
        sg = -1 if hi >> 31 else 1
        out.append([sg * dd for dd in digits(v)])
    return ecm >> 20, out


def order_sums(row_digits, col_digits):
    s = [0] * ORDERS
    for i in range(SLICES):
        for j in range(SLICES):
            if i + j < ORDERS:
                s[i + j] += sum(c[i] * r[j] for c, r in zip(col_digits, row_digits))
    assert all(abs(v) < 2 ** 22 for v in s), s  # the integer extraction's range
    return s


def combine(s):
    """combine_orders: int64 Y (orders 6, 7 through one floor shift)."""
    p01 = s[0] * 256 + s[1]
    p23 = s[2] * 256 + s[3]
    p45 = s[4] * 256 + s[5]
    p67 = (s[6] * 256 + s[7]) >> 16
    assert all(abs(p) < 2 ** 31 for p in (p01, p23, p45))
    y = (p01 << 32) + (p23 << 16) + (p45 + p67)
    assert abs(y) < 2 ** 63
    return y


def key(s, ec):
    mag = f32(f32(abs(s[1]) * 0.00390625 + abs(s[0])) + 65.0)  # one FMA rounding, then the add
    return ec + (f32_bits(mag) >> 23)


def to_fp64(y, p):
    """tensor64.cu to_fp64: the correctly rounded double of y, times 2^p."""
    if y == 0:
        return 0.0
    d = float(y)  # round to nearest even, as cvt.rn.f64.s64
    e = ((f64_bits(d) >> 52) & 0x7FF) + p
    if e <= 0:
        return 0.0
    return bits_f64(f64_bits(d) + (p << 52))


def real_embedding(m):
    return np.block([[m.real, -m.imag], [m.imag, m.real]])


def emulate_pass(u, v, x):
    """One D x D group: y = V-side applied to (U x) columns, as the kernel's two
    steps: rho'[a][b] = sum_{c,d} U[a][c] V[b][d] x[c][d]."""
    d = u.shape[0]
    wu, wv = real_embedding(u), real_embedding(v)
    rows_u = [host_row(wu[n]) for n in range(2 * d)]
    rows_v = [host_row(wv[n]) for n in range(2 * d)]
    assert all(rows_u[a][0] == rows_u[a + d][0] for a in range(d))
    # ket step: column b holds x[.][b] as [re; im]
    Y = np.zeros((2 * d, d), dtype=object)  # [re/im output a][column b]
    Ec = []
    for b in range(d):
        col = list(x[:, b].real) + list(x[:, b].imag)
        ec, cd = column_digits_fp64(col)
        Ec.append(ec)
        for n in range(2 * d):
            Y[n, b] = combine(order_sums(rows_u[n][1], cd))
    # the bra columns' magnitude keys, then the bra step on column a
    out = np.zeros((d, d), dtype=complex)
    for a in range(d):
        mkey = 0
        for b in range(d):
            for n in (a, a + d):
                col = list(x[:, b].real) + list(x[:, b].imag)
                _, cd = column_digits_fp64(col)
                mkey = max(mkey, key(order_sums(rows_u[n][1], cd), Ec[b]))
        vals = []
        for n in (a, a + d):  # real parts then imaginary parts of row a
            for b in range(d):
                sh = mkey - 141 - Ec[b]
                y = Y[n, b] >> sh if sh >= 0 else Y[n, b] << (-sh)
                assert abs(y) < 2 ** 55 * (1 + 2 ** -23)
                vals.append(y)
        cd = [digits(vv) for vv in vals]
        ew_a = rows_u[a][0]
        for n in range(2 * d):
            yy = combine(order_sums(rows_v[n][1], cd))
            bidx = n % d
            p = mkey + ew_a + rows_v[bidx][0] - 1106
            val = to_fp64(yy, p)
            if n < d:
                out[a, bidx] += val
            else:
                out[a, bidx] += 1j * val
    return out


def exact_pass(u, v, x):
    d = u.shape[0]
    F = Fraction
    U = [[(F(u[i, j].real), F(u[i, j].imag)) for j in range(d)] for i in range(d)]
    V = [[(F(v[i, j].real), F(v[i, j].imag)) for j in range(d)] for i in range(d)]
    X = [[(F(x[i, j].real), F(x[i, j].imag)) for j in range(d)] for i in range(d)]

    def mul(p, q):
        return (p[0] * q[0] - p[1] * q[1], p[0] * q[1] + p[1] * q[0])

    T = [[(F(0), F(0)) for _ in range(d)] for _ in range(d)]
    for a in range(d):
        for b in range(d):
            re = im = F(0)
            for c in range(d):
                pr = mul(U[a][c], X[c][b])
                re += pr[0]
                im += pr[1]
            T[a][b] = (re, im)
    out = np.zeros((d, d), dtype=complex)
    for a in range(d):
        for b in range(d):
            re = im = F(0)
            for c in range(d):
                pr = mul(V[b][c], T[a][c])
                re += pr[0]
                im += pr[1]
            out[a, b] = float(re) + 1j * float(im)
    return out


@pytest.mark.parametrize("d,trial", [(8, 0), (8, 1), (16, 2), (16, 3), (16, 4), (16, 5)])
def test_fp64_width_pass_matches_exact_arithmetic(d, trial):
    """Every value is held with 55 significant bits relative to its column's
    largest (block floating point per column of 2^K entries), so the error of
    an output is bounded by its operator row's 1-norm times its column's
    largest value, per step (2^-54 of that, asserted).  The largest absolute
    error stays at or below FP64 arithmetic's on the same inputs, and with
    dense rows within 3 bits of FP64's componentwise bound."""
    rng = np.random.default_rng(100 + trial)
    u, _ = np.linalg.qr(rng.normal(size=(d, d)) + 1j * rng.normal(size=(d, d)))
    sparse = trial in (1, 3)
    if sparse:
        u[np.abs(u) < 0.15] = 0  # sparse rows
    v = u.conj()  # the superoperator's bra factor
    x = rng.normal(size=(d, d)) + 1j * rng.normal(size=(d, d))
    x *= 10.0 ** rng.uniform(-12, 0, size=(1, d))  # columns of very different sizes
    if trial == 4:
        x[:, 3] = 0.0  # an all-zero column
        x[5, :] *= 1e-30
    if trial == 5:
        x = x.conj().T @ x  # Hermitian positive: a density-matrix block
        x /= np.trace(x).real
    got = emulate_pass(u, v, x)
    ref = exact_pass(u, v, x)
    # per step: |U_a|_1 times the ket column's largest |x|, then |V_b|_1 times
    # the bra column's largest of those
    ket_scale = np.abs(u).sum(axis=1)[:, None] * np.abs(x).max(axis=0)[None, :]  # [a, c]
    nw = np.abs(v).sum(axis=1)[None, :] * ket_scale.max(axis=1)[:, None]  # [a, b]
    err = np.abs(got - ref)
    f64 = np.abs(u @ x @ v.T - ref)  # numpy's FP64 evaluation of the same product
    assert (err / np.maximum(nw, 1e-300)).max() <= 2.0 ** -54
    # in absolute terms no worse than FP64 arithmetic
    assert err.max() <= 2 * f64.max() + 1e-300, (float(err.max()), float(f64.max()))
    if not sparse:
        # dense rows: within 3 bits of FP64's componentwise bound, whose
        # scale is sum_c |V_bc| sum_k |U_ak| |x_kc|, even with columns 12
        # orders of magnitude apart
        scale = np.abs(u) @ np.abs(x) @ np.abs(v).T
        assert (err / np.maximum(scale, 1e-300)).max() <= 2.0 ** -50
