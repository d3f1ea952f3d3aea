"""The arithmetic of the tensor-core passes, emulated in numpy float32 (CPU):
BF16 slices at true scale, exact FP32 sums per slice-pair order, double-float
recombination.  Checks the two facts the kernel relies on -- every slice has
at most 8 significant bits and every order sum is exact in FP32 -- and the
error bound (2^-46 of |W row|_2 |x|_2) on random unitaries and columns."""
import numpy as np

f32 = np.float32
S = 6


def host_slices(wrow):
    """Row slices as plan.cpp: build_tc_k computes them (|t| <= 128 units of 2^(e-7-8j))."""
    mx = np.abs(wrow).max()
    t = np.zeros((S, wrow.size))
    if mx == 0:
        return t
    _, e = np.frexp(mx)
    v = wrow.copy()
    for j in range(S):
        u = 2.0 ** (e - 7 - 8 * j)
        t[j] = np.rint(v / u) * u
        assert np.abs(t[j] / u).max() <= 128
        v = v - t[j]
    return t


def magic(eb, i):
    return np.array([((eb + 17 - 8 * i) << 23) | 0x400000], dtype=np.int32).view(f32)[0]


def device_slices(hi, lo):
    """Column slices as tensor.cu: slice_df computes them."""
    mx = f32(np.abs(hi).max())
    eb = max(int((mx.view(np.int32) >> 23) & 0xFF), 40)
    s = np.zeros((S, hi.size), dtype=f32)
    v = hi.copy()
    for i in range(3):
        c = magic(eb, i)
        s[i] = ((v + c).astype(f32) - c).astype(f32)
        v = (v - s[i]).astype(f32)
    v = (v + lo).astype(f32)
    for i in range(3, S):
        c = magic(eb, i)
        s[i] = ((v + c).astype(f32) - c).astype(f32)
        v = (v - s[i]).astype(f32)
    for i in range(S):
        q = s[i].astype(np.float64) / 2.0 ** (eb - 133 - 8 * i)
        assert np.all(q == np.rint(q)) and np.abs(q).max() <= 256
    return s


def two_sum(a, b):
    s = f32(a + b)
    v = f32(s - a)
    return s, f32(f32(a - f32(s - v)) + f32(b - v))


def recombine(d):
    lo = f32(f32(d[6] + d[5]) + d[4])
    h1, l1 = two_sum(d[0], d[1])
    h2, l2 = two_sum(h1, d[2])
    h3, l3 = two_sum(h2, d[3])
    t = f32(f32(f32(l1 + l2) + l3) + lo)
    s = f32(h3 + t)
    return np.float64(s) + np.float64(f32(t - f32(s - h3)))


def test_slices_exact_sums_and_error_bound():
    rng = np.random.default_rng(9)
    worst = 0.0
    for trial in range(120):
        d = 16 if trial % 2 else 8
        r = 2 * d
        q, _ = np.linalg.qr(rng.normal(size=(d, d)) + 1j * rng.normal(size=(d, d)))
        if trial % 3 == 0:
            q[np.abs(q) < 0.2] = 0  # sparse rows
        w = np.block([[q.real, -q.imag], [q.imag, q.real]])
        x = (rng.normal(size=d) + 1j * rng.normal(size=d)) * 10.0 ** rng.uniform(-8, 2)
        if trial % 5 == 0:
            x[rng.integers(0, d, 3)] *= 1e-9
        xv = np.concatenate([x.real, x.imag])
        hi = xv.astype(f32)
        lo = (xv - hi.astype(np.float64)).astype(f32)
        xd = hi.astype(np.float64) + lo.astype(np.float64)
        s = device_slices(hi, lo)
        exact = w @ xd
        for n in range(r):
            t = host_slices(w[n])
            sums = np.zeros(S + 1)
            for o in range(S + 1):
                for i in range(max(0, o - S + 1), min(o, S - 1) + 1):
                    sums[o] += np.dot(s[i].astype(np.float64), t[o - i])
            assert np.all(sums.astype(f32).astype(np.float64) == sums)  # the tensor cores add exactly
            y = recombine(sums.astype(f32))
            worst = max(worst, abs(y - exact[n]) / (np.linalg.norm(w[n]) * np.linalg.norm(xd)))
    assert worst < 2.0 ** -46, worst
