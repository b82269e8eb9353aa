"""The double-float arithmetic of the packed analytic-signal stage
(fastpcc_gb300/csrc/dfloat.cuh), emulated in float32 with numpy: Knuth's
two-sum, Dekker's fast two-sum and addition, the exact product error (here by
Veltkamp splitting instead of an FMA).  A radix-2 transform built from them
stays within a few 1e-15 of the norm of an FP64 transform, with Dekker's
addition as with the longer form that also two-sums the low parts, and the
analytic signal inside a run of zeros keeps ~1e-12 relative precision, where
FP32 rounding (of the samples alone, here) already moves it by more than 1e-7
relative."""
import numpy as np
import pytest

f32 = np.float32


def two_sum(a, b):
    s = (a + b).astype(f32)
    bb = (s - a).astype(f32)
    return s, ((a - (s - bb).astype(f32)).astype(f32) + (b - bb).astype(f32)).astype(f32)


def fast_two_sum(a, b):
    s = (a + b).astype(f32)
    return s, (b - (s - a).astype(f32)).astype(f32)


def split(a):
    c = (f32(4097) * a).astype(f32)
    hi = (c - (c - a).astype(f32)).astype(f32)
    return hi, (a - hi).astype(f32)


def two_prod(a, b):
    p = (a * b).astype(f32)
    ah, al = split(a)
    bh, bl = split(b)
    e = ((((ah * bh).astype(f32) - p).astype(f32) + (ah * bl).astype(f32)).astype(f32) + (al * bh).astype(f32))
    return p, (e.astype(f32) + (al * bl).astype(f32)).astype(f32)


def add_long(a, b):
    s, e1 = two_sum(a[0], b[0])
    t, e2 = two_sum(a[1], b[1])
    u = fast_two_sum(s, (e1 + t).astype(f32))
    return fast_two_sum(u[0], (u[1] + e2).astype(f32))


def add_dekker(a, b):   # the form the kernels use
    s, e = two_sum(a[0], b[0])
    return fast_two_sum(s, ((e + a[1]).astype(f32) + b[1]).astype(f32))


def mul(a, b):
    p, e = two_prod(a[0], b[0])
    e = ((e + (a[0] * b[1]).astype(f32)).astype(f32) + (a[1] * b[0]).astype(f32)).astype(f32)
    return fast_two_sum(p, e)


def neg(a):
    return (-a[0], -a[1])


def to_df(x):
    h = x.astype(f32)
    return (h, (x - h.astype(np.float64)).astype(f32))


def value(a):
    return a[0].astype(np.float64) + a[1].astype(np.float64)


def fft_df(xr, xi, add):
    n = xr[0].size
    lev = int(np.log2(n))
    idx = np.arange(n)
    rev = np.zeros(n, int)
    for b in range(lev):
        rev |= ((idx >> b) & 1) << (lev - 1 - b)
    re = [xr[0][rev].copy(), xr[1][rev].copy()]
    im = [xi[0][rev].copy(), xi[1][rev].copy()]
    size = 2
    while size <= n:
        h = size // 2
        ang = -2 * np.pi * np.arange(h) / size
        wr, wi = to_df(np.cos(ang)), to_df(np.sin(ang))
        for st in range(0, n, size):
            a, b = slice(st, st + h), slice(st + h, st + size)
            br, bi = (re[0][b], re[1][b]), (im[0][b], im[1][b])
            tr = add(mul(br, wr), neg(mul(bi, wi)))
            ti = add(mul(br, wi), mul(bi, wr))
            ar, ai = (re[0][a].copy(), re[1][a].copy()), (im[0][a].copy(), im[1][a].copy())
            nr, ni, mr, mi = add(ar, tr), add(ai, ti), add(ar, neg(tr)), add(ai, neg(ti))
            re[0][a], re[1][a] = nr
            im[0][a], im[1][a] = ni
            re[0][b], re[1][b] = mr
            im[0][b], im[1][b] = mi
        size *= 2
    return value(re) + 1j * value(im)


@pytest.mark.parametrize("add", [add_long, add_dekker], ids=["long", "dekker"])
def test_double_float_transform_precision(add):
    rng = np.random.default_rng(1)
    n = 2048
    x = rng.standard_normal(n)
    x[500:700] = 0.0
    X64 = np.fft.fft(x)
    X = fft_df(to_df(x), to_df(np.zeros(n)), add)
    assert np.linalg.norm(X - X64) / np.linalg.norm(X64) < 3e-14
    # analytic signal inside the run of zeros (mask product in FP64, inverse by conjugation)
    h = np.zeros(n)
    h[0], h[1:n // 2], h[n // 2] = 1.0, 2.0, 1.0
    a64 = np.fft.ifft(X64 * h)
    Y = X * h
    y = np.conj(fft_df(to_df(Y.real), to_df(-Y.imag), add)) / n
    g = slice(550, 650)
    assert np.max(np.abs(y[g] - a64[g]) / np.abs(a64[g])) < 1e-10
    # FP32 samples alone (the transform itself in FP64) move it far more
    y32 = np.fft.ifft((np.fft.fft(x.astype(f32)).astype(np.complex64) * h.astype(f32))).astype(np.complex64)
    assert np.max(np.abs(y32[g] - a64[g]) / np.abs(a64[g])) > 1e-7
