"""CPU model of the split form's df64 lambda recursion (legendre_split.cu k_lambda_digits and
its synthesis / spin-2 forms): the same FP32 operation sequence as dd::dot2 (products exact
through a wider format, as fmaf is), the per-step rescaling of the state into 2^-32 .. 2^32,
and the FP32 digit sequence of tc::digits4_df.  It checks the two facts the kernels
rely on: the state never leaves FP32's normal range, and the recursion stays within a small
part of the 2^-31 digit quantum of the FP64 recursion over thousands of steps."""
import math

import numpy as np
import pytest

f32 = np.float32


def _two_sum(a, b):
    s = f32(a + b)
    v = f32(s - a)
    return s, f32(f32(a - f32(s - v)) + f32(b - v))


def _fmaf(a, b, c):
    return f32(float(a) * float(b) + float(c))


def _dot2(x1h, x1l, y1h, y1l, x2h, x2l, y2h, y2l):
    p1 = f32(x1h * y1h)
    e1 = _fmaf(x1h, y1h, -p1)
    p2 = f32(x2h * y2h)
    e2 = _fmaf(x2h, y2h, -p2)
    s, e = _two_sum(p1, p2)
    t = f32(e1 + e2)
    for a, b in ((x1h, y1l), (x1l, y1h), (x2h, y2l), (x2l, y2h)):
        t = _fmaf(a, b, t)
    h = f32(s + f32(e + t))
    return h, f32(f32(e + t) - f32(h - s))


def _pair(v):
    h = f32(v)
    return h, f32(v - float(h))


def _coeffs(l, m):
    a = math.sqrt((2 * l - 1) * (2 * l + 1) / (l * l - m * m))
    b = math.sqrt(((l - 1) ** 2 - m * m) / ((2 * l - 3) * (2 * l - 1))) * a
    return a, b


def _digits_df(hi, lo, E):
    """tc::digits4_df: the FP32 operation sequence (exponent moves are exact)."""
    wh, wl = f32(math.ldexp(float(hi), 6 - E)), f32(math.ldexp(float(lo), 6 - E))
    assert abs(wh) <= 64.5
    d0 = f32(np.rint(wh))
    r = f32(f32(wh - d0) + wl)
    t = f32(r * f32(256))
    d1 = f32(np.rint(t))
    t = f32(f32(t - d1) * f32(256))
    d2 = f32(np.rint(t))
    t = f32(f32(t - d2) * f32(256))
    d3 = f32(np.rint(t))
    return [float(d) for d in (d0, d1, d2, d3)], float(wh) + float(wl)


@pytest.mark.parametrize("m,x,lmax", [(2000, 0.0, 2047), (1000, 0.99, 2047), (3000, 1e-4, 4095),
                                      (0, 0.01, 2047), (10, 0.5, 2047)])
def test_df64_recursion_tracks_fp64(m, x, lmax):
    s1d, s2d, ed = 0.75, 0.0, 0
    s1h, s1l = _pair(0.75)
    s2h = s2l = f32(0)
    et = 0
    xh, xl = _pair(x)
    a_prev = None
    worst = 0.0
    for l in range(m + 1, lmax + 1):
        a, b = _coeffs(l, m)
        beta = 0.0 if l == m + 1 else b / (a * a_prev)
        a_prev = a
        s1d, s2d = x * s1d - beta * s2d, s1d
        am = max(abs(s1d), abs(s2d))
        if am > 2.0 ** 300:
            s1d, s2d, ed = s1d * 2.0 ** -600, s2d * 2.0 ** -600, ed + 600
        elif 0 < am < 2.0 ** -300:
            s1d, s2d, ed = s1d * 2.0 ** 600, s2d * 2.0 ** 600, ed - 600
        bh, bl = _pair(-beta)
        nh, nl = _dot2(xh, xl, s1h, s1l, bh, bl, s2h, s2l)
        s2h, s2l, s1h, s1l = s1h, s1l, nh, nl
        amf = max(abs(s1h), abs(s2h))
        if amf > f32(2.0 ** 32):
            s1h, s1l, s2h, s2l = (f32(v * f32(2.0 ** -64)) for v in (s1h, s1l, s2h, s2l))
            et += 64
        elif 0 < amf < f32(2.0 ** -32):
            s1h, s1l, s2h, s2l = (f32(v * f32(2.0 ** 64)) for v in (s1h, s1l, s2h, s2l))
            et -= 64
        hi = max(abs(s1h), abs(s2h))
        assert hi == 0 or 2.0 ** -46 <= hi <= 2.0 ** 33     # normal, with room for lo
        ref = math.ldexp(s1d, ed)
        got = math.ldexp(float(s1h) + float(s1l), et)
        scale = math.ldexp(max(abs(s1d), abs(s2d)), ed)
        if scale > 0:
            worst = max(worst, abs(got - ref) / scale)
    assert worst < 2.0 ** -31 / 2, worst


def test_fp32_digits_reconstruct_the_value():
    """digits4_df's digits are integers within the bounds the exact UMMA levels need, and
    d0 + d1 2^-8 + d2 2^-16 + d3 2^-24 is within 1.5 2^-25 of (hi + lo) 2^(6 - E)."""
    rng = np.random.default_rng(1)
    for _ in range(20000):
        E = int(rng.integers(-90, 90))
        v = rng.uniform(-1, 1) * 2.0 ** (E - int(rng.integers(0, 40)))
        hi, lo = _pair(v)
        d, w = _digits_df(hi, lo, E)
        assert all(x == int(x) for x in d)
        assert abs(d[0]) <= 64 and all(abs(x) <= 128 for x in d[1:])
        rec = d[0] + d[1] * 2.0 ** -8 + d[2] * 2.0 ** -16 + d[3] * 2.0 ** -24
        assert abs(rec - w) <= 1.5 * 2.0 ** -25


def _digits_f(v, E):
    """tc::digits4_f: the FP32 pair cut from the FP64 bits, then the FP32 digit sequence."""
    b = int(np.float64(v).view(np.uint64))
    hw, lw = b >> 32, b & 0xFFFFFFFF
    eb = (hw >> 20) & 0x7FF
    ew = eb - 1023 + 6 - E
    if eb == 0 or ew < -40:
        return [0.0] * 4, 0.0
    sign = hw & 0x80000000
    wh = np.uint32(sign | ((ew + 127) << 23) | ((hw & 0xFFFFF) << 3) | (lw >> 29)).view(np.float32)
    r = lw & 0x1FFFFFFF
    wl = f32(0)
    if r:
        pbit = r.bit_length() - 1
        mr = r >> (pbit - 23) if pbit >= 23 else r << (23 - pbit)
        wl = np.uint32(sign | ((ew - 52 + pbit + 127) << 23) | (mr & 0x7FFFFF)).view(np.float32)
    assert abs(wh) <= 64.5
    rint = lambda x: f32(f32(x + f32(12582912.0)) - f32(12582912.0))
    d0 = rint(wh)
    t = f32(f32(f32(wh - d0) + wl) * f32(256))
    d1 = rint(t)
    t = f32(f32(t - d1) * f32(256))
    d2 = rint(t)
    t = f32(f32(t - d2) * f32(256))
    d3 = rint(t)
    return [float(d) for d in (d0, d1, d2, d3)], v * 2.0 ** (6 - E)


def test_fp64_digits_on_the_fp32_pipe():
    """digits4_f reconstructs v 2^(6 - E) to 1.5 2^-25 with digits inside the exact bounds."""
    rng = np.random.default_rng(2)
    for _ in range(20000):
        E = int(rng.integers(-900, 900))
        v = rng.uniform(-1, 1) * 2.0 ** (E - int(rng.integers(0, 45)))
        d, w = _digits_f(v, E)
        assert abs(d[0]) <= 64 and all(abs(x) <= 128 for x in d[1:])
        rec = d[0] + d[1] * 2.0 ** -8 + d[2] * 2.0 ** -16 + d[3] * 2.0 ** -24
        assert abs(rec - w) <= 1.5 * 2.0 ** -25, (v, E, d, w)
