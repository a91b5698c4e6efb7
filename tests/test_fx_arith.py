"""The FX integer formulas, restated in Python big integers on the CPU: the
rounded high product FX::mh and the four-product complex twiddle product
FX::mul of fft_fast.cuh, and the per-tile rounded shift.

Python integers do not overflow, so each check also asserts the bound the
kernel relies on for its 64-bit intermediates (every partial sum below 2^63)
at the largest magnitudes the stages feed in (|x| < 2^61, twiddle parts at
most 2^62).
"""
import random

U32 = (1 << 32) - 1


def split(x):
    """x = hi * 2^32 + lo, lo the signed low word (the kernels' xh, xl)."""
    lo = x & U32
    lo_s = lo - (1 << 32) if lo >= 1 << 31 else lo
    return (x >> 32) + (lo >> 31), lo_s


def round_hi(s):
    """(s >> 32) + bit 31 of s: s / 2^32 rounded to nearest (ties up)."""
    return (s >> 32) + ((s & U32) >> 31)


def mh(x, w):
    xh, xl = split(x)
    wh, wl = split(w)
    s = xh * wl + xl * wh
    assert abs(s) < 1 << 63
    return xh * wh + round_hi(s)


def mul(x, y, c, s):
    """(x + i y)(c + i s) / 2^64 as FX::mul: c, s and -s split on their own."""
    xh, xl = split(x)
    yh, yl = split(y)
    ch, cl = split(c)
    sh, sl = split(s)
    nsh, nsl = split(-s)
    rm = xh * cl + xl * ch + yh * nsl + yl * nsh
    im = xh * sl + xl * sh + yh * cl + yl * ch
    assert abs(rm) < 1 << 63 and abs(im) < 1 << 63
    re_ = xh * ch + yh * nsh + round_hi(rm)
    im_ = xh * sh + yh * ch + round_hi(im)
    assert abs(re_) < 1 << 63 and abs(im_) < 1 << 63
    return re_, im_


def test_mh_is_the_rounded_high_product():
    rng = random.Random(3)
    worst = 0.0
    bias = 0
    for _ in range(20000):
        x = rng.randrange(-(1 << 61), 1 << 61) >> rng.randrange(0, 50)
        w = rng.randrange(1, (1 << 63) - (1 << 32))  # a constant whose high word fits an int32
        got = mh(x, w)
        exact = x * w  # / 2^64
        err = got * (1 << 64) - exact
        worst = max(worst, abs(err) / (1 << 64))
        bias += err
    assert worst <= 0.75
    assert abs(bias / 20000 / (1 << 64)) < 0.02  # no steady loss
    assert mh(0, 12345678912345) == 0


def test_twiddle_product_within_one_unit():
    rng = random.Random(5)
    worst = 0.0
    for _ in range(20000):
        # twiddle w / 4 = c + i s at 2^64 scale, |c|, |s| <= 2^62
        c = rng.randrange(-(1 << 62), 1 << 62)
        s = rng.randrange(-(1 << 62), 1 << 62)
        sh = rng.randrange(0, 40)
        x = rng.randrange(-(1 << 61), 1 << 61) >> sh
        y = rng.randrange(-(1 << 61), 1 << 61) >> sh
        re_, im_ = mul(x, y, c, s)
        er = re_ * (1 << 64) - (x * c - y * s)
        ei = im_ * (1 << 64) - (x * s + y * c)
        worst = max(worst, abs(er) / (1 << 64), abs(ei) / (1 << 64))
    assert worst <= 1.0
    assert mul(0, 0, 1 << 62, 12345) == (0, 0)


def test_rounded_shift_and_half_even():
    """The renormalisation's right shift rounds to nearest (ties up); the
    mixed-radix halving rounds half to even (no steady bias on ties)."""
    rng = random.Random(7)
    for _ in range(5000):
        x = rng.randrange(-(1 << 62), 1 << 62)
        s = rng.randrange(1, 32)
        got = (x + (1 << (s - 1))) >> s
        assert abs(got * (1 << s) - x) <= 1 << (s - 1)
    half = lambda x: (x + ((x >> 1) & 1)) >> 1  # noqa: E731
    assert [half(v) for v in (1, 3, 5, -1, -3, 4, -4)] == [0, 2, 2, 0, -2, 2, -2]
    assert sum(half(2 * k + 1) * 2 - (2 * k + 1) for k in range(-1000, 1000)) == 0
