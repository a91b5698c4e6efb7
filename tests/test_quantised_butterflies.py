"""CPU model of the block-quantised float-float butterflies (no GPU).

The double API's default arithmetic (fft_fast.cuh bf8q, fft_mixed.cuh
fq_bf3 / fq_bf5 / the radix-2 and radix-4 branch of bfR) rounds the high
words of a butterfly's inputs to a grid q = ulp(c1), c1 = 1.5 * 2^(T-1),
T = e(m) - 126 + H (m the largest high word, e its biased exponent), and
relies on two facts: the rounding stays in c1's binade, so every rounded
value is a multiple of q, and every partial sum of the butterfly stays
below 2^T, so every addition of high words is exact in float32.  This test
emulates the butterflies operation by operation in float32 (numpy) with the
kernels' headroom H (radix 2, 3, 4: 2; radix 5: 3; radix 8: 4) and the
constant products re-gridded with c2 = 2 c1, and checks both facts on random
inputs and on adversarial ones (components at +-m, all of one sign, and the
near -m values that break a 1-bit grid): every float32 high-word addition
must equal its exact (float64) value.
"""
import numpy as np
import pytest

f32 = np.float32
HEAD = {2: 2, 3: 2, 4: 2, 5: 3, 8: 4}  # fq_head<R>() / bf8q
K = {"s3": 0.86602540378443864676372317075294, "c1": 0.30901699437494742410229341718282,
     "c2": -0.80901699437494742410229341718282, "s1": 0.95105651629515357211643933337938,
     "s2": 0.58778525229247312916870595463907, "c8": 0.70710678118654752440}


class Exact:
    """float32 high-word arithmetic that records whether each addition was exact."""

    def __init__(self):
        self.inexact = 0
        self.off_grid = 0

    def add(self, a, b):
        s = (a + b).astype(f32)
        self.inexact += int(np.count_nonzero(s.astype(np.float64) != a.astype(np.float64) + b.astype(np.float64)))
        return s

    def sub(self, a, b):
        return self.add(a, -b)


def grid_constants(h, H):
    """c1, c2 of the kernels from the largest |component| of the inputs."""
    m = np.max(np.abs(np.stack(h)), axis=0).astype(f32)
    eb = m.view(np.uint32) & np.uint32(0x7F800000)
    eb = np.minimum(eb, np.uint32((253 - H) << 23))
    c1 = (eb + np.uint32(H << 23) + np.uint32(0x400000)).view(f32)
    c2 = (eb + np.uint32((H + 1) << 23) + np.uint32(0x400000)).view(f32)
    return c1, c2


def on_grid(x, c):
    q = np.spacing(c).astype(np.float64)
    r = x.astype(np.float64) / q
    return np.count_nonzero(r != np.round(r))


def rnd(x, c, ex):
    """(x + c) - c in float32; counts results off the grid of c."""
    y = ((x + c).astype(f32) - c).astype(f32)
    ex.off_grid += on_grid(y, c)
    return y


def mulc(x, k, c, ex):
    """high word of k * x (the kernels' exact product of high words), back on the grid of c"""
    p = (x * f32(k)).astype(f32)
    return rnd(p, c, ex)


# complex high words as (re, im) pairs of float32 arrays
def cadd(a, b, ex):
    return (ex.add(a[0], b[0]), ex.add(a[1], b[1]))


def csub(a, b, ex):
    return (ex.sub(a[0], b[0]), ex.sub(a[1], b[1]))


def msi(a):  # * (-i): the forward direction
    return (a[1], -a[0])


def cmulc(a, k, c, ex):
    return (mulc(a[0], k, c, ex), mulc(a[1], k, c, ex))


def bf4(v, ex):
    t0, t1 = cadd(v[0], v[2], ex), csub(v[0], v[2], ex)
    t2, t3 = cadd(v[1], v[3], ex), msi(csub(v[1], v[3], ex))
    return [cadd(t0, t2, ex), cadd(t1, t3, ex), csub(t0, t2, ex), csub(t1, t3, ex)]


def butterfly(R, v, ex, H=None):
    """One quantised radix-R butterfly as the kernels compute its high words."""
    H = HEAD[R] if H is None else H
    c1, c2 = grid_constants([x for z in v for x in z], H)
    v = [(rnd(z[0], c1, ex), rnd(z[1], c1, ex)) for z in v]
    if R == 2:
        return [cadd(v[0], v[1], ex), csub(v[0], v[1], ex)]
    if R == 4:
        return bf4(v, ex)
    if R == 3:
        t, u, a0 = cadd(v[1], v[2], ex), csub(v[1], v[2], ex), v[0]
        m = csub(a0, cmulc(t, 0.5, c2, ex), ex)
        su = msi(cmulc(u, K["s3"], c2, ex))
        return [cadd(a0, t, ex), cadd(m, su, ex), csub(m, su, ex)]
    if R == 5:
        a0 = v[0]
        t1, t2 = cadd(v[1], v[4], ex), cadd(v[2], v[3], ex)
        u1, u2 = csub(v[1], v[4], ex), csub(v[2], v[3], ex)
        m1 = cadd(a0, cadd(cmulc(t1, K["c1"], c2, ex), cmulc(t2, K["c2"], c2, ex), ex), ex)
        m2 = cadd(a0, cadd(cmulc(t1, K["c2"], c2, ex), cmulc(t2, K["c1"], c2, ex), ex), ex)
        n1 = msi(cadd(cmulc(u1, K["s1"], c2, ex), cmulc(u2, K["s2"], c2, ex), ex))
        n2 = msi(csub(cmulc(u1, K["s2"], c2, ex), cmulc(u2, K["s1"], c2, ex), ex))
        return [cadd(a0, cadd(t1, t2, ex), ex), cadd(m1, n1, ex), cadd(m2, n2, ex), csub(m2, n2, ex),
                csub(m1, n1, ex)]
    assert R == 8
    e = bf4([v[0], v[2], v[4], v[6]], ex)
    o = bf4([v[1], v[3], v[5], v[7]], ex)
    o1 = cmulc(cadd(o[1], msi(o[1]), ex), K["c8"], c2, ex)
    o3 = cmulc(csub(msi(o[3]), o[3], ex), K["c8"], c2, ex)
    o2 = msi(o[2])
    oo = [o[0], o1, o2, o3]
    return [cadd(e[j], oo[j], ex) for j in range(4)] + [csub(e[j], oo[j], ex) for j in range(4)]


def inputs(R, kind, n, rng):
    """R complex inputs of n butterflies: random, or adversarial patterns."""
    if kind == "random":
        scale = np.exp2(rng.integers(-60, 60, n)).astype(np.float64)
        return [(f32(rng.uniform(-1, 1, n) * scale), f32(rng.uniform(-1, 1, n) * scale)) for _ in range(R)]
    m = f32(np.nextafter(f32(2.0 ** rng.integers(-30, 30)), f32(0)))  # just below a power of two
    if kind == "neg":
        return [(np.full(n, -m, f32), np.full(n, -m, f32)) for _ in range(R)]
    if kind == "pos":
        return [(np.full(n, m, f32), np.full(n, m, f32)) for _ in range(R)]
    sg = rng.choice([-1.0, 1.0], (R, 2, n)).astype(f32)
    return [(sg[r, 0] * m, sg[r, 1] * m) for r in range(R)]


@pytest.mark.parametrize("R", [2, 3, 4, 5, 8])
@pytest.mark.parametrize("kind", ["random", "neg", "pos", "signs"])
def test_high_word_additions_are_exact(R, kind):
    rng = np.random.default_rng(R * 10 + len(kind))
    ex = Exact()
    butterfly(R, inputs(R, kind, 4096, rng), ex)
    assert ex.off_grid == 0 and ex.inexact == 0, (ex.off_grid, ex.inexact)


@pytest.mark.parametrize("R", [2, 3, 4, 5, 8])
def test_one_bit_less_headroom_breaks_exactness(R):
    """The model detects grids the kernels must not use: with one bit less
    headroom than the kernels' (radix 2 with one bit rounds values near -m
    into the binade below c1; radix 8 with three lets the sqrt(1/2) sums
    overflow the grid) some rounding leaves the grid or some addition is no
    longer exact, so the kernels' headroom is the smallest that keeps every
    high-word addition exact."""
    bad = 0
    for kind in ("random", "neg", "pos", "signs"):
        ex = Exact()
        butterfly(R, inputs(R, kind, 4096, np.random.default_rng(3)), ex, H=HEAD[R] - 1)
        bad += ex.off_grid + ex.inexact
    assert bad > 0
