"""The 64-bit fixed-point constants of the FX butterflies, read from the kernel
sources, against high-precision values (CPU).

Each constant is stored as make_int2(hi, lo) with value hi * 2^32 + lo equal
to c * 2^64 rounded to the nearest integer, lo signed: the sqrt(1/2) rotation
of the radix-8 butterfly (as 1 - sqrt(1/2)), the radix-3 constant
(1 - sqrt(3)/2) and the radix-5 ones (cos 2pi/5, 1 + cos 4pi/5, 1 - sin 2pi/5,
1 - sin 4pi/5).  A wrong digit in any of them would bias every transform of
the lengths that use it.
"""
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "pfft_gb300", "csrc")


def _constants(path):
    """(hi, lo, comment) of every make_int2 constant with a trailing comment."""
    out = []
    pat = re.compile(r"make_int2\((-?\d+),\s*(-?\d+)\);\s*//\s*(.*)$")
    with open(path) as f:
        for line in f:
            m = pat.search(line)
            if m:
                out.append((int(m.group(1)), int(m.group(2)), m.group(3).strip()))
    return out


def _expected(sp):
    pi = sp.pi
    return {
        "(1 - sqrt(1/2)) 2^64": 1 - sp.sqrt(2) / 2,
        "(1 - sqrt(3)/2) 2^64": 1 - sp.sqrt(3) / 2,
        "cos(2 pi / 5) 2^64": sp.cos(2 * pi / 5),
        "(1 + cos(4 pi / 5)) 2^64": 1 + sp.cos(4 * pi / 5),
        "(1 - sin(2 pi / 5)) 2^64": 1 - sp.sin(2 * pi / 5),
        "(1 - sin(4 pi / 5)) 2^64": 1 - sp.sin(4 * pi / 5),
    }


def test_fx_constants_are_the_rounded_fractions():
    sp = pytest.importorskip("sympy")
    found = _constants(os.path.join(CSRC, "fft_fast.cuh")) + _constants(os.path.join(CSRC, "fft_mixed.cuh"))
    expected = _expected(sp)
    seen = set()
    for hi, lo, name in found:
        if name not in expected:
            continue
        seen.add(name)
        assert -2 ** 31 <= lo < 2 ** 31 and 0 <= hi < 2 ** 31, name
        stored = hi * 2 ** 32 + lo
        exact = sp.Integer(2) ** 64 * expected[name]
        want = int(sp.floor(sp.N(exact, 60) + sp.Rational(1, 2)))
        assert stored == want, (name, stored, want)
        assert stored < 2 ** 63, name  # an int64 operand
    assert seen == set(expected), sorted(set(expected) - seen)
