"""The reference suite's own acceptance checks, run through the drop-in C API.

tests/c/roundtrip_checks.c is a plain C program built against include/pfft.h
and the library; each case plans a forward and a backward transform, fills the
input with the golden generator, runs both, normalises and reports the maximum
absolute error, as the reference's check programs do.  The reference accepts a
case below 1e-12 (tests/run_checks.sh:75); so does this test with the default
double arithmetic (64-bit fixed point on the radix-8 passes, FP64 elsewhere)
and with native FP64 everywhere, on the reference's sizes and on the large_*
cases (up to 512 x 256 x 128 and 256^3 r2c) added to the program.

The opt-in float-float arithmetics do not meet that absolute bound and are
held to their own: the golden data reaches magnitude 1500, and a float-float
value keeps 48-49 significant bits, so the representation alone is good to
1500 * 2^-49 = 2.7e-12 - above the reference's bound, which assumes 53-bit
doubles.  TwoSum float-float (df) stays below 2e-11; the block-quantised form
(dfq), whose low words carry remainders of a butterfly grid, below 2e-10.
"""
import os
import re
import subprocess

import pytest

import pfft_gb300 as pg

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "c", "roundtrip_checks.c")
CASES = re.findall(r'^\s*\{"(\w+)",', open(SRC).read(), flags=re.M)
TOL = {"auto": 1e-12, "native": 1e-12, "df": 2e-11, "dfq": 2e-10}


@pytest.fixture(scope="module")
def exe(cuda, pfft_lib, tmp_path_factory):
    path = str(tmp_path_factory.mktemp("rt") / "roundtrip_checks")
    libdir = os.path.dirname(pg.LIBPATH)
    subprocess.run(["gcc", "-O1", "-I", os.path.join(ROOT, "include"), SRC, "-L", libdir, "-lpfft_gb300",
                    "-Wl,-rpath," + libdir, "-o", path], check=True)
    return path


_CACHE = {}


def results(exe, mode):
    if mode in _CACHE:
        return _CACHE[mode]
    env = dict(os.environ, PFFT_GB300_F64_ARITH=mode)
    out = subprocess.run([exe], capture_output=True, text=True, timeout=900, env=env)
    res = {}
    for ln in out.stdout.splitlines():
        m = re.match(r"(\w+) maxerror = ([^;]+);", ln)
        if m:
            res[m.group(1)] = float(m.group(2))
        elif ln.strip():
            res[ln.split()[0]] = ln
    _CACHE[mode] = (res, out)
    return res, out


def test_all_cases_listed():
    assert len(CASES) >= 30


@pytest.mark.parametrize("mode", ["auto", "native", "df", "dfq"])
@pytest.mark.parametrize("name", CASES)
def test_roundtrip_maxerror(exe, name, mode):
    res, out = results(exe, mode)
    assert name in res, out.stdout[-2000:] + out.stderr[-2000:]
    assert isinstance(res[name], float), res[name]
    assert res[name] < TOL[mode], (name, mode, res[name])
