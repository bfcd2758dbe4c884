"""The modular scheme's last step, ozd::i128_scaled (csrc/ozaki_digits.cuh):
a two's-complement 128-bit integer times 2^x0 rounded to the nearest double
(ties to even) with integer operations, ok = false outside the normal range.
The function is compiled as host code (nvcc, no GPU) and checked against
Python's correctly rounded int/int division on random magnitudes of every
length, exact ties with and without bits below them (in the low word and in
the high word), carries into the next power of two, +-2^127 and the range
ends."""
from __future__ import annotations

import math
import os
import random
import shutil
import struct
import subprocess
from fractions import Fraction

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "..", "openblas_gb300", "csrc")

DRIVER = r"""
#include <cstdio>
#include <cstring>
#include "ozaki_digits.cuh"
int main() {
  unsigned long long hi, lo;
  int x0;
  while (scanf("%llu %llu %d", &hi, &lo, &x0) == 3) {
    bool ok;
    const double v = gb::ozd::i128_scaled(hi, lo, x0, ok);
    unsigned long long b;
    memcpy(&b, &v, sizeof b);
    printf("%d %llu\n", ok ? 1 : 0, b);
  }
  return 0;
}
"""


def _nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    return None


def _expected(v, x0):
    if v == 0:
        return True, 0.0
    num, den = (v << x0, 1) if x0 >= 0 else (v, 1 << -x0)
    try:
        d = num / den  # correctly rounded (ties to even)
    except OverflowError:
        return False, None
    if math.isinf(d) or abs(d) < 2.0 ** -1022:
        return False, None
    return True, d


def _cases():
    rng = random.Random(20261204)
    out = [(0, 0), (1, 0), (-1, 0), (-(1 << 127), 0), ((1 << 127) - 1, 0), ((1 << 127) - 1, -60),
           (1, 1023), (1, 1024), (1, -1022), (1, -1023), (3, -1024), ((1 << 53) - 1, 971),
           ((1 << 53) - 1, 972), ((1 << 54) - 1, 970)]
    for _ in range(3000):
        bits = rng.randint(1, 127)
        v = rng.getrandbits(bits) | (1 << (bits - 1))
        if rng.random() < 0.5:
            v = -v
        out.append((v, rng.randint(-300, 300)))
    # exact ties below a 53-bit significand, with and without sticky bits, at
    # shifts that put the rounding bit in the low word, across the words and in
    # the high word; odd and even significands; all-ones significands that
    # carry into the next power of two
    for s in (1, 5, 11, 31, 40, 63, 64, 65, 70, 74):
        for mant in ((1 << 52) | 12345, (1 << 52) | 12346, (1 << 53) - 1, 1 << 52):
            tie = (mant << s) | (1 << (s - 1))
            for extra in (0, 1, -1):
                for sign in (1, -1):
                    v = sign * (tie + extra)
                    if -(1 << 127) <= v < (1 << 127):
                        out.append((v, rng.randint(-100, 100)))
    return out


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    nvcc = _nvcc()
    if nvcc is None:
        pytest.skip("nvcc not available")
    d = tmp_path_factory.mktemp("i128")
    src = d / "drv.cu"
    src.write_text(DRIVER)
    exe = d / "drv"
    r = subprocess.run([nvcc, "-O2", "-std=c++17", "-I", CSRC, str(src), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return str(exe)


def test_i128_scaled_rounds_like_exact_division(driver):
    cases = _cases()
    lines = []
    for v, x0 in cases:
        u = v & ((1 << 128) - 1)
        lines.append(f"{u >> 64} {u & ((1 << 64) - 1)} {x0}")
    r = subprocess.run([driver], input="\n".join(lines) + "\n", capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    got = r.stdout.split("\n")
    bad = []
    for (v, x0), line in zip(cases, got):
        ok_s, bits_s = line.split()
        ok = ok_s == "1"
        val = struct.unpack("<d", struct.pack("<Q", int(bits_s)))[0]
        eok, ev = _expected(v, x0)
        if ok != eok or (ok and (val != ev or math.copysign(1, val) != math.copysign(1, ev))):
            bad.append((v, x0, ok, val, eok, ev))
    assert not bad, f"{len(bad)} of {len(cases)} differ, first {bad[:3]}"
    assert len(got) - 1 == len(cases)
