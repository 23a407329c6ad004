"""The integer arithmetic of the tensor-core Cholesky (librpa_gb300/csrc/ozaki_fixed.h),
compiled for the host and checked against exact rational arithmetic:

- slice_digits: the 8 signed 7-bit digits of each entry of a row rebuild the entry truncated to
  2^-56 of the row scale, and each digit fits BF16 exactly;
- combine_groups: W = round(U / 2^7) for U = sum_d T_d 2^{7(7-d)}, over the group sums the
  tensor core can produce (|T_d| below the exactness bound of FP32 accumulation);
- fixed_to_double: w 2^e0 rounded to the nearest double.
"""
import math
import random
import struct
import subprocess
from fractions import Fraction
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    exe = tmp_path_factory.mktemp("oz") / "ozaki_fixed_check"
    subprocess.run(["g++", "-O2", "-std=c++17", "-I", str(ROOT / "librpa_gb300" / "csrc"),
                    str(ROOT / "tests" / "ozaki_fixed_check.cpp"), "-o", str(exe)], check=True)

    def run(lines):
        out = subprocess.run([str(exe)], input="\n".join(lines) + "\n", capture_output=True, text=True, check=True)
        return out.stdout.split("\n")[:len(lines)]
    return run


def _bits(x):
    return struct.unpack("<Q", struct.pack("<d", x))[0]


def _double(b):
    return struct.unpack("<d", struct.pack("<Q", b))[0]


def test_slice_digits_rebuild_the_truncated_entry(checker):
    rng = random.Random(11)
    cases = []
    for _ in range(3000):
        row = [rng.uniform(-1, 1) * 10.0 ** rng.uniform(-6, 6) for _ in range(4)]
        if rng.random() < 0.1:
            row[rng.randrange(4)] = 0.0
        m = max(abs(v) for v in row)
        x = row[rng.randrange(4)]
        cases.append((x, m))
    cases += [(0.0, 0.0), (1.0, 1.0), (-1.0, 1.0), (0.5, 1.0), (2.0 ** -40, 3.0)]
    out = checker([f"S {_bits(x):x} {_bits(m):x}" for x, m in cases])
    for (x, m), line in zip(cases, out):
        f = [int(t) for t in line.split()]
        e, dig = f[0], f[1:]
        assert all(-127 <= d <= 127 for d in dig)
        if m == 0.0:
            assert dig == [0] * 8
            continue
        assert m < 2.0 ** e <= 2 * m  # the row scale is the smallest power of two above the maximum
        rebuilt = sum(Fraction(d) * Fraction(2) ** (-7 * (p + 1)) for p, d in enumerate(dig)) * Fraction(2) ** e
        exact = Fraction(x)
        # truncation toward zero at 2^(e - 56)
        step = Fraction(2) ** (e - 56)
        want = (abs(exact) // step) * step * (1 if x >= 0 else -1)
        assert rebuilt == want, (x, m, dig)


def test_combine_groups_rounds_the_exact_sum(checker):
    rng = random.Random(5)
    cases = []
    for _ in range(3000):
        # group d sums d + 1 slice products of 64 terms (|s_p s_q| <= 127^2); group 0's digits
        # come from |v| < 1 (|s_0| <= 127 as well)
        T = [rng.randint(-(d + 1) * 64 * 127 * 127, (d + 1) * 64 * 127 * 127) for d in range(8)]
        cases.append(T)
    lines = []
    for T in cases:
        u = [T[2 * g] * 128 + T[2 * g + 1] for g in range(4)]
        lines.append("C " + " ".join(str(x) for x in u))
    out = checker(lines)
    for T, line in zip(cases, out):
        U = sum(T[d] * 2 ** (7 * (7 - d)) for d in range(8))
        W = int(line)
        assert W == math.floor(Fraction(U, 128) + Fraction(1, 2)), T  # round half up


def test_fixed_to_double_is_correctly_rounded(checker):
    rng = random.Random(7)
    cases = [(rng.randint(-2 ** 62, 2 ** 62), rng.randint(-300, 60)) for _ in range(4000)]
    cases += [(rng.randint(-2 ** 30, 2 ** 30), rng.randint(-100, 10)) for _ in range(1000)]
    cases += [(1, 0), (-1, 0), (2 ** 53 + 1, 0), (-(2 ** 53 + 1), 0), (2 ** 62, -56), (2 ** 54 - 1, 0), (0, 5)]
    out = checker([f"F {w} {e0}" for w, e0 in cases])
    for (w, e0), line in zip(cases, out):
        got = _double(int(line, 16))
        exact = Fraction(w) * Fraction(2) ** e0
        if w == 0:
            assert got == 0.0
            continue
        # nearest double; a tie may go either way
        err = abs(Fraction(got) - exact)
        ulp = Fraction(2) ** (math.frexp(float(exact))[1] - 53)
        assert err <= ulp / 2, (w, e0, got)
