"""The rounding multiplications of the fixed-point Jacobi cell, checked in
exact integer arithmetic on the CPU with the constants and shifts read from
the device source (csrc/k_common.cuh).

The cell multiplies its exact neighbour sum by fl(1/7), the double the
reference's cell multiplies by.  fx_mul7_round(sum) must equal the exact
product rounded to nearest (ties away from zero) for every sum of seven
values |k| < 2^57; fx_mul49_round(sum) (the two-step pass: an exact sum of
exact sums times fl(1/7)^2) must equal round(sum * M49 / 2^69) and differ
from the exact product by less than 0.006 units before rounding.  The
device forms are one 64 x 64-bit multiply-high, an add and a shift on |sum|,
with the sign put back afterwards."""
import os
import random
import re
import struct
from fractions import Fraction

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "libgeodecomp_gb300", "csrc", "k_common.cuh")
MASK64 = (1 << 64) - 1


def source():
    return open(SRC).read()


def define(name):
    m = re.search(r"#define %s (0x[0-9a-fA-F]+|\d+)(ull)?" % name, source())
    return int(m.group(1), 0)


def device_form(name):
    """(multiplier, added, shift) of a magnitude helper, parsed from its body."""
    body = re.search(r"long long %s\(long long sum\)\s*\{(.*?)\n\}" % name, source(), re.S).group(1)
    const, add, shift = re.search(
        r"__umul64hi\(\(unsigned long long\)sum, (LGD_FIX_M\d+)\) \+ (\d+)ull\) >> (\d+)", body).groups()
    return define(const), int(add), int(shift)


def emulate(form, s):
    """The signed helper: sign-magnitude around the magnitude helper."""
    mul, add, shift = form
    a = abs(s)
    q = (((a * mul) >> 64) + add) >> shift
    assert q <= MASK64
    return -q if s < 0 else q


def round_half_away(fr: Fraction) -> int:
    a = abs(fr)
    q = int(a + Fraction(1, 2))     # floor(|x| + 1/2)
    return -q if fr < 0 else q


def fl_one_seventh() -> Fraction:
    return Fraction(1.0 / 7.0)


def samples(limit, count, seed):
    rng = random.Random(seed)
    pts = {0, 1, -1, 2, -2, 3, 4, 7, 49, limit, -limit, limit - 1, -(limit - 1)}
    for _ in range(count):
        pts.add(rng.randint(-limit, limit))
    for _ in range(200):            # small sums, where every rounding shows
        pts.add(rng.randint(-1000, 1000))
    return sorted(pts)


def test_c7_is_the_double_nearest_one_seventh():
    c7 = define("LGD_FIX_C7")
    assert Fraction(c7, 1 << 54) == fl_one_seventh()
    assert struct.pack("<d", float(Fraction(c7, 1 << 54))) == struct.pack("<Q", 0x3FC2492492492492)
    bits = define("LGD_FIX_BITS")
    assert bits == 57


def test_m7_is_exact_and_fits():
    c7 = define("LGD_FIX_C7")
    mul, add, shift = device_form("fx_mul7_round_nonneg")
    assert mul == c7 << 11 and mul < (1 << 63)
    assert add == 1 and shift == 1      # (P + 2^64) >> 65


def test_m49_is_the_rounded_square():
    c7 = define("LGD_FIX_C7")
    mul, add, shift = device_form("fx_mul49_round_nonneg")
    assert add == 16 and shift == 5     # (P + 2^68) >> 69
    exact = Fraction(c7 * c7, 1 << 39)  # fl(1/7)^2 * 2^69
    assert abs(Fraction(mul) - exact) <= Fraction(1, 2)
    assert mul < (1 << 64)


def test_single_step_rounding_is_exact():
    form = device_form("fx_mul7_round_nonneg")
    c = fl_one_seventh()
    limit = 7 << define("LGD_FIX_BITS")
    assert limit < (1 << 63)
    for s in samples(limit, 20000, seed=7):
        assert emulate(form, s) == round_half_away(s * c), s


def test_two_step_rounding_matches_its_constant_and_the_exact_square():
    form = device_form("fx_mul49_round_nonneg")
    mul = form[0]
    c2 = fl_one_seventh() ** 2
    limit = (49 << define("LGD_FIX_BITS")) - 1
    assert limit < (1 << 63)
    bound = Fraction(limit, 1 << 70)        # |M49 / 2^69 - fl(1/7)^2| <= 2^-70
    assert bound < Fraction(6, 1000)
    near_ties = 0
    pts = samples(limit, 20000, seed=49)
    for s in pts:
        got = emulate(form, s)
        assert got == round_half_away(Fraction(s * mul, 1 << 69)), s
        exact = s * c2
        # the constant's error moves the product by less than 0.006 units
        assert abs(Fraction(s * mul, 1 << 69) - exact) <= bound
        frac = abs(exact) - int(abs(exact))
        if abs(frac - Fraction(1, 2)) <= bound:
            near_ties += 1
            assert abs(got - round_half_away(exact)) <= 1
        else:
            assert got == round_half_away(exact), s
    # only products within the constant's error of a half unit may round
    # differently from the exact square: about 2 * bound of all samples
    assert near_ties <= 3 * float(bound) * len(pts)


def test_sign_symmetry():
    bits = define("LGD_FIX_BITS")
    for name, limit in (("fx_mul7_round_nonneg", 7 << bits), ("fx_mul49_round_nonneg", (49 << bits) - 1)):
        form = device_form(name)
        for s in samples(limit, 2000, seed=3):
            assert emulate(form, -s) == -emulate(form, s)


@pytest.mark.parametrize("name", ["fx_mul7_round", "fx_mul49_round"])
def test_signed_helpers_wrap_the_magnitude_helpers(name):
    body = re.search(r"long long %s\(long long sum\)\s*\{(.*?)\n\}" % name, source(), re.S).group(1)
    assert "const long long s = sum >> 63;" in body
    assert "%s_nonneg((sum ^ s) - s)" % name in body
    assert "return (q ^ s) - s;" in body
