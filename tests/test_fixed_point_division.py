"""The rounding divisions of the fixed-point Jacobi cell, checked in exact
integer arithmetic on the CPU with the constants read from the device
source (csrc/k_common.cuh): fx_div7_round(sum) must equal round(sum / 7)
for every sum of seven values |k| <= 2^56, and fx_div49_round(sum) must
equal round(sum / 49) for every |sum| < 49 * 2^56 (the two-step pass's sum
of sums).  Neither division has ties (7 and 49 are odd).  The device forms
are an unsigned offset, one 64 x 64-bit multiply-high and a shift."""
import os
import random
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "libgeodecomp_gb300", "csrc", "k_common.cuh")
MASK64 = (1 << 64) - 1


def device_form(name):
    """(add, offset multiple, multiplier, shift, fraction bits) of a division
    helper, parsed from its source."""
    text = open(SRC).read()
    bits = int(re.search(r"#define LGD_FIX_BITS (\d+)", text).group(1))
    body = re.search(r"long long %s\(long long sum\)\s*\{(.*?)\n\}" % name, text, re.S).group(1)
    off = int(re.search(r"const unsigned long long off = (\d+)ull << LGD_FIX_BITS;", body).group(1))
    add = int(re.search(r"\(unsigned long long\)\(sum \+ (\d+)\) \+ off", body).group(1))
    mul, shift = re.search(r"__umul64hi\(n, (0x[0-9a-fA-F]+)ull\) >> (\d+)", body).groups()
    return add, off, int(mul, 16), int(shift), bits


def emulate(form, s):
    add, off, mul, shift, bits = form
    n = (s + add + (off << bits)) & MASK64
    q = ((n * mul) >> 64) >> shift
    r = (q - (1 << bits)) & MASK64
    return r - (1 << 64) if r >> 63 else r


def samples(limit, div, count, seed):
    rng = random.Random(seed)
    pts = {0, 1, -1, limit, -limit, limit - 1, -(limit - 1)}
    for _ in range(count):
        pts.add(rng.randint(-limit, limit))
    # every residue around a few multiples, where rounding changes
    for base in (0, limit // div, -(limit // div), rng.randint(-limit // div, limit // div)):
        for r in range(-2 * div, 2 * div + 1):
            v = base * div + r
            if -limit <= v <= limit:
                pts.add(v)
    return sorted(pts)


@pytest.mark.parametrize("name,div,limit", [("fx_div7_round", 7, 7 << 56), ("fx_div49_round", 49, (49 << 56) - 1)])
def test_rounding_division_is_exact(name, div, limit):
    form = device_form(name)
    assert form[1] == div and form[0] == div // 2
    for s in samples(limit, div, 20000, seed=div):
        want = (s + div // 2) // div            # round(s / div): odd div, no ties
        assert emulate(form, s) == want, (name, s)


def test_division_constants_are_the_ceilings_stated():
    """M = ceil(2^(64 + shift) / div) for both helpers, and 49 M - 2^69 = 34."""
    for name, div in (("fx_div7_round", 7), ("fx_div49_round", 49)):
        _, _, mul, shift, _ = device_form(name)
        k = 64 + shift
        assert mul == -(-(1 << k) // div)
    _, _, m49, s49, _ = device_form("fx_div49_round")
    assert 49 * m49 - (1 << (64 + s49)) == 34
