"""The bit-sliced Game of Life pass (gol_bits_kernel in csrc/k_gol.cu),
checked on the CPU where it is plain integer arithmetic:
  - the byte <-> bit packing: (w * P) >> 28 gathers bytes 0..3 of w (each 0
    or 1) into bits 0..3, and (nibble * U) & 0x01010101 spreads them back,
    for all 16 patterns, with P and U read from the device source;
  - the per-row logic (column sums as two bit planes, neighbour columns by
    funnel shifts across words, T = u0 + 2k, next = (u0 & k == 1) |
    (~u0 & alive & k == 2)), restated on numpy words of a torus, gives the
    oracle's generations.
The GPU tests compare the kernel itself with the oracle."""
import os
import re

import numpy as np

import oracle
from libgeodecomp_gb300 import workloads

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "libgeodecomp_gb300", "csrc", "k_gol.cu")


def constants():
    text = open(SRC).read()
    pack = int(re.search(r"\(w\[i\] \* (0x[0-9a-fA-F]+)u\) >> 28", text).group(1), 16)
    unpack = int(re.search(r"\* (0x[0-9a-fA-F]+)u\) & 0x01010101u", text).group(1), 16)
    return pack, unpack


def test_pack_and_unpack_all_nibbles():
    pack, unpack = constants()
    for nib in range(16):
        w = sum(((nib >> j) & 1) << (8 * j) for j in range(4))        # bytes 0/1
        assert ((w * pack) & 0xFFFFFFFF) >> 28 == nib
        assert (nib * unpack) & 0x01010101 == w


def bits_generation(words):
    """One generation on a torus of 32-bit words (rows x words per row)."""
    w = words.astype(np.uint64)
    a = np.roll(w, 1, axis=0)                     # row above
    c = np.roll(w, -1, axis=0)                    # row below
    m = w
    s0 = a ^ m ^ c
    s1 = (a & m) | (a & c) | (m & c)
    mask = np.uint64(0xFFFFFFFF)

    def left(p):                                  # column x - 1: funnel shift with the word to the left
        return ((p << np.uint64(1)) | (np.roll(p, 1, axis=1) >> np.uint64(31))) & mask

    def right(p):                                 # column x + 1
        return ((p >> np.uint64(1)) | (np.roll(p, -1, axis=1) << np.uint64(31))) & mask

    x0, x1, z0, z1 = left(s0), left(s1), right(s0), right(s1)
    u0 = x0 ^ s0 ^ z0
    c0 = (x0 & s0) | (x0 & z0) | (s0 & z0)
    a1, a2 = x1 ^ s1, x1 & s1
    b1, b2 = z1 ^ c0, z1 & c0
    k1 = (a1 ^ b1) & ~(a2 | b2) & mask
    k2 = ((a2 & ~(b1 | b2)) | (b2 & ~(a1 | a2)) | (a1 & b1)) & mask
    return ((u0 & k1) | (~u0 & m & k2)) & mask


def to_words(cells):
    ny, nx = cells.shape
    bits = cells.reshape(ny, nx // 32, 32).astype(np.uint64)
    return (bits << np.arange(32, dtype=np.uint64)).sum(axis=2)


def from_words(words):
    ny, nw = words.shape
    return ((words[:, :, None] >> np.arange(32, dtype=np.uint64)) & np.uint64(1)).astype(np.uint8).reshape(ny, nw * 32)


def test_bit_logic_matches_the_oracle():
    for ny, nx, seed in ((48, 64, 5), (33, 96, 6), (7, 32, 7)):
        c0 = workloads.gol_initial(nx, ny, seed=seed)
        w = to_words(c0)
        for gen in range(1, 9):
            w = bits_generation(w)
            np.testing.assert_array_equal(from_words(w), oracle.gol(c0, gen))
