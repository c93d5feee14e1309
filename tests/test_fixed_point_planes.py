"""The deposit's shared tile keeps each 64-bit fixed-point cell as two 32-bit planes
(tile_add in particlesimulation_gb300/csrc/deposit_body.cuh): a 64-bit add is a 32-bit add of
the low word, whose carry out goes with the high word's add.  This restates that arithmetic in
numpy and checks that, for signed contributions of any size the deposit produces (TSC weights
can be negative), in any order, the two planes hold exactly the 64-bit sum modulo 2^64, which
is what the device's bit-exact density tests then see."""
import numpy as np

M32 = (1 << 32) - 1


def plane_add(lo, hi, v):
    u = v & ((1 << 64) - 1)  # two's complement of the signed contribution
    l, h = u & M32, u >> 32
    old = lo
    lo = (lo + l) & M32
    carry = 1 if lo < old else 0  # the low-word add wrapped (old + l >= 2^32)
    hc = (h + carry) & M32
    if hc:
        hi = (hi + hc) & M32
    return lo, hi


def planes_sum(values):
    lo = hi = 0
    for v in values:
        lo, hi = plane_add(lo, hi, int(v))
    return (hi << 32) | lo


def test_planes_equal_64bit_sum_in_any_order():
    rng = np.random.default_rng(7)
    for trial in range(40):
        n = int(rng.integers(1, 600))
        scale = int(rng.integers(1, 62))
        mag = rng.integers(0, 1 << scale, n, dtype=np.int64)
        sign = np.where(rng.random(n) < 0.15, -1, 1)
        vals = [int(m) * int(s) for m, s in zip(mag, sign)]
        want = sum(vals) & ((1 << 64) - 1)
        assert planes_sum(vals) == want
        perm = rng.permutation(n)
        assert planes_sum([vals[i] for i in perm]) == want


def test_planes_carry_edge_cases():
    # low words that wrap on every add, exact multiples of 2^32, -1 and the extremes
    cases = [
        [M32, 1, M32, 1],
        [1 << 32, 1 << 32, -(1 << 32)],
        [-1, -1, 2],
        [(1 << 62) - 1, (1 << 62) - 1, -(1 << 62)],
        [-(1 << 62), 1, -1, (1 << 62)],
    ]
    for vals in cases:
        assert planes_sum(vals) == sum(vals) & ((1 << 64) - 1)
