"""The integer row step of the float scans (add_bits in verkehrt_gb300/csrc/k_canon.cu), restated
in Python integers and checked against IEEE-754 double addition (numpy) on the cases the GPU
data rarely reaches: states at the edge of the rule's range (exponent field 64 and 2046), zero
and subnormal rows, rows one binade below the state, sums that land exactly on or past 2^53
units, and exact halfway rows of both parities. The rule: for a positive normal state
s = S * 2^(E-52) with exponent field KE = E + 1023 in [64, 2046] and a non-negative row x whose
exponent field is below KE, fl(s + x) = (S + RNE(x / 2^(E-52))) * 2^(E-52) with ties to the
even S, as long as the sum stays below 2^53 units; every other case takes the FP64 add."""

import numpy as np

MANT = (1 << 52) - 1
ONE52 = 1 << 52


def bits(v):
    return int(np.float64(v).view(np.uint64))


def f64(b):
    return float(np.uint64(b).view(np.float64))


def add_bits(s, x):
    """The device rule on bit patterns; None where it hands over to the FP64 add."""
    KE, ex = s >> 52, x >> 52  # the sign bit makes a negative state or row exceed 2047
    if not (64 <= KE <= 2046 and ex < KE):
        return None
    k = min(KE - ex, 63)
    w = ((x & MANT) | ONE52) + (1 << (k - 1))
    inc = w >> k
    S = (s & MANT) | ONE52
    if (w << (64 - k)) & ((1 << 64) - 1) == 0:  # exactly halfway
        inc -= 1
        inc += (S + inc) & 1
    S2 = S + inc
    if S2 >= 2 * ONE52:
        return None
    return (KE << 52) | (S2 & MANT)


def check(s_val, x_val):
    s, x = bits(s_val), bits(x_val)
    got = add_bits(s, x)
    if got is not None:
        want = bits(np.float64(s_val) + np.float64(x_val))
        assert got == want, (s_val, x_val, hex(got), hex(want))
    return got is not None


def test_edges():
    taken = 0
    tiny = 2.0 ** -959  # exponent field 64, the lowest the rule takes
    for s_val in (tiny, tiny * 1.75, 1.0, 1.5, 2.0 ** 53, 2.0 ** 53 + 2, 2.0 ** 1023, 1.999 * 2.0 ** 1023):
        ulp = np.spacing(np.float64(s_val))
        for x_val in (0.0, 5e-324, 2.0 ** -1022 * 0.75, ulp / 2, ulp * 1.5, ulp * 2.5, ulp / 4, ulp / 2 * 3,
                      s_val / 2, s_val / 2 * 0.999, np.nextafter(s_val / 2, 0)):
            taken += check(s_val, float(x_val))
    # a sum that lands exactly on 2^53 units and one just below
    s_val = 2.0 - 2.0 ** -52
    assert add_bits(bits(s_val), bits(2.0 ** -52)) is None
    assert check(s_val - 2.0 ** -52, 2.0 ** -52)
    # negative states and rows, infinities and NaN hand over
    for s_val, x_val in ((-1.0, 0.5), (1.0, -0.25), (1.0, float("inf")), (1.0, float("nan")), (2.0 ** -1000, 1e-310)):
        assert add_bits(bits(s_val), bits(x_val)) is None
    assert taken > 40


def test_random_pairs_and_ties():
    rng = np.random.default_rng(5)
    taken = 0
    for _ in range(20000):
        e = int(rng.integers(-950, 1000))
        s_val = float(np.ldexp(1.0 + rng.random(), e))
        d = int(rng.integers(1, 70))
        x_val = float(np.ldexp(1.0 + rng.random(), e - d))
        taken += check(s_val, x_val)
        # a halfway row: an odd multiple of half the state's ulp
        ulp = float(np.spacing(np.float64(s_val)))
        m = 2 * int(rng.integers(0, 1 << 20)) + 1
        if m * ulp / 2 < s_val:
            taken += check(s_val, m * ulp / 2)
    assert taken > 30000
