"""Shared inputs of the parity tests (src/kernels tests and tests/isa_variants.rs shapes)."""

import numpy as np

import oracle

# tests/isa_variants.rs:17 (LENGTHS) plus its TILED_LEN, LONG_LEN and lengths that cross the
# GPU tiles (4096-row selection/scan tiles, 8192-row canonical tiles) and the end of the
# short paths (argsort to 2048 and to 8192 rows, the canonical sums to 4096).
LENGTHS = [0, 1, 3, 4, 7, 8, 15, 16, 17, 31, 32, 63, 64, 65, 300, 1000, 4500]
GPU_LENGTHS = [4095, 4096, 4097, 4111, 4112, 8191, 8192, 8193, 8192 * 3 + 17, 100_003]
# tests/isa_variants.rs:28-30
REDUCE_CUTS = [64, 384, 992]
TILE_CUTS = [37, 100]


def bits(x):
    return int(np.float64(x).view(np.uint64))


def same_f64(a, b):
    """Equal bits, except that a NaN only has to be NaN (tests/isa_variants.rs:300-309)."""
    if np.isnan(a):
        return bool(np.isnan(b))
    return bits(a) == bits(b)


def varied(n, seed=0):
    """Magnitudes 1e0..1e16 with both signs (src/kernels/tests.rs:664-673 shape)."""
    u = oracle.rand_f64(n, seed)
    return (u - 0.5) * 10.0 ** ((np.arange(n) % 9) * 2)


def with_specials(n, seed=0):
    """Finite values plus signed zeros, infinities and NaN (tests/isa_variants.rs:57-66)."""
    x = (oracle.rand_f64(n, seed) - 0.5) * 8.0
    sp = np.array([0.0, -0.0, np.inf, -np.inf, np.nan])
    pick = oracle.rand_i64(n, seed + 99) % 23
    for i, s in enumerate(sp):
        x = np.where(pick == i, s, x)
    return x


def uniform(n, seed=1):
    return oracle.rand_f64(n, seed)
