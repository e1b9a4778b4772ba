"""FastDiv (csrc/nsw6_common.cuh): the multiply-and-shift quotient of a
32-bit unsigned n by a divisor fixed for a launch, restated in Python integer
arithmetic, against n // d on edge and random cases.  The multiplier rests on
Granlund and Montgomery's bound 2^(32+s) < M d <= 2^(32+s) + 2^s, checked
here for every divisor tested."""
from __future__ import annotations

import numpy as np


def make(d: int) -> tuple[int, int]:
    s = 0
    while (1 << s) < d:
        s += 1
    m = ((1 << 32) * ((1 << s) - d)) // d + 1
    assert 0 <= m < (1 << 32)
    big_m = m + (1 << 32)
    assert (1 << (32 + s)) < big_m * d <= (1 << (32 + s)) + (1 << s)
    return m, s


def div(n: int, m: int, s: int) -> int:
    return (((n * m) >> 32) + n) >> s


def test_fastdiv_matches_integer_division():
    rng = np.random.default_rng(11)
    divisors = [1, 2, 3, 5, 7, 40, 42, 160, 641, 16900, 2 ** 31 - 1, 2 ** 31, 2 ** 31 + 1, 2 ** 32 - 1]
    divisors += [int(x) for x in rng.integers(1, 2 ** 32, 40)] + [int(x) for x in rng.integers(1, 70000, 40)]
    for d in divisors:
        m, s = make(d)
        ns = [0, 1, d - 1, d, d + 1, 2 ** 32 - 1, 2 ** 32 - 2, (2 ** 32 - 1) // d * d, (2 ** 32 - 1) // d * d - 1]
        ns += [int(x) for x in rng.integers(0, 2 ** 32, 2000)]
        for n in ns:
            if 0 <= n < 2 ** 32:
                assert div(n, m, s) == n // d, (n, d)


def test_fastdiv_exhaustive_small_divisors():
    # every n of a 2^20 window at the top of the range and at the bottom
    for d in (3, 7, 42, 16900):
        m, s = make(d)
        for base in (0, 2 ** 32 - 2 ** 20):
            n = np.arange(base, base + 2 ** 20, dtype=np.uint64)
            q = (((n * np.uint64(m)) >> np.uint64(32)) + n) >> np.uint64(s)
            assert np.array_equal(q, n // np.uint64(d))
