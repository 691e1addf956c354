"""The multiply-high division by frame-invariant integers (udiv_magic / udiv
in voxeltoy_gb300/csrc/vt_internal.h): floor(n * M / 2^64) with
M = ceil(2^64 / d) equals floor(n / d) for every n < 2^32, checked here in
exact integer arithmetic over divisors and numerators that stress it."""
import numpy as np


def magic(d: int) -> int:
    return 0 if d <= 1 else ((1 << 64) - 1) // d + 1


def udiv(n: int, m: int) -> int:
    return n if m == 0 else (n * m) >> 64


def test_invariant_division_is_exact():
    rng = np.random.default_rng(7)
    divisors = [1, 2, 3, 5, 7, 255, 256, 257, 1000, 1023, 1024, 1025, 65535, 65536, 65537, 1 << 20,
                (1 << 20) + 1, 1048576 * 3, 2147483647, 2147483648, 4294967295]
    divisors += [int(x) for x in rng.integers(2, 1 << 32, 200, dtype=np.uint64)]
    for d in divisors:
        m = magic(d)
        assert m < (1 << 64)
        ns = [0, 1, d - 1, d, d + 1, 2 * d - 1, (1 << 32) - 1, (1 << 31) - 1, (1 << 32) - 1 - ((1 << 32) - 1) % d - 1]
        ns += [int(x) for x in rng.integers(0, 1 << 32, 500, dtype=np.uint64)]
        # the largest multiples of d below 2^32 and their neighbours, where rounding up of M bites first
        top = ((1 << 32) - 1) // d * d
        ns += [top, top - 1, max(top - d, 0), max(top - d - 1, 0)]
        for n in ns:
            if 0 <= n < (1 << 32):
                assert udiv(n, m) == n // d, (n, d)
