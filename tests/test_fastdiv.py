"""The multiply-high division used to decode cell coordinates on the GPU
(FastDiv in ofblend_gb300/csrc/flof_common.cuh), emulated with Python
integers: exact for every 32-bit dividend of the divisors the grids use."""
import numpy as np


def magic(d):
    l = 0
    while (1 << l) < d:
        l += 1
    m = ((1 << 32) * ((1 << l) - d)) // d + 1
    return m & 0xFFFFFFFF, l


def fastdiv(n, d):
    m, l = magic(d)
    hi = (n * m) >> 32
    return (hi + n) >> l


def test_fastdiv_exact():
    rng = np.random.default_rng(7)
    divisors = list(range(1, 300)) + [510, 511, 512, 1000, 4094, 16384, 65535, 65536, 123457]
    samples = [0, 1, 2, 3, 2**31 - 1, 2**31, 2**32 - 1, 2**32 - 2] + \
        [int(v) for v in rng.integers(0, 2**32, size=400)]
    for d in divisors:
        for n in samples + [d - 1, d, d + 1, 2 * d - 1, 2 * d]:
            n &= 0xFFFFFFFF
            assert fastdiv(n, d) == n // d, (n, d)
