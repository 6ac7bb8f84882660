"""The invariant-divisor division used by the kernels' index loops (q = umulhi(n, mul) >> shr,
mul = ceil(2^(31+l) / d), l = ceil(log2 d)) is exact for every dividend below 2^31."""
import numpy as np
import pytest


def make(d):
    if d <= 1:
        return 0, 0
    l = (d - 1).bit_length()
    p = 31 + l
    return -(-(1 << p) // d), p - 32


def fdiv(n, mul, shr):
    n = np.asarray(n, np.uint64)
    return n if mul == 0 else ((n * np.uint64(mul)) >> np.uint64(32)) >> np.uint64(shr)


@pytest.mark.parametrize("d", [1, 2, 3, 8, 16, 24, 32, 48, 96, 129, 256, 257, 384, 1024, 1025, 4096, 65536, 99991])
def test_fastdiv_exact(d):
    mul, shr = make(d)
    assert mul < 2 ** 32
    rng = np.random.default_rng(d)
    n = np.concatenate([np.arange(0, 200000, dtype=np.uint64),
                        rng.integers(0, 2 ** 31, 200000, dtype=np.uint64),
                        np.array([2 ** 31 - 1, 2 ** 31 - 2], np.uint64)])
    assert np.array_equal(fdiv(n, mul, shr), n // np.uint64(d))
