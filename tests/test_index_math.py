"""The multiply-high divider of the kernels' index math (FastDiv in
mepinterp_gb300/csrc/mepi_internal.cuh): q = (e * m) >> 32 with
m = floor((2^32 - 1) / d) + 1 equals e // d whenever e * d < 2^32.  Checked
exhaustively for the divisors the kernels use (N and N^2, N <= 64) over the
element indices they divide (e < 6 N^2), and on a sample of larger products."""
import numpy as np


def _fastdiv(e, d):
    m = (0xFFFFFFFF // d) + 1
    return (e.astype(np.uint64) * np.uint64(m)) >> np.uint64(32)


def test_divisors_of_band_counts():
    for n in range(1, 65):
        for d in (n, n * n):
            e = np.arange(6 * n * n + 64, dtype=np.uint64)
            assert np.array_equal(_fastdiv(e, d), e // np.uint64(d)), d


def test_bound_e_times_d_below_2_32():
    rng = np.random.default_rng(0)
    for d in rng.integers(1, 1 << 16, size=200):
        e = rng.integers(0, (1 << 32) // int(d), size=2000, dtype=np.uint64)
        assert np.array_equal(_fastdiv(e, int(d)), e // np.uint64(d)), d
