"""The kernels' small-integer division (small_div in csrc/rtg_internal.h):
q = trunc((a + 1/2) * rb) with rb = 1/b rounded to the nearest float equals
a // b for 0 <= a < 2^22.  Checked here with IEEE float32 arithmetic (numpy
rounds every product to nearest, as the device does) over the ranges the
kernels use: a < 2^16 for every divisor up to 512, and sampled a up to 2^22
for divisors up to 2^10."""
import numpy as np


def _small_div(a, b):
    rb = (np.float32(1.0) / b.astype(np.float32)).astype(np.float32)
    t = (a.astype(np.float32) + np.float32(0.5)).astype(np.float32)
    return np.trunc((t * rb).astype(np.float32)).astype(np.int64)


def test_exact_for_kernel_ranges():
    a = np.arange(1 << 16, dtype=np.int64)
    for b in range(1, 513):
        bb = np.full_like(a, b)
        assert np.array_equal(_small_div(a, bb), a // b), b


def test_exact_up_to_2_pow_22():
    rng = np.random.default_rng(0)
    a = rng.integers(0, 1 << 22, size=2_000_000, dtype=np.int64)
    b = rng.integers(1, 1 << 10, size=a.size, dtype=np.int64)
    assert np.array_equal(_small_div(a, b), a // b)
    # the values right below and at multiples of b, where truncation is tightest
    for bv in (3, 7, 9, 13, 16, 81, 127, 1023):
        m = np.arange(1, ((1 << 22) - 1) // bv, dtype=np.int64) * bv
        for off in (-1, 0):
            aa = m + off
            assert np.array_equal(_small_div(aa, np.full_like(aa, bv)), aa // bv), (bv, off)
