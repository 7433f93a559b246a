"""The force accumulators' FP32 -> 64-bit fixed-point conversion
(komd_gb300/csrc/atm_device.cuh, fix32_rn): round(x * 2^32) as int64 built
from two 32-bit conversions.  This restates the kernel's FP32 steps in numpy
float32 (the same IEEE operations) and checks them bit for bit against the
direct rounding of x * 2^32 over random bit patterns and the edge cases: values
next to integers, the ulp boundary at 2^-9, ties to even, and the signs."""
import numpy as np

TWO32 = np.float32(4294967296.0)


def split_conversion(x):
    x = np.asarray(x, np.float32)
    a = np.abs(x)
    fl = np.floor(a)                                       # floorf
    hi = fl.astype(np.int64)                               # __float2int_rz of an integral value
    lo = np.rint((a - fl) * TWO32).astype(np.int64)        # __float2uint_rn of the exact low part
    m = (hi << 32) | lo
    return np.where(x < 0, -m, m)


def direct(x):
    return np.rint(np.asarray(x, np.float32).astype(np.float64) * 2.0 ** 32).astype(np.int64)


def test_split_conversion_equals_direct_rounding():
    rng = np.random.default_rng(5)
    bits = rng.integers(0, 2 ** 32, size=4_000_000, dtype=np.uint64).astype(np.uint32)
    x = bits.view(np.float32)
    x = x[np.isfinite(x) & (np.abs(x) < 2.0 ** 31)]
    assert x.size > 2_000_000
    assert np.array_equal(split_conversion(x), direct(x))


def test_split_conversion_edge_cases():
    one = np.float32(1.0)
    edge = [0.0, -0.0, 1.0, -1.0, np.nextafter(one, np.float32(0)), np.nextafter(one, np.float32(2)),
            2.0 ** -9, np.nextafter(np.float32(2.0 ** -9), np.float32(0)), 2.0 ** -33, 3 * 2.0 ** -33,
            5 * 2.0 ** -34, 2.0 ** -40, 0.3, 0.5, 0.7, 123.456, 2.0 ** 31 - 128, 1e-30, 1.17549435e-38]
    x = np.array(edge + [-e for e in edge], np.float32)
    assert np.array_equal(split_conversion(x), direct(x))
    # ties go to even: 0.5 and 1.5 units of 2^-32
    assert split_conversion(np.float32(2.0 ** -33)) == 0
    assert split_conversion(np.float32(3 * 2.0 ** -33)) == 2
    assert split_conversion(np.float32(-3 * 2.0 ** -33)) == -2
