"""Two conversions the kernels build from other instructions, restated in
numpy with the same IEEE operations and checked bit for bit:
  * the force accumulators' FP32 -> 64-bit fixed-point conversion
    (komd_gb300/csrc/atm_device.cuh, fix32_rn): round(x * 2^32) as int64 from
    two 32-bit conversions, over random bit patterns and the edge cases
    (values next to integers, the ulp boundary at 2^-9, ties to even, signs);
  * the fused drift's FP64 -> FP32 rounding from the bits
    (komd_gb300/csrc/kernels.cu, d2f_rn)."""
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


def d2f_rn(x):
    """The fused drift's FP64 -> FP32 rounding from the bits
    (komd_gb300/csrc/kernels.cu, d2f_rn), the conversion instruction outside
    the FP32 normal range."""
    x = np.asarray(x, np.float64)
    b = x.view(np.uint64)
    e = ((b >> np.uint64(52)) & np.uint64(0x7ff)).astype(np.int64) - 1023 + 127
    mant = b & np.uint64(0xfffffffffffff)
    f = ((np.clip(e, 0, 255).astype(np.uint64) << np.uint64(23)) | (mant >> np.uint64(29))).astype(np.uint64)
    rest = mant & np.uint64(0x1fffffff)
    half = np.uint64(0x10000000)
    up = (rest > half) | ((rest == half) & ((f & np.uint64(1)) == 1))
    f = (f + up.astype(np.uint64)) | ((b >> np.uint64(32)) & np.uint64(0x80000000))
    bits = f.astype(np.uint32).view(np.float32)
    normal = (e >= 1) & (e <= 254)
    return np.where(normal, bits, x.astype(np.float32))


def test_d2f_rn_equals_conversion():
    rng = np.random.default_rng(13)
    n = 2_000_000
    x = rng.standard_normal(n) * 10.0 ** rng.uniform(-45, 40, n)
    # values on and next to the FP32 rounding ties
    t = rng.standard_normal(200_000).astype(np.float32).astype(np.float64)
    ulp = np.spacing(np.abs(t).astype(np.float32)).astype(np.float64)
    x = np.concatenate([x, t, t + ulp / 2, t - ulp / 2, t + ulp / 2 * (1 + 2.0 ** -30), np.nextafter(t + ulp / 2, 0),
                        [0.0, -0.0, 3.4028234663852886e38, 3.4028235677973366e38, 1.1754943508222875e-38,
                         1.1754942e-38, np.inf, -np.inf]])
    with np.errstate(over="ignore"):
        got = d2f_rn(x)
        want = x.astype(np.float32)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
