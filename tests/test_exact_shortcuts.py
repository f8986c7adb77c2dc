"""The exact integer-pipe forms the throughput kernels use in place of FP64
instructions (nsg_internal.cuh: add_1em30, mul4; nsg_div.cuh: div_recip_seed's
integer built from the float's bits), restated with numpy bit operations and
compared with the IEEE operations they replace."""
import numpy as np


def _rand_doubles(rng, n, lo_exp, hi_exp):
    mant = rng.integers(0, 1 << 52, n, dtype=np.uint64)
    exp = rng.integers(lo_exp, hi_exp + 1, n).astype(np.uint64)
    sign = rng.integers(0, 2, n).astype(np.uint64) << np.uint64(63)
    return (sign | (exp << np.uint64(52)) | mant).view(np.float64)


def test_add_1em30_is_identity_from_2_pow_minus_46():
    rng = np.random.default_rng(1)
    x = np.abs(_rand_doubles(rng, 200000, 977, 2046))
    x = np.concatenate([x, [2.0 ** -46, np.nextafter(2.0 ** -46, 1.0), np.inf]])
    assert np.array_equal((x + 1.0e-30).view(np.uint64), x.view(np.uint64))
    # below the threshold the addition is not the identity everywhere: the shortcut must not apply
    y = np.abs(_rand_doubles(rng, 20000, 900, 976))
    assert np.any((y + 1.0e-30) != y)
    assert (np.float64(2.0 ** -46).view(np.uint64) >> np.uint64(52)) == 977


def test_mul4_by_exponent_field():
    rng = np.random.default_rng(2)
    x = _rand_doubles(rng, 200000, 1, 2044)
    bits = x.view(np.int64) + (np.int64(2) << np.int64(52))
    assert np.array_equal(bits.view(np.float64), 4.0 * x)


def test_recip_seed_from_float_bits():
    # y = 1/fb for fb in [2^23, 2^24): y 2^76 as an integer equals the significand
    # shifted by (biased exponent of y) - 74
    fb = np.arange(1 << 23, 1 << 24, 977, dtype=np.uint32)
    fb = np.concatenate([fb, [1 << 23, (1 << 24) - 1]]).astype(np.uint32)
    y = (np.float32(1.0) / fb.astype(np.float32)).astype(np.float32)
    fy = y.view(np.uint32)
    built = ((fy & np.uint32(0x7FFFFF)) | np.uint32(0x800000)).astype(np.int64) << ((fy >> np.uint32(23)).astype(np.int64) - 74)
    direct = (y.astype(np.float64) * 2.0 ** 76).astype(np.int64)
    assert np.array_equal(built, direct)
    # the 24-bit divisor top as a float from its bits
    f24 = ((np.uint32(150) << np.uint32(23)) | (fb & np.uint32(0x7FFFFF))).view(np.float32)
    assert np.array_equal(f24, fb.astype(np.float32))


def _ratio_bound(tol):
    b = int(np.float64(tol).view(np.uint64))
    et = (b >> 52) & 0x7FF
    if (b >> 63) or et == 0 or et == 0x7FF:
        return None
    mt = (b & ((1 << 52) - 1)) | (1 << 52)
    if mt == 1 << 52:
        return (1 << 54) - 1, 1077 - et
    return 2 * mt - 1, 1076 - et


def _ratio_lt(x, y, rb):
    """RN(x/y) < tol decided from the bits (ratio_lt); None where the kernel divides."""
    bx, by = int(np.float64(x).view(np.uint64)), int(np.float64(y).view(np.uint64))
    ex, ey = (bx >> 52) & 0x7FF, (by >> 52) & 0x7FF
    if rb is None or not (1 <= ey <= 2046) or not (bx == 0 or 1 <= ex <= 2046):
        return None
    if bx == 0:
        return True
    B, doff = rb
    D = ex - ey + doff
    if D <= 52:
        return True
    if D >= 55:
        return False
    mx = (bx & ((1 << 52) - 1)) | (1 << 52)
    my = (by & ((1 << 52) - 1)) | (1 << 52)
    return (mx << D) < B * my   # the kernel's 128-bit comparison


def test_ratio_test_matches_division():
    rng = np.random.default_rng(3)
    x = np.abs(_rand_doubles(rng, 20000, 800, 1200))
    y = np.abs(_rand_doubles(rng, 20000, 800, 1200))
    q = x / y
    qb = q.view(np.uint64)
    cases = 0
    for k in range(len(x)):
        for tol in (q[k], (qb[k] + np.uint64(1)).view(np.float64), (qb[k] - np.uint64(1)).view(np.float64),
                    1e-7, 2.0 ** -23, np.nextafter(2.0 ** -23, 0.0)):
            got = _ratio_lt(x[k], y[k], _ratio_bound(tol))
            if got is not None:
                cases += 1
                assert got == bool(q[k] < tol), (x[k], y[k], tol)
    assert cases > 100000
    # zero dividends, and the kernels' typical relative differences near tol = 1e-7
    assert _ratio_lt(0.0, 3.0, _ratio_bound(1e-7)) is True
    rf = np.float64(0.731)
    for d in np.linspace(-2e-7, 2e-7, 4001):
        xr, yr = abs(np.float64(rf * d)), abs(rf) + 1e-30
        assert _ratio_lt(xr, yr, _ratio_bound(1e-7)) == bool(xr / yr < 1e-7)
