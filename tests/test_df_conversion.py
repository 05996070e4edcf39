"""The double -> double-float conversion of csrc/df64.cuh (``to_df``) restated
in numpy (CPU): hi from bits 60..29 of the double plus 2^30 with the sign
or-ed in, lo the signed 29-bit remainder converted to float toward zero and
scaled by 2^(e-52).  This checks the bit arithmetic against the
conversion's definition -- hi the 24 leading significand bits, lo the next
24, both truncated -- and its error bound, not the device code (the GPU
parity tests run that end to end)."""
from __future__ import annotations

import numpy as np

U32 = np.uint32


def _bits(v):
    b = np.asarray(v, dtype=np.float64).view(np.uint64)
    return (b & np.uint64(0xFFFFFFFF)).astype(U32), (b >> np.uint64(32)).astype(U32)


def _funnel29(lo32, hi32):
    """__funnelshift_r(lo, hi, 29): the low 32 bits of (hi:lo) >> 29."""
    return ((lo32 >> U32(29)) | (hi32 << U32(3))).astype(U32)


def to_df(v):
    lo32, hi32 = _bits(v)
    sign = hi32 & U32(0x80000000)
    de = (hi32 >> U32(20)) & U32(0x7FF)
    fast = (de - U32(949)) <= U32(201)          # unsigned wrap, as on the device
    with np.errstate(over="ignore"):
        hb_fast = (_funnel29(lo32, hi32) + U32(0x40000000)) | sign
        scale_bits = ((de - U32(948)) << U32(23)) | sign
    scale = (scale_bits & U32(0x7FFFFFFF)).view(np.float32)
    r = (lo32 & U32(0x1FFFFFFF)).astype(np.int64)
    # __int2float_rz: keep the 24 leading bits of |r|
    drop = np.maximum(np.floor(np.log2(np.maximum(r, 1))).astype(np.int64) - 23, 0)
    rz = ((r >> drop) << drop).astype(np.float32)
    lo_fast = np.where(sign != 0, -rz, rz) * scale
    mid = (de >= U32(897)) & (de <= U32(1150))
    nan = (de == U32(0x7FF)) & (((hi32 & U32(0xFFFFF)) | lo32) != U32(0))
    hb_edge = np.where(mid, hb_fast, np.where(de < U32(897), sign,
                       np.where(nan, sign | U32(0x7FC00000), sign | U32(0x7F800000))))
    hi = np.where(fast, hb_fast, hb_edge).astype(U32).view(np.float32)
    lo = np.where(fast, lo_fast, np.float32(0.0))
    return hi, lo


def test_in_range_error_bound():
    rng = np.random.default_rng(5)
    n = 400_000
    v = np.ldexp(1.0 + rng.random(n), rng.integers(-74, 128, n))
    v = np.where(rng.random(n) < 0.5, v, -v)
    hi, lo = to_df(v)
    # hi is v truncated to 24 significand bits: same sign, |hi| <= |v|
    # within one FP32 ulp
    assert np.all(np.signbit(hi) == np.signbit(v))
    assert np.all(np.abs(hi.astype(np.float64)) <= np.abs(v))
    assert np.all(np.abs(v - hi) < np.abs(v) * 2.0 ** -23)
    # exact reconstruction of the 53-bit value up to lo's truncation, 2^-47
    err = np.abs((v - hi.astype(np.float64)) - lo.astype(np.float64))
    assert np.max(err / np.abs(v)) < 2.0 ** -47
    # lo is the remainder truncated: same sign as v, never larger in size
    rem = v - hi.astype(np.float64)
    assert np.all(np.abs(lo.astype(np.float64)) <= np.abs(rem))
    assert np.all((lo == 0) | (np.signbit(lo) == np.signbit(v)))
    assert not np.any((lo == 0) & np.signbit(lo))
    # lo never exceeds one ulp of hi
    ulp_hi = np.spacing(np.abs(hi)).astype(np.float64)
    assert np.all(np.abs(lo.astype(np.float64)) <= ulp_hi)


def test_exact_when_the_remainder_fits_a_float():
    rng = np.random.default_rng(6)
    v = np.ldexp(1.0 + np.floor(rng.random(10_000) * 2.0 ** 47) * 2.0 ** -47, rng.integers(-70, 120, 10_000))
    hi, lo = to_df(v)
    assert np.array_equal(hi.astype(np.float64) + lo.astype(np.float64), v)


def test_range_edges():
    v = np.array([0.0, -0.0, 2.0 ** -74, -(2.0 ** -74) * 1.5, 2.0 ** -75 * 1.25, 2.0 ** -126,
                  2.0 ** -127, 1e-300, 5e-324, 2.0 ** 127 * 1.999, 2.0 ** 128, -1e300,
                  np.inf, -np.inf, np.nan, 1.0, -1.0, 1.125, 1.0 / 3.0])
    hi, lo = to_df(v)
    h, l = hi.astype(np.float64), lo.astype(np.float64)
    assert h[0] == 0 and not np.signbit(h[0]) and l[0] == 0
    assert h[1] == 0 and np.signbit(h[1]) and l[1] == 0
    assert h[2] == 2.0 ** -74 and l[2] == 0
    assert h[3] + l[3] == v[3]
    # below 2^-74: the truncated high word alone
    assert l[4] == 0 and h[4] == np.float32(2.0 ** -75 * 1.25)
    assert l[5] == 0 and h[5] == 2.0 ** -126
    for i in (6, 7, 8):   # below the normal float range: a signed zero
        assert h[i] == 0 and l[i] == 0
    assert np.isfinite(h[9]) and abs((h[9] + l[9]) / v[9] - 1) < 2.0 ** -47
    assert h[10] == np.inf and h[11] == -np.inf and l[10] == 0 and l[11] == 0
    assert h[12] == np.inf and h[13] == -np.inf
    assert np.isnan(h[14]) and l[14] == 0
    assert h[15] == 1.0 and l[15] == 0 and h[16] == -1.0 and h[17] == 1.125
    assert abs(h[18] + l[18] - v[18]) < v[18] * 2.0 ** -47


def _reference_split(v):
    """The definition with exact rationals: hi = v truncated to 24 significand
    bits, lo = the remainder truncated to 24 significant bits."""
    from fractions import Fraction
    import math
    out = []
    for x in v:
        f = Fraction(float(x))
        e = math.floor(math.log2(abs(float(x))))
        q = Fraction(2) ** (e - 23)
        hi = (abs(f) // q) * q
        rem = abs(f) - hi
        if rem == 0:
            lo = Fraction(0)
        else:
            e2 = math.floor(math.log2(float(rem)))
            q2 = Fraction(2) ** (e2 - 23)
            lo = (rem // q2) * q2
        sgn = -1 if x < 0 else 1
        out.append((float(sgn * hi), float(sgn * lo)))
    return out


def test_matches_the_truncating_definition():
    rng = np.random.default_rng(8)
    v = np.ldexp(1.0 + rng.random(3000), rng.integers(-74, 128, 3000))
    v = np.where(rng.random(3000) < 0.5, v, -v)
    hi, lo = to_df(v)
    for (h, l), a, b in zip(_reference_split(v), hi, lo):
        assert float(a) == h and float(b) == l
