"""The refinement steps of csrc/fastmath.cuh restated in numpy (CPU): from an
FP32 estimate (relative error near 2^-23), one third-order step reaches FP64
accuracy.  This checks the series, y (1 + e + e^2) for 1/x with e = 1 - x y
and y (1 + r/3 + 2 r^2/9) for x^(-1/3) with r = 1 - x y^3, not the device
code (tests/test_gpu_math.py compares that with CUDA's functions); numpy has
no fused multiply-add, so the residuals here carry one rounding more than on
the GPU, and the bound is an ulp looser."""
from __future__ import annotations

import numpy as np

ULP = 2.0 ** -52


def _args(n=200_000, seed=7):
    rng = np.random.default_rng(seed)
    # |x| in [2^-125, 2^125), both signs for the reciprocal
    return np.ldexp(1.0 + rng.random(n), rng.integers(-125, 124, n))


def _approx(y, seed):
    """An FP32 estimate as the hardware's approximate instructions give it:
    the correctly rounded value moved by up to 2 ulps of FP32."""
    rng = np.random.default_rng(seed)
    return y * (1.0 + rng.uniform(-2.0, 2.0, y.size) * 2.0 ** -23)


def test_reciprocal_series():
    x = _args()
    x = np.where(np.arange(x.size) % 2 == 0, x, -x)
    y = _approx((np.float32(1.0) / x.astype(np.float32)).astype(np.float64), 1)   # FP32 estimate
    assert np.max(np.abs(y * x - 1.0)) < 2.0 ** -21
    e = 1.0 - x * y
    r = y + y * (e + e * e)
    err = np.abs(r * x - 1.0)
    assert np.max(err) <= 3 * ULP, np.max(err) / ULP


def test_inverse_cube_root_series():
    x = np.abs(_args(seed=11))
    y = np.cbrt(x.astype(np.float32)).astype(np.float64)
    y = _approx((np.float32(1.0) / y.astype(np.float32)).astype(np.float64), 2)   # estimate of x^(-1/3)
    exact = 1.0 / np.cbrt(x)
    assert np.max(np.abs(y / exact - 1.0)) < 2.0 ** -20
    r = 1.0 - x * (y * y) * y
    z = y + (y * r) * (r * (2.0 / 9.0) + 1.0 / 3.0)
    err = np.abs(z / exact - 1.0)
    assert np.max(err) <= 4 * ULP, np.max(err) / ULP


def test_second_order_would_not_do():
    """One Newton (second-order) step from the same estimate leaves ~2^-44:
    the third-order term is what reaches FP64."""
    x = np.abs(_args(seed=3))
    y = _approx((np.float32(1.0) / x.astype(np.float32)).astype(np.float64), 3)
    e = 1.0 - x * y
    newton = y + y * e
    assert np.max(np.abs(newton * x - 1.0)) > 64 * ULP
