"""The library's own FP64 root functions against CUDA's: the Newton inverse
cube root of the hourglass coefficient against rcbrt, and the sound speed's
x*rsqrt(x) against sqrt, over 2^20 arguments in [2^-60, 2^60]."""
from __future__ import annotations

import pytest

pytestmark = pytest.mark.gpu

ULP = 2.0 ** -52


def test_roots_agree_with_cuda(pkg):
    e = pkg.probe_math()
    assert e["inv_cbrt_vs_rcbrt"] <= 4 * ULP, e
    assert e["x_rsqrt_x_vs_sqrt"] <= 4 * ULP, e
