"""The library's own FP64 root and reciprocal functions against CUDA's: the
inverse cube root of the hourglass coefficient against rcbrt, the sound
speed's x*rsqrt(x) against sqrt, the reciprocal and the quotient refined from
FP32 estimates against __drcp_rn and the correctly rounded division, over
2^20 arguments in [2^-140, 2^140] (inside and outside the range where the
FP32 estimate is used)."""
from __future__ import annotations

import pytest

pytestmark = pytest.mark.gpu

ULP = 2.0 ** -52


def test_roots_and_reciprocals_agree_with_cuda(pkg):
    e = pkg.probe_math()
    assert e["rcbrt"] <= 4 * ULP, e
    assert e["sqrt"] <= 4 * ULP, e
    assert e["rcp"] <= 2 * ULP, e
    assert e["quot"] <= 3 * ULP, e
