// fastmath.cuh -- FP64 reciprocal, quotient and inverse cube root refined
// from FP32 estimates.
//
// GB300's FP64 pipe issues at 1/64 of the FP32 rate, and the FP64 step is
// bound by it, so these functions spend FP32 and integer instructions to save
// FP64 ones.  Each takes an FP32 hardware estimate (relative error below
// 2^-22) and applies one third-order correction: with the residual r of the
// estimate y, the exact value is y (1 - r)^(-1/n), and the series
// 1 + r/n + ((1+n)/(2n^2)) r^2 leaves an error of order r^3 (~2^-66), below
// FP64 rounding.  1/x costs 3 FP64 operations (5 for __drcp_rn), a/x 4 (8 for
// the correctly rounded quotient), x^(-1/3) 6; results are within an ulp or
// so of the correctly rounded values (tested against CUDA's functions).
//
// The estimate is read and written with integer bit operations (the
// FP64<->FP32 conversion instructions also take FP64 issue slots), which is
// exact only where x and the estimate are normal FP32 numbers: for |x|
// outside [2^-125, 2^125) (and for zeros, infinities and NaNs) the functions
// fall back to CUDA's correctly rounded ones.
#pragma once

namespace lulesh {

// |x| in [2^-125, 2^125)
__device__ __forceinline__ bool f32_range(double x)
{
    const unsigned e = ((unsigned)__double2hiint(x) >> 20) & 0x7ffu;
    return e - 898u <= 249u;
}

// x truncated to FP32 (x in f32_range)
__device__ __forceinline__ float f32_trunc(double x)
{
    const unsigned hi = (unsigned)__double2hiint(x), lo = (unsigned)__double2loint(x);
    return __uint_as_float((hi & 0x80000000u) | ((((hi >> 20) & 0x7ffu) - 896u) << 23) |
                           ((hi & 0xfffffu) << 3) | (lo >> 29));
}

// a normal FP32 value as FP64 (exact)
__device__ __forceinline__ double f64_exact(float f)
{
    const unsigned u = __float_as_uint(f);
    const unsigned hi = (u & 0x80000000u) | ((((u >> 23) & 0xffu) + 896u) << 20) | ((u >> 3) & 0xfffffu);
    return __hiloint2double((int)hi, (int)(u << 29));
}

// 1/x: e = 1 - x y, 1/x = y / (1 - e) = y (1 + e + e^2 + ...)
__device__ __forceinline__ double rcp_fast(double x)
{
    if (!f32_range(x)) return __drcp_rn(x);
    float yf;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(yf) : "f"(f32_trunc(x)));
    const double y = f64_exact(yf);
    const double e = fma(-x, y, 1.0);
    return fma(y, fma(e, e, e), y);
}

// a/x as a times the reciprocal (within about an ulp of the quotient)
__device__ __forceinline__ double quot_fast(double a, double x) { return a * rcp_fast(x); }

// x^(-1/3) for x > 0: r = 1 - x y^3, x^(-1/3) = y (1 - r)^(-1/3)
// = y (1 + r/3 + 2 r^2/9 + ...)
__device__ __forceinline__ double rcbrt_fast(double x)
{
    if (!f32_range(x)) return rcbrt(x);
    const double y = f64_exact(rcbrtf(f32_trunc(x)));
    const double r = fma(-x, (y * y) * y, 1.0);
    return fma(y * r, fma(r, 2.0 / 9.0, 1.0 / 3.0), y);
}

}  // namespace lulesh
