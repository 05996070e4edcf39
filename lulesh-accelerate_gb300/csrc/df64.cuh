// df64.cuh -- double-float arithmetic on the FP32 pipe.
//
// GB300 issues FP32 at 64 times its FP64 rate, so element arithmetic that
// the step would otherwise spend FP64 issue slots on runs here as pairs of
// floats: a value is the unevaluated sum hi + lo of two floats with
// |lo| <= ulp(hi)/2, which carries about 48 significant bits (relative
// rounding near 2^-47 per operation, against 2^-53 in FP64).
//
// The algorithms are the published error-free transformations and the
// double-word operations built on them, restated:
//   - two_sum: Knuth's two-sum (TAOCP vol. 2, 4.2.2), s + e == a + b exactly;
//   - fast_two_sum: Dekker's (1971) variant for |a| >= |b|;
//   - two_prod: the product and its exact remainder through one fused
//     multiply-add;
//   - df_add / df_mul / df_fma: the "sloppy" double-word sum and the
//     double-word product of Hida, Li and Bailey's QD library (2001) --
//     addition through two_sum of the high words, product through two_prod
//     plus the cross terms, each renormalised by fast_two_sum;
//   - reciprocal, quotient and inverse square root: an FP32 estimate refined
//     by Newton steps carried out in double-float.
// Every operation is written with the _rn intrinsics, which the compiler
// neither contracts nor reorders, so any kernel that inlines them rounds the
// same way.
//
// Conversions never touch the FP64 pipe: to_df splits a double's bit
// pattern with integer operations (hi = its leading 24 significand bits, lo
// = the next 24 of the remaining 29, both truncated), and to_double joins
// the two words with one FP64 addition.
#pragma once

#include <cuda_runtime.h>

namespace lulesh {

using ::fabs;
using ::fma;
using ::fmax;

struct df64 {
    float hi, lo;
    df64() = default;
    __host__ __device__ constexpr df64(float h, float l) : hi(h), lo(l) {}
    // compile-time constants only (a run-time double goes through to_df)
    __host__ __device__ constexpr explicit df64(double v) : hi((float)v), lo((float)(v - (double)(float)v)) {}
};

__device__ __forceinline__ df64 two_sum(float a, float b)
{
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    return {s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb))};
}

__device__ __forceinline__ df64 fast_two_sum(float a, float b)
{
    const float s = __fadd_rn(a, b);
    return {s, __fsub_rn(b, __fsub_rn(s, a))};
}

__device__ __forceinline__ df64 two_prod(float a, float b)
{
    const float p = __fmul_rn(a, b);
    return {p, __fmaf_rn(a, b, -p)};
}

__device__ __forceinline__ df64 df_add(df64 a, df64 b)
{
    const df64 s = two_sum(a.hi, b.hi);
    return fast_two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo)));
}

__device__ __forceinline__ df64 df_mul(df64 a, df64 b)
{
    const df64 p = two_prod(a.hi, b.hi);
    return fast_two_sum(p.hi, __fmaf_rn(a.hi, b.lo, __fmaf_rn(a.lo, b.hi, p.lo)));
}

// a * b + c with one renormalisation
__device__ __forceinline__ df64 df_fma(df64 a, df64 b, df64 c)
{
    const df64 p = two_prod(a.hi, b.hi);
    const float t = __fmaf_rn(a.hi, b.lo, __fmaf_rn(a.lo, b.hi, p.lo));
    const df64 s = two_sum(p.hi, c.hi);
    return fast_two_sum(s.hi, __fadd_rn(__fadd_rn(s.lo, t), c.lo));
}

// A sum of products c + sum_i a_i b_i accumulated with one renormalisation
// at the end: each product's high word joins the running high word through
// two_sum and every low-order term collects in one float (the compensated
// dot product Dot2 of Ogita, Rump and Oishi, 2005, on pairs).  12 FP32
// operations per term against 15 for a chain of df_fma, to the same order
// of accuracy.
struct DfDot {
    float s, e;
    __device__ explicit DfDot(df64 c) : s(c.hi), e(c.lo) {}
    __device__ void add(df64 a, df64 b)
    {
        const df64 p = two_prod(a.hi, b.hi);
        const df64 q = two_sum(s, p.hi);
        s = q.hi;
        e = __fadd_rn(e, __fadd_rn(q.lo, __fmaf_rn(a.hi, b.lo, __fmaf_rn(a.lo, b.hi, p.lo))));
    }
    __device__ df64 value() const { return two_sum(s, e); }
};

// a times a float (exact in hi)
__device__ __forceinline__ df64 df_mul_f(df64 a, float b)
{
    const df64 p = two_prod(a.hi, b);
    return fast_two_sum(p.hi, __fmaf_rn(a.lo, b, p.lo));
}

// a times a power of two: exact
__device__ __forceinline__ df64 df_scale(df64 a, float pow2) { return {__fmul_rn(a.hi, pow2), __fmul_rn(a.lo, pow2)}; }

__device__ __forceinline__ df64 operator+(df64 a, df64 b) { return df_add(a, b); }
__device__ __forceinline__ df64 operator-(df64 a) { return {-a.hi, -a.lo}; }
__device__ __forceinline__ df64 operator-(df64 a, df64 b) { return df_add(a, -b); }
__device__ __forceinline__ df64 operator*(df64 a, df64 b) { return df_mul(a, b); }
__device__ __forceinline__ df64 fma(df64 a, df64 b, df64 c) { return df_fma(a, b, c); }
// the sign of a renormalised pair is the sign of its high word
__device__ __forceinline__ df64 fabs(df64 a) { return a.hi < 0.f ? -a : a; }
__device__ __forceinline__ bool df_gt(df64 a, df64 b) { return a.hi > b.hi || (a.hi == b.hi && a.lo > b.lo); }
__device__ __forceinline__ df64 fmax(df64 a, df64 b) { return df_gt(b, a) ? b : a; }

// Reciprocal: r0 = the FP32 reciprocal, then two Newton steps
// r <- r + r (1 - b r) with the residual formed in double-float; each step
// squares the relative error (2^-23 -> 2^-46 -> below the format's
// rounding).
__device__ __forceinline__ df64 df_rcp(df64 b)
{
    const float r0 = __frcp_rn(b.hi);
    df64 r{r0, 0.f};
#pragma unroll
    for (int it = 0; it < 2; ++it) {
        const df64 e = df_add(df64(1.0), -df_mul(b, r));
        r = df_fma(r, e, r);
    }
    return r;
}

// a / b: the quotient through the reciprocal, corrected once by the
// remainder a - q b.
__device__ __forceinline__ df64 df_div(df64 a, df64 b)
{
    const df64 r = df_rcp(b);
    const df64 q = df_mul(a, r);
    const df64 rem = df_add(a, -df_mul(q, b));
    return df_fma(rem, r, q);
}

// 1 / sqrt(a), a > 0: the FP32 estimate, then two Newton steps
// y <- y + y (1 - a y^2) / 2 in double-float.
__device__ __forceinline__ df64 df_rsqrt(df64 a)
{
    df64 y{rsqrtf(a.hi), 0.f};
#pragma unroll
    for (int it = 0; it < 2; ++it) {
        const df64 e = df_add(df64(1.0), -df_mul(a, df_mul(y, y)));
        y = df_fma(df_scale(y, 0.5f), e, y);
    }
    return y;
}

// ---- conversions --------------------------------------------------------

// double -> pair without the FP64 pipe.  hi takes the 24 leading
// significand bits, lo the next 24 of the remaining 29, both truncated:
// |v - (hi + lo)| < 2^-47 |v|.  For an exponent e of v (v = 1.f 2^e) the
// float exponent field of hi is e + 127, which the bits 60..29 of v plus
// 2^30 give directly (the low nine bits of v's biased exponent, minus 384,
// modulo 2^32); lo is the 29-bit remainder r, signed, converted to float
// rounding toward zero (its 24 leading bits) and scaled by 2^(e-52).
// Magnitudes outside [2^-74, 2^128), where lo or hi would leave the normal
// float range, keep hi only (an error below 2^-98 absolute): zeros,
// infinities and NaNs map to themselves.
__device__ __forceinline__ df64 to_df(double v)
{
    const unsigned lo32 = (unsigned)__double2loint(v), hi32 = (unsigned)__double2hiint(v);
    const unsigned sign = hi32 & 0x80000000u;
    const unsigned de = (hi32 >> 20) & 0x7ffu;   // biased exponent, e + 1023
    if (de - 949u <= 201u) {                     // e in [-74, 127]
        const float hi = __uint_as_float((__funnelshift_r(lo32, hi32, 29) + 0x40000000u) | sign);
        const int m = (int)hi32 >> 31;            // 0 or -1
        const int r = (int)(((lo32 & 0x1fffffffu) ^ (unsigned)m) - (unsigned)m);   // +-remainder
        return {hi, __int2float_rz(r) * __uint_as_float((de - 948u) << 23)};
    }
    // outside the split's range: the high word alone (FP32 truncation,
    // signed zero below the float range, infinity above, NaN kept)
    unsigned hb;
    if (de >= 897u && de <= 1150u) hb = (__funnelshift_r(lo32, hi32, 29) + 0x40000000u) | sign;
    else if (de < 897u) hb = sign;
    else if (de == 0x7ffu && ((hi32 & 0xfffffu) | lo32) != 0u) hb = sign | 0x7fc00000u;
    else hb = sign | 0x7f800000u;
    return {__uint_as_float(hb), 0.f};
}

// float -> double with integer operations (normal floats and zeros exact;
// subnormals flush to a signed zero, infinities and NaNs kept).
__device__ __forceinline__ double df_f2d(float f)
{
    const unsigned u = __float_as_uint(f);
    const unsigned long long sign = (unsigned long long)(u & 0x80000000u) << 32;
    const unsigned fe = (u >> 23) & 0xffu;
    const unsigned long long mant = (unsigned long long)(u & 0x7fffffu) << 29;
    if (fe == 0) return __longlong_as_double((long long)sign);
    const unsigned long long de = (fe == 0xff) ? 0x7ffULL : (unsigned long long)(fe - 127 + 1023);
    return __longlong_as_double((long long)(sign | (de << 52) | mant));
}

// pair -> double: one FP64 addition (the correctly rounded sum of the words)
__device__ __forceinline__ double to_double(df64 a) { return df_f2d(a.hi) + df_f2d(a.lo); }

// quotient overload for the geometry templates (hexmodes.cuh)
__device__ __forceinline__ df64 quot_fast(df64 a, df64 b) { return df_div(a, b); }

__device__ __forceinline__ float2 as_float2(df64 a) { return make_float2(a.hi, a.lo); }
__device__ __forceinline__ df64 as_df(float2 f) { return {f.x, f.y}; }

}  // namespace lulesh
