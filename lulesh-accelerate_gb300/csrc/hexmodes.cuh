// hexmodes.cuh -- hexahedron geometry through the Walsh modes of its corners.
//
// A trilinear hexahedron x(xi,eta,zeta), xi,eta,zeta in [-1,1], with the
// reference's corner order (corner c at signs s(c) = (-,-,-) (+,-,-) (+,+,-)
// (-,+,-) (-,-,+) (+,-,+) (+,+,+) (-,+,+)) is
//     x = (M0 + M1 xi + M2 eta + M3 zeta + M4 xi eta + M5 xi zeta
//          + M6 eta zeta + M7 xi eta zeta) / 8,
// where the modes M_i = sum_c s_i(c) x_c are the Walsh transform of the
// corner coordinates (three butterfly stages, 24 additions).  Everything the
// step needs from the corner coordinates is a short expression in these
// modes:
//   - the Jacobian columns at the centre (CalcElemShapeFunctionDerivatives,
//     LULESH-OMP.cc:650-660) are M1/8, M2/8, M3/8;
//   - the monotonic-Q logical differences (:2066-2076) are M1/4, M2/4, M3/4;
//   - the four hourglass base vectors gamma (:1252-1285) are the sign
//     patterns eta zeta, xi zeta, xi eta, xi eta zeta, so the hourglass mode
//     projections sum_c gamma_m(c) x_c are M6, M5, M4, M7;
//   - the exact volume (CalcElemVolume, :1706-1790) integrates det J over the
//     cube: V = [M1.(M2xM3) + (M4.(M2xM6) + M5.(M6xM3) + M1.(M4xM5))/3] / 64;
//   - its derivative with respect to corner c (CalcElemVolumeDerivative,
//     :1008-1048) is (1/64) sum_{i=1..6} s_i(c) W_i with the W_i below, an
//     inverse Walsh transform of six vectors.
// These are the reference's quantities, not approximations of them; only the
// rounding differs (relative differences of a few 1e-16 on distorted
// elements, checked against the reference formulas).
#pragma once

#include "fastmath.cuh"
#include "df64.cuh"

#include <type_traits>

namespace lulesh {

template <typename T>
struct V3 {
    T x, y, z;
};

// The products and sums below are written as explicit fused multiply-adds,
// so that every kernel that inlines them rounds the same way: the compiler
// is otherwise free to fuse either product of a*b - c*d into the add, and
// its choice may differ between a single-instance kernel and the batched
// kernel that runs the same element body.
template <typename T>
__device__ __forceinline__ V3<T> cross3(const V3<T> &a, const V3<T> &b)
{
    return {fma(a.y, b.z, -(a.z * b.y)), fma(a.z, b.x, -(a.x * b.z)), fma(a.x, b.y, -(a.y * b.x))};
}

template <typename T>
__device__ __forceinline__ T dot3(const V3<T> &a, const V3<T> &b)
{
    return fma(a.z, b.z, fma(a.y, b.y, a.x * b.x));
}

// acc + a.b as one chain of three fused multiply-adds
template <typename T>
__device__ __forceinline__ T dot3_acc(const V3<T> &a, const V3<T> &b, T acc)
{
    return fma(a.z, b.z, fma(a.y, b.y, fma(a.x, b.x, acc)));
}

// a x b + c x d, four operations per component (one product and three
// fused multiply-adds) instead of the five of two crosses and a sum
template <typename T>
__device__ __forceinline__ V3<T> cross_sum(const V3<T> &a, const V3<T> &b, const V3<T> &c, const V3<T> &d)
{
    return {fma(a.y, b.z, fma(-a.z, b.y, fma(c.y, d.z, -(c.z * d.y)))),
            fma(a.z, b.x, fma(-a.x, b.z, fma(c.z, d.x, -(c.x * d.z)))),
            fma(a.x, b.y, fma(-a.y, b.x, fma(c.x, d.y, -(c.y * d.x))))};
}

// Modes m[0..6] = M1..M7 (xi, eta, zeta, xi eta, xi zeta, eta zeta,
// xi eta zeta) of 8 corner values.
template <typename T>
__device__ __forceinline__ void walsh8(const T c[8], T m[7])
{
    const T s01 = c[0] + c[1], d01 = c[1] - c[0];
    const T s32 = c[3] + c[2], d32 = c[2] - c[3];
    const T s45 = c[4] + c[5], d45 = c[5] - c[4];
    const T s76 = c[7] + c[6], d76 = c[6] - c[7];
    const T ssm = s01 + s32, dsm = s32 - s01;    // zeta = -1 face
    const T ssp = s45 + s76, dsp = s76 - s45;    // zeta = +1 face
    const T sdm = d01 + d32, ddm = d32 - d01;
    const T sdp = d45 + d76, ddp = d76 - d45;
    m[0] = sdm + sdp;    // xi
    m[1] = dsm + dsp;    // eta
    m[2] = ssp - ssm;    // zeta
    m[3] = ddm + ddp;    // xi eta
    m[4] = sdp - sdm;    // xi zeta
    m[5] = dsp - dsm;    // eta zeta
    m[6] = ddp - ddm;    // xi eta zeta
}

// The three linear modes only (17 additions).
template <typename T>
__device__ __forceinline__ void walsh_linear(const T c[8], T m[3])
{
    const T s01 = c[0] + c[1], d01 = c[1] - c[0];
    const T s32 = c[3] + c[2], d32 = c[2] - c[3];
    const T s45 = c[4] + c[5], d45 = c[5] - c[4];
    const T s76 = c[7] + c[6], d76 = c[6] - c[7];
    m[0] = (d01 + d32) + (d45 + d76);
    m[1] = (s32 - s01) + (s76 - s45);
    m[2] = (s45 + s76) - (s01 + s32);
}

template <typename T>
__device__ __forceinline__ V3<T> mode(const T mx[7], const T my[7], const T mz[7], int i)
{
    return {mx[i], my[i], mz[i]};
}

// Corner values of sum_{i=1..6} s_i(c) q_i (inverse Walsh transform with
// the constant and xi eta zeta modes zero), 20 additions.
template <typename T>
__device__ __forceinline__ void inv_walsh6(T q1, T q2, T q3, T q4, T q5, T q6, T v[8])
{
    const T bp = q1 + q4, bm = q1 - q4;
    const T cp = q3 + q6, cm = q3 - q6;
    const T epp = q2 + bp, emp = q2 - bp;        // E(+,+), E(-,+)
    const T epm = bm - q2, emm = -(q2 + bm);     // E(+,-), E(-,-)
    const T fpp = cp + q5, fmp = cp - q5;        // F(+,+), F(-,+)
    const T fpm = cm + q5, fmm = cm - q5;        // F(+,-), F(-,-)
    v[0] = emm - fmm;
    v[1] = epm - fpm;
    v[2] = epp - fpp;
    v[3] = emp - fmp;
    v[4] = emm + fmm;
    v[5] = epm + fpm;
    v[6] = epp + fpp;
    v[7] = emp + fmp;
}

// The six cross products of the modes that the volume, the node normals, the
// Q gradients and the face areas share: c23 = M2xM3, c31 = M3xM1, c12 = M1xM2,
// c45 = M4xM5, c64 = M6xM4, c56 = M5xM6.
template <typename T>
struct ModeCrosses {
    V3<T> c23, c31, c12, c45, c64, c56;
};

template <typename T>
__device__ __forceinline__ ModeCrosses<T> mode_crosses(const V3<T> &M1, const V3<T> &M2, const V3<T> &M3,
                                                       const V3<T> &M4, const V3<T> &M5, const V3<T> &M6)
{
    return {cross3(M2, M3), cross3(M3, M1), cross3(M1, M2), cross3(M4, M5), cross3(M6, M4), cross3(M5, M6)};
}

// 192 x the volume derivative of each corner (dx/dy/dz[c] = 192 dV/dx_c)
// and the three vectors nx[0..2] = X1, X2, X3 that give the node normals,
// from the modes and their shared cross products C.
// The node normals, sums of the quarter-area vectors of each corner's three
// faces (CalcElemNodeNormals :708-799), are linear in the corner's signs:
// pf[c] = (s_xi X1 + s_eta X2 + s_zeta X3)/64 with X1 = M2xM3 + M4xM5,
// X2 = M3xM1 + M6xM4, X3 = M1xM2 + M5xM6 (the mixed terms of the three faces
// cancel), so the normals of corners 4..7 are those of 2, 3, 0, 1 negated.
// The same six cross products enter the volume derivative, whose six Walsh
// coefficients are taken three times over (3 W1 = 3 M2xM3 + M4xM5,
// 3 W4 = M2xM6 + M5xM1, ...) so that no multiplication by 1/3 is needed.
template <typename T>
__device__ __forceinline__ void volume_derivative(const V3<T> &M1, const V3<T> &M2, const V3<T> &M3,
                                                  const V3<T> &M4, const V3<T> &M5, const V3<T> &M6,
                                                  const ModeCrosses<T> &C, T dx[8], T dy[8], T dz[8])
{
    const V3<T> &c23 = C.c23, &c45 = C.c45, &c31 = C.c31, &c64 = C.c64, &c12 = C.c12, &c56 = C.c56;
    auto add3 = [](const V3<T> &a, T s, const V3<T> &b) {
        return V3<T>{a.x * s + b.x, a.y * s + b.y, a.z * s + b.z};
    };
    const V3<T> W1 = add3(c23, T(3.0), c45);
    const V3<T> W2 = add3(c31, T(3.0), c64);
    const V3<T> W3 = add3(c12, T(3.0), c56);
    const V3<T> W4 = cross_sum(M2, M6, M5, M1);
    const V3<T> W5 = cross_sum(M6, M3, M1, M4);
    const V3<T> W6 = cross_sum(M4, M2, M3, M5);
    inv_walsh6(W1.x, W2.x, W3.x, W4.x, W5.x, W6.x, dx);
    inv_walsh6(W1.y, W2.y, W3.y, W4.y, W5.y, W6.y, dy);
    inv_walsh6(W1.z, W2.z, W3.z, W4.z, W5.z, W6.z, dz);
}

template <typename T>
__device__ __forceinline__ void normal_generators(const ModeCrosses<T> &C, V3<T> nx[3])
{
    auto sum3 = [](const V3<T> &a, const V3<T> &b) { return V3<T>{a.x + b.x, a.y + b.y, a.z + b.z}; };
    nx[0] = sum3(C.c23, C.c45);
    nx[1] = sum3(C.c31, C.c64);
    nx[2] = sum3(C.c12, C.c56);
}

template <typename T>
__device__ __forceinline__ void force_geometry(const V3<T> &M1, const V3<T> &M2, const V3<T> &M3,
                                               const V3<T> &M4, const V3<T> &M5, const V3<T> &M6,
                                               const ModeCrosses<T> &C, T dx[8], T dy[8], T dz[8], V3<T> nx[3])
{
    volume_derivative(M1, M2, M3, M4, M5, M6, C, dx, dy, dz);
    normal_generators(C, nx);
}

// 64 x volume through the shared crosses: the bilinear terms of the volume formula above are
// scalar triple products, M4.(M2xM6) = M2.(M6xM4) and M5.(M6xM3) = M3.(M5xM6).
template <typename T>
__device__ __forceinline__ T volume64_shared(const V3<T> &M1, const V3<T> &M2, const V3<T> &M3,
                                             const ModeCrosses<T> &C)
{
    const T third = T(1.0 / 3.0);
    return fma(dot3_acc(M1, C.c45, dot3_acc(M3, C.c56, dot3(M2, C.c64))), third, dot3(M1, C.c23));
}

// 64 x the largest |u x v|^2 over the six faces (u, v the face diagonals),
// through the modes.  On the face xi = s the surface is bilinear in (eta,
// zeta) with edge vectors (M2 + s M4)/8 and (M3 + s M5)/8, and u x v is 8
// times their cross product: (X1 + s Y1)/8 with X1 = M2xM3 + M4xM5 and
// Y1 = M2xM5 + M4xM3; likewise X2 = M3xM1 + M6xM4, Y2 = M6xM1 + M3xM4 for
// eta = s and X3 = M1xM2 + M5xM6, Y3 = M1xM6 + M5xM2 for zeta = s.  The
// larger of the two faces of a direction is |X|^2 + |Y|^2 + 2|X.Y|.
template <typename T>
__device__ __forceinline__ T max_face_cross2_64(const V3<T> &M1, const V3<T> &M2, const V3<T> &M3,
                                                const V3<T> &M4, const V3<T> &M5, const V3<T> &M6,
                                                const ModeCrosses<T> &C)
{
    const V3<T> a = cross3(M3, M4), b = cross3(M2, M5), c = cross3(M6, M1);
    auto pair = [](const V3<T> &p, const V3<T> &q, const V3<T> &r, const V3<T> &t, T sy) {
        const V3<T> X{p.x + q.x, p.y + q.y, p.z + q.z};
        const V3<T> Y{fma(sy, t.x, r.x), fma(sy, t.y, r.y), fma(sy, t.z, r.z)};
        return fma(T(2.0), fabs(dot3(X, Y)), dot3_acc(Y, Y, dot3(X, X)));
    };
    const T f1 = pair(C.c23, C.c45, b, a, T(-1.0));   // Y1 = b - a
    const T f2 = pair(C.c31, C.c64, c, a, T(1.0));    // Y2 = c + a
    const T f3 = pair(C.c12, C.c56, c, b, T(1.0));    // |Y3| = |c + b|
    if constexpr (std::is_same<T, double>::value) {
        // the three are >= 0, so their bit patterns order like the values:
        // compare those on the integer pipes instead of two FP64 max slots
        unsigned long long k1, k2, k3;
        asm("mov.b64 %0, %1;" : "=l"(k1) : "d"(f1));
        asm("mov.b64 %0, %1;" : "=l"(k2) : "d"(f2));
        asm("mov.b64 %0, %1;" : "=l"(k3) : "d"(f3));
        const T m12 = k1 > k2 ? f1 : f2;
        return (k1 > k2 ? k1 : k2) > k3 ? m12 : f3;
    } else {
        return fmax(fmax(f1, f2), f3);
    }
}

// The strain rate tr(grad v) at the half step (CalcElemVelocityGrandient +
// trace, LULESH-OMP.cc:1864-1925, 1975-2020): the half-step Jacobian has
// columns (M - dt2 Mv)/8 for the position modes M1..M3 and velocity modes
// V1..V3, and the trace is sum(cofactor . velocity mode) / det.
template <typename T>
__device__ __forceinline__ T strain_rate(const V3<T> &M1, const V3<T> &M2, const V3<T> &M3, const V3<T> &V1,
                                         const V3<T> &V2, const V3<T> &V3m, T dt2)
{
    const V3<T> A{M1.x - dt2 * V1.x, M1.y - dt2 * V1.y, M1.z - dt2 * V1.z};
    const V3<T> B{M2.x - dt2 * V2.x, M2.y - dt2 * V2.y, M2.z - dt2 * V2.z};
    const V3<T> C{M3.x - dt2 * V3m.x, M3.y - dt2 * V3m.y, M3.z - dt2 * V3m.z};
    const V3<T> cxi = cross3(B, C), cet = cross3(C, A), cze = cross3(A, B);
    const T num = dot3_acc(cze, V3m, dot3_acc(cet, V2, dot3(cxi, V1)));
    return quot_fast(num, dot3(B, cet));
}

}  // namespace lulesh
