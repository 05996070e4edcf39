// hourglass_df.cuh -- the Flanagan-Belytschko hourglass forces of one
// element in double-float (CalcFBHourglassForceForElems and
// CalcElemFBHourglassForce, LULESH-OMP.cc:1233-1501, :1050-1231).
//
// This is the bulk of the element force kernel's arithmetic (about 300 of
// its 472 FP64 instructions per element: the hourglass shape vectors, their
// projections on the corner velocities and the corner forces), and the
// hourglass forces are a correction beside the stress forces, so the plain
// FP64 path evaluates them as double-float pairs on the FP32 pipe
// (df64.cuh) and keeps the stress force in FP64.
#pragma once

#include "common.cuh"
#include "hexmodes.cuh"

namespace lulesh {

// hourgam = gamma - volinv (dV/dx . hourmod), with hourmod the projections
// of the coordinates on the gamma vectors (the modes H = M6, M5, M4, M7);
// then for each velocity component u the corner forces
// coefficient * hourgam (hourgam^T u).  dvd*: 192 x dV/dx per corner,
// volinv192 = determ^-1 / 192, coefficient = -hgcoef 0.01 ss mass
// determ^-1/3.  emit(dim, hgf) receives the 8 corner forces of one
// component.
template <class Emit>
__device__ __forceinline__ void fb_hourglass_df(const Dom &d, const int nl[8], const df64 dvdx[8],
                                                const df64 dvdy[8], const df64 dvdz[8], const V3<df64> H[4],
                                                df64 volinv192, df64 coefficient, Emit &&emit)
{
    // gamma (LULESH-OMP.cc:1252-1285): the sign patterns eta zeta, xi zeta,
    // xi eta and xi eta zeta of the corners
    const float gam[4][8] = {
        { 1.f,  1.f, -1.f, -1.f, -1.f, -1.f,  1.f,  1.f},
        { 1.f, -1.f, -1.f,  1.f, -1.f,  1.f,  1.f, -1.f},
        { 1.f, -1.f,  1.f, -1.f,  1.f, -1.f,  1.f, -1.f},
        {-1.f,  1.f, -1.f,  1.f,  1.f, -1.f,  1.f, -1.f}};
    df64 hg[8][4];
#pragma unroll
    for (int m = 0; m < 4; ++m) {
        // the projection enters negated, so gamma is the addend of the
        // three multiply-adds
        const df64 hx = -(volinv192 * H[m].x), hy = -(volinv192 * H[m].y), hz = -(volinv192 * H[m].z);
#pragma unroll
        for (int c = 0; c < 8; ++c) {
            DfDot acc(df64(gam[m][c], 0.f));
            acc.add(dvdx[c], hx);
            acc.add(dvdy[c], hy);
            acc.add(dvdz[c], hz);
            hg[c][m] = acc.value();
        }
    }
    // One velocity component per iteration, the loop kept rolled: the body is
    // the same code three times over, and the smaller instruction footprint
    // ran the force kernel 5 % faster at s=192 (2.09 -> 1.99 ms).  Each
    // iteration issues the next component's corner gather before its own
    // arithmetic, so those loads are in flight while it computes
    // (1.87 -> 1.82 ms; staging all 24 in shared memory at the start instead
    // ran at 2.03).
    double un[8];
    gather8(d.xd, nl, un);
#pragma unroll 1
    for (int dim = 0; dim < 3; ++dim) {
        df64 u[8];
#pragma unroll
        for (int c = 0; c < 8; ++c) u[c] = to_df(un[c]);
        if (dim < 2) gather8(dim == 0 ? d.yd : d.zd, nl, un);
        df64 h[4];
#pragma unroll
        for (int m = 0; m < 4; ++m) {
            DfDot acc(df64(0.f, 0.f));
#pragma unroll
            for (int c = 0; c < 8; ++c) acc.add(hg[c][m], u[c]);
            h[m] = coefficient * acc.value();
        }
        df64 f[8];
#pragma unroll
        for (int c = 0; c < 8; ++c) {
            DfDot acc(df64(0.f, 0.f));
#pragma unroll
            for (int m = 0; m < 4; ++m) acc.add(hg[c][m], h[m]);
            f[c] = acc.value();
        }
        emit(dim, f);
    }
}

}  // namespace lulesh
