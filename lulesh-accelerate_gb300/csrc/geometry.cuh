// geometry.cuh -- per-element hexahedron geometry in FP64, device side.
//
// Each function keeps the floating-point association of the reference
// routine it restates (reference/C/LULESH-OMP.cc, lines cited per function);
// only multiply-add contraction, which nvcc applies by default, differs.
#pragma once

namespace lulesh {

// Jacobian columns of one coordinate at the element centre, scaled by 1/8
// (LULESH-OMP.cc:650-660).
template <typename T>
__device__ __forceinline__ void jac_column(const T c[8], T &xi, T &et, T &ze)
{
    const T d60 = c[6] - c[0], d53 = c[5] - c[3];
    const T d71 = c[7] - c[1], d42 = c[4] - c[2];
    xi = T(.125) * (((d60 + d53) - d71) - d42);
    et = T(.125) * (((d60 - d53) + d71) - d42);
    ze = T(.125) * (((d60 + d53) + d71) + d42);
}

// Jacobian volume only (the determinant IntegrateStressForElems checks).
template <typename T>
__device__ __forceinline__ T jacobian_volume(const T x[8], const T y[8], const T z[8])
{
    T a[3], t[3], c[3];
    jac_column(x, a[0], t[0], c[0]);
    jac_column(y, a[1], t[1], c[1]);
    jac_column(z, a[2], t[2], c[2]);
    const T cet0 = (a[2] * c[1]) - (a[1] * c[2]);
    const T cet1 = (a[0] * c[2]) - (a[2] * c[0]);
    const T cet2 = (a[1] * c[0]) - (a[0] * c[1]);
    return T(8.0) * ((t[0] * cet0 + t[1] * cet1) + t[2] * cet2);
}

// Node normals from the face diagonals, for the split-precision step.  For a
// face (n0,n1,n2,n3) the reference's quarter-area vector
// 0.25*(b0 x b1), with bisectors b0 = (u+v)/2, b1 = (u-v)/2 of the diagonals
// u = x[n2]-x[n0], v = x[n3]-x[n1], equals 0.125*(v x u): the same value with
// 12 operations instead of 27 and no cancellation in the bisector sums.
template <typename T>
__device__ __forceinline__ void face_area_diag(const T x[8], const T y[8], const T z[8],
                                               int n0, int n1, int n2, int n3, T &ax, T &ay, T &az)
{
    const T ux = x[n2] - x[n0], uy = y[n2] - y[n0], uz = z[n2] - z[n0];
    const T vx = x[n3] - x[n1], vy = y[n3] - y[n1], vz = z[n3] - z[n1];
    ax = T(0.125) * (vy * uz - vz * uy);
    ay = T(0.125) * (vz * ux - vx * uz);
    az = T(0.125) * (vx * uy - vy * ux);
}

template <typename T>
__device__ __forceinline__ void node_normals_diag(T pf[3][8], const T x[8], const T y[8], const T z[8])
{
    T a[6][3];
    face_area_diag(x, y, z, 0, 1, 2, 3, a[0][0], a[0][1], a[0][2]);
    face_area_diag(x, y, z, 0, 4, 5, 1, a[1][0], a[1][1], a[1][2]);
    face_area_diag(x, y, z, 1, 5, 6, 2, a[2][0], a[2][1], a[2][2]);
    face_area_diag(x, y, z, 2, 6, 7, 3, a[3][0], a[3][1], a[3][2]);
    face_area_diag(x, y, z, 3, 7, 4, 0, a[4][0], a[4][1], a[4][2]);
    face_area_diag(x, y, z, 4, 7, 6, 5, a[5][0], a[5][1], a[5][2]);
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        pf[d][0] = (a[0][d] + a[1][d]) + a[4][d];
        pf[d][1] = (a[0][d] + a[1][d]) + a[2][d];
        pf[d][2] = (a[0][d] + a[2][d]) + a[3][d];
        pf[d][3] = (a[0][d] + a[3][d]) + a[4][d];
        pf[d][4] = (a[1][d] + a[4][d]) + a[5][d];
        pf[d][5] = (a[1][d] + a[2][d]) + a[5][d];
        pf[d][6] = (a[2][d] + a[3][d]) + a[5][d];
        pf[d][7] = (a[3][d] + a[4][d]) + a[5][d];
    }
}

// VoluDer (LULESH-OMP.cc:978-1006) on six corners given by index.
template <typename T>
__device__ __forceinline__ void volu_der(const T x[8], const T y[8], const T z[8],
                                         int i0, int i1, int i2, int i3, int i4, int i5,
                                         T &dx, T &dy, T &dz)
{
    const T twelfth = T(1.0) / T(12.0);
    const T x0 = x[i0], x1 = x[i1], x2 = x[i2], x3 = x[i3], x4 = x[i4], x5 = x[i5];
    const T y0 = y[i0], y1 = y[i1], y2 = y[i2], y3 = y[i3], y4 = y[i4], y5 = y[i5];
    const T z0 = z[i0], z1 = z[i1], z2 = z[i2], z3 = z[i3], z4 = z[i4], z5 = z[i5];
    const T vx =
        (y1 + y2) * (z0 + z1) - (y0 + y1) * (z1 + z2) +
        (y0 + y4) * (z3 + z4) - (y3 + y4) * (z0 + z4) -
        (y2 + y5) * (z3 + z5) + (y3 + y5) * (z2 + z5);
    const T vy =
        -(x1 + x2) * (z0 + z1) + (x0 + x1) * (z1 + z2) -
        (x0 + x4) * (z3 + z4) + (x3 + x4) * (z0 + z4) +
        (x2 + x5) * (z3 + z5) - (x3 + x5) * (z2 + z5);
    const T vz =
        -(y1 + y2) * (x0 + x1) + (y0 + y1) * (x1 + x2) -
        (y0 + y4) * (x3 + x4) + (y3 + y4) * (x0 + x4) +
        (y2 + y5) * (x3 + x5) - (y3 + y5) * (x2 + x5);
    dx = vx * twelfth;
    dy = vy * twelfth;
    dz = vz * twelfth;
}

// CalcElemVolumeDerivative (LULESH-OMP.cc:1008-1048).
template <typename T>
__device__ __forceinline__ void volume_derivative(T dvdx[8], T dvdy[8], T dvdz[8],
                                                  const T x[8], const T y[8], const T z[8])
{
    volu_der(x, y, z, 1, 2, 3, 4, 5, 7, dvdx[0], dvdy[0], dvdz[0]);
    volu_der(x, y, z, 0, 1, 2, 7, 4, 6, dvdx[3], dvdy[3], dvdz[3]);
    volu_der(x, y, z, 3, 0, 1, 6, 7, 5, dvdx[2], dvdy[2], dvdz[2]);
    volu_der(x, y, z, 2, 3, 0, 5, 6, 4, dvdx[1], dvdy[1], dvdz[1]);
    volu_der(x, y, z, 7, 6, 5, 0, 3, 1, dvdx[4], dvdy[4], dvdz[4]);
    volu_der(x, y, z, 4, 7, 6, 1, 0, 2, dvdx[5], dvdy[5], dvdz[5]);
    volu_der(x, y, z, 5, 4, 7, 2, 1, 3, dvdx[6], dvdy[6], dvdz[6]);
    volu_der(x, y, z, 6, 5, 4, 3, 2, 0, dvdx[7], dvdy[7], dvdz[7]);
}

}  // namespace lulesh
