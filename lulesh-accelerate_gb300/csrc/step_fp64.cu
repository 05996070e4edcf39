// step_fp64.cu -- the plain FP64 Lagrange leapfrog step on sm_103a.
//
// One cycle is six launches on one stream:
//   k_time_increment   1 thread   TimeIncrement                (LULESH-OMP.cc:557-604)
//   k_elem_force       1 thr/elem IntegrateStressForElems + CalcHourglassControlForElems
//                                 + CalcFBHourglassForceForElems, element half
//                                 (:853-931, :1233-1558): 8 corner forces (stress
//                                 plus hourglass) per element, corner-major SoA
//   k_node_update      1 thr/node the corner gather (:905-926, :1475-1496) in
//                                 nodeElemCornerList order, CalcAccelerationForNodes,
//                                 the symmetry-plane conditions, velocity and position
//                                 (:1613-1683)
//   k_elem_kinematics  1 thr/elem CalcKinematicsForElems + CalcLagrangeElements +
//                                 CalcMonotonicQGradientsForElems (:1927-2180); keeps
//                                 the element geometry (Walsh modes and cross products
//                                 of the new positions) for the next k_elem_force
//   k_elem_material    1 thr/elem CalcMonotonicQRegionForElems, the qstop test,
//                                 ApplyMaterialPropertiesForElems / EvalEOSForElems /
//                                 CalcEnergyForElems / CalcSoundSpeedForElems,
//                                 UpdateVolumesForElems and the Courant/hydro
//                                 constraint minima (:2182-2933)
//   k_finalize         1 thread   publishes dtcourant/dthydro (k_run_epilogue in the
//                                 run loop, which also decides whether another cycle
//                                 follows)
// No floating-point atomics: node sums run in the reference's fixed corner
// order and the constraint minima use an order-independent integer min.
#include "lulesh_internal.h"
#include "kernels.h"
#include "hexmodes.cuh"
#include "common.cuh"
#include "batch_kernels.cuh"

#include <cuda_runtime.h>

namespace lulesh {

// ---------------------------------------------------------------------
// TimeIncrement (LULESH-OMP.cc:557-604)
// ---------------------------------------------------------------------
__global__ void k_time_increment(const __grid_constant__ Dom d)
{
    if (skip_step(d)) return;
    time_increment(d.sc, d.prm);
}

// ---------------------------------------------------------------------
// Geometry cache (Dom::geo): modes M1..M7 of x, y, z, then the six shared
// cross products, one word per element per plane
// ---------------------------------------------------------------------
__device__ __forceinline__ void store_geometry(double *__restrict__ g, size_t ne, int k, const double mx[7],
                                               const double my[7], const double mz[7], const ModeCrosses<double> &X)
{
#pragma unroll
    for (int i = 0; i < 7; ++i) {
        g[(3 * i + 0) * ne + k] = mx[i];
        g[(3 * i + 1) * ne + k] = my[i];
        g[(3 * i + 2) * ne + k] = mz[i];
    }
    const V3<double> c[6] = {X.c23, X.c31, X.c12, X.c45, X.c64, X.c56};
#pragma unroll
    for (int i = 0; i < 6; ++i) {
        g[(21 + 3 * i) * ne + k] = c[i].x;
        g[(22 + 3 * i) * ne + k] = c[i].y;
        g[(23 + 3 * i) * ne + k] = c[i].z;
    }
}

__device__ __forceinline__ void load_geometry(const double *__restrict__ g, size_t ne, int k, double mx[7],
                                              double my[7], double mz[7], ModeCrosses<double> &X)
{
#pragma unroll
    for (int i = 0; i < 7; ++i) {
        mx[i] = __ldg(g + (3 * i + 0) * ne + k);
        my[i] = __ldg(g + (3 * i + 1) * ne + k);
        mz[i] = __ldg(g + (3 * i + 2) * ne + k);
    }
    V3<double> c[6];
#pragma unroll
    for (int i = 0; i < 6; ++i)
        c[i] = {__ldg(g + (21 + 3 * i) * ne + k), __ldg(g + (22 + 3 * i) * ne + k), __ldg(g + (23 + 3 * i) * ne + k)};
    X = {c[0], c[1], c[2], c[3], c[4], c[5]};
}

// ---------------------------------------------------------------------
// Element force: stress + Flanagan-Belytschko hourglass
// ---------------------------------------------------------------------
__device__ __forceinline__ void elem_force_fp64(const Dom &d, int k, DevScalars *sc)
{
    const size_t ne = (size_t)d.ne;
    int nl[8];
    load_nodelist(d.nodelist, k, nl);
    // The Walsh modes of the corner coordinates and their shared cross
    // products: left by the previous cycle's kinematics kernel for these
    // same positions when it kept them (the same functions of the same
    // values, so the same bits), else formed here.  The node update that
    // follows moves the positions and clears the mark.
    double mx[7], my[7], mz[7];
    ModeCrosses<double> X;
    if (d.geo && sc->geo_valid) {
        load_geometry(d.geo, ne, k, mx, my, mz, X);
    } else {
        double x[8], y[8], z[8];
        gather8(d.x, nl, x);
        gather8(d.y, nl, y);
        gather8(d.z, nl, z);
        walsh8(x, mx);
        walsh8(y, my);
        walsh8(z, mz);
        X = mode_crosses(mode(mx, my, mz, 0), mode(mx, my, mz, 1), mode(mx, my, mz, 2), mode(mx, my, mz, 3),
                         mode(mx, my, mz, 4), mode(mx, my, mz, 5));
    }
    const V3<double> M1 = mode(mx, my, mz, 0), M2 = mode(mx, my, mz, 1), M3 = mode(mx, my, mz, 2);
    const V3<double> M4 = mode(mx, my, mz, 3), M5 = mode(mx, my, mz, 4), M6 = mode(mx, my, mz, 5);
    double dvdx[8], dvdy[8], dvdz[8];
    V3<double> nx[3];
    force_geometry(M1, M2, M3, M4, M5, M6, X, dvdx, dvdy, dvdz, nx);   // 192 x dV/dx, normal generators

    // IntegrateStressForElems (LULESH-OMP.cc:853-903): sig = -p - q and the
    // corner force -sig * (area-weighted node normal).  The normal of the
    // corner with signs s is (s_xi X1 + s_eta X2 + s_zeta X3)/64, so the
    // stress forces are s . (Y1, Y2, Y3) with Y = ((p + q)/64) X, and those
    // of corners 4..7 are the forces of corners 2, 3, 0, 1 negated.  The
    // Jacobian volume it checks is 8 t.(c x a) = M2.(M3 x M1) / 64; only its
    // sign matters.
    double Y[3][3];
    {
        const double w = (1.0 / 64.0) * (d.p[k] + d.q[k]);
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            Y[i][0] = w * nx[i].x;
            Y[i][1] = w * nx[i].y;
            Y[i][2] = w * nx[i].z;
        }
        const double determ64 = dot3(M2, X.c31);
        if (determ64 <= 0.0) flag_error(sc, ERR_K1_DETERM, k);
    }
    // stress force of corners 0..3 in one component (corners 4..7: 2, 3,
    // 0, 1 negated)
    auto stress4 = [&](int dim, double f[4]) {
        const double a = Y[0][dim] + Y[1][dim], b = Y[0][dim] - Y[1][dim], z = Y[2][dim];
        f[0] = -(a + z);   // (-,-,-)
        f[1] = b - z;      // (+,-,-)
        f[2] = a - z;      // (+,+,-)
        f[3] = -(b + z);   // (-,+,-)
    };
    double *out[3] = {d.fcx, d.fcy, d.fcz};

    // CalcHourglassControlForElems (:1503-1558)
    const double vk = d.v[k];
    const double determ = d.volo[k] * vk;
    if (vk <= 0.0) flag_error(sc, ERR_K1_VOLUME, k);

    const double hourg = d.prm.hgcoef;
    if (!gt(hourg, 0.0)) {
#pragma unroll
        for (int dim = 0; dim < 3; ++dim) {
            double f[4];
            stress4(dim, f);
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                out[dim][c * ne + k] = f[c];
                out[dim][(c ^ 6) * ne + k] = neg(f[c]);
            }
        }
        return;
    }

    // CalcFBHourglassForceForElems (:1291-1473): hourgam = gamma -
    // volinv * (dV/dx . hourmod), with hourmod the gamma projections of the
    // coordinates (modes M6, M5, M4, M7).
    const double r = rcbrt_fast(determ);                    // determ^(-1/3)
    const double volinv192 = (r * r * r) * (1.0 / 192.0);   // the 1/192 of the derivative
    double hg[8][4];
    {
        const V3<double> M7 = mode(mx, my, mz, 6);
        const V3<double> H[4] = {M6, M5, M4, M7};
        const double gam[4][8] = {
            { 1.,  1., -1., -1., -1., -1.,  1.,  1.},
            { 1., -1., -1.,  1., -1.,  1.,  1., -1.},
            { 1., -1.,  1., -1.,  1., -1.,  1., -1.},
            {-1.,  1., -1.,  1.,  1., -1.,  1., -1.}};
#pragma unroll
        for (int m = 0; m < 4; ++m) {
            // the projection enters negated, so gamma is the addend of the
            // three fused multiply-adds
            const double hx = -(volinv192 * H[m].x), hy = -(volinv192 * H[m].y), hz = -(volinv192 * H[m].z);
#pragma unroll
            for (int c = 0; c < 8; ++c)
                hg[c][m] = fma(dvdz[c], hz, fma(dvdy[c], hy, fma(dvdx[c], hx, gam[m][c])));
        }
    }
    const double coefficient = -hourg * 0.01 * d.ss[k] * d.elem_mass[k] * r;

    // CalcElemFBHourglassForce (:1050-1231), one velocity component at a
    // time; each corner's stress force is the addend of its hourglass sum
    // (the reference adds the two node sums instead, :905-926 and
    // :1475-1496: the same total up to rounding, with one gather instead of
    // two)
    const double *vel[3] = {d.xd, d.yd, d.zd};
#pragma unroll
    for (int dim = 0; dim < 3; ++dim) {
        double u[8];
        gather8(vel[dim], nl, u);
        double h[4];
#pragma unroll
        for (int m = 0; m < 4; ++m) {
            double acc = hg[0][m] * u[0];
#pragma unroll
            for (int c = 1; c < 8; ++c) acc = acc + hg[c][m] * u[c];
            h[m] = coefficient * acc;
        }
        double f[4];
        stress4(dim, f);
        const double st[8] = {f[0], f[1], f[2], f[3], -f[2], -f[3], -f[0], -f[1]};
#pragma unroll
        for (int c = 0; c < 8; ++c)
            out[dim][c * ne + k] = (((st[c] + hg[c][0] * h[0]) + hg[c][1] * h[1]) + hg[c][2] * h[2]) + hg[c][3] * h[3];
    }
}

__global__ void __launch_bounds__(kBlockElem, 4) k_elem_force(const __grid_constant__ Dom d)
{
    if (skip_step(d)) return;
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= d.ne) return;
    elem_force_fp64(d, k, d.sc);
}

// ---------------------------------------------------------------------
// Node update: fixed-order corner gather + acceleration, BC, velocity,
// position
// ---------------------------------------------------------------------
__device__ __forceinline__ void node_update_fp64(const Dom &d, int n, const DevScalars *sc)
{

    // the sums start from the first corner rather than from 0.0 (the same
    // value: x + 0.0 == x, up to the sign of a zero sum), one FP64 add fewer
    // per component; every node belongs to at least one element
    double fx = 0.0, fy = 0.0, fz = 0.0;
    for_node_corners(d, sc, n, [&](int c, bool first) {
        if (first) {
            fx = d.fcx[c];
            fy = d.fcy[c];
            fz = d.fcz[c];
        } else {
            fx += d.fcx[c];
            fy += d.fcy[c];
            fz += d.fcz[c];
        }
    });
    node_integrate(d, n, sc, fx, fy, fz);
}

__global__ void __launch_bounds__(kBlockNode) k_node_update(const __grid_constant__ Dom d)
{
    if (skip_step(d)) return;
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= d.nn) return;
    if (n == 0 && d.geo) d.sc->geo_valid = 0;   // the positions move: the geometry cache goes stale
    node_update_fp64(d, n, d.sc);
}

// ---------------------------------------------------------------------
// Element kinematics + monotonic-Q gradients
// ---------------------------------------------------------------------
__device__ __forceinline__ void elem_kinematics_fp64(const Dom &d, int k, DevScalars *sc)
{
    int nl[8];
    load_nodelist(d.nodelist, k, nl);
    double x[8], y[8], z[8];
    gather8(d.x, nl, x);
    gather8(d.y, nl, y);
    gather8(d.z, nl, z);
    double mx[7], my[7], mz[7];
    walsh8(x, mx);
    walsh8(y, my);
    walsh8(z, mz);
    const V3<double> M1 = mode(mx, my, mz, 0), M2 = mode(mx, my, mz, 1), M3 = mode(mx, my, mz, 2);
    double vx[3], vy[3], vz[3];
    {
        double u[8];
        gather8(d.xd, nl, u);
        walsh_linear(u, vx);
        gather8(d.yd, nl, u);
        walsh_linear(u, vy);
        gather8(d.zd, nl, u);
        walsh_linear(u, vz);
    }
    const V3<double> V1{vx[0], vy[0], vz[0]}, V2{vx[1], vy[1], vz[1]}, V3v{vx[2], vy[2], vz[2]};

    // CalcKinematicsForElems, volume part (:1950-1964)
    const V3<double> M4 = mode(mx, my, mz, 3), M5 = mode(mx, my, mz, 4), M6 = mode(mx, my, mz, 5);
    const ModeCrosses<double> X = mode_crosses(M1, M2, M3, M4, M5, M6);
    // The next cycle's force kernel works on these same positions.  Every
    // context that runs this kernel keeps the cache (only the nodal-only
    // entry point has none), and the store is unconditional: behind a branch
    // the compiler formed the cross products twice (36 more FP64 operations).
    store_geometry(d.geo, (size_t)d.ne, k, mx, my, mz, X);
    if (k == sc->elem_begin) sc->geo_valid = 1;
    const double volo = d.volo[k];
    const double vol64 = volume64_shared(M1, M2, M3, X);
    const double volume = vol64 * (1.0 / 64.0);
    // volume / volo, as a product with the reciprocal taken at set-up (within
    // an ulp of the quotient)
    const double rel = volume * __ldg(d.inv_volo + k);
    d.vnew[k] = rel;
    d.delv[k] = rel - d.v[k];
    // CalcElemCharacteristicLength (:1821-1862): 4V / sqrt(max AreaFace) with
    // AreaFace = 4|u x v|^2 = (64 |u x v|^2) / 16
    d.arealg[k] = (0.25 * vol64) * rsqrt(max_face_cross2_64(M1, M2, M3, M4, M5, M6, X));
    if (rel <= 0.0) flag_error(sc, ERR_K3_VNEW, k);

    // CalcMonotonicQGradientsForElems (:2034-2180): the logical differences
    // are M/4, so each cross product is (M x M')/16 and each velocity
    // difference Mv/4.
    {
        const double ptiny = 1.e-36;
        const double vol = volo * rel;
        // (1/16) (1/4) / (vol + ptiny), the power-of-two scale taken inside
        const double vscale = rcp_fast(fma(vol, 64.0, 64.0 * ptiny));
        const V3<double> &Az = X.c12, &Ax = X.c23, &Ae = X.c31;
        d.delx_zeta[k] = vol * rsqrt(0.00390625 * dot3(Az, Az) + ptiny);
        d.delv_zeta[k] = vscale * dot3(Az, V3v);
        d.delx_xi[k] = vol * rsqrt(0.00390625 * dot3(Ax, Ax) + ptiny);
        d.delv_xi[k] = vscale * dot3(Ax, V1);
        d.delx_eta[k] = vol * rsqrt(0.00390625 * dot3(Ae, Ae) + ptiny);
        d.delv_eta[k] = vscale * dot3(Ae, V2);
    }

    // CalcKinematicsForElems, strain-rate part (:1975-2020)
    d.vdov[k] = strain_rate(M1, M2, M3, V1, V2, V3v, 0.5 * sc->deltatime);
}

__global__ void __launch_bounds__(kBlockElem) k_elem_kinematics(const __grid_constant__ Dom d)
{
    if (skip_step(d)) return;
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= d.ne) return;
    elem_kinematics_fp64(d, k, d.sc);
}

// ---------------------------------------------------------------------
// Q limiter + EOS + volume update + time constraints
// ---------------------------------------------------------------------

// Monotonic-Q region + material update of element k; with kConstraints the
// element's Courant/hydro keys are returned in kc/kh.
template <bool kConstraints>
__device__ __forceinline__ void elem_material_fp64(const Dom &d, int k, DevScalars *sc,
                                                   unsigned long long &kc, unsigned long long &kh)
{
    const lulesh_params &P = d.prm;
    {
        // CalcMonotonicQRegionForElems (:2182-2320)
        const int bc = __ldg(d.elem_bc + k);
        const FaceNeighbours nb = face_neighbours(d, sc, k);
        const double lim = P.monoq_limiter_mult, maxs = P.monoq_max_slope;
        const double phixi = limiter_phi(d.delv_xi, k, bc & BC_XI_M, bc & BC_XI_P, BC_XI_M_SYMM,
                                         BC_XI_M_FREE, BC_XI_P_SYMM, BC_XI_P_FREE,
                                         nb.xim, nb.xip, lim, maxs);
        const double phieta = limiter_phi(d.delv_eta, k, bc & BC_ETA_M, bc & BC_ETA_P, BC_ETA_M_SYMM,
                                          BC_ETA_M_FREE, BC_ETA_P_SYMM, BC_ETA_P_FREE,
                                          nb.etam, nb.etap, lim, maxs);
        const double phizeta = limiter_phi(d.delv_zeta, k, bc & BC_ZETA_M, bc & BC_ZETA_P,
                                           BC_ZETA_M_SYMM, BC_ZETA_M_FREE, BC_ZETA_P_SYMM,
                                           BC_ZETA_P_FREE, nb.zetam, nb.zetap,
                                           lim, maxs);
        const double vnew = d.vnew[k], volo = d.volo[k], vdov = d.vdov[k];
        double qlin, qquad;
        if (gt(vdov, 0.)) {
            qlin = 0.;
            qquad = 0.;
        } else {
            double dxi = d.delv_xi[k] * d.delx_xi[k];
            double deta = d.delv_eta[k] * d.delx_eta[k];
            double dzeta = d.delv_zeta[k] * d.delx_zeta[k];
            if (gt(dxi, 0.)) dxi = 0.;
            if (gt(deta, 0.)) deta = 0.;
            if (gt(dzeta, 0.)) dzeta = 0.;
            const double rho = quot_fast(d.elem_mass[k], volo * vnew);
            qlin = -P.qlc_monoq * rho *
                   ((dxi * (1. - phixi) + deta * (1. - phieta)) + dzeta * (1. - phizeta));
            qquad = P.qqc_monoq * rho *
                    ((dxi * dxi * (1. - phixi * phixi) + deta * deta * (1. - phieta * phieta)) +
                     dzeta * dzeta * (1. - phizeta * phizeta));
        }
        if (d.keep & 2) {
            d.ql[k] = qlin;
            d.qq[k] = qquad;
        }

        const double ssn = material_update(d, k, sc, vnew, qlin, qquad, d.reps ? __ldg(d.reps + k) : 1);

        if (kConstraints) constraint_keys(ssn, vdov, d.arealg[k], P, kc, kh);
    }
}

template <bool kConstraints>
__global__ void __launch_bounds__(kBlockElem) k_elem_material(const __grid_constant__ Dom d)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    unsigned long long kc = ~0ULL, kh = ~0ULL;
    if (t < d.ne && !skip_step(d)) {
        // with regions, threads take elements in cost-grouped order (the
        // reference's region element lists, lulesh-2.0.3/lulesh.cc:2410-2424)
        const int k = d.mat_order ? __ldg(d.mat_order + t) : t;
        elem_material_fp64<kConstraints>(d, k, d.sc, kc, kh);
    }
    if (kConstraints) block_min_publish(kc, kh, d.sc);
}

// CalcTimeConstraintsForElems on its own (:2935-2942).
__global__ void __launch_bounds__(kBlockElem) k_time_constraints(const __grid_constant__ Dom d)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    unsigned long long kc = ~0ULL, kh = ~0ULL;
    if (k < d.ne && !skip_step(d)) {
        if (d.df == kArithDF64) constraint_keys_df(d.ss[k], d.vdov[k], d.arealg[k], d.prm, kc, kh);
        else constraint_keys(d.ss[k], d.vdov[k], d.arealg[k], d.prm, kc, kh);
    }
    block_min_publish(kc, kh, d.sc);
}

__global__ void k_finalize(const __grid_constant__ Dom d)
{
    finalize_constraints(d.sc);
}

__global__ void k_run_prologue(const __grid_constant__ Dom d, const int *max_cycles,
                               cudaGraphConditionalHandle handle, int *active)
{
    d.sc->run_cycles = 0;
    d.sc->run_max = *max_cycles;
    const unsigned go = run_continue(d.sc, d.prm);
    *active = (int)go;
    if (handle) cudaGraphSetConditional(handle, go);
}

__global__ void k_run_epilogue(const __grid_constant__ Dom d, cudaGraphConditionalHandle handle,
                               int *active)
{
    if (!*active) return;
    finalize_constraints(d.sc);
    d.sc->run_cycles++;
    const unsigned go = run_continue(d.sc, d.prm);
    *active = (int)go;
    if (handle) cudaGraphSetConditional(handle, go);
}


// ---------------------------------------------------------------------
// Launchers
// ---------------------------------------------------------------------
static inline unsigned blocks_for(long n, int bs) { return (unsigned)((n + bs - 1) / bs); }

void launch_time_increment(const Dom &d, cudaStream_t st)
{
    k_time_increment<<<1, 1, 0, st>>>(d);
}

// Dom::df: kArithDF64 the element geometry and forces in double-float
// (step_df.cu), kArithIEEE every operation in FP64 (this file's kernels)
static void launch_elem_force(const Dom &d, cudaStream_t st)
{
    if (d.df == kArithDF64) launch_elem_force_df(d, st);
    else k_elem_force<<<blocks_for(d.ne, elem_block(d)), elem_block(d), 0, st>>>(d);
}

static void launch_node_update(const Dom &d, cudaStream_t st)
{
    if (d.df == kArithDF64) launch_node_update_df(d, st);
    else k_node_update<<<blocks_for(d.nn, node_block(d)), node_block(d), 0, st>>>(d);
}

static void launch_elem_kinematics(const Dom &d, cudaStream_t st)
{
    if (d.df == kArithDF64) launch_elem_kinematics_df(d, st);
    else k_elem_kinematics<<<blocks_for(d.ne, elem_block(d)), elem_block(d), 0, st>>>(d);
}

void launch_lagrange_nodal(const Dom &d, cudaStream_t st)
{
    launch_elem_force(d, st);
    launch_node_update(d, st);
}

void launch_lagrange_elements(const Dom &d, cudaStream_t st, bool with_constraints)
{
    launch_elem_kinematics(d, st);
    if (d.df == kArithDF64)
        launch_elem_material_df(d, st, with_constraints);
    else if (with_constraints)
        k_elem_material<true><<<blocks_for(d.ne, elem_block(d)), elem_block(d), 0, st>>>(d);
    else
        k_elem_material<false><<<blocks_for(d.ne, elem_block(d)), elem_block(d), 0, st>>>(d);
}

void launch_time_constraints(const Dom &d, cudaStream_t st)
{
    k_time_constraints<<<blocks_for(d.ne, elem_block(d)), elem_block(d), 0, st>>>(d);
    k_finalize<<<1, 1, 0, st>>>(d);
}

void launch_finalize(const Dom &d, cudaStream_t st)
{
    k_finalize<<<1, 1, 0, st>>>(d);
}

void launch_run_epilogue(const Dom &d, cudaStream_t st, cudaGraphConditionalHandle h, int *active)
{
    k_run_epilogue<<<1, 1, 0, st>>>(d, h, active);
}

void launch_run_prologue(const Dom &d, cudaStream_t st, const int *max_cycles,
                         cudaGraphConditionalHandle h, int *active)
{
    k_run_prologue<<<1, 1, 0, st>>>(d, max_cycles, h, active);
}

// One cycle of the run loop.  In the graph with a conditional while node
// d.gate is null and the node stops the loop; in the host-driven fallback
// d.gate == active and the cycles after the last one return at once.
void launch_run_body(const Dom &d, cudaStream_t st, cudaGraphConditionalHandle h, int *active)
{
    k_time_increment<<<1, 1, 0, st>>>(d);
    launch_lagrange_nodal(d, st);
    launch_lagrange_elements(d, st, true);
    k_run_epilogue<<<1, 1, 0, st>>>(d, h, active);
}

int kernels_per_cycle() { return 6; }

// Kernels of one cycle launched one by one, with an event recorded before
// each (ev[0..6]); for per-kernel timing.
void launch_cycle_timed(const Dom &d, cudaStream_t st, cudaEvent_t ev[7])
{
    cudaEventRecord(ev[0], st);
    k_time_increment<<<1, 1, 0, st>>>(d);
    cudaEventRecord(ev[1], st);
    launch_elem_force(d, st);
    cudaEventRecord(ev[2], st);
    launch_node_update(d, st);
    cudaEventRecord(ev[3], st);
    launch_elem_kinematics(d, st);
    cudaEventRecord(ev[4], st);
    if (d.df == kArithDF64) launch_elem_material_df(d, st, true);
    else k_elem_material<true><<<blocks_for(d.ne, elem_block(d)), elem_block(d), 0, st>>>(d);
    cudaEventRecord(ev[5], st);
    k_finalize<<<1, 1, 0, st>>>(d);
    cudaEventRecord(ev[6], st);
}

// FP64 issue-rate probe: independent FMA chains, 8 per thread.
__global__ void k_fp64_probe(double *out, int iters, double a, double b)
{
    double r[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) r[j] = threadIdx.x * 1e-3 + j;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int j = 0; j < 8; ++j) r[j] = fma(r[j], a, b);
    }
    double s = 0.0;
#pragma unroll
    for (int j = 0; j < 8; ++j) s += r[j];
    if (s == 12345.678) out[0] = s;   // keeps the chains live
}

void launch_fp64_probe(double *out, int blocks, int threads, int iters, cudaStream_t st)
{
    k_fp64_probe<<<blocks, threads, 0, st>>>(out, iters, 0.999999, 1e-7);
}

// Accuracy probe of the FP64 root and reciprocal functions against CUDA's.
// Arguments 2^(280 u - 140) (1 + v) over a grid of u, v (both sides of the
// range the fastmath.cuh functions refine, and its fallbacks); the relative
// differences of rcbrt_fast from rcbrt, x*rsqrt(x) from sqrt, rcp_fast from
// __drcp_rn and quot_fast(a, x) from a / x, reduced as the bit patterns of
// non-negative doubles (which order like the values).
__global__ void k_math_probe(unsigned long long *keys, int n)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double u = (double)(i >> 10) / 1024.0, v = (double)(i & 1023) / 1024.0;
    const double x = ldexp(1.0 + v, (int)(280.0 * u) - 140);
    const double num = (i & 1) ? -(1.0 + u) : 0.75 + v;
    const double rel[4] = {
        fabs(rcbrt_fast(x) - rcbrt(x)) / rcbrt(x),
        fabs(x * rsqrt(x) - sqrt(x)) / sqrt(x),
        fabs(rcp_fast(x) - __drcp_rn(x)) / __drcp_rn(x),
        fabs(quot_fast(num, x) - num / x) / fabs(num / x)};
#pragma unroll
    for (int j = 0; j < 4; ++j) atomicMax(keys + j, (unsigned long long)__double_as_longlong(rel[j]));
}

void launch_math_probe(unsigned long long *keys, int n, cudaStream_t st)
{
    k_math_probe<<<(n + 255) / 256, 256, 0, st>>>(keys, n);
}

// Issue-rate probes: 8 independent chains per thread of one operation; each
// thread writes one value (keeps the chains live).
__global__ void k_probe_ffma(float *out, int iters, float a, float b)
{
    float r[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) r[j] = threadIdx.x * 1e-3f + j;
    for (int i = 0; i < iters; ++i)
#pragma unroll
        for (int j = 0; j < 8; ++j) r[j] = fmaf(r[j], a, b);
    float s = 0.f;
#pragma unroll
    for (int j = 0; j < 8; ++j) s += r[j];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

// double -> float conversions (each iteration: one conversion, one DADD).
__global__ void k_probe_d2f(float *out, int iters, double a)
{
    double r[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) r[j] = threadIdx.x * 1e-3 + j;
    float acc = 0.f;
    for (int i = 0; i < iters; ++i)
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            acc += __double2float_rn(r[j]);
            r[j] += a;
        }
    out[blockIdx.x * blockDim.x + threadIdx.x] = acc;
}

// correctly rounded FP64 division
__global__ void k_probe_ddiv(float *out, int iters, double a)
{
    double r[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) r[j] = threadIdx.x * 1e-3 + j + 1.0;
    for (int i = 0; i < iters; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) r[j] = a / r[j];
    double s = 0.0;
#pragma unroll
    for (int j = 0; j < 4; ++j) s += r[j];
    out[blockIdx.x * blockDim.x + threadIdx.x] = (float)s;
}

void launch_rate_probe(int which, float *out, int blocks, int threads, int iters, cudaStream_t st)
{
    switch (which) {
    case 0: k_probe_ffma<<<blocks, threads, 0, st>>>(out, iters, 0.9999f, 1e-7f); break;
    case 1: k_probe_d2f<<<blocks, threads, 0, st>>>(out, iters, 1e-9); break;
    default: k_probe_ddiv<<<blocks, threads, 0, st>>>(out, iters, 1.2345); break;
    }
}

// ---------------------------------------------------------------------
// Batched ensembles: the same bodies over the active tiles of one class
// ---------------------------------------------------------------------
void launch_batch_kernel_fp64(const Dom &d, const BatchView &b, cudaStream_t st, int kernel, int cls,
                              LaunchCfg cfg)
{
    if (d.df == kArithDF64) {
        launch_batch_kernel_df(d, b, st, kernel, cls, cfg);
        return;
    }
    switch (kernel) {
    case 0: kb_elem<elem_force_fp64><<<cfg.grid, cfg.block, 0, st>>>(d, b, cls); break;
    case 1: kb_node<node_update_fp64><<<cfg.grid, cfg.block, 0, st>>>(d, b, cls); break;
    case 2: kb_elem<elem_kinematics_fp64><<<cfg.grid, cfg.block, 0, st>>>(d, b, cls); break;
    default: kb_material<elem_material_fp64<true>><<<cfg.grid, cfg.block, 0, st>>>(d, b, cls); break;
    }
}

// Resident blocks per SM of a batched kernel at a block size.
int batch_max_blocks_fp64(int kernel, int block, int arith)
{
    if (arith == kArithDF64) return batch_max_blocks_df(kernel, block);
    int n = 0;
    cudaError_t e;
    switch (kernel) {
    case 0: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kb_elem<elem_force_fp64>, block, 0); break;
    case 1: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kb_node<node_update_fp64>, block, 0); break;
    case 2: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kb_elem<elem_kinematics_fp64>, block, 0); break;
    default: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kb_material<elem_material_fp64<true>>, block, 0); break;
    }
    return e == cudaSuccess ? n : 0;
}

}  // namespace lulesh
