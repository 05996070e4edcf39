// step_df.cu -- the plain path's element geometry and forces in double-float.
//
// The plain FP64 step is bound by GB300's FP64 pipe (2 FMA per SM per clock),
// not by HBM: ~990 FP64 instructions per zone-cycle against ~1.6 kB moved.
// The element geometry (Walsh modes, cross products, volume derivative, node
// normals, volume, face areas, strain rate) and the stress and
// Flanagan-Belytschko hourglass forces are therefore evaluated here as
// double-float pairs on the FP32 pipe (df64.cuh; ~48 significant bits), with
// the same formulas as the FP64 kernels of step_fp64.cu:
//
//   k_elem_force_df      IntegrateStressForElems + CalcHourglassControlForElems
//                        + CalcFBHourglassForceForElems (LULESH-OMP.cc:853-931,
//                        :1233-1558); corner forces stored as pairs
//   k_node_update_df     the corner gather in nodeElemCornerList order, summed
//                        as pairs and joined once in FP64, then the FP64 node
//                        update (:1613-1683)
//   k_elem_kinematics_df CalcKinematicsForElems + CalcLagrangeElements +
//                        CalcMonotonicQGradientsForElems (:1927-2180); keeps
//                        the geometry as pairs for the next force kernel
//
// What stays FP64: the nodal state (positions, velocities, their update),
// the element state and the whole material kernel (monotonic-Q limiter,
// EOS, energy, pressure, sound speed, volume update) and the time
// constraints, plus the corner-relative differences that every geometric
// quantity starts from: a mode is a signed sum of corner differences, and
// the differences of neighbouring coordinates are exact in FP64, so the
// pairs carry each mode to ~2^-47 of its own size (the FP64 transform of the
// absolute coordinates carries it to 2^-53 of the coordinates).
#include "lulesh_internal.h"
#include "kernels.h"
#include "hexmodes.cuh"
#include "common.cuh"
#include "hourglass_df.cuh"
#include "eos_df.cuh"
#include "batch_kernels.cuh"

#include <cuda_runtime.h>

namespace lulesh {

// Modes M1..M7 of one coordinate of the 8 corners: the corners relative to
// corner 0 formed in FP64 and split into pairs (the modes do not see a
// translation).
__device__ __forceinline__ void rel_modes_df(const double *__restrict__ f, const int nl[8], df64 m[7])
{
    double c[8];
    gather8(f, nl, c);
    df64 r[8];
    r[0] = df64(0.f, 0.f);
#pragma unroll
    for (int i = 1; i < 8; ++i) r[i] = to_df(c[i] - c[0]);
    walsh8(r, m);
}

// The three linear modes of the 8 corner velocities, likewise.
__device__ __forceinline__ void rel_linear_df(const double *__restrict__ f, const int nl[8], df64 m[3])
{
    double c[8];
    gather8(f, nl, c);
    df64 r[8];
    r[0] = df64(0.f, 0.f);
#pragma unroll
    for (int i = 1; i < 8; ++i) r[i] = to_df(c[i] - c[0]);
    walsh_linear(r, m);
}

// Geometry cache as pairs: the layout of step_fp64.cu's store_geometry, one
// float2 per word.
__device__ __forceinline__ void store_geometry_df(double *__restrict__ geo, size_t ne, int k, const df64 mx[7],
                                                  const df64 my[7], const df64 mz[7], const ModeCrosses<df64> &X)
{
    float2 *g = reinterpret_cast<float2 *>(geo);
#pragma unroll
    for (int i = 0; i < 7; ++i) {
        g[(3 * i + 0) * ne + k] = as_float2(mx[i]);
        g[(3 * i + 1) * ne + k] = as_float2(my[i]);
        g[(3 * i + 2) * ne + k] = as_float2(mz[i]);
    }
    const V3<df64> c[6] = {X.c23, X.c31, X.c12, X.c45, X.c64, X.c56};
#pragma unroll
    for (int i = 0; i < 6; ++i) {
        g[(21 + 3 * i) * ne + k] = as_float2(c[i].x);
        g[(22 + 3 * i) * ne + k] = as_float2(c[i].y);
        g[(23 + 3 * i) * ne + k] = as_float2(c[i].z);
    }
}

__device__ __forceinline__ void load_geometry_df(const double *__restrict__ geo, size_t ne, int k, df64 mx[7],
                                                 df64 my[7], df64 mz[7], ModeCrosses<df64> &X)
{
    const float2 *g = reinterpret_cast<const float2 *>(geo);
#pragma unroll
    for (int i = 0; i < 7; ++i) {
        mx[i] = as_df(__ldg(g + (3 * i + 0) * ne + k));
        my[i] = as_df(__ldg(g + (3 * i + 1) * ne + k));
        mz[i] = as_df(__ldg(g + (3 * i + 2) * ne + k));
    }
    V3<df64> c[6];
#pragma unroll
    for (int i = 0; i < 6; ++i)
        c[i] = {as_df(__ldg(g + (21 + 3 * i) * ne + k)), as_df(__ldg(g + (22 + 3 * i) * ne + k)),
                as_df(__ldg(g + (23 + 3 * i) * ne + k))};
    X = {c[0], c[1], c[2], c[3], c[4], c[5]};
}

// ---------------------------------------------------------------------
// Element force: stress + Flanagan-Belytschko hourglass, as pairs
// ---------------------------------------------------------------------
__device__ __forceinline__ void elem_force_df(const Dom &d, int k, DevScalars *sc)
{
    const size_t ne = (size_t)d.ne;
    // the element scalars first: their loads are in flight with the geometry's
    const double pk = __ldg(d.p + k), qk = __ldg(d.q + k), vk = __ldg(d.v + k), volok = __ldg(d.volo + k);
    const double ssk = __ldg(d.ss + k), massk = __ldg(d.elem_mass + k);
    int nl[8];
    load_nodelist(d.nodelist, k, nl);
    // the modes and shared cross products: kept by the previous cycle's
    // kinematics kernel for these positions, else formed here by the same
    // functions (the same bits either way)
    df64 mx[7], my[7], mz[7];
    ModeCrosses<df64> X;
    if (d.geo && sc->geo_valid) {
        load_geometry_df(d.geo, ne, k, mx, my, mz, X);
    } else {
        rel_modes_df(d.x, nl, mx);
        rel_modes_df(d.y, nl, my);
        rel_modes_df(d.z, nl, mz);
        X = mode_crosses(mode(mx, my, mz, 0), mode(mx, my, mz, 1), mode(mx, my, mz, 2), mode(mx, my, mz, 3),
                         mode(mx, my, mz, 4), mode(mx, my, mz, 5));
    }
    const V3<df64> M1 = mode(mx, my, mz, 0), M2 = mode(mx, my, mz, 1), M3 = mode(mx, my, mz, 2);
    const V3<df64> M4 = mode(mx, my, mz, 3), M5 = mode(mx, my, mz, 4), M6 = mode(mx, my, mz, 5);
    df64 dvdx[8], dvdy[8], dvdz[8];
    V3<df64> nx[3];
    force_geometry(M1, M2, M3, M4, M5, M6, X, dvdx, dvdy, dvdz, nx);   // 192 x dV/dx, normal generators

    // IntegrateStressForElems (LULESH-OMP.cc:853-903), as in step_fp64.cu:
    // the stress forces are s . (Y1, Y2, Y3) with Y = ((p + q)/64) X; corners
    // 4..7 carry the forces of corners 2, 3, 0, 1 negated; only the sign of
    // the Jacobian volume M2.(M3 x M1)/64 is tested.
    df64 Y[3][3];
    {
        const df64 w = to_df((1.0 / 64.0) * (pk + qk));
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            Y[i][0] = w * nx[i].x;
            Y[i][1] = w * nx[i].y;
            Y[i][2] = w * nx[i].z;
        }
        if (dot3(M2, X.c31).hi <= 0.f) flag_error(sc, ERR_K1_DETERM, k);
    }
    // (dim may be a run-time value: the component is selected, not indexed,
    // so that Y stays in registers)
    auto comp = [&](int i, int dim) { return dim == 0 ? Y[i][0] : (dim == 1 ? Y[i][1] : Y[i][2]); };
    auto stress8 = [&](int dim, df64 f[8]) {
        const df64 y0 = comp(0, dim), y1 = comp(1, dim);
        const df64 a = y0 + y1, b = y0 - y1, z = comp(2, dim);
        f[0] = -(a + z);   // (-,-,-)
        f[1] = b - z;      // (+,-,-)
        f[2] = a - z;      // (+,+,-)
        f[3] = -(b + z);   // (-,+,-)
        f[4] = -f[2];
        f[5] = -f[3];
        f[6] = -f[0];
        f[7] = -f[1];
    };
    auto out_of = [&](int dim) {
        return reinterpret_cast<float2 *>(dim == 0 ? d.fcx : (dim == 1 ? d.fcy : d.fcz));
    };

    // CalcHourglassControlForElems (:1503-1558)
    const double determ = volok * vk;
    if (vk <= 0.0) flag_error(sc, ERR_K1_VOLUME, k);

    const double hourg = d.prm.hgcoef;
    if (!gt(hourg, 0.0)) {
#pragma unroll
        for (int dim = 0; dim < 3; ++dim) {
            df64 f[8];
            stress8(dim, f);
#pragma unroll
            for (int c = 0; c < 8; ++c) out_of(dim)[c * ne + k] = as_float2(f[c]);
        }
        return;
    }

    // CalcFBHourglassForceForElems (:1291-1473); the scalar factors are FP64
    // (a handful of operations), everything per corner is pairs
    const double r = rcbrt_fast(determ);                    // determ^(-1/3)
    const V3<df64> H[4] = {M6, M5, M4, mode(mx, my, mz, 6)};
    fb_hourglass_df(d, nl, dvdx, dvdy, dvdz, H, to_df((r * r * r) * (1.0 / 192.0)),
                    to_df(-hourg * 0.01 * ssk * massk * r), [&](int dim, const df64 hgf[8]) {
                        // each corner's stress force plus its hourglass force
                        df64 f[8];
                        stress8(dim, f);
#pragma unroll
                        for (int c = 0; c < 8; ++c) out_of(dim)[c * ne + k] = as_float2(f[c] + hgf[c]);
                    });
}

__global__ void __launch_bounds__(kBlockElem) k_elem_force_df(const __grid_constant__ Dom d)
{
    if (skip_step(d)) return;
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= d.ne) return;
    elem_force_df(d, k, d.sc);
}

// ---------------------------------------------------------------------
// Node update: the corner gather as pairs, joined once in FP64
// ---------------------------------------------------------------------
__device__ __forceinline__ void node_update_df(const Dom &d, int n, const DevScalars *sc)
{
    const float2 *cx = reinterpret_cast<const float2 *>(d.fcx);
    const float2 *cy = reinterpret_cast<const float2 *>(d.fcy);
    const float2 *cz = reinterpret_cast<const float2 *>(d.fcz);
    df64 fx(0.f, 0.f), fy(0.f, 0.f), fz(0.f, 0.f);
    for_node_corners(d, sc, n, [&](int c, bool first) {
        if (first) {
            fx = as_df(cx[c]);
            fy = as_df(cy[c]);
            fz = as_df(cz[c]);
        } else {
            fx = fx + as_df(cx[c]);
            fy = fy + as_df(cy[c]);
            fz = fz + as_df(cz[c]);
        }
    });
    node_integrate(d, n, sc, to_double(fx), to_double(fy), to_double(fz));
}

__global__ void __launch_bounds__(kBlockNode) k_node_update_df(const __grid_constant__ Dom d)
{
    if (skip_step(d)) return;
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= d.nn) return;
    if (n == 0 && d.geo) d.sc->geo_valid = 0;   // the positions move: the geometry cache goes stale
    node_update_df(d, n, d.sc);
}

// ---------------------------------------------------------------------
// Element kinematics + monotonic-Q gradients, as pairs
// ---------------------------------------------------------------------
__device__ __forceinline__ void elem_kinematics_df(const Dom &d, int k, DevScalars *sc)
{
    int nl[8];
    load_nodelist(d.nodelist, k, nl);
    df64 mx[7], my[7], mz[7];
    rel_modes_df(d.x, nl, mx);
    rel_modes_df(d.y, nl, my);
    rel_modes_df(d.z, nl, mz);
    df64 vx[3], vy[3], vz[3];
    rel_linear_df(d.xd, nl, vx);
    rel_linear_df(d.yd, nl, vy);
    rel_linear_df(d.zd, nl, vz);
    const V3<df64> M1 = mode(mx, my, mz, 0), M2 = mode(mx, my, mz, 1), M3 = mode(mx, my, mz, 2);
    const V3<df64> M4 = mode(mx, my, mz, 3), M5 = mode(mx, my, mz, 4), M6 = mode(mx, my, mz, 5);
    const V3<df64> V1{vx[0], vy[0], vz[0]}, V2{vx[1], vy[1], vz[1]}, V3v{vx[2], vy[2], vz[2]};

    // CalcKinematicsForElems, volume part (:1950-1964)
    const ModeCrosses<df64> X = mode_crosses(M1, M2, M3, M4, M5, M6);
    store_geometry_df(d.geo, (size_t)d.ne, k, mx, my, mz, X);
    if (k == sc->elem_begin) sc->geo_valid = 1;
    const df64 vol64 = volume64_shared(M1, M2, M3, X);
    // volume / volo, as a product with the reciprocal taken at set-up
    const df64 rel_df = df_scale(vol64 * to_df(__ldg(d.inv_volo + k)), 1.f / 64.f);
    const double rel = to_double(rel_df);
    d.vnew[k] = rel;
    d.delv[k] = rel - d.v[k];
    // CalcElemCharacteristicLength (:1821-1862): 4V / sqrt(max AreaFace)
    d.arealg[k] = to_double(df_scale(vol64, 0.25f) * df_rsqrt(max_face_cross2_64(M1, M2, M3, M4, M5, M6, X)));
    if (rel <= 0.0) flag_error(sc, ERR_K3_VNEW, k);

    // CalcMonotonicQGradientsForElems (:2034-2180): the logical differences
    // are M/4, so each cross product is (M x M')/16 and each velocity
    // difference Mv/4
    {
        const df64 ptiny(1.e-36);
        const df64 vol = to_df(d.volo[k]) * rel_df;
        // (1/16) (1/4) / (vol + ptiny)
        const df64 vscale = df_rcp(df_scale(vol + ptiny, 64.f));
        const V3<df64> &Az = X.c12, &Ax = X.c23, &Ae = X.c31;
        d.delx_zeta[k] = to_double(vol * df_rsqrt(df_scale(dot3(Az, Az), 0.00390625f) + ptiny));
        d.delv_zeta[k] = to_double(vscale * dot3(Az, V3v));
        d.delx_xi[k] = to_double(vol * df_rsqrt(df_scale(dot3(Ax, Ax), 0.00390625f) + ptiny));
        d.delv_xi[k] = to_double(vscale * dot3(Ax, V1));
        d.delx_eta[k] = to_double(vol * df_rsqrt(df_scale(dot3(Ae, Ae), 0.00390625f) + ptiny));
        d.delv_eta[k] = to_double(vscale * dot3(Ae, V2));
    }

    // CalcKinematicsForElems, strain-rate part (:1975-2020)
    d.vdov[k] = to_double(strain_rate(M1, M2, M3, V1, V2, V3v, to_df(0.5 * sc->deltatime)));
}

__global__ void __launch_bounds__(kKinBlockFactor * kBlockElem, 2) k_elem_kinematics_df(const __grid_constant__ Dom d)
{
    if (skip_step(d)) return;
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= d.ne) return;
    elem_kinematics_df(d, k, d.sc);
}

// ---------------------------------------------------------------------
// Monotonic-Q limiter and viscosity coefficients as pairs, then the FP64
// material update, volume update and constraint candidates
// ---------------------------------------------------------------------

// One direction of the monotonic limiter (LULESH-OMP.cc:2198-2228) as
// pairs.  The neighbour slopes are divided by the element's own (plus
// 1e-36): in FP64 a vanishing own slope makes the ratios huge but finite,
// and the clamp to [0, max_slope] absorbs them; in pairs the product would
// overflow (and its remainder turn into a NaN), so a ratio whose magnitude
// exceeds 2^100 -- judged from the high words before multiplying -- is
// taken as +-2^100.  That changes no outcome: a ratio beyond it is never the
// minimum unless both are, and then the result is max_slope either way; a
// negative one makes the result 0 either way.
__device__ __forceinline__ df64 limiter_phi_df(const double *__restrict__ delv, int i, int bm, int bp,
                                               int m_symm, int m_free, int p_symm, int p_free, int lm, int lp,
                                               df64 limiter, df64 max_slope)
{
    const double own = delv[i];
    const df64 norm = df_rcp(to_df(own) + df64(1.e-36));
    double dm = 0.0, dp = 0.0;
    if (bm == 0) dm = delv[lm];
    else if (bm == m_symm) dm = own;
    if (bp == 0) dp = delv[lp];
    else if (bp == p_symm) dp = own;
    (void)m_free;
    (void)p_free;
    const float big = 1.2676506e30f;   // 2^100
    auto ratio = [&](double x) {
        const df64 a = to_df(x);
        if (fabsf(a.hi) * fabsf(norm.hi) > big)   // may be inf: still > big
            return (a.hi < 0.f) != (norm.hi < 0.f) ? df64(-big, 0.f) : df64(big, 0.f);
        return a * norm;
    };
    df64 delvm = ratio(dm), delvp = ratio(dp);
    df64 phi = df_scale(delvm + delvp, 0.5f);
    delvm = delvm * limiter;
    delvp = delvp * limiter;
    if (df_gt(phi, delvm)) phi = delvm;
    if (df_gt(phi, delvp)) phi = delvp;
    if (phi.hi < 0.f) phi = df64(0.f, 0.f);
    if (df_gt(phi, max_slope)) phi = max_slope;
    return phi;
}

// Monotonic-Q region (:2182-2320) and the material update as pairs (the
// energy accumulated in FP64), and the element's constraint keys in pairs
// when kConstraints.
template <bool kConstraints>
__device__ __forceinline__ void elem_material_df(const Dom &d, int k, DevScalars *sc, unsigned long long &kc,
                                                 unsigned long long &kh)
{
    const lulesh_params &P = d.prm;
    const int bc = __ldg(d.elem_bc + k);
    const FaceNeighbours nb = face_neighbours(d, sc, k);
    const df64 lim = to_df(P.monoq_limiter_mult), maxs = to_df(P.monoq_max_slope);
    const df64 phixi = limiter_phi_df(d.delv_xi, k, bc & BC_XI_M, bc & BC_XI_P, BC_XI_M_SYMM, BC_XI_M_FREE,
                                      BC_XI_P_SYMM, BC_XI_P_FREE, nb.xim, nb.xip, lim, maxs);
    const df64 phieta = limiter_phi_df(d.delv_eta, k, bc & BC_ETA_M, bc & BC_ETA_P, BC_ETA_M_SYMM, BC_ETA_M_FREE,
                                       BC_ETA_P_SYMM, BC_ETA_P_FREE, nb.etam, nb.etap, lim,
                                       maxs);
    const df64 phizeta = limiter_phi_df(d.delv_zeta, k, bc & BC_ZETA_M, bc & BC_ZETA_P, BC_ZETA_M_SYMM,
                                        BC_ZETA_M_FREE, BC_ZETA_P_SYMM, BC_ZETA_P_FREE, nb.zetam,
                                        nb.zetap, lim, maxs);
    const double vnew = d.vnew[k], vdov = d.vdov[k];
    df64 qlin(0.f, 0.f), qquad(0.f, 0.f);
    if (!gt(vdov, 0.)) {
        // the products delv * delx; a positive one contributes nothing
        auto prod = [](double dv, double dx) {
            const df64 p = to_df(dv) * to_df(dx);
            return p.hi > 0.f ? df64(0.f, 0.f) : p;
        };
        const df64 dxi = prod(d.delv_xi[k], d.delx_xi[k]);
        const df64 deta = prod(d.delv_eta[k], d.delx_eta[k]);
        const df64 dzeta = prod(d.delv_zeta[k], d.delx_zeta[k]);
        const df64 rho = df_div(to_df(d.elem_mass[k]), to_df(d.volo[k]) * to_df(vnew));
        const df64 one(1.f, 0.f);
        const df64 lin = (dxi * (one - phixi) + deta * (one - phieta)) + dzeta * (one - phizeta);
        const df64 quad = (dxi * dxi * (one - phixi * phixi) + deta * deta * (one - phieta * phieta)) +
                          dzeta * dzeta * (one - phizeta * phizeta);
        qlin = -(to_df(P.qlc_monoq) * rho) * lin;
        qquad = to_df(P.qqc_monoq) * rho * quad;
    }
    if (d.keep & 2) {
        d.ql[k] = to_double(qlin);
        d.qq[k] = to_double(qquad);
    }
    const double ssn = material_update_df(d, k, sc, vnew, qlin, qquad, d.reps ? __ldg(d.reps + k) : 1);
    if (kConstraints) constraint_keys_df(ssn, vdov, d.arealg[k], P, kc, kh);
}

// Eight blocks per SM (64 registers, ~40 bytes spilled; 80 registers at six
// blocks): the kernel waits on its neighbour loads, and the extra warps hide
// them better than the spills cost (0.88 ms at six blocks, 0.81 at seven,
// 0.78 at eight, s=192).
template <bool kConstraints>
__global__ void __launch_bounds__(kBlockElem, 8) k_elem_material_df(const __grid_constant__ Dom d)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    unsigned long long kc = ~0ULL, kh = ~0ULL;
    if (t < d.ne && !skip_step(d)) {
        // with regions, threads take elements in cost-grouped order
        const int k = d.mat_order ? __ldg(d.mat_order + t) : t;
        elem_material_df<kConstraints>(d, k, d.sc, kc, kh);
    }
    if (kConstraints) block_min_publish(kc, kh, d.sc);
}

// ---------------------------------------------------------------------
// Launchers
// ---------------------------------------------------------------------
static inline unsigned blocks_for(long n, int bs) { return (unsigned)((n + bs - 1) / bs); }

void launch_elem_force_df(const Dom &d, cudaStream_t st)
{
    k_elem_force_df<<<blocks_for(d.ne, elem_block(d)), elem_block(d), 0, st>>>(d);
}

void launch_node_update_df(const Dom &d, cudaStream_t st)
{
    k_node_update_df<<<blocks_for(d.nn, node_block(d)), node_block(d), 0, st>>>(d);
}

void launch_elem_kinematics_df(const Dom &d, cudaStream_t st)
{
    k_elem_kinematics_df<<<blocks_for(d.ne, kin_block(d)), kin_block(d), 0, st>>>(d);
}

void launch_elem_material_df(const Dom &d, cudaStream_t st, bool with_constraints)
{
    if (with_constraints)
        k_elem_material_df<true><<<blocks_for(d.ne, elem_block(d)), elem_block(d), 0, st>>>(d);
    else
        k_elem_material_df<false><<<blocks_for(d.ne, elem_block(d)), elem_block(d), 0, st>>>(d);
}

// Batched ensembles: kernels 0..3 (force, node update, kinematics, material)
// over the active tiles of one class.
void launch_batch_kernel_df(const Dom &d, const BatchView &b, cudaStream_t st, int kernel, int cls, LaunchCfg cfg)
{
    switch (kernel) {
    case 0: kb_elem<elem_force_df><<<cfg.grid, cfg.block, 0, st>>>(d, b, cls); break;
    case 1: kb_node<node_update_df><<<cfg.grid, cfg.block, 0, st>>>(d, b, cls); break;
    case 2: kb_elem<elem_kinematics_df><<<cfg.grid, cfg.block, 0, st>>>(d, b, cls); break;
    default: kb_material_capped<elem_material_df<true>, 4><<<cfg.grid, cfg.block, 0, st>>>(d, b, cls); break;
    }
}

int batch_max_blocks_df(int kernel, int block)
{
    int n = 0;
    cudaError_t e;
    switch (kernel) {
    case 0: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kb_elem<elem_force_df>, block, 0); break;
    case 1: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kb_node<node_update_df>, block, 0); break;
    case 2: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kb_elem<elem_kinematics_df>, block, 0); break;
    default: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kb_material_capped<elem_material_df<true>, 4>, block, 0); break;
    }
    return e == cudaSuccess ? n : 0;
}

}  // namespace lulesh
