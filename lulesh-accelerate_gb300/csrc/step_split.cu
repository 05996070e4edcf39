// step_split.cu -- the split-precision Lagrange leapfrog step on sm_103a.
//
// GB300 issues FP32 at 64x its FP64 rate, so this step moves the geometry-
// heavy work to FP32 and keeps FP64 where the solution's stability needs it:
//
//   FP32  shape-function geometry, stress and Flanagan-Belytschko hourglass
//         corner forces (IntegrateStressForElems, CalcFBHourglassForceForElems,
//         LULESH-OMP.cc:853-931, :1233-1558), the monotonic-Q gradients and
//         limiter (:2034-2320);
//   FP64  node accelerations, velocities and positions (:1613-1683), the
//         energy (:2415-2541, accumulated in FP64), the element state and
//         the constraint minima (:2799-2933); the relative volume and its
//         change, the strain rate vdov and the characteristic length
//         (:1799-1862, :1927-2032), the pressure, viscosity and sound speed
//         of the EOS (:2384-2782) and the constraint candidates are
//         evaluated to FP64 grade (~2^-47) as double-float pairs on the FP32
//         pipe (df64.cuh, eos_df.cuh) and stored in FP64.
//
// Corner forces are FP32 and summed per node with a compensated (Kahan)
// FP32 sum whose two words are combined in FP64.  FP32 geometry never sees an
// absolute coordinate: the force kernel works on the corners relative to
// corner 0, formed from a hi/lo float pair that the node kernel keeps beside
// each FP64 position and velocity ((hi_c - hi_0) + (lo_c - lo_0) carries the
// difference to ~2^-48 of the coordinate), and the kinematics kernel on the
// Walsh modes of the corners (differences only), summed exactly from the
// same pairs; so FP32 round-off is relative to the element size, not to the
// mesh extent.
//
// Launch structure and error handling are those of step_fp64.cu.
#include "lulesh_internal.h"
#include "kernels.h"
#include "hexmodes.cuh"
#include "common.cuh"
#include "eos_df.cuh"
#include "tile.cuh"
#include "batch_kernels.cuh"

#include <cuda_runtime.h>

namespace lulesh {

// v = hi + lo with hi = v truncated to FP32 precision (exact in FP32) and
// lo = the remainder (exact in FP64, truncated to FP32): hi + lo carries v to
// ~2^-46 relative.  One FP64 subtraction, the rest integer operations.
__device__ __forceinline__ float2 split_hi_lo(double v)
{
    const unsigned long long b = (unsigned long long)__double_as_longlong(v);
    const double hid = __longlong_as_double((long long)(b & ~((1ULL << 29) - 1)));
    return make_float2(d2f(hid), d2f(v - hid));
}

// Corner values relative to corner 0, from hi/lo pairs.
__device__ __forceinline__ void rel8(const float2 *__restrict__ f, const int nl[8], float out[8])
{
    const float2 a0 = __ldg(f + nl[0]);
    out[0] = 0.f;
#pragma unroll
    for (int c = 1; c < 8; ++c) {
        const float2 a = __ldg(f + nl[c]);
        out[c] = (a.x - a0.x) + (a.y - a0.y);
    }
}

// ---- compensated FP32 sums of hi/lo pairs ---------------------------------
// A value carried as an unevaluated sum hi + lo of two floats.
struct DF {
    float hi, lo;
};

// hi + lo as the FP32 rounding of the sum and its exact remainder (Knuth's
// two-sum), so that |lo| <= 2^-24 |hi|.
__device__ __forceinline__ DF df_renorm(DF a)
{
    const float s = a.hi + a.lo;
    const float bb = s - a.hi;
    return {s, (a.hi - (s - bb)) + (a.lo - bb)};
}

// A value carried as h + e: h a float, e the exact rounding errors of the
// sums that formed h plus the low words, gathered in one float.
__device__ __forceinline__ DF bf_add(DF a, DF b)
{
    const float s = a.hi + b.hi;
    const float bb = s - a.hi;
    return {s, ((a.hi - (s - bb)) + (b.hi - bb)) + (a.lo + b.lo)};
}
__device__ __forceinline__ DF bf_sub(DF a, DF b) { return bf_add(a, {-b.hi, -b.lo}); }

// The Walsh modes M1..M6 of one coordinate of the 8 corners, from hi/lo
// pairs, as renormalised hi/lo pairs: the three butterfly stages of walsh8
// (hexmodes.cuh) with every high-word sum formed exactly (Knuth's two-sum)
// and its error carried, with the low words, in the second float; one
// renormalisation per mode.  With linear_only, M1..M3 alone.
template <bool kLinearOnly>
__device__ __forceinline__ void df_modes(const float2 *__restrict__ f, const int nl[8], DF m[6])
{
    DF c[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        const float2 v = __ldg(f + nl[i]);
        c[i] = {v.x, v.y};
    }
    const DF s01 = bf_add(c[0], c[1]), d01 = bf_sub(c[1], c[0]);
    const DF s32 = bf_add(c[3], c[2]), d32 = bf_sub(c[2], c[3]);
    const DF s45 = bf_add(c[4], c[5]), d45 = bf_sub(c[5], c[4]);
    const DF s76 = bf_add(c[7], c[6]), d76 = bf_sub(c[6], c[7]);
    const DF dsm = bf_sub(s32, s01), dsp = bf_sub(s76, s45);   // eta differences of the zeta faces
    const DF sdm = bf_add(d01, d32), sdp = bf_add(d45, d76);   // xi differences of the zeta faces
    m[0] = df_renorm(bf_add(sdm, sdp));                          // xi
    m[1] = df_renorm(bf_add(dsm, dsp));                          // eta
    m[2] = df_renorm(bf_sub(bf_add(s45, s76), bf_add(s01, s32)));   // zeta
    if (!kLinearOnly) {
        const DF ddm = bf_sub(d32, d01), ddp = bf_sub(d76, d45);
        m[3] = df_renorm(bf_add(ddm, ddp));                      // xi eta
        m[4] = df_renorm(bf_sub(sdp, sdm));                      // xi zeta
        m[5] = df_renorm(bf_sub(dsp, dsm));                      // eta zeta
    }
}

// FP64 state -> hi/lo pairs and reciprocal masses (after any host upload).
__global__ void __launch_bounds__(kBlockNode) k_split_sync(const __grid_constant__ Dom d)
{
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= d.nn) return;
    d.xs[n] = split_hi_lo(d.x[n]);
    d.ys[n] = split_hi_lo(d.y[n]);
    d.zs[n] = split_hi_lo(d.z[n]);
    d.xds[n] = split_hi_lo(d.xd[n]);
    d.yds[n] = split_hi_lo(d.yd[n]);
    d.zds[n] = split_hi_lo(d.zd[n]);
    d.inv_mass[n] = 1.0 / d.nodal_mass[n];
}

// ---------------------------------------------------------------------
// Element force in FP32
// ---------------------------------------------------------------------
// The hi/lo pairs of field f: 0..5 = x, y, z, xd, yd, zd.
__device__ __forceinline__ const float2 *pair_field(const Dom &d, int f)
{
    return f == 0 ? d.xs : f == 1 ? d.ys : f == 2 ? d.zs : f == 3 ? d.xds : f == 4 ? d.yds : d.zds;
}

// An element's corner values relative to corner 0, gathered from global
// memory through its node list (any mesh).
struct GlobalCorners {
    const Dom &d;
    int nl[8];
    __device__ GlobalCorners(const Dom &dom, int k) : d(dom) { load_nodelist(d.nodelist, k, nl); }
    __device__ void rel(int f, float out[8]) const { rel8(pair_field(d, f), nl, out); }
};

template <class Shape>
struct TileCorners {
    const float2 *tile;   // [6][Shape::kNodes]
    int li[8];            // the corners' places in the tile, in the reference's corner order
    __device__ TileCorners(const float2 *t, int rr, int cc) : tile(t) { Shape::corners(rr, cc, li); }
    __device__ void rel(int f, float out[8]) const
    {
        const float2 *t = tile + f * Shape::kNodes;
        const float2 a0 = t[li[0]];
        out[0] = 0.f;
#pragma unroll
        for (int c = 1; c < 8; ++c) {
            const float2 a = t[li[c]];
            out[c] = (a.x - a0.x) + (a.y - a0.y);
        }
    }
};

// The element scalars the force body reads, as FP32 (v also as its sign).
struct ForceIn {
    float p, q, v, volo, ss, mass;
    bool v_bad;
};
__device__ __forceinline__ ForceIn load_force_in(const Dom &d, int k)
{
    const double v = d.v[k];
    return {d2f(d.p[k]), d2f(d.q[k]), d2f(v), d2f(d.volo[k]), d2f(d.ss[k]), d2f(d.elem_mass[k]), v <= 0.0};
}

template <class Corners>
__device__ __forceinline__ void elem_force_split_from(const Dom &d, int k, DevScalars *sc, const Corners &cn,
                                                      const ForceIn &in)
{
    const size_t ne = (size_t)d.ne;

    // The geometry of the FP64 kernel (the Walsh-mode identities of
    // hexmodes.cuh) in FP32, on corner coordinates relative to corner 0: the
    // modes M1..M7 do not see a translation.
    V3<float> M[7];
    {
        float x[8], y[8], z[8], mx[7], my[7], mz[7];
        cn.rel(0, x);
        cn.rel(1, y);
        cn.rel(2, z);
        walsh8(x, mx);
        walsh8(y, my);
        walsh8(z, mz);
#pragma unroll
        for (int i = 0; i < 7; ++i) M[i] = mode(mx, my, mz, i);
    }
    float dvdx[8], dvdy[8], dvdz[8];
    V3<float> nx[3];
    const ModeCrosses<float> C = mode_crosses(M[0], M[1], M[2], M[3], M[4], M[5]);
    force_geometry(M[0], M[1], M[2], M[3], M[4], M[5], C, dvdx, dvdy, dvdz, nx);   // 192 x dV/dx, normal generators

    // IntegrateStressForElems (LULESH-OMP.cc:853-903): the stress force of
    // the corner with signs s is s . (Y1, Y2, Y3) with Y = ((p + q)/64) X;
    // corners 4..7 carry the forces of corners 2, 3, 0, 1 negated.  Only the
    // sign of the Jacobian volume M2.(M3 x M1) / 64 is tested.
    if (dot3(M[1], C.c31) <= 0.f) flag_error(sc, ERR_K1_DETERM, k);
    const float w = (1.f / 64.f) * (in.p + in.q);
    float f[3][8];
#pragma unroll
    for (int dim = 0; dim < 3; ++dim) {
        const float y1 = w * (dim == 0 ? nx[0].x : dim == 1 ? nx[0].y : nx[0].z);
        const float y2 = w * (dim == 0 ? nx[1].x : dim == 1 ? nx[1].y : nx[1].z);
        const float y3 = w * (dim == 0 ? nx[2].x : dim == 1 ? nx[2].y : nx[2].z);
        const float a = y1 + y2, b = y1 - y2;
        f[dim][0] = -(a + y3);   // (-,-,-)
        f[dim][1] = b - y3;      // (+,-,-)
        f[dim][2] = a - y3;      // (+,+,-)
        f[dim][3] = -(b + y3);   // (-,+,-)
        f[dim][4] = -f[dim][2];
        f[dim][5] = -f[dim][3];
        f[dim][6] = -f[dim][0];
        f[dim][7] = -f[dim][1];
    }

    if (in.v_bad) flag_error(sc, ERR_K1_VOLUME, k);
    const float hourg = d2f(d.prm.hgcoef);
    if (hourg > 0.f) {
        // CalcFBHourglassForceForElems (:1291-1473): hourgam = gamma -
        // volinv (dV/dx . hourmod), the hourglass projections being the
        // modes M6, M5, M4, M7
        const float r = rcbrtf(in.volo * in.v);      // determ^(-1/3)
        const float volinv192 = ((r * r) * r) * (1.f / 192.f);
        const V3<float> H[4] = {M[5], M[4], M[3], M[6]};
        const float gam[4][8] = {
            { 1.f,  1.f, -1.f, -1.f, -1.f, -1.f,  1.f,  1.f},
            { 1.f, -1.f, -1.f,  1.f, -1.f,  1.f,  1.f, -1.f},
            { 1.f, -1.f,  1.f, -1.f,  1.f, -1.f,  1.f, -1.f},
            {-1.f,  1.f, -1.f,  1.f,  1.f, -1.f,  1.f, -1.f}};
        float hg[8][4];
#pragma unroll
        for (int m = 0; m < 4; ++m) {
            const float hx = -(volinv192 * H[m].x), hy = -(volinv192 * H[m].y), hz = -(volinv192 * H[m].z);
#pragma unroll
            for (int c = 0; c < 8; ++c)
                hg[c][m] = fmaf(dvdz[c], hz, fmaf(dvdy[c], hy, fmaf(dvdx[c], hx, gam[m][c])));
        }
        const float coefficient = (((-hourg) * 0.01f) * in.ss) * in.mass * r;
        // velocities relative to corner 0: the hourglass modes are blind to
        // a uniform velocity (sum over corners of each hourgam column is 0)
#pragma unroll
        for (int dim = 0; dim < 3; ++dim) {
            float u[8];
            cn.rel(3 + dim, u);
            float h[4];
#pragma unroll
            for (int m = 0; m < 4; ++m) {
                float acc = hg[1][m] * u[1];
#pragma unroll
                for (int c = 2; c < 8; ++c) acc = fmaf(hg[c][m], u[c], acc);
                h[m] = coefficient * acc;
            }
#pragma unroll
            for (int c = 0; c < 8; ++c)
                f[dim][c] = fmaf(hg[c][3], h[3], fmaf(hg[c][2], h[2], fmaf(hg[c][1], h[1], fmaf(hg[c][0], h[0], f[dim][c]))));
        }
    }
#pragma unroll
    for (int c = 0; c < 8; ++c) {
        d.f32x[c * ne + k] = f[0][c];
        d.f32y[c * ne + k] = f[1][c];
        d.f32z[c * ne + k] = f[2][c];
    }
}

__device__ __forceinline__ void elem_force_split(const Dom &d, int k, DevScalars *sc)
{
    elem_force_split_from(d, k, sc, GlobalCorners(d, k), load_force_in(d, k));
}

// The staged force kernel of a structured s^3 cube (Dom::s > 0, the node
// and element numbering of the reference's set-up): block b covers plane p,
// rows r0..r0+1 and columns c0..c0+63 of elements.  The same arithmetic as
// k_elem_force_split, so the same bits.  Each thread issues its element's
// scalar loads (p, q, v, volo, ss, mass) before the block stages the tile,
// so they are in flight during the tile's loads and its barrier
// (0.41 -> 0.37 ms at s=192).  The skip decision is taken once per block (an
// error word another block sets meanwhile must not split the block at its
// barrier).
__global__ void __launch_bounds__(SoloTile::kThreads, 8) k_elem_force_split_tiled(const __grid_constant__ Dom d)
{
    __shared__ float2 tile[6 * SoloTile::kNodes];
    __shared__ int skip;
    const TileCoord t = SoloTile::coord(d.s, blockIdx.x);
    if (threadIdx.x == 0) skip = skip_step(d) ? 1 : 0;
    int k, rr, cc;
    const bool mine = SoloTile::element(d.s, t, k, rr, cc);
    ForceIn in{};
    if (mine) in = load_force_in(d, k);   // in flight while the tile loads
    SoloTile::load(tile, d.s, t, 0, 0, 6, [&](int f) { return pair_field(d, f); });
    __syncthreads();
    if (skip || !mine) return;
    elem_force_split_from(d, k, d.sc, TileCorners<SoloTile>(tile, rr, cc), in);
}

// The staged force kernel over the structured cubes of one size class of a
// batched ensemble (every instance of the class has s >= kTileCols): a
// persistent grid walks the class's staged tiles, instance by instance
// (StagedClass::tile_begin), skipping instances that have retired or
// failed; each tile is staged and computed as in k_elem_force_split_tiled,
// with the instance's element and node offsets and its own scalar block.
// ROWS (2 or 4 element rows per tile of 64 columns) is the staging depth the
// autotuner chooses.  The same arithmetic as the gathering batch kernel, so
// the same bits.
template <int ROWS>
__global__ void __launch_bounds__(TileShape<ROWS>::kThreads, 1024 / TileShape<ROWS>::kThreads)
    kb_force_split_staged(const __grid_constant__ Dom d, const __grid_constant__ BatchView b,
                          const __grid_constant__ StagedClass sc)
{
    using Shape = TileShape<ROWS>;
    __shared__ float2 tile[6 * Shape::kNodes];
    __shared__ int s_j, s_skip;
    const long long total = sc.tile_begin[sc.n];
    for (long long t = blockIdx.x; t < total; t += gridDim.x) {
        if (threadIdx.x == 0) {
            // the last instance whose first tile is at or before t
            int lo = 0, hi = sc.n - 1;
            while (lo < hi) {
                const int mid = (lo + hi + 1) / 2;
                if (sc.tile_begin[mid] <= t) lo = mid;
                else hi = mid - 1;
            }
            s_j = lo;
            const int inst = sc.inst[lo];
            s_skip = (!b.inst_active[inst] || d.sc[inst].err_any) ? 1 : 0;
        }
        __syncthreads();
        if (!s_skip) {   // the same for the whole block
            const int j = s_j, s = sc.s[j];
            const TileCoord tc = Shape::coord(s, t - sc.tile_begin[j]);
            Shape::load(tile, s, tc, sc.node_base[j], 0, 6, [&](int f) { return pair_field(d, f); });
            __syncthreads();
            int k, rr, cc;
            if (Shape::element(s, tc, k, rr, cc))
                elem_force_split_from(d, sc.elem_base[j] + k, d.sc + sc.inst[j], TileCorners<Shape>(tile, rr, cc),
                                      load_force_in(d, sc.elem_base[j] + k));
        }
        __syncthreads();   // the tile and s_j are rewritten for the next tile
    }
}

// The FP32 force kernel waits on its corner gathers rather than on an
// arithmetic pipe, so it is held to 64 registers (eight 128-thread blocks
// per SM instead of four; ~200 bytes spilled): 0.48 -> 0.43 ms at s=192.
__global__ void __launch_bounds__(kBlockElem, 8) k_elem_force_split(const __grid_constant__ Dom d)
{
    if (skip_step(d)) return;
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= d.ne) return;
    elem_force_split(d, k, d.sc);
}

// ---------------------------------------------------------------------
// Node update: compensated gather, FP64 integration
// ---------------------------------------------------------------------
__device__ __forceinline__ void kahan_add(float &s, float &c, float v)
{
    const float y = v - c;
    const float t = s + y;
    c = (t - s) - y;
    s = t;
}

__device__ __forceinline__ void node_update_split(const Dom &d, int n, const DevScalars *sc)
{

    float sx = 0.f, sy = 0.f, sz = 0.f, cx = 0.f, cy = 0.f, cz = 0.f;
    for_node_corners(d, sc, n, [&](int c, bool) {
        kahan_add(sx, cx, d.f32x[c]);
        kahan_add(sy, cy, d.f32y[c]);
        kahan_add(sz, cz, d.f32z[c]);
    });
    const double fx = f2d(sx) - f2d(cx);
    const double fy = f2d(sy) - f2d(cy);
    const double fz = f2d(sz) - f2d(cz);
    if (d.keep & 1) {
        d.fx[n] = fx;
        d.fy[n] = fy;
        d.fz[n] = fz;
    }
    const double dt = sc->deltatime, u_cut = d.prm.u_cut;
    const double im = d.inv_mass[n];
    const unsigned bc = __ldg(d.node_bc + n);
    const double ax = (bc & 1) ? 0.0 : fx * im;
    const double ay = (bc & 2) ? 0.0 : fy * im;
    const double az = (bc & 4) ? 0.0 : fz * im;
    double t, p;
    t = d.xd[n] + ax * dt; if (abs_lt(t, u_cut)) t = 0.0; p = d.x[n] + t * dt;
    d.xd[n] = t; d.x[n] = p; d.xds[n] = split_hi_lo(t); d.xs[n] = split_hi_lo(p);
    t = d.yd[n] + ay * dt; if (abs_lt(t, u_cut)) t = 0.0; p = d.y[n] + t * dt;
    d.yd[n] = t; d.y[n] = p; d.yds[n] = split_hi_lo(t); d.ys[n] = split_hi_lo(p);
    t = d.zd[n] + az * dt; if (abs_lt(t, u_cut)) t = 0.0; p = d.z[n] + t * dt;
    d.zd[n] = t; d.z[n] = p; d.zds[n] = split_hi_lo(t); d.zs[n] = split_hi_lo(p);
}

__global__ void __launch_bounds__(kBlockNode) k_node_update_split(const __grid_constant__ Dom d)
{
    if (skip_step(d)) return;
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= d.nn) return;
    node_update_split(d, n, d.sc);
}

// ---------------------------------------------------------------------
// Element kinematics: FP64 volume and strain rate, FP32 length and Q
// gradients
// ---------------------------------------------------------------------
__device__ __forceinline__ void elem_kinematics_split(const Dom &d, int k, DevScalars *sc)
{
    const size_t ne = (size_t)d.ne;

    int nl[8];
    load_nodelist(d.nodelist, k, nl);

    // Relative volume, half-step strain rate and characteristic length
    // through the Walsh modes of the corner coordinates and velocities
    // (CalcKinematicsForElems :1950-1958, :1975-2020, CalcElemCharacteristic-
    // Length :1821-1862; the identities of hexmodes.cuh).  The modes come
    // from the hi/lo pairs by an error-free FP32 butterfly (df_modes) as
    // hi + lo with |lo| <= 2^-24 |hi|, and the cross products, volume, strain
    // rate, face areas and divisions run on them as double-float pairs
    // (df64.cuh): FP64-grade (~2^-47) results without the FP64 pipe.  The
    // characteristic length sets the Courant time step, which every
    // instance's result is sensitive to; in FP32 it moved the origin energy of
    // small ensemble instances (s = 13, 18) up to 1.9e-6 from the reference.
    DF mx[6], my[6], mz[6];
    df_modes<false>(d.xs, nl, mx);
    df_modes<false>(d.ys, nl, my);
    df_modes<false>(d.zs, nl, mz);
    DF vx[6], vy[6], vz[6];
    df_modes<true>(d.xds, nl, vx);
    df_modes<true>(d.yds, nl, vy);
    df_modes<true>(d.zds, nl, vz);
    auto pair = [](const DF &a) { return df64(a.hi, a.lo); };
    V3<df64> M[6], V[3];
#pragma unroll
    for (int i = 0; i < 6; ++i) M[i] = {pair(mx[i]), pair(my[i]), pair(mz[i])};
#pragma unroll
    for (int i = 0; i < 3; ++i) V[i] = {pair(vx[i]), pair(vy[i]), pair(vz[i])};
    const ModeCrosses<df64> X = mode_crosses(M[0], M[1], M[2], M[3], M[4], M[5]);
    const df64 vol64 = volume64_shared(M[0], M[1], M[2], X);
    // volume / volo, as a product with the reciprocal taken at set-up
    const df64 rel_df = df_scale(vol64 * to_df(__ldg(d.inv_volo + k)), 1.f / 64.f);
    const double rel = to_double(rel_df);
    d.vnew[k] = rel;
    d.delv[k] = rel - d.v[k];
    d.vdov[k] = to_double(strain_rate(M[0], M[1], M[2], V[0], V[1], V[2], to_df(0.5 * sc->deltatime)));
    d.arealg[k] = to_double(df_scale(vol64, 0.25f) * df_rsqrt(max_face_cross2_64(M[0], M[1], M[2], M[3], M[4], M[5], X)));
    if (rel <= 0.0) flag_error(sc, ERR_K3_VNEW, k);

    // FP32: monotonic-Q gradients (:2034-2180) through the high words of the
    // modes' cross products, with the formulas of the FP64 kernel (the
    // logical differences are M/4, so each cross product is (M x M')/16 and
    // each velocity difference Mv/4); the roots are the correctly rounded
    // sqrtf and division.
    auto hi3 = [](const V3<df64> &v) { return V3<float>{v.x.hi, v.y.hi, v.z.hi}; };
    const V3<float> c12 = hi3(X.c12), c23 = hi3(X.c23), c31 = hi3(X.c31);
    const V3<float> V1 = hi3(V[0]), V2 = hi3(V[1]), V3f = hi3(V[2]);
    const float vol = vol64.hi * (1.f / 64.f);
    const float ptiny = 1.e-36f;
    const float vscale = 1.f / fmaf(vol, 64.f, 64.f * ptiny);     // (1/16) (1/4) / (vol + ptiny)
    float *gq = d.gq;
    gq[5 * ne + k] = vol / sqrtf(fmaf(0.00390625f, dot3(c12, c12), ptiny));   // delx_zeta
    gq[2 * ne + k] = vscale * dot3(c12, V3f);                                 // delv_zeta
    gq[3 * ne + k] = vol / sqrtf(fmaf(0.00390625f, dot3(c23, c23), ptiny));   // delx_xi
    gq[0 * ne + k] = vscale * dot3(c23, V1);                                  // delv_xi
    gq[4 * ne + k] = vol / sqrtf(fmaf(0.00390625f, dot3(c31, c31), ptiny));   // delx_eta
    gq[1 * ne + k] = vscale * dot3(c31, V2);                                  // delv_eta
}

// Two 256-thread blocks per SM (128 registers: the pairs need them; see
// kin_block).
__global__ void __launch_bounds__(kKinBlockFactor * kBlockElem, 2) k_elem_kinematics_split(const __grid_constant__ Dom d)
{
    if (skip_step(d)) return;
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= d.ne) return;
    elem_kinematics_split(d, k, d.sc);
}

// ---------------------------------------------------------------------
// Q limiter in FP32; EOS and constraints in pairs, the energy in FP64
// ---------------------------------------------------------------------
template <bool kConstraints>
__device__ __forceinline__ void elem_material_split(const Dom &d, int k, DevScalars *sc,
                                                    unsigned long long &kc, unsigned long long &kh)
{
    const lulesh_params &P = d.prm;
    {
        const size_t ne = (size_t)d.ne;
        const float *dv_xi = d.gq, *dv_eta = d.gq + ne, *dv_zeta = d.gq + 2 * ne;
        const int bc = __ldg(d.elem_bc + k);
        const FaceNeighbours nb = face_neighbours(d, sc, k);
        const float lim = d2f(P.monoq_limiter_mult), maxs = d2f(P.monoq_max_slope);
        const float phixi = limiter_phi<float>(dv_xi, k, bc & BC_XI_M, bc & BC_XI_P, BC_XI_M_SYMM,
                                               BC_XI_M_FREE, BC_XI_P_SYMM, BC_XI_P_FREE,
                                               nb.xim, nb.xip, lim, maxs);
        const float phieta = limiter_phi<float>(dv_eta, k, bc & BC_ETA_M, bc & BC_ETA_P, BC_ETA_M_SYMM,
                                                BC_ETA_M_FREE, BC_ETA_P_SYMM, BC_ETA_P_FREE,
                                                nb.etam, nb.etap, lim, maxs);
        const float phizeta = limiter_phi<float>(dv_zeta, k, bc & BC_ZETA_M, bc & BC_ZETA_P,
                                                 BC_ZETA_M_SYMM, BC_ZETA_M_FREE, BC_ZETA_P_SYMM,
                                                 BC_ZETA_P_FREE, nb.zetam, nb.zetap,
                                                 lim, maxs);
        const double vnew = d.vnew[k], vdov = d.vdov[k];
        float qlin = 0.f, qquad = 0.f;
        if (!gt(vdov, 0.)) {
            float dxi = dv_xi[k] * d.gq[3 * ne + k];
            float deta = dv_eta[k] * d.gq[4 * ne + k];
            float dzeta = dv_zeta[k] * d.gq[5 * ne + k];
            if (dxi > 0.f) dxi = 0.f;
            if (deta > 0.f) deta = 0.f;
            if (dzeta > 0.f) dzeta = 0.f;
            const float rho = d2f(d.elem_mass[k]) / (d2f(d.volo[k]) * d2f(vnew));
            const float sl = (dxi * (1.f - phixi) + deta * (1.f - phieta)) + dzeta * (1.f - phizeta);
            const float sq = (dxi * dxi * (1.f - phixi * phixi) + deta * deta * (1.f - phieta * phieta)) +
                             dzeta * dzeta * (1.f - phizeta * phizeta);
            qlin = -d2f(P.qlc_monoq) * rho * sl;
            qquad = d2f(P.qqc_monoq) * rho * sq;
        }
        if (d.keep & 2) {
            d.ql[k] = f2d(qlin);
            d.qq[k] = f2d(qquad);
        }
        // the EOS, energy, sound speed and constraint candidates in pairs,
        // the energy accumulated in FP64 (eos_df.cuh)
        const double ssn = material_update_df(d, k, sc, vnew, df64(qlin, 0.f), df64(qquad, 0.f),
                                              d.reps ? __ldg(d.reps + k) : 1);
        if (kConstraints) constraint_keys_df(ssn, vdov, d.arealg[k], P, kc, kh);
    }
}

// Eight blocks per SM (64 registers, ~30 bytes spilled): the kernel waits on
// its neighbour loads, and the extra warps hide them better than the spills
// cost (0.61 ms at six blocks, 0.56 at seven, 0.55 at eight, s=192).
template <bool kConstraints>
__global__ void __launch_bounds__(kBlockElem, 8) k_elem_material_split(const __grid_constant__ Dom d)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    unsigned long long kc = ~0ULL, kh = ~0ULL;
    if (t < d.ne && !skip_step(d)) {
        const int k = d.mat_order ? __ldg(d.mat_order + t) : t;   // cost-grouped order with regions
        elem_material_split<kConstraints>(d, k, d.sc, kc, kh);
    }
    if (kConstraints) block_min_publish(kc, kh, d.sc);
}

// ---------------------------------------------------------------------
// Launchers
// ---------------------------------------------------------------------
static inline unsigned blocks_for(long n, int bs) { return (unsigned)((n + bs - 1) / bs); }

// The force kernel: staged tiles on structured cubes wide enough to fill
// them (s >= 64 columns), the gather kernel otherwise (unstructured meshes,
// small cubes).
static void launch_elem_force_split(const Dom &d, cudaStream_t st)
{
    if (d.s >= kTileCols) {
        k_elem_force_split_tiled<<<(unsigned)SoloTile::tiles(d.s), SoloTile::kThreads, 0, st>>>(d);
    } else {
        k_elem_force_split<<<blocks_for(d.ne, elem_block(d)), elem_block(d), 0, st>>>(d);
    }
}

void launch_split_sync(const Dom &d, cudaStream_t st)
{
    k_split_sync<<<blocks_for(d.nn, node_block(d)), node_block(d), 0, st>>>(d);
}

void launch_lagrange_nodal_split(const Dom &d, cudaStream_t st)
{
    launch_elem_force_split(d, st);
    k_node_update_split<<<blocks_for(d.nn, node_block(d)), node_block(d), 0, st>>>(d);
}

void launch_lagrange_elements_split(const Dom &d, cudaStream_t st, bool with_constraints)
{
    k_elem_kinematics_split<<<blocks_for(d.ne, kin_block(d)), kin_block(d), 0, st>>>(d);
    if (with_constraints)
        k_elem_material_split<true><<<blocks_for(d.ne, elem_block(d)), elem_block(d), 0, st>>>(d);
    else
        k_elem_material_split<false><<<blocks_for(d.ne, elem_block(d)), elem_block(d), 0, st>>>(d);
}

void launch_run_body_split(const Dom &d, cudaStream_t st, cudaGraphConditionalHandle h, int *active)
{
    launch_time_increment(d, st);
    launch_lagrange_nodal_split(d, st);
    launch_lagrange_elements_split(d, st, true);
    launch_run_epilogue(d, st, h, active);
}

void launch_cycle_timed_split(const Dom &d, cudaStream_t st, cudaEvent_t ev[kTimedKernels + 1])
{
    cudaEventRecord(ev[0], st);
    launch_time_increment(d, st);
    cudaEventRecord(ev[1], st);
    launch_elem_force_split(d, st);
    cudaEventRecord(ev[2], st);
    k_node_update_split<<<blocks_for(d.nn, node_block(d)), node_block(d), 0, st>>>(d);
    cudaEventRecord(ev[3], st);
    k_elem_kinematics_split<<<blocks_for(d.ne, kin_block(d)), kin_block(d), 0, st>>>(d);
    cudaEventRecord(ev[4], st);
    k_elem_material_split<true><<<blocks_for(d.ne, elem_block(d)), elem_block(d), 0, st>>>(d);
    cudaEventRecord(ev[5], st);
    launch_finalize(d, st);
    cudaEventRecord(ev[6], st);
}

// ---------------------------------------------------------------------
// Batched ensembles: the same bodies over the active tiles of one class
// ---------------------------------------------------------------------
void launch_batch_kernel_split(const Dom &d, const BatchView &b, cudaStream_t st, int kernel, int cls,
                              LaunchCfg cfg)
{
    switch (kernel) {
    case 0: kb_elem<elem_force_split><<<cfg.grid, cfg.block, 0, st>>>(d, b, cls); break;
    case 1: kb_node<node_update_split><<<cfg.grid, cfg.block, 0, st>>>(d, b, cls); break;
    case 2: kb_elem_capped<elem_kinematics_split, 2><<<cfg.grid, cfg.block, 0, st>>>(d, b, cls); break;
    default: kb_material_capped<elem_material_split<true>, 4><<<cfg.grid, cfg.block, 0, st>>>(d, b, cls); break;
    }
}

// The staged batched force kernel of one class with `rows` element rows per
// tile (cfg.block is then rows x kTileCols).
void launch_batch_force_split_staged(const Dom &d, const BatchView &b, const StagedClass &sc, int rows,
                                     LaunchCfg cfg, cudaStream_t st)
{
    if (rows == 4) kb_force_split_staged<4><<<cfg.grid, TileShape<4>::kThreads, 0, st>>>(d, b, sc);
    else kb_force_split_staged<2><<<cfg.grid, TileShape<2>::kThreads, 0, st>>>(d, b, sc);
}

int batch_max_blocks_split_staged(int rows)
{
    int n = 0;
    const cudaError_t e =
        rows == 4 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kb_force_split_staged<4>, TileShape<4>::kThreads, 0)
                  : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kb_force_split_staged<2>, TileShape<2>::kThreads, 0);
    return e == cudaSuccess ? n : 0;
}

// Resident blocks per SM of a batched kernel at a block size.
int batch_max_blocks_split(int kernel, int block)
{
    int n = 0;
    cudaError_t e;
    switch (kernel) {
    case 0: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kb_elem<elem_force_split>, block, 0); break;
    case 1: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kb_node<node_update_split>, block, 0); break;
    case 2: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kb_elem_capped<elem_kinematics_split, 2>, block, 0); break;
    default: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kb_material_capped<elem_material_split<true>, 4>, block, 0); break;
    }
    return e == cudaSuccess ? n : 0;
}

}  // namespace lulesh
