// common.cuh -- device helpers shared by the FP64 and split-precision steps.
#pragma once

#include "lulesh_internal.h"
#include "fastmath.cuh"
#include "df64.cuh"

#include <cuda_runtime.h>

namespace lulesh {

__device__ __forceinline__ void load_nodelist(const int *nodelist, int k, int nl[8])
{
    const int4 *p = reinterpret_cast<const int4 *>(nodelist + 8 * (size_t)k);
    const int4 a = __ldg(p), b = __ldg(p + 1);
    nl[0] = a.x; nl[1] = a.y; nl[2] = a.z; nl[3] = a.w;
    nl[4] = b.x; nl[5] = b.y; nl[6] = b.z; nl[7] = b.w;
}

__device__ __forceinline__ void gather8(const double *__restrict__ f, const int nl[8], double out[8])
{
#pragma unroll
    for (int c = 0; c < 8; ++c) out[c] = __ldg(f + nl[c]);
}

__device__ __forceinline__ void flag_error(DevScalars *sc, int site, int elem)
{
    sc->err[site] = elem + 1;
    sc->err_any = 1;
}

// A kernel of the step does nothing once an earlier phase of the cycle has
// flagged an error (the reference would have exited), or when the run loop
// has been stopped (only in the host-driven fallback loop, where d.gate is
// set).  Kernels that use a block barrier evaluate this into a flag instead
// of returning, so that every thread reaches the barrier.
__device__ __forceinline__ bool skip_step(const Dom &d)
{
    return d.sc->err_any != 0 || (d.gate != nullptr && *d.gate == 0);
}

// ---------------------------------------------------------------------
// TimeIncrement (LULESH-OMP.cc:557-604)
// ---------------------------------------------------------------------
__device__ __forceinline__ void time_increment(DevScalars *sc, const lulesh_params &P)
{
    double targetdt = P.stoptime - sc->time;
    if ((P.dtfixed <= 0.0) && (sc->cycle != 0)) {
        const double olddt = sc->deltatime;
        double newdt = 1.0e+20;
        if (sc->dtcourant < newdt) newdt = sc->dtcourant / 2.0;
        if (sc->dthydro < newdt) newdt = sc->dthydro * 2.0 / 3.0;
        const double ratio = newdt / olddt;
        if (ratio >= 1.0) {
            if (ratio < P.deltatimemultlb) newdt = olddt;
            else if (ratio > P.deltatimemultub) newdt = olddt * P.deltatimemultub;
        }
        if (newdt > P.dtmax) newdt = P.dtmax;
        sc->deltatime = newdt;
    }
    if ((targetdt > sc->deltatime) && (targetdt < (4.0 * sc->deltatime / 3.0)))
        targetdt = 2.0 * sc->deltatime / 3.0;
    if (targetdt < sc->deltatime) sc->deltatime = targetdt;
    sc->time += sc->deltatime;
    ++sc->cycle;
}

// Comparisons of doubles on the integer pipes.  The FP64 unit of this part
// retires two lanes per SM per clock and an FP64 compare takes one of those
// slots like an FMA; the integer units are many times wider.  ikey maps a
// double onto an int64 that orders like the value (sign-magnitude to two's
// complement; -0 and +0 both map to 0), so for non-NaN operands these give
// the IEEE results.  The keys are formed in inline PTX so that the compiler
// keeps them integer work.  The step's error tests (volume, qstop) stay IEEE
// compares, so that a NaN never raises or hides them differently.
__device__ __forceinline__ long long ikey(double x)
{
    long long k;
    asm("{\n\t.reg .b64 b, m, s;\n\t"
        "mov.b64 b, %1;\n\t"
        "and.b64 m, b, 0x7fffffffffffffff;\n\t"
        "shr.s64 s, b, 63;\n\t"
        "xor.b64 m, m, s;\n\t"
        "sub.s64 %0, m, s;\n\t}"
        : "=l"(k) : "d"(x));
    return k;
}
// |x| as its bit pattern (orders like |x| for non-NaN x)
__device__ __forceinline__ unsigned long long iabs(double x)
{
    unsigned long long k;
    asm("{\n\t.reg .b64 b;\n\tmov.b64 b, %1;\n\tand.b64 %0, b, 0x7fffffffffffffff;\n\t}" : "=l"(k) : "d"(x));
    return k;
}
// -x by flipping the sign bit on the integer pipes (a negation the compiler
// cannot fold into a neighbouring operation otherwise costs an FP64 add)
__device__ __forceinline__ double neg(double x)
{
    double r;
    asm("{\n\t.reg .b64 b;\n\tmov.b64 b, %1;\n\txor.b64 b, b, 0x8000000000000000;\n\tmov.b64 %0, b;\n\t}"
        : "=d"(r) : "d"(x));
    return r;
}
__device__ __forceinline__ bool lt(double a, double b) { return ikey(a) < ikey(b); }
__device__ __forceinline__ bool le(double a, double b) { return ikey(a) <= ikey(b); }
__device__ __forceinline__ bool gt(double a, double b) { return ikey(a) > ikey(b); }
__device__ __forceinline__ bool ge(double a, double b) { return ikey(a) >= ikey(b); }
// |a| < |c|
__device__ __forceinline__ bool abs_lt(double a, double c) { return iabs(a) < iabs(c); }
// FP32 compares are cheap already
__device__ __forceinline__ bool lt(float a, float b) { return a < b; }
__device__ __forceinline__ bool gt(float a, float b) { return a > b; }

// 1/x: in FP64 refined from the FP32 estimate (fastmath.cuh, within an ulp
// or so of the quotient), in FP32 correctly rounded.
__device__ __forceinline__ double recip(double x) { return rcp_fast(x); }
__device__ __forceinline__ float recip(float x) { return __frcp_rn(x); }

// Conversions between FP64 and FP32 run on GB300's FP64 pipe at the FP64
// rate (2 per SM per clock), so this file converts with integer bit
// operations instead.  Values below FP32's normal range (|v| < 2^-126)
// become signed zeros; positions, velocities, forces and the element scalars
// converted here never live there.

// double -> float, mantissa truncated to 23 bits (error < 2^-23 relative).
__device__ __forceinline__ float d2f(double v)
{
    const unsigned long long b = (unsigned long long)__double_as_longlong(v);
    const unsigned hi = (unsigned)(b >> 32);
    const unsigned sign = hi & 0x80000000u;
    const int de = (int)((hi >> 20) & 0x7ffu);
    const unsigned mant = (unsigned)(b >> 29) & 0x7fffffu;
    if (de == 0x7ff) return __uint_as_float(sign | 0x7f800000u | (mant ? 0x400000u : 0u));   // inf, nan
    const int fe = de - 1023 + 127;
    if (fe <= 0) return __uint_as_float(sign);
    if (fe >= 255) return __uint_as_float(sign | 0x7f800000u);
    return __uint_as_float(sign | ((unsigned)fe << 23) | mant);
}

// float -> double, exact (FP32 subnormals become zeros).
__device__ __forceinline__ double f2d(float f) { return df_f2d(f); }

// The node update after the corner gather: CalcAccelerationForNodes, the
// symmetry-plane conditions, CalcVelocityForNodes and CalcPositionForNodes
// (LULESH-OMP.cc:1613-1683) for node n with nodal force (fx, fy, fz).
__device__ __forceinline__ void node_integrate(const Dom &d, int n, const DevScalars *sc, double fx, double fy,
                                               double fz)
{
    if (d.keep & 1) {
        d.fx[n] = fx;
        d.fy[n] = fy;
        d.fz[n] = fz;
    }
    const double dt = sc->deltatime, u_cut = d.prm.u_cut;
    const unsigned bc = __ldg(d.node_bc + n);
    double ax, ay, az;
    if (d.inv_mass) {
        // f * (1/m) with the reciprocal precomputed: within an ulp of f / m
        const double im = __ldg(d.inv_mass + n);
        ax = (bc & 1) ? 0.0 : fx * im;
        ay = (bc & 2) ? 0.0 : fy * im;
        az = (bc & 4) ? 0.0 : fz * im;
    } else {
        const double m = __ldg(d.nodal_mass + n);
        ax = (bc & 1) ? 0.0 : fx / m;
        ay = (bc & 2) ? 0.0 : fy / m;
        az = (bc & 4) ? 0.0 : fz / m;
    }
    double t;
    t = d.xd[n] + ax * dt; if (abs_lt(t, u_cut)) t = 0.0; d.xd[n] = t; d.x[n] += t * dt;
    t = d.yd[n] + ay * dt; if (abs_lt(t, u_cut)) t = 0.0; d.yd[n] = t; d.y[n] += t * dt;
    t = d.zd[n] + az * dt; if (abs_lt(t, u_cut)) t = 0.0; d.zd[n] = t; d.z[n] += t * dt;
}

// The six face neighbours of element k (lxim, lxip, letam, letap, lzetam,
// lzetap).  On the structured s^3 cube of the reference's set-up (Dom::s > 0,
// or a batch instance's DevScalars::edge > 0, whose elements are contiguous)
// they are k -+ 1, k -+ s and k -+ s^2 across every interior face, the only
// faces whose neighbour the limiter reads (a boundary face carries a BC
// flag), so there they are formed instead of loaded: the limiter's
// neighbour slopes then depend on no earlier load.
struct FaceNeighbours {
    int xim, xip, etam, etap, zetam, zetap;
};
__device__ __forceinline__ FaceNeighbours face_neighbours(const Dom &d, const DevScalars *sc, int k)
{
    const int s = d.s > 0 ? d.s : sc->edge;
    if (s > 0) {
        const int s2 = s * s;
        return {k - 1, k + 1, k - s, k + s, k - s2, k + s2};
    }
    return {__ldg(d.lxim + k), __ldg(d.lxip + k), __ldg(d.letam + k),
            __ldg(d.letap + k), __ldg(d.lzetam + k), __ldg(d.lzetap + k)};
}

// Node n's corner slots (corner * ne + element), in the order of the
// reference's node-to-corner lists (AllocateNodeElemIndexes,
// LULESH-OMP.cc:209-268: the node's elements in increasing order), each
// passed to f(slot, first).  On the structured s^3 cube (Dom::s > 0, or a
// batch instance's DevScalars::edge > 0, whose nodes and elements are
// contiguous from node_begin and elem_begin) they are formed from the
// node's coordinates -- the element below, behind and left of the node
// first -- instead of loaded from the corner tables, which takes the
// tables' loads and their dependent level off the node update.
template <class F>
__device__ __forceinline__ void for_node_corners(const Dom &d, const DevScalars *sc, int n, F &&f)
{
    const int s = d.s > 0 ? d.s : sc->edge;
    if (s > 0) {
        const int en = s + 1;
        const size_t ne = (size_t)d.ne;
        const int e0 = d.s > 0 ? 0 : sc->elem_begin;
        if (d.s <= 0) n -= sc->node_begin;
        const int c = n % en, r = (n / en) % en, p = n / (en * en);
        bool first = true;
#pragma unroll
        for (int dp = 1; dp >= 0; --dp)
#pragma unroll
            for (int dr = 1; dr >= 0; --dr)
#pragma unroll
                for (int dc = 1; dc >= 0; --dc) {
                    const int ep = p - dp, er = r - dr, ec = c - dc;
                    if (ep < 0 || ep >= s || er < 0 || er >= s || ec < 0 || ec >= s) continue;
                    // the node is the corner at offset (dc, dr, dp) of its element
                    const int corner = dp ? (dr ? (dc ? 6 : 7) : (dc ? 5 : 4)) : (dr ? (dc ? 2 : 3) : (dc ? 1 : 0));
                    f((int)(corner * ne + (size_t)(e0 + (ep * s + er) * s + ec)), first);
                    first = false;
                }
        return;
    }
    const int st = __ldg(d.corner_start + n), en = __ldg(d.corner_start + n + 1);
    for (int i = st; i < en; ++i) f(__ldg(d.corner_list + i), i == st);
}

// One direction of the monotonic limiter (:2198-2228).
template <typename T>
__device__ __forceinline__ T limiter_phi(const T *__restrict__ delv, int i, int bm, int bp,
                                         int m_symm, int m_free, int p_symm, int p_free,
                                         int lm, int lp, T limiter, T max_slope)
{
    const T ptiny = T(1.e-36);
    const T own = delv[i];
    const T norm = recip(own + ptiny);
    T delvm = T(0.0), delvp = T(0.0);
    if (bm == 0) delvm = delv[lm];
    else if (bm == m_symm) delvm = own;
    else if (bm == m_free) delvm = 0.0;
    if (bp == 0) delvp = delv[lp];
    else if (bp == p_symm) delvp = own;
    else if (bp == p_free) delvp = 0.0;
    delvm = delvm * norm;
    delvp = delvp * norm;
    T phi = T(.5) * (delvm + delvp);
    delvm *= limiter;
    delvp *= limiter;
    if (lt(delvm, phi)) phi = delvm;
    if (lt(delvp, phi)) phi = delvp;
    if (lt(phi, T(0.))) phi = T(0.);
    if (gt(phi, max_slope)) phi = max_slope;
    return phi;
}

// CalcPressureForElems for one element (:2384-2413).
__device__ __forceinline__ double eos_pressure(double &bvc, double e, double comp, double vnewc,
                                               const lulesh_params &P)
{
    const double c1s = 2.0 / 3.0;
    bvc = c1s * (comp + 1.);
    double p = bvc * e;
    if (abs_lt(p, P.p_cut)) p = 0.0;
    if (ge(vnewc, P.eosvmax)) p = 0.0;
    if (lt(p, P.pmin)) p = P.pmin;
    return p;
}

// sqrt((pbvc*e + vv^2*bvc*p)/rho0) with the reference's floor (:2485-2493).
__device__ __forceinline__ double sound_term(double pbvc, double e, double vv, double bvc, double p,
                                             double rho0, bool unit_rho0)
{
    double ssc = pbvc * e + vv * vv * bvc * p;
    if (!unit_rho0) ssc = ssc / rho0;   // x / 1.0 == x: the division is skipped only then
    // sqrt(x) as x * rsqrt(x) (x > 1.1e-37 here): within a few ulps of the
    // correctly rounded root at a fraction of its FP64 instructions
    if (le(ssc, .111111e-36)) ssc = .333333e-18;
    else ssc = ssc * rsqrt(ssc);
    return ssc;
}

// ssc * qlin + qquad with ssc the sound term of the viscosity update.  With
// kF32Q (split precision, whose Q coefficients qlin/qquad are FP32) the term
// is formed in FP32: the coefficients carry FP32 precision already, so an
// FP64 square root would add FP64 work and no accuracy.
template <bool kF32Q>
__device__ __forceinline__ double q_term(double pbvc, double e, double vv, double bvc, double p,
                                         double rho0, bool unit_rho0, double qlin, double qquad)
{
    if constexpr (kF32Q) {
        const float vvf = d2f(vv);
        float ssc = d2f(pbvc) * d2f(e) + vvf * vvf * d2f(bvc) * d2f(p);
        if (!unit_rho0) ssc = ssc / d2f(rho0);
        ssc = (ssc <= .111111e-36f) ? .333333e-18f : sqrtf(ssc);
        return f2d(ssc * d2f(qlin) + d2f(qquad));
    } else {
        return sound_term(pbvc, e, vv, bvc, p, rho0, unit_rho0) * qlin + qquad;
    }
}

// The qstop test, ApplyMaterialPropertiesForElems, EvalEOSForElems +
// CalcEnergyForElems + CalcSoundSpeedForElems and UpdateVolumesForElems for
// element k (LULESH-OMP.cc:2369-2381, :2384-2782), given its monotonic-Q
// terms; every loop of the reference there is element-local.  Writes
// p, e, q, ss and v and returns the new sound speed.
//
// rep > 1 evaluates the EOS rep times from the same inputs, as LULESH 2.0
// does for its costly regions (lulesh-2.0.3/lulesh.cc:2265-2323, called with
// rep from :2410-2424): the results are those of one evaluation, and the
// empty asm statements keep the compiler from merging or dropping the
// repeated evaluations.
__device__ __forceinline__ void opaque(double &v) { asm volatile("" : "+d"(v)); }
__device__ __forceinline__ void consume(double v) { asm volatile("" ::"d"(v)); }

template <bool kF32Q = false>
__device__ __forceinline__ double material_update(const Dom &d, int k, DevScalars *sc, double vnew,
                                                  double qlin, double qquad, int rep = 1)
{
    const lulesh_params &P = d.prm;
    if (rep < 1) rep = 1;
    // CalcQForElems qstop test on the old q (:2369-2381)
    const double q_old_in = d.q[k];
    if (q_old_in > P.qstop) flag_error(sc, ERR_K3_QSTOP, k);

    // ApplyMaterialPropertiesForElems (:2703-2761)
    const double eosvmin = P.eosvmin, eosvmax = P.eosvmax;
    double vnewc_in = vnew;
    // eosvmin/eosvmax != 0 (a zero bound switches the bound off)
    const bool has_vmin = iabs(eosvmin) != 0ULL, has_vmax = iabs(eosvmax) != 0ULL;
    if (has_vmin && lt(vnewc_in, eosvmin)) vnewc_in = eosvmin;
    if (has_vmax && gt(vnewc_in, eosvmax)) vnewc_in = eosvmax;
    const double qlin_in = qlin, qquad_in = qquad;
    const double v_old = d.v[k];
    double vc = v_old;
    if (has_vmin && lt(vc, eosvmin)) vc = eosvmin;
    if (has_vmax && gt(vc, eosvmax)) vc = eosvmax;
    if (vc <= 0.) flag_error(sc, ERR_K3_MATV, k);

    // EvalEOSForElems + CalcEnergyForElems (:2415-2701); work == 0
    const double delvc_in = d.delv[k], e_old_in = d.e[k], p_old_in = d.p[k];
    const double rho0 = P.refdens;
    const bool unit_rho0 = ikey(rho0) == ikey(1.0);
    const double pbvc = 2.0 / 3.0;
    double p_new, e_new, q_new, bvc, ssn;
    for (int j = 0; j < rep; ++j) {
        double delvc = delvc_in, e_old = e_old_in, p_old = p_old_in, q_old = q_old_in, vnewc = vnewc_in;
        double qlin = qlin_in, qquad = qquad_in;
        if (rep > 1) {
            opaque(delvc); opaque(e_old); opaque(p_old); opaque(q_old); opaque(vnewc);
            opaque(qlin); opaque(qquad);
        }
        double compression = rcp_fast(vnewc) - 1.;
        const double vchalf = vnewc - delvc * .5;
        double comp_half = rcp_fast(vchalf) - 1.;
        // vhalf = 1 / (1 + comp_half) (:2460), which is vchalf, vnewc or 1 in the
        // three cases below; taken directly instead of through two divisions
        double vhalf = vchalf;
        if (has_vmin && le(vnewc, eosvmin)) {
            comp_half = compression;
            vhalf = vnewc;
        }
        if (has_vmax && ge(vnewc, eosvmax)) {
            p_old = 0.;
            compression = 0.;
            comp_half = 0.;
            vhalf = 1.;
        }
        const double emin = P.emin, e_cut = P.e_cut;

        e_new = e_old - .5 * delvc * (p_old + q_old);
        if (lt(e_new, emin)) e_new = emin;
        const double p_half = eos_pressure(bvc, e_new, comp_half, vnewc, P);
        q_new = 0.;
        if (!gt(delvc, 0.)) q_new = q_term<kF32Q>(pbvc, e_new, vhalf, bvc, p_half, rho0, unit_rho0, qlin, qquad);
        e_new = e_new + .5 * delvc * (3.0 * (p_old + q_old) - 4.0 * (p_half + q_new));
        if (abs_lt(e_new, e_cut)) e_new = 0.;
        if (lt(e_new, emin)) e_new = emin;

        p_new = eos_pressure(bvc, e_new, compression, vnewc, P);
        double q_tilde = 0.;
        if (!gt(delvc, 0.)) q_tilde = q_term<kF32Q>(pbvc, e_new, vnewc, bvc, p_new, rho0, unit_rho0, qlin, qquad);
        const double sixth = 1.0 / 6.0;
        e_new = e_new - (7.0 * (p_old + q_old) - 8.0 * (p_half + q_new) + (p_new + q_tilde)) * delvc * sixth;
        if (abs_lt(e_new, e_cut)) e_new = 0.;
        if (lt(e_new, emin)) e_new = emin;

        p_new = eos_pressure(bvc, e_new, compression, vnewc, P);
        // CalcSoundSpeedForElems (:2543-2561) takes the last evaluation's
        ssn = sound_term(pbvc, e_new, vnewc, bvc, p_new, rho0, unit_rho0);
        if (le(delvc, 0.)) {
            q_new = ssn * qlin + qquad;
            if (abs_lt(q_new, P.q_cut)) q_new = 0.;
        }
        if (rep > 1) {
            consume(p_new); consume(e_new); consume(q_new); consume(ssn);
        }
    }
    d.p[k] = p_new;
    d.e[k] = e_new;
    d.q[k] = q_new;
    d.ss[k] = ssn;

    // UpdateVolumesForElems (:2763-2782)
    double vt = vnew;
    if (abs_lt(vt - 1.0, P.v_cut)) vt = 1.0;
    d.v[k] = vt;
    return ssn;
}

// Order-preserving map of a double onto uint64 (NaN maps to the maximum, so
// it never wins a minimum, as in the reference's '<' tests).
__device__ __forceinline__ unsigned long long order_key(double v)
{
    const unsigned long long b = (unsigned long long)__double_as_longlong(v);
    if (iabs(v) > 0x7ff0000000000000ULL) return ~0ULL;   // NaN
    return (b & 0x8000000000000000ULL) ? ~b : (b | 0x8000000000000000ULL);
}
__device__ __forceinline__ double key_value(unsigned long long k)
{
    const unsigned long long b = (k & 0x8000000000000000ULL) ? (k & 0x7fffffffffffffffULL) : ~k;
    return __longlong_as_double((long long)b);
}

__device__ __forceinline__ unsigned long long warp_min_u64(unsigned long long v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long w = __shfl_xor_sync(0xffffffffu, v, o);
        v = w < v ? w : v;
    }
    return v;
}

// Block-wide minimum of two keys, one atomicMin each per block.
__device__ __forceinline__ void block_min_publish(unsigned long long kc, unsigned long long kh,
                                                  DevScalars *sc)
{
    __shared__ unsigned long long s_c[32], s_h[32];
    kc = warp_min_u64(kc);
    kh = warp_min_u64(kh);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) { s_c[warp] = kc; s_h[warp] = kh; }
    __syncthreads();
    if (warp == 0) {
        const int nw = (blockDim.x + 31) >> 5;
        kc = lane < nw ? s_c[lane] : ~0ULL;
        kh = lane < nw ? s_h[lane] : ~0ULL;
        kc = warp_min_u64(kc);
        kh = warp_min_u64(kh);
        if (lane == 0) {
            if (kc != ~0ULL) atomicMin(&sc->courant_key, kc);
            if (kh != ~0ULL) atomicMin(&sc->hydro_key, kh);
        }
    }
}

// Constraint candidates of one element (:2820-2855, :2897-2915).
__device__ __forceinline__ void constraint_keys(double ss, double vdov, double arealg,
                                                const lulesh_params &P,
                                                unsigned long long &kc, unsigned long long &kh)
{
    kc = ~0ULL;
    kh = ~0ULL;
    if (iabs(vdov) != 0ULL) {
        const double qqc2 = 64.0 * P.qqc * P.qqc;
        double dtf = ss * ss;
        if (lt(vdov, 0.)) dtf = dtf + qqc2 * arealg * arealg * vdov * vdov;
        dtf = arealg * rsqrt(dtf);      // arealg / sqrt(dtf)
        kc = order_key(dtf);
        kh = order_key(quot_fast(P.dvovmax, fabs(vdov) + 1.e-20));
    }
}

// The same candidates with the arithmetic in double-float pairs (the
// default plain path): the comparisons that decide which terms enter stay
// on the FP64 values.
__device__ __forceinline__ void constraint_keys_df(double ss, double vdov, double arealg,
                                                   const lulesh_params &P,
                                                   unsigned long long &kc, unsigned long long &kh)
{
    kc = ~0ULL;
    kh = ~0ULL;
    if (iabs(vdov) != 0ULL) {
        const df64 s = to_df(ss), a = to_df(arealg), v = to_df(vdov);
        df64 dtf = s * s;
        if (lt(vdov, 0.)) dtf = fma(to_df(64.0 * P.qqc * P.qqc) * (a * a), v * v, dtf);
        kc = order_key(to_double(a * df_rsqrt(dtf)));          // arealg / sqrt(dtf)
        kh = order_key(to_double(df_div(to_df(P.dvovmax), fabs(v) + df64(1.e-20))));
    }
}

// Publish the constraint minima: a value is registered only when some
// element was active and it is below the 1e20 start value (:2869-2871,
// :2928-2930); otherwise the previous dtcourant/dthydro stay.
__device__ __forceinline__ void finalize_constraints(DevScalars *sc)
{
    const unsigned long long limit = order_key(1.0e+20);
    if (sc->courant_key < limit) sc->dtcourant = key_value(sc->courant_key);
    if (sc->hydro_key < limit) sc->dthydro = key_value(sc->hydro_key);
    sc->courant_key = ~0ULL;
    sc->hydro_key = ~0ULL;
}

// Run-loop control: may another cycle start?  Besides the reference's
// time < stoptime test and the caller's cap, the loop stops when the time
// step is no longer positive (the reference would spin forever there) and
// after kRunCycleLimit cycles, so a device-side loop always ends.
__device__ __forceinline__ unsigned run_continue(const DevScalars *sc, const lulesh_params &P)
{
    const int cap = (sc->run_max > 0 && sc->run_max < kRunCycleLimit) ? sc->run_max : kRunCycleLimit;
    return (sc->err_any == 0) && (sc->time < P.stoptime) && (sc->deltatime > 0.0) &&
           (sc->run_cycles < cap);
}

}  // namespace lulesh
