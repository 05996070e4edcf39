// eos_df.cuh -- the material update with its arithmetic in double-float
// pairs (df64.cuh): pressures, viscosities, sound speeds and the energy
// increments as pairs, the energy itself accumulated in FP64.
#pragma once

#include "common.cuh"

namespace lulesh {

// ---- the EOS with its arithmetic in pairs --------------------------------
// The EOS parameters that the pair arithmetic compares against, converted
// once per element.
struct EosCuts {
    df64 p_cut, pmin, q_cut;
    __device__ explicit EosCuts(const lulesh_params &P) : p_cut(to_df(P.p_cut)), pmin(to_df(P.pmin)), q_cut(to_df(P.q_cut)) {}
};

// CalcPressureForElems (:2384-2413): p = (2/3)(1 + compression) e with the
// reference's cuts (p_zero: vnewc >= eosvmax, tested by the reference
// whether or not the bound is switched on); bvc receives
// (2/3)(1 + compression).  e is the energy as a pair.
__device__ __forceinline__ df64 eos_pressure_df(df64 &bvc, df64 e, df64 comp, bool p_zero, const EosCuts &cut)
{
    bvc = df64(2.0 / 3.0) * (comp + df64(1.f, 0.f));
    df64 p = bvc * e;
    if (df_gt(cut.p_cut, fabs(p))) p = df64(0.f, 0.f);
    if (p_zero) p = df64(0.f, 0.f);
    if (df_gt(cut.pmin, p)) p = cut.pmin;
    return p;
}

// sqrt((pbvc e + vv^2 bvc p) / rho0) with the reference's floor (:2485-2493)
__device__ __forceinline__ df64 sound_term_df(df64 e, df64 vv, df64 bvc, df64 p, double rho0, bool unit_rho0)
{
    df64 ssc = fma(df64(2.0 / 3.0), e, vv * vv * bvc * p);
    if (!unit_rho0) ssc = df_div(ssc, to_df(rho0));
    if (!df_gt(ssc, df64(.111111e-36))) return df64(.333333e-18);
    return ssc * df_rsqrt(ssc);
}

__device__ __forceinline__ void opaque_df(df64 &v) { asm volatile("" : "+f"(v.hi), "+f"(v.lo)); }

// The qstop test, ApplyMaterialPropertiesForElems, EvalEOSForElems +
// CalcEnergyForElems + CalcSoundSpeedForElems and UpdateVolumesForElems
// (LULESH-OMP.cc:2369-2381, :2384-2782), as material_update of common.cuh,
// with the pressures, viscosities, sound speeds and the energy increments
// in pairs.  The energy is state carried from cycle to cycle, so each of the
// three energy stages adds its increment to the FP64 energy with one FP64
// addition: the energy keeps its FP64 precision, and only the increments
// carry the pairs' ~2^-47.  The comparisons against the cuts and bounds use
// the same quantities as the FP64 kernel, in whichever form they are held.
__device__ __forceinline__ double material_update_df(const Dom &d, int k, DevScalars *sc, double vnew,
                                                     df64 qlin_in, df64 qquad_in, int rep)
{
    const lulesh_params &P = d.prm;
    if (rep < 1) rep = 1;
    const double q_old_in = d.q[k];
    if (q_old_in > P.qstop) flag_error(sc, ERR_K3_QSTOP, k);

    const double eosvmin = P.eosvmin, eosvmax = P.eosvmax;
    double vnewc_in = vnew;
    const bool has_vmin = iabs(eosvmin) != 0ULL, has_vmax = iabs(eosvmax) != 0ULL;
    if (has_vmin && lt(vnewc_in, eosvmin)) vnewc_in = eosvmin;
    if (has_vmax && gt(vnewc_in, eosvmax)) vnewc_in = eosvmax;
    double vc = d.v[k];
    if (has_vmin && lt(vc, eosvmin)) vc = eosvmin;
    if (has_vmax && gt(vc, eosvmax)) vc = eosvmax;
    if (vc <= 0.) flag_error(sc, ERR_K3_MATV, k);

    const double delvc_in = d.delv[k], e_old_in = d.e[k], p_old_in = d.p[k];
    const double rho0 = P.refdens;
    const bool unit_rho0 = ikey(rho0) == ikey(1.0);
    const double emin = P.emin, e_cut = P.e_cut;
    const EosCuts cut(P);
    df64 p_new(0.f, 0.f), q_new(0.f, 0.f), ssn(0.f, 0.f), bvc;
    double e_new = 0.0;
    for (int j = 0; j < rep; ++j) {
        double delvc = delvc_in, e_old = e_old_in, p_old = p_old_in, q_old = q_old_in, vnewc = vnewc_in;
        df64 qlin = qlin_in, qquad = qquad_in;
        if (rep > 1) {
            opaque(delvc); opaque(e_old); opaque(p_old); opaque(q_old); opaque(vnewc);
            opaque_df(qlin); opaque_df(qquad);
        }
        const df64 one(1.f, 0.f);
        const df64 dvc = to_df(delvc), vn = to_df(vnewc);
        df64 compression = df_rcp(vn) - one;
        const df64 vchalf = vn - df_scale(dvc, 0.5f);
        df64 comp_half = df_rcp(vchalf) - one;
        df64 vhalf = vchalf;
        if (has_vmin && le(vnewc, eosvmin)) {
            comp_half = compression;
            vhalf = vn;
        }
        const bool p_zero = ge(vnewc, eosvmax);
        const bool at_vmax = has_vmax && p_zero;
        df64 pq_old = to_df(p_old) + to_df(q_old);
        if (at_vmax) {
            pq_old = to_df(q_old);   // p_old = 0
            compression = df64(0.f, 0.f);
            comp_half = df64(0.f, 0.f);
            vhalf = one;
        }

        e_new = e_old + to_double(-df_scale(dvc * pq_old, 0.5f));
        if (lt(e_new, emin)) e_new = emin;
        df64 e_df = to_df(e_new);
        const df64 p_half = eos_pressure_df(bvc, e_df, comp_half, p_zero, cut);
        q_new = df64(0.f, 0.f);
        if (!gt(delvc, 0.)) q_new = fma(sound_term_df(e_df, vhalf, bvc, p_half, rho0, unit_rho0), qlin, qquad);
        const df64 pq_half = p_half + q_new;
        e_new = e_new + to_double(df_scale(dvc * (df_mul_f(pq_old, 3.f) - df_mul_f(pq_half, 4.f)), 0.5f));
        if (abs_lt(e_new, e_cut)) e_new = 0.;
        if (lt(e_new, emin)) e_new = emin;

        e_df = to_df(e_new);
        p_new = eos_pressure_df(bvc, e_df, compression, p_zero, cut);
        df64 q_tilde(0.f, 0.f);
        if (!gt(delvc, 0.)) q_tilde = fma(sound_term_df(e_df, vn, bvc, p_new, rho0, unit_rho0), qlin, qquad);
        const df64 combo = (df_mul_f(pq_old, 7.f) - df_mul_f(pq_half, 8.f)) + (p_new + q_tilde);
        e_new = e_new - to_double(combo * dvc * df64(1.0 / 6.0));
        if (abs_lt(e_new, e_cut)) e_new = 0.;
        if (lt(e_new, emin)) e_new = emin;

        e_df = to_df(e_new);
        p_new = eos_pressure_df(bvc, e_df, compression, p_zero, cut);
        ssn = sound_term_df(e_df, vn, bvc, p_new, rho0, unit_rho0);
        if (le(delvc, 0.)) {
            q_new = fma(ssn, qlin, qquad);
            if (df_gt(cut.q_cut, fabs(q_new))) q_new = df64(0.f, 0.f);
        }
        if (rep > 1) {
            consume(e_new); opaque_df(p_new); opaque_df(q_new); opaque_df(ssn);
        }
    }
    const double ss_d = to_double(ssn);
    d.p[k] = to_double(p_new);
    d.e[k] = e_new;
    d.q[k] = to_double(q_new);
    d.ss[k] = ss_d;

    // UpdateVolumesForElems (:2763-2782)
    double vt = vnew;
    if (abs_lt(vt - 1.0, P.v_cut)) vt = 1.0;
    d.v[k] = vt;
    return ss_d;
}

}  // namespace lulesh
