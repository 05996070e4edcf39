/*
 * lulesh_oracle.c -- CPU restatement of the LULESH 1.0 Lagrange leapfrog step.
 *
 * TEST INFRASTRUCTURE ONLY (see lulesh_oracle.h).  Never linked into the
 * product library.
 *
 * Every floating-point expression keeps the association of the reference
 * (reference/C/LULESH-OMP.cc), so that built with -ffp-contract=off it agrees
 * with the reference bit for bit; the structure (arrays of corners, loops,
 * tables of corner permutations) is this file's own.
 */
#include "lulesh_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <sys/time.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* Element boundary-condition bits, LULESH-OMP.cc:231-253. */
#define BC_XI_M      0x003
#define BC_XI_M_SYMM 0x001
#define BC_XI_M_FREE 0x002
#define BC_XI_P      0x00c
#define BC_XI_P_SYMM 0x004
#define BC_XI_P_FREE 0x008
#define BC_ETA_M      0x030
#define BC_ETA_M_SYMM 0x010
#define BC_ETA_M_FREE 0x020
#define BC_ETA_P      0x0c0
#define BC_ETA_P_SYMM 0x040
#define BC_ETA_P_FREE 0x080
#define BC_ZETA_M      0x300
#define BC_ZETA_M_SYMM 0x100
#define BC_ZETA_M_FREE 0x200
#define BC_ZETA_P      0xc00
#define BC_ZETA_P_SYMM 0x400
#define BC_ZETA_P_FREE 0x800

struct lo_domain {
    int s, nelem, nnode;
    lo_params prm;
    double time, deltatime, dtcourant, dthydro;
    int cycle;

    /* nodal */
    double *x, *y, *z, *xd, *yd, *zd, *xdd, *ydd, *zdd, *fx, *fy, *fz, *nodal_mass;
    /* element */
    double *e, *p, *q, *ql, *qq, *v, *volo, *vnew, *delv, *vdov, *arealg, *ss, *elem_mass;
    double *delv_xi, *delv_eta, *delv_zeta, *delx_xi, *delx_eta, *delx_zeta;
    double *determ;
    /* per-corner temporaries (8 per element) */
    double *fx_elem, *fy_elem, *fz_elem;
    double *dvdx, *dvdy, *dvdz, *x8n, *y8n, *z8n;
    /* connectivity */
    int *nodelist, *lxim, *lxip, *letam, *letap, *lzetam, *lzetap, *elem_bc;
    int *node_elem_start, *node_elem_count, *node_elem_corner_list;
    int *symm_x, *symm_y, *symm_z;
    int nsymm_x, nsymm_y, nsymm_z;       /* (s+1)^2 each on the cube */
    int origin;                          /* element holding the initial energy */
};

/* ------------------------------------------------------------------ */
/* Parameters                                                           */
/* ------------------------------------------------------------------ */

/* LULESH-OMP.cc:3051-3087 */
void lo_default_params(lo_params *p)
{
    memset(p, 0, sizeof *p);
    p->dtfixed = -1.0e-7;
    p->deltatimemultlb = 1.1;
    p->deltatimemultub = 1.2;
    p->stoptime = 1.0e-2;
    p->dtmax = 1.0e-2;
    p->e_cut = 1.0e-7;
    p->p_cut = 1.0e-7;
    p->q_cut = 1.0e-7;
    p->u_cut = 1.0e-7;
    p->v_cut = 1.0e-10;
    p->hgcoef = 3.0;
    p->ss4o3 = 4.0 / 3.0;
    p->qstop = 1.0e+12;
    p->monoq_max_slope = 1.0;
    p->monoq_limiter_mult = 2.0;
    p->qlc_monoq = 0.5;
    p->qqc_monoq = 2.0 / 3.0;
    p->qqc = 2.0;
    p->pmin = 0.0;
    p->emin = -1.0e+15;
    p->dvovmax = 0.1;
    p->eosvmax = 1.0e+9;
    p->eosvmin = 1.0e-9;
    p->refdens = 1.0;
}

int lo_num_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* ------------------------------------------------------------------ */
/* Element geometry kernels                                             */
/* ------------------------------------------------------------------ */

/* Jacobian columns of the trilinear map at the element centre for one
 * coordinate: d/dxi, d/deta, d/dzeta, each scaled by 1/8.
 * LULESH-OMP.cc:650-660 (fjxxi..fjzze). */
static inline void jac_column(const double c[8], double *xi, double *et, double *ze)
{
    const double d60 = c[6] - c[0], d53 = c[5] - c[3];
    const double d71 = c[7] - c[1], d42 = c[4] - c[2];
    *xi = .125 * (((d60 + d53) - d71) - d42);
    *et = .125 * (((d60 - d53) + d71) - d42);
    *ze = .125 * (((d60 + d53) + d71) + d42);
}

/* CalcElemShapeFunctionDerivatives, LULESH-OMP.cc:619-706.
 * b[dim][corner] for corners 0..7 and the Jacobian volume. */
static void shape_derivs(const double x[8], const double y[8], const double z[8],
                         double b[3][8], double *volume)
{
    double a[3], t[3], c[3];           /* d/dxi, d/deta, d/dzeta (per coordinate) */
    jac_column(x, &a[0], &t[0], &c[0]);
    jac_column(y, &a[1], &t[1], &c[1]);
    jac_column(z, &a[2], &t[2], &c[2]);

    /* cofactors: cxi = t x c, cet = c x a, cze = a x t (component-wise the
     * same products and differences as the reference's cj** terms) */
    double cxi[3], cet[3], cze[3];
    cxi[0] = (t[1] * c[2]) - (t[2] * c[1]);
    cxi[1] = (t[2] * c[0]) - (t[0] * c[2]);
    cxi[2] = (t[0] * c[1]) - (t[1] * c[0]);
    cet[0] = (a[2] * c[1]) - (a[1] * c[2]);
    cet[1] = (a[0] * c[2]) - (a[2] * c[0]);
    cet[2] = (a[1] * c[0]) - (a[0] * c[1]);
    cze[0] = (a[1] * t[2]) - (a[2] * t[1]);
    cze[1] = (a[2] * t[0]) - (a[0] * t[2]);
    cze[2] = (a[0] * t[1]) - (a[1] * t[0]);

    for (int d = 0; d < 3; ++d) {
        b[d][0] = ((-cxi[d]) - cet[d]) - cze[d];
        b[d][1] = (cxi[d] - cet[d]) - cze[d];
        b[d][2] = (cxi[d] + cet[d]) - cze[d];
        b[d][3] = ((-cxi[d]) + cet[d]) - cze[d];
        b[d][4] = -b[d][2];
        b[d][5] = -b[d][3];
        b[d][6] = -b[d][0];
        b[d][7] = -b[d][1];
    }
    *volume = 8.0 * ((t[0] * cet[0] + t[1] * cet[1]) + t[2] * cet[2]);
}

/* Faces of the hexahedron in the reference's evaluation order with the
 * corner order used by SumElemFaceNormal, LULESH-OMP.cc:747-798. */
static const int k_face[6][4] = {
    {0, 1, 2, 3}, {0, 4, 5, 1}, {1, 5, 6, 2}, {2, 6, 7, 3}, {3, 7, 4, 0}, {4, 7, 6, 5}
};

/* CalcElemNodeNormals + SumElemFaceNormal, LULESH-OMP.cc:708-799. */
static void node_normals(double pf[3][8], const double x[8], const double y[8], const double z[8])
{
    for (int d = 0; d < 3; ++d)
        for (int i = 0; i < 8; ++i) pf[d][i] = 0.0;
    for (int f = 0; f < 6; ++f) {
        const int n0 = k_face[f][0], n1 = k_face[f][1], n2 = k_face[f][2], n3 = k_face[f][3];
        const double bx0 = 0.5 * (((x[n3] + x[n2]) - x[n1]) - x[n0]);
        const double by0 = 0.5 * (((y[n3] + y[n2]) - y[n1]) - y[n0]);
        const double bz0 = 0.5 * (((z[n3] + z[n2]) - z[n1]) - z[n0]);
        const double bx1 = 0.5 * (((x[n2] + x[n1]) - x[n3]) - x[n0]);
        const double by1 = 0.5 * (((y[n2] + y[n1]) - y[n3]) - y[n0]);
        const double bz1 = 0.5 * (((z[n2] + z[n1]) - z[n3]) - z[n0]);
        const double ax = 0.25 * (by0 * bz1 - bz0 * by1);
        const double ay = 0.25 * (bz0 * bx1 - bx0 * bz1);
        const double az = 0.25 * (bx0 * by1 - by0 * bx1);
        for (int k = 0; k < 4; ++k) {
            const int n = k_face[f][k];
            pf[0][n] += ax;
            pf[1][n] += ay;
            pf[2][n] += az;
        }
    }
}

/* VoluDer, LULESH-OMP.cc:978-1006: derivative of the volume with respect to
 * one corner, given the six corners it depends on (permuted order). */
static inline void volu_der(const double x[6], const double y[6], const double z[6],
                            double *dx, double *dy, double *dz)
{
    const double twelfth = 1.0 / 12.0;
    double vx =
        (y[1] + y[2]) * (z[0] + z[1]) - (y[0] + y[1]) * (z[1] + z[2]) +
        (y[0] + y[4]) * (z[3] + z[4]) - (y[3] + y[4]) * (z[0] + z[4]) -
        (y[2] + y[5]) * (z[3] + z[5]) + (y[3] + y[5]) * (z[2] + z[5]);
    double vy =
        -(x[1] + x[2]) * (z[0] + z[1]) + (x[0] + x[1]) * (z[1] + z[2]) -
        (x[0] + x[4]) * (z[3] + z[4]) + (x[3] + x[4]) * (z[0] + z[4]) +
        (x[2] + x[5]) * (z[3] + z[5]) - (x[3] + x[5]) * (z[2] + z[5]);
    double vz =
        -(y[1] + y[2]) * (x[0] + x[1]) + (y[0] + y[1]) * (x[1] + x[2]) -
        (y[0] + y[4]) * (x[3] + x[4]) + (y[3] + y[4]) * (x[0] + x[4]) +
        (y[2] + y[5]) * (x[3] + x[5]) - (y[3] + y[5]) * (x[2] + x[5]);
    *dx = vx * twelfth;
    *dy = vy * twelfth;
    *dz = vz * twelfth;
}

/* Corner permutations of CalcElemVolumeDerivative, LULESH-OMP.cc:1008-1048,
 * indexed by the corner whose derivative is produced. */
static const int k_voluder[8][6] = {
    {1, 2, 3, 4, 5, 7}, {2, 3, 0, 5, 6, 4}, {3, 0, 1, 6, 7, 5}, {0, 1, 2, 7, 4, 6},
    {7, 6, 5, 0, 3, 1}, {4, 7, 6, 1, 0, 2}, {5, 4, 7, 2, 1, 3}, {6, 5, 4, 3, 2, 0}
};

static void volume_derivative(double dvdx[8], double dvdy[8], double dvdz[8],
                              const double x[8], const double y[8], const double z[8])
{
    for (int c = 0; c < 8; ++c) {
        double px[6], py[6], pz[6];
        for (int k = 0; k < 6; ++k) {
            px[k] = x[k_voluder[c][k]];
            py[k] = y[k_voluder[c][k]];
            pz[k] = z[k_voluder[c][k]];
        }
        volu_der(px, py, pz, &dvdx[c], &dvdy[c], &dvdz[c]);
    }
}

/* Hourglass base vectors, LULESH-OMP.cc:1252-1285. */
static const double k_gamma[4][8] = {
    { 1.,  1., -1., -1., -1., -1.,  1.,  1.},
    { 1., -1., -1.,  1., -1.,  1.,  1., -1.},
    { 1., -1.,  1., -1.,  1., -1.,  1., -1.},
    {-1.,  1., -1.,  1.,  1., -1.,  1., -1.}
};

/* CalcElemVolume, LULESH-OMP.cc:1706-1790. */
static double elem_volume(const double x[8], const double y[8], const double z[8])
{
    const double twelveth = 1.0 / 12.0;
#define D(a, b) (x[a] - x[b])
#define DY(a, b) (y[a] - y[b])
#define DZ(a, b) (z[a] - z[b])
    const double dx61 = D(6, 1), dy61 = DY(6, 1), dz61 = DZ(6, 1);
    const double dx70 = D(7, 0), dy70 = DY(7, 0), dz70 = DZ(7, 0);
    const double dx63 = D(6, 3), dy63 = DY(6, 3), dz63 = DZ(6, 3);
    const double dx20 = D(2, 0), dy20 = DY(2, 0), dz20 = DZ(2, 0);
    const double dx50 = D(5, 0), dy50 = DY(5, 0), dz50 = DZ(5, 0);
    const double dx64 = D(6, 4), dy64 = DY(6, 4), dz64 = DZ(6, 4);
    const double dx31 = D(3, 1), dy31 = DY(3, 1), dz31 = DZ(3, 1);
    const double dx72 = D(7, 2), dy72 = DY(7, 2), dz72 = DZ(7, 2);
    const double dx43 = D(4, 3), dy43 = DY(4, 3), dz43 = DZ(4, 3);
    const double dx57 = D(5, 7), dy57 = DY(5, 7), dz57 = DZ(5, 7);
    const double dx14 = D(1, 4), dy14 = DY(1, 4), dz14 = DZ(1, 4);
    const double dx25 = D(2, 5), dy25 = DY(2, 5), dz25 = DZ(2, 5);
#undef D
#undef DY
#undef DZ
#define TRIPLE(x1, y1, z1, x2, y2, z2, x3, y3, z3) \
    ((x1) * ((y2) * (z3) - (z2) * (y3)) + (x2) * ((z1) * (y3) - (y1) * (z3)) + (x3) * ((y1) * (z2) - (z1) * (y2)))
    double vol =
        TRIPLE(dx31 + dx72, dx63, dx20, dy31 + dy72, dy63, dy20, dz31 + dz72, dz63, dz20) +
        TRIPLE(dx43 + dx57, dx64, dx70, dy43 + dy57, dy64, dy70, dz43 + dz57, dz64, dz70) +
        TRIPLE(dx14 + dx25, dx61, dx50, dy14 + dy25, dy61, dy50, dz14 + dz25, dz61, dz50);
#undef TRIPLE
    return vol * twelveth;
}

/* AreaFace, LULESH-OMP.cc:1799-1819 (corner indices into x/y/z). */
static inline double area_face(const double x[8], const double y[8], const double z[8],
                               int a, int b, int c, int d)
{
    const double fx = (x[c] - x[a]) - (x[d] - x[b]);
    const double fy = (y[c] - y[a]) - (y[d] - y[b]);
    const double fz = (z[c] - z[a]) - (z[d] - z[b]);
    const double gx = (x[c] - x[a]) + (x[d] - x[b]);
    const double gy = (y[c] - y[a]) + (y[d] - y[b]);
    const double gz = (z[c] - z[a]) + (z[d] - z[b]);
    const double fg = fx * gx + fy * gy + fz * gz;
    return (fx * fx + fy * fy + fz * fz) * (gx * gx + gy * gy + gz * gz) - fg * fg;
}

/* CalcElemCharacteristicLength, LULESH-OMP.cc:1821-1862 (face order kept). */
static double char_length(const double x[8], const double y[8], const double z[8], double volume)
{
    static const int faces[6][4] = {
        {0, 1, 2, 3}, {4, 5, 6, 7}, {0, 1, 5, 4}, {1, 2, 6, 5}, {2, 3, 7, 6}, {3, 0, 4, 7}
    };
    double m = 0.0;
    for (int f = 0; f < 6; ++f) {
        const double a = area_face(x, y, z, faces[f][0], faces[f][1], faces[f][2], faces[f][3]);
        m = (m < a) ? a : m;               /* std::max(a, charLength) */
    }
    return 4.0 * volume / sqrt(m);
}

/* ------------------------------------------------------------------ */
/* Phases                                                               */
/* ------------------------------------------------------------------ */

static inline void gather8(const double *f, const int *nl, double out[8])
{
    for (int k = 0; k < 8; ++k) out[k] = f[nl[k]];
}

/* Corner -> node gather in nodeElemCornerList order, LULESH-OMP.cc:905-926
 * (assign) and :1475-1496 (accumulate). */
static void gather_corner_forces(lo_domain *d, int accumulate)
{
    const int nn = d->nnode;
#pragma omp parallel for
    for (int n = 0; n < nn; ++n) {
        const int cnt = d->node_elem_count[n], st = d->node_elem_start[n];
        double fx = 0.0, fy = 0.0, fz = 0.0;
        for (int i = 0; i < cnt; ++i) {
            const int c = d->node_elem_corner_list[st + i];
            fx += d->fx_elem[c];
            fy += d->fy_elem[c];
            fz += d->fz_elem[c];
        }
        if (accumulate) {
            d->fx[n] += fx; d->fy[n] += fy; d->fz[n] += fz;
        } else {
            d->fx[n] = fx; d->fy[n] = fy; d->fz[n] = fz;
        }
    }
}

/* IntegrateStressForElems, LULESH-OMP.cc:853-931, with
 * InitStressTermsForElems (:606-617) folded in (sig = -p - q). */
static void integrate_stress(lo_domain *d)
{
    const int ne = d->nelem;
#pragma omp parallel for
    for (int k = 0; k < ne; ++k) {
        const int *nl = &d->nodelist[8 * k];
        double x[8], y[8], z[8], b[3][8];
        gather8(d->x, nl, x);
        gather8(d->y, nl, y);
        gather8(d->z, nl, z);
        shape_derivs(x, y, z, b, &d->determ[k]);
        node_normals(b, x, y, z);
        const double sig = -d->p[k] - d->q[k];
        for (int c = 0; c < 8; ++c) {
            d->fx_elem[8 * k + c] = -(sig * b[0][c]);
            d->fy_elem[8 * k + c] = -(sig * b[1][c]);
            d->fz_elem[8 * k + c] = -(sig * b[2][c]);
        }
    }
    gather_corner_forces(d, 0);
}

/* CalcFBHourglassForceForElems + CalcElemFBHourglassForce,
 * LULESH-OMP.cc:1050-1501. */
static void fb_hourglass(lo_domain *d, double hourg)
{
    const int ne = d->nelem;
#pragma omp parallel for
    for (int i2 = 0; i2 < ne; ++i2) {
        const int i3 = 8 * i2;
        const int *nl = &d->nodelist[i3];
        const double volinv = 1.0 / d->determ[i2];
        double hg[8][4];                       /* hourgam[corner][mode] */
        for (int m = 0; m < 4; ++m) {
            double hx = d->x8n[i3] * k_gamma[m][0];
            double hy = d->y8n[i3] * k_gamma[m][0];
            double hz = d->z8n[i3] * k_gamma[m][0];
            for (int c = 1; c < 8; ++c) {
                hx = hx + d->x8n[i3 + c] * k_gamma[m][c];
                hy = hy + d->y8n[i3 + c] * k_gamma[m][c];
                hz = hz + d->z8n[i3 + c] * k_gamma[m][c];
            }
            for (int c = 0; c < 8; ++c)
                hg[c][m] = k_gamma[m][c] - volinv * (d->dvdx[i3 + c] * hx +
                                                     d->dvdy[i3 + c] * hy +
                                                     d->dvdz[i3 + c] * hz);
        }
        const double ss1 = d->ss[i2];
        const double mass1 = d->elem_mass[i2];
        const double volume13 = cbrt(d->determ[i2]);
        const double coefficient = -hourg * 0.01 * ss1 * mass1 / volume13;

        const double *vel[3] = {d->xd, d->yd, d->zd};
        double *out[3] = {d->fx_elem, d->fy_elem, d->fz_elem};
        for (int dim = 0; dim < 3; ++dim) {
            double v8[8];
            gather8(vel[dim], nl, v8);
            double h[4];
            for (int m = 0; m < 4; ++m) {
                double acc = hg[0][m] * v8[0];
                for (int c = 1; c < 8; ++c) acc = acc + hg[c][m] * v8[c];
                h[m] = acc;
            }
            for (int c = 0; c < 8; ++c)
                out[dim][i3 + c] = coefficient *
                    (((hg[c][0] * h[0] + hg[c][1] * h[1]) + hg[c][2] * h[2]) + hg[c][3] * h[3]);
        }
    }
    gather_corner_forces(d, 1);
}

/* CalcHourglassControlForElems, LULESH-OMP.cc:1503-1558. */
static int hourglass_control(lo_domain *d)
{
    const int ne = d->nelem;
    int bad = 0;
#pragma omp parallel for reduction(|:bad)
    for (int i = 0; i < ne; ++i) {
        const int *nl = &d->nodelist[8 * i];
        double x[8], y[8], z[8], px[8], py[8], pz[8];
        gather8(d->x, nl, x);
        gather8(d->y, nl, y);
        gather8(d->z, nl, z);
        volume_derivative(px, py, pz, x, y, z);
        for (int c = 0; c < 8; ++c) {
            d->dvdx[8 * i + c] = px[c];
            d->dvdy[8 * i + c] = py[c];
            d->dvdz[8 * i + c] = pz[c];
            d->x8n[8 * i + c] = x[c];
            d->y8n[8 * i + c] = y[c];
            d->z8n[8 * i + c] = z[c];
        }
        d->determ[i] = d->volo[i] * d->v[i];
        if (d->v[i] <= 0.0) bad = 1;
    }
    if (bad) return LO_VOLUME_ERROR;
    if (d->prm.hgcoef > 0.0) fb_hourglass(d, d->prm.hgcoef);
    return LO_OK;
}

/* LagrangeNodal, LULESH-OMP.cc:1685-1704 (CalcForceForNodes :1595,
 * CalcVolumeForceForElems :1560-1593, acceleration :1613-1623, boundary
 * conditions :1626-1645, velocity :1647-1669, position :1671-1683). */
int lo_lagrange_nodal(lo_domain *d)
{
    const double dt = d->deltatime, u_cut = d->prm.u_cut;
    const int nn = d->nnode, ne = d->nelem;

    integrate_stress(d);
    for (int k = 0; k < ne; ++k)
        if (d->determ[k] <= 0.0) return LO_VOLUME_ERROR;
    int rc = hourglass_control(d);
    if (rc) return rc;

#pragma omp parallel for
    for (int i = 0; i < nn; ++i) {
        d->xdd[i] = d->fx[i] / d->nodal_mass[i];
        d->ydd[i] = d->fy[i] / d->nodal_mass[i];
        d->zdd[i] = d->fz[i] / d->nodal_mass[i];
    }
    for (int i = 0; i < d->nsymm_x; ++i) d->xdd[d->symm_x[i]] = 0.0;
    for (int i = 0; i < d->nsymm_y; ++i) d->ydd[d->symm_y[i]] = 0.0;
    for (int i = 0; i < d->nsymm_z; ++i) d->zdd[d->symm_z[i]] = 0.0;

#pragma omp parallel for
    for (int i = 0; i < nn; ++i) {
        double t;
        t = d->xd[i] + d->xdd[i] * dt;
        if (fabs(t) < u_cut) t = 0.0;
        d->xd[i] = t;
        t = d->yd[i] + d->ydd[i] * dt;
        if (fabs(t) < u_cut) t = 0.0;
        d->yd[i] = t;
        t = d->zd[i] + d->zdd[i] * dt;
        if (fabs(t) < u_cut) t = 0.0;
        d->zd[i] = t;
    }
#pragma omp parallel for
    for (int i = 0; i < nn; ++i) {
        d->x[i] += d->xd[i] * dt;
        d->y[i] += d->yd[i] * dt;
        d->z[i] += d->zd[i] * dt;
    }
    return LO_OK;
}

/* CalcKinematicsForElems + CalcLagrangeElements, LULESH-OMP.cc:1927-2032.
 * Only the trace vdov of the velocity gradient is kept: the deviatoric
 * components the reference stores in dxx/dyy/dzz are never read again. */
static int kinematics(lo_domain *d)
{
    const int ne = d->nelem;
    const double dt = d->deltatime;
    int bad = 0;
#pragma omp parallel for reduction(|:bad)
    for (int k = 0; k < ne; ++k) {
        const int *nl = &d->nodelist[8 * k];
        double x[8], y[8], z[8], xv[8], yv[8], zv[8], b[3][8], detJ;
        gather8(d->x, nl, x);
        gather8(d->y, nl, y);
        gather8(d->z, nl, z);
        const double volume = elem_volume(x, y, z);
        const double rel = volume / d->volo[k];
        d->vnew[k] = rel;
        d->delv[k] = rel - d->v[k];
        d->arealg[k] = char_length(x, y, z, volume);

        gather8(d->xd, nl, xv);
        gather8(d->yd, nl, yv);
        gather8(d->zd, nl, zv);
        const double dt2 = 0.5 * dt;
        for (int j = 0; j < 8; ++j) {
            x[j] -= dt2 * xv[j];
            y[j] -= dt2 * yv[j];
            z[j] -= dt2 * zv[j];
        }
        shape_derivs(x, y, z, b, &detJ);

        /* CalcElemVelocityGrandient, LULESH-OMP.cc:1864-1925 (diagonal) */
        const double inv = 1.0 / detJ;
        const double *vel[3] = {xv, yv, zv};
        double dd[3];
        for (int dim = 0; dim < 3; ++dim) {
            const double *u = vel[dim];
            dd[dim] = inv * (((b[dim][0] * (u[0] - u[6]) + b[dim][1] * (u[1] - u[7])) +
                              b[dim][2] * (u[2] - u[4])) + b[dim][3] * (u[3] - u[5]));
        }
        d->vdov[k] = (dd[0] + dd[1]) + dd[2];
        if (rel <= 0.0) bad = 1;
    }
    return bad ? LO_VOLUME_ERROR : LO_OK;
}

static inline double sum4(double a, double b, double c, double e) { return ((a + b) + c) + e; }

/* CalcMonotonicQGradientsForElems, LULESH-OMP.cc:2034-2180. */
static void q_gradients(lo_domain *d)
{
    const int ne = d->nelem;
    const double ptiny = 1.e-36;
#pragma omp parallel for
    for (int i = 0; i < ne; ++i) {
        const int *nl = &d->nodelist[8 * i];
        double x[8], y[8], z[8], xv[8], yv[8], zv[8];
        gather8(d->x, nl, x);
        gather8(d->y, nl, y);
        gather8(d->z, nl, z);
        gather8(d->xd, nl, xv);
        gather8(d->yd, nl, yv);
        gather8(d->zd, nl, zv);

        const double vol = d->volo[i] * d->vnew[i];
        const double norm = 1.0 / (vol + ptiny);

        /* logical-direction differences of a corner field */
#define DJ(f) (-0.25 * (sum4(f[0], f[1], f[5], f[4]) - sum4(f[3], f[2], f[6], f[7])))
#define DI(f) ( 0.25 * (sum4(f[1], f[2], f[6], f[5]) - sum4(f[0], f[3], f[7], f[4])))
#define DK(f) ( 0.25 * (sum4(f[4], f[5], f[6], f[7]) - sum4(f[0], f[1], f[2], f[3])))
        const double dxj = DJ(x), dyj = DJ(y), dzj = DJ(z);
        const double dxi = DI(x), dyi = DI(y), dzi = DI(z);
        const double dxk = DK(x), dyk = DK(y), dzk = DK(z);
        double ax, ay, az, dxv, dyv, dzv;

        /* zeta: i cross j */
        ax = dyi * dzj - dzi * dyj;
        ay = dzi * dxj - dxi * dzj;
        az = dxi * dyj - dyi * dxj;
        d->delx_zeta[i] = vol / sqrt(ax * ax + ay * ay + az * az + ptiny);
        ax *= norm; ay *= norm; az *= norm;
        dxv = DK(xv); dyv = DK(yv); dzv = DK(zv);
        d->delv_zeta[i] = ax * dxv + ay * dyv + az * dzv;

        /* xi: j cross k */
        ax = dyj * dzk - dzj * dyk;
        ay = dzj * dxk - dxj * dzk;
        az = dxj * dyk - dyj * dxk;
        d->delx_xi[i] = vol / sqrt(ax * ax + ay * ay + az * az + ptiny);
        ax *= norm; ay *= norm; az *= norm;
        dxv = DI(xv); dyv = DI(yv); dzv = DI(zv);
        d->delv_xi[i] = ax * dxv + ay * dyv + az * dzv;

        /* eta: k cross i */
        ax = dyk * dzi - dzk * dyi;
        ay = dzk * dxi - dxk * dzi;
        az = dxk * dyi - dyk * dxi;
        d->delx_eta[i] = vol / sqrt(ax * ax + ay * ay + az * az + ptiny);
        ax *= norm; ay *= norm; az *= norm;
        dxv = DJ(xv); dyv = DJ(yv); dzv = DJ(zv);
        d->delv_eta[i] = ax * dxv + ay * dyv + az * dzv;
#undef DJ
#undef DI
#undef DK
    }
}

/* One direction of the monotonic limiter, LULESH-OMP.cc:2198-2228. */
static inline double limiter_phi(const double *delv, int i, int bc, int m_mask, int m_symm,
                                 int m_free, int p_mask, int p_symm, int p_free,
                                 int lm, int lp, double limiter, double max_slope, double ptiny)
{
    const double norm = 1. / (delv[i] + ptiny);
    double delvm = 0.0, delvp = 0.0;
    const int bm = bc & m_mask, bp = bc & p_mask;
    if (bm == 0) delvm = delv[lm];
    else if (bm == m_symm) delvm = delv[i];
    else if (bm == m_free) delvm = 0.0;
    if (bp == 0) delvp = delv[lp];
    else if (bp == p_symm) delvp = delv[i];
    else if (bp == p_free) delvp = 0.0;
    delvm = delvm * norm;
    delvp = delvp * norm;
    double phi = .5 * (delvm + delvp);
    delvm *= limiter;
    delvp *= limiter;
    if (delvm < phi) phi = delvm;
    if (delvp < phi) phi = delvp;
    if (phi < 0.) phi = 0.;
    if (phi > max_slope) phi = max_slope;
    return phi;
}

/* CalcMonotonicQRegionForElems, LULESH-OMP.cc:2182-2320. */
static void q_region(lo_domain *d)
{
    const int ne = d->nelem;
    const double ptiny = 1.e-36;
    const double qlc = d->prm.qlc_monoq, qqc = d->prm.qqc_monoq;
    const double lim = d->prm.monoq_limiter_mult, maxs = d->prm.monoq_max_slope;
#pragma omp parallel for
    for (int i = 0; i < ne; ++i) {
        const int bc = d->elem_bc[i];
        const double phixi = limiter_phi(d->delv_xi, i, bc, BC_XI_M, BC_XI_M_SYMM, BC_XI_M_FREE,
                                         BC_XI_P, BC_XI_P_SYMM, BC_XI_P_FREE,
                                         d->lxim[i], d->lxip[i], lim, maxs, ptiny);
        const double phieta = limiter_phi(d->delv_eta, i, bc, BC_ETA_M, BC_ETA_M_SYMM, BC_ETA_M_FREE,
                                          BC_ETA_P, BC_ETA_P_SYMM, BC_ETA_P_FREE,
                                          d->letam[i], d->letap[i], lim, maxs, ptiny);
        const double phizeta = limiter_phi(d->delv_zeta, i, bc, BC_ZETA_M, BC_ZETA_M_SYMM, BC_ZETA_M_FREE,
                                           BC_ZETA_P, BC_ZETA_P_SYMM, BC_ZETA_P_FREE,
                                           d->lzetam[i], d->lzetap[i], lim, maxs, ptiny);
        double qlin, qquad;
        if (d->vdov[i] > 0.) {
            qlin = 0.;
            qquad = 0.;
        } else {
            double dxi = d->delv_xi[i] * d->delx_xi[i];
            double deta = d->delv_eta[i] * d->delx_eta[i];
            double dzeta = d->delv_zeta[i] * d->delx_zeta[i];
            if (dxi > 0.) dxi = 0.;
            if (deta > 0.) deta = 0.;
            if (dzeta > 0.) dzeta = 0.;
            const double rho = d->elem_mass[i] / (d->volo[i] * d->vnew[i]);
            qlin = -qlc * rho *
                   ((dxi * (1. - phixi) + deta * (1. - phieta)) + dzeta * (1. - phizeta));
            qquad = qqc * rho *
                    ((dxi * dxi * (1. - phixi * phixi) + deta * deta * (1. - phieta * phieta)) +
                     dzeta * dzeta * (1. - phizeta * phizeta));
        }
        d->qq[i] = qquad;
        d->ql[i] = qlin;
    }
}

/* CalcPressureForElems for one element, LULESH-OMP.cc:2384-2413. */
static inline double pressure(double *bvc, double *pbvc, double e, double comp, double vnewc,
                              double pmin, double p_cut, double eosvmax)
{
    const double c1s = 2.0 / 3.0;
    *bvc = c1s * (comp + 1.);
    *pbvc = c1s;
    double p = *bvc * e;
    if (fabs(p) < p_cut) p = 0.0;
    if (vnewc >= eosvmax) p = 0.0;
    if (p < pmin) p = pmin;
    return p;
}

static inline double sound_term(double pbvc, double e, double vv, double bvc, double p, double rho0)
{
    double ssc = (pbvc * e + vv * vv * bvc * p) / rho0;
    if (ssc <= .111111e-36) ssc = .333333e-18;
    else ssc = sqrt(ssc);
    return ssc;
}

/* ApplyMaterialPropertiesForElems + EvalEOSForElems + CalcEnergyForElems +
 * CalcSoundSpeedForElems, LULESH-OMP.cc:2415-2761, evaluated per element
 * (every loop of the reference is element-local). */
static int material(lo_domain *d)
{
    const int ne = d->nelem;
    const lo_params *P = &d->prm;
    const double e_cut = P->e_cut, p_cut = P->p_cut, q_cut = P->q_cut;
    const double eosvmax = P->eosvmax, eosvmin = P->eosvmin, pmin = P->pmin, emin = P->emin;
    const double rho0 = P->refdens;
    int bad = 0;
#pragma omp parallel for reduction(|:bad)
    for (int i = 0; i < ne; ++i) {
        double vnewc = d->vnew[i];
        if (eosvmin != 0.) { if (vnewc < eosvmin) vnewc = eosvmin; }
        if (eosvmax != 0.) { if (vnewc > eosvmax) vnewc = eosvmax; }
        double vc = d->v[i];
        if (eosvmin != 0.) { if (vc < eosvmin) vc = eosvmin; }
        if (eosvmax != 0.) { if (vc > eosvmax) vc = eosvmax; }
        if (vc <= 0.) bad = 1;

        const double e_old = d->e[i], delvc = d->delv[i], q_old = d->q[i];
        double p_old = d->p[i];
        double compression = 1. / vnewc - 1.;
        const double vchalf = vnewc - delvc * .5;
        double comp_half = 1. / vchalf - 1.;
        if (eosvmin != 0. && vnewc <= eosvmin) comp_half = compression;
        if (eosvmax != 0. && vnewc >= eosvmax) {
            p_old = 0.;
            compression = 0.;
            comp_half = 0.;
        }
        const double ql = d->ql[i], qq = d->qq[i], work = 0.;
        double bvc, pbvc;

        double e_new = e_old - .5 * delvc * (p_old + q_old) + .5 * work;
        if (e_new < emin) e_new = emin;

        const double p_half = pressure(&bvc, &pbvc, e_new, comp_half, vnewc, pmin, p_cut, eosvmax);
        const double vhalf = 1. / (1. + comp_half);
        double q_new;
        if (delvc > 0.) {
            q_new = 0.;
        } else {
            const double ssc = sound_term(pbvc, e_new, vhalf, bvc, p_half, rho0);
            q_new = (ssc * ql + qq);
        }
        e_new = e_new + .5 * delvc * (3.0 * (p_old + q_old) - 4.0 * (p_half + q_new));

        e_new += .5 * work;
        if (fabs(e_new) < e_cut) e_new = 0.;
        if (e_new < emin) e_new = emin;

        double p_new = pressure(&bvc, &pbvc, e_new, compression, vnewc, pmin, p_cut, eosvmax);
        double q_tilde;
        if (delvc > 0.) {
            q_tilde = 0.;
        } else {
            const double ssc = sound_term(pbvc, e_new, vnewc, bvc, p_new, rho0);
            q_tilde = (ssc * ql + qq);
        }
        const double sixth = 1.0 / 6.0;
        e_new = e_new - (7.0 * (p_old + q_old) - 8.0 * (p_half + q_new) + (p_new + q_tilde)) * delvc * sixth;
        if (fabs(e_new) < e_cut) e_new = 0.;
        if (e_new < emin) e_new = emin;

        p_new = pressure(&bvc, &pbvc, e_new, compression, vnewc, pmin, p_cut, eosvmax);
        if (delvc <= 0.) {
            const double ssc = sound_term(pbvc, e_new, vnewc, bvc, p_new, rho0);
            q_new = (ssc * ql + qq);
            if (fabs(q_new) < q_cut) q_new = 0.;
        }
        d->p[i] = p_new;
        d->e[i] = e_new;
        d->q[i] = q_new;
        d->ss[i] = sound_term(pbvc, e_new, vnewc, bvc, p_new, rho0);
    }
    return bad ? LO_VOLUME_ERROR : LO_OK;
}

/* LagrangeElements, LULESH-OMP.cc:2784-2797, with CalcQForElems
 * (:2351-2382) and UpdateVolumesForElems (:2763-2782). */
int lo_lagrange_elements(lo_domain *d)
{
    const int ne = d->nelem;
    int rc = kinematics(d);
    if (rc) return rc;
    q_gradients(d);
    q_region(d);
    for (int i = 0; i < ne; ++i)                  /* qstop test on the old q */
        if (d->q[i] > d->prm.qstop) return LO_QSTOP_ERROR;
    rc = material(d);
    if (rc) return rc;
    const double v_cut = d->prm.v_cut;
#pragma omp parallel for
    for (int i = 0; i < ne; ++i) {
        double t = d->vnew[i];
        if (fabs(t - 1.0) < v_cut) t = 1.0;
        d->v[i] = t;
    }
    return LO_OK;
}

/* CalcCourantConstraintForElems + CalcHydroConstraintForElems,
 * LULESH-OMP.cc:2799-2942.  A minimum is independent of evaluation order,
 * so the per-thread split of the reference is not reproduced. */
void lo_time_constraints(lo_domain *d)
{
    const int ne = d->nelem;
    const double qqc2 = 64.0 * d->prm.qqc * d->prm.qqc;
    const double dvovmax = d->prm.dvovmax;
    double dtc = 1.0e+20, dth = 1.0e+20;
    int found_c = 0, found_h = 0;
#pragma omp parallel
    {
        double lc = 1.0e+20, lh = 1.0e+20;
        int fc = 0, fh = 0;
#pragma omp for nowait
        for (int i = 0; i < ne; ++i) {
            const double vdov = d->vdov[i];
            double dtf = d->ss[i] * d->ss[i];
            if (vdov < 0.) dtf = dtf + qqc2 * d->arealg[i] * d->arealg[i] * vdov * vdov;
            dtf = sqrt(dtf);
            dtf = d->arealg[i] / dtf;
            if (vdov != 0.) {
                if (dtf < lc) { lc = dtf; fc = 1; }
                const double dtdvov = dvovmax / (fabs(vdov) + 1.e-20);
                if (lh > dtdvov) { lh = dtdvov; fh = 1; }
            }
        }
#pragma omp critical
        {
            if (fc && lc < dtc) { dtc = lc; found_c = 1; }
            if (fh && lh < dth) { dth = lh; found_h = 1; }
        }
    }
    if (found_c) d->dtcourant = dtc;
    if (found_h) d->dthydro = dth;
}

/* TimeIncrement, LULESH-OMP.cc:557-604. */
void lo_time_increment(lo_domain *d)
{
    const lo_params *P = &d->prm;
    double targetdt = P->stoptime - d->time;
    if ((P->dtfixed <= 0.0) && (d->cycle != 0)) {
        const double olddt = d->deltatime;
        double newdt = 1.0e+20;
        if (d->dtcourant < newdt) newdt = d->dtcourant / 2.0;
        if (d->dthydro < newdt) newdt = d->dthydro * 2.0 / 3.0;
        const double ratio = newdt / olddt;
        if (ratio >= 1.0) {
            if (ratio < P->deltatimemultlb) newdt = olddt;
            else if (ratio > P->deltatimemultub) newdt = olddt * P->deltatimemultub;
        }
        if (newdt > P->dtmax) newdt = P->dtmax;
        d->deltatime = newdt;
    }
    if ((targetdt > d->deltatime) && (targetdt < (4.0 * d->deltatime / 3.0)))
        targetdt = 2.0 * d->deltatime / 3.0;
    if (targetdt < d->deltatime) d->deltatime = targetdt;
    d->time += d->deltatime;
    ++d->cycle;
}

/* LagrangeLeapFrog, LULESH-OMP.cc:2944-2958. */
int lo_lagrange_leapfrog(lo_domain *d)
{
    int rc = lo_lagrange_nodal(d);
    if (rc) return rc;
    rc = lo_lagrange_elements(d);
    if (rc) return rc;
    lo_time_constraints(d);
    return LO_OK;
}

int lo_run(lo_domain *d, int max_cycles, double *elapsed)
{
    struct timeval t0, t1;
    gettimeofday(&t0, NULL);
    int rc = LO_OK, n = 0;
    while (d->time < d->prm.stoptime && (max_cycles <= 0 || n < max_cycles)) {
        lo_time_increment(d);
        rc = lo_lagrange_leapfrog(d);
        ++n;
        if (rc) break;
    }
    gettimeofday(&t1, NULL);
    if (elapsed) *elapsed = (double)(t1.tv_sec - t0.tv_sec) + 1e-6 * (double)(t1.tv_usec - t0.tv_usec);
    return rc;
}

/* LULESH-OMP.cc:3197-3223 */
void lo_symmetry(lo_domain *d, double *max_abs, double *total_abs, double *max_rel)
{
    const int s = d->s;                           /* 0 on an unstructured mesh: no test */
    double ma = 0.0, ta = 0.0, mr = 0.0;
    for (int j = 0; j < s; ++j)
        for (int k = j + 1; k < s; ++k) {
            const double a = fabs(d->e[j * s + k] - d->e[k * s + j]);
            ta += a;
            if (ma < a) ma = a;
            const double r = a / d->e[k * s + j];
            if (mr < r) mr = r;
        }
    *max_abs = ma;
    *total_abs = ta;
    *max_rel = mr;
}

/* ------------------------------------------------------------------ */
/* Construction: the Sedov cube of LULESH-OMP.cc:2960-3171               */
/* ------------------------------------------------------------------ */

#define ALLOC_D(n) ((double *)calloc((size_t)(n), sizeof(double)))
#define ALLOC_I(n) ((int *)calloc((size_t)(n), sizeof(int)))

static lo_domain *alloc_domain(int ne, int nn, int nx, int ny, int nz)
{
    lo_domain *d = (lo_domain *)calloc(1, sizeof *d);
    d->nelem = ne;
    d->nnode = nn;
    lo_default_params(&d->prm);
    d->x = ALLOC_D(nn); d->y = ALLOC_D(nn); d->z = ALLOC_D(nn);
    d->xd = ALLOC_D(nn); d->yd = ALLOC_D(nn); d->zd = ALLOC_D(nn);
    d->xdd = ALLOC_D(nn); d->ydd = ALLOC_D(nn); d->zdd = ALLOC_D(nn);
    d->fx = ALLOC_D(nn); d->fy = ALLOC_D(nn); d->fz = ALLOC_D(nn);
    d->nodal_mass = ALLOC_D(nn);
    d->e = ALLOC_D(ne); d->p = ALLOC_D(ne); d->q = ALLOC_D(ne);
    d->ql = ALLOC_D(ne); d->qq = ALLOC_D(ne); d->v = ALLOC_D(ne);
    d->volo = ALLOC_D(ne); d->vnew = ALLOC_D(ne); d->delv = ALLOC_D(ne);
    d->vdov = ALLOC_D(ne); d->arealg = ALLOC_D(ne); d->ss = ALLOC_D(ne);
    d->elem_mass = ALLOC_D(ne); d->determ = ALLOC_D(ne);
    d->delv_xi = ALLOC_D(ne); d->delv_eta = ALLOC_D(ne); d->delv_zeta = ALLOC_D(ne);
    d->delx_xi = ALLOC_D(ne); d->delx_eta = ALLOC_D(ne); d->delx_zeta = ALLOC_D(ne);
    d->fx_elem = ALLOC_D(8L * ne); d->fy_elem = ALLOC_D(8L * ne); d->fz_elem = ALLOC_D(8L * ne);
    d->dvdx = ALLOC_D(8L * ne); d->dvdy = ALLOC_D(8L * ne); d->dvdz = ALLOC_D(8L * ne);
    d->x8n = ALLOC_D(8L * ne); d->y8n = ALLOC_D(8L * ne); d->z8n = ALLOC_D(8L * ne);
    d->nodelist = ALLOC_I(8L * ne);
    d->lxim = ALLOC_I(ne); d->lxip = ALLOC_I(ne);
    d->letam = ALLOC_I(ne); d->letap = ALLOC_I(ne);
    d->lzetam = ALLOC_I(ne); d->lzetap = ALLOC_I(ne);
    d->elem_bc = ALLOC_I(ne);
    d->node_elem_start = ALLOC_I(nn); d->node_elem_count = ALLOC_I(nn);
    d->node_elem_corner_list = ALLOC_I(8L * ne);
    d->nsymm_x = nx; d->nsymm_y = ny; d->nsymm_z = nz;
    d->symm_x = ALLOC_I(nx > 0 ? nx : 1); d->symm_y = ALLOC_I(ny > 0 ? ny : 1);
    d->symm_z = ALLOC_I(nz > 0 ? nz : 1);
    return d;
}

/* Corner lists, reference volumes and masses of a filled-in nodelist. */
static void mesh_derived(lo_domain *d)
{
    const int ne = d->nelem, nn = d->nnode;
    /* node -> corner lists, AllocateNodeElemIndexes LULESH-OMP.cc:209-268:
     * corners sorted by element, then by local corner number. */
    for (int i = 0; i < 8 * ne; ++i) d->node_elem_count[d->nodelist[i]]++;
    d->node_elem_start[0] = 0;
    for (int i = 1; i < nn; ++i)
        d->node_elem_start[i] = d->node_elem_start[i - 1] + d->node_elem_count[i - 1];
    memset(d->node_elem_count, 0, sizeof(int) * (size_t)nn);
    for (int i = 0; i < ne; ++i)
        for (int j = 0; j < 8; ++j) {
            const int m = d->nodelist[8 * i + j];
            d->node_elem_corner_list[d->node_elem_start[m] + d->node_elem_count[m]] = 8 * i + j;
            d->node_elem_count[m]++;
        }

    /* masses and reference volumes, LULESH-OMP.cc:3089-3109 */
    for (int i = 0; i < ne; ++i) {
        double x[8], y[8], z[8];
        gather8(d->x, &d->nodelist[8 * i], x);
        gather8(d->y, &d->nodelist[8 * i], y);
        gather8(d->z, &d->nodelist[8 * i], z);
        const double vol = elem_volume(x, y, z);
        d->volo[i] = vol;
        d->elem_mass[i] = vol;
        for (int j = 0; j < 8; ++j) d->nodal_mass[d->nodelist[8 * i + j]] += vol / 8.0;
    }
    for (int i = 0; i < ne; ++i) d->v[i] = 1.0;
    d->time = 0.0;
    d->cycle = 0;
    d->dtcourant = 1.0e+20;
    d->dthydro = 1.0e+20;
}

lo_domain *lo_create(int s, int init_mode)
{
    if (s < 1) return NULL;
    const int en = s + 1;
    const int ne = s * s * s, nn = en * en * en;
    lo_domain *d = alloc_domain(ne, nn, en * en, en * en, en * en);
    d->s = s;

    /* coordinates, LULESH-OMP.cc:2996-3015 */
    int n = 0;
    for (int pl = 0; pl < en; ++pl)
        for (int row = 0; row < en; ++row)
            for (int col = 0; col < en; ++col, ++n) {
                d->x[n] = (col == 0) ? 0.0 : 1.125 * (double)col / (double)s;
                d->y[n] = (row == 0) ? 0.0 : 1.125 * (double)row / (double)s;
                d->z[n] = (pl == 0) ? 0.0 : 1.125 * (double)pl / (double)s;
            }

    /* hexahedra, LULESH-OMP.cc:3020-3042 */
    int e = 0;
    for (int pl = 0; pl < s; ++pl)
        for (int row = 0; row < s; ++row)
            for (int col = 0; col < s; ++col, ++e) {
                const int n0 = (pl * en + row) * en + col;
                int *l = &d->nodelist[8 * e];
                l[0] = n0;
                l[1] = n0 + 1;
                l[2] = n0 + en + 1;
                l[3] = n0 + en;
                l[4] = n0 + en * en;
                l[5] = n0 + en * en + 1;
                l[6] = n0 + en * en + en + 1;
                l[7] = n0 + en * en + en;
            }
    mesh_derived(d);

    d->origin = 0;
    if (init_mode == LO_INIT_V2) {
        /* lulesh-2.0.3/lulesh-init.cc:171-182 */
        const double ebase = 3.948746e+7;
        const double scale = (double)s / 45.0;
        const double einit = ebase * scale * scale * scale;
        d->e[0] = einit;
        d->deltatime = (.5 * cbrt(d->volo[0])) / sqrt(2.0 * einit);
    } else {
        d->e[0] = 3.948746e+7;                    /* LULESH-OMP.cc:3112 */
        d->deltatime = 1.0e-7;                    /* LULESH-OMP.cc:3053 */
    }

    /* symmetry node sets, LULESH-OMP.cc:3114-3125 */
    n = 0;
    for (int i = 0; i < en; ++i)
        for (int j = 0; j < en; ++j, ++n) {
            d->symm_x[n] = i * en * en + j * en;
            d->symm_y[n] = i * en * en + j;
            d->symm_z[n] = i * en + j;
        }

    /* face neighbours, LULESH-OMP.cc:3127-3151 */
    d->lxim[0] = 0;
    for (int i = 1; i < ne; ++i) { d->lxim[i] = i - 1; d->lxip[i - 1] = i; }
    d->lxip[ne - 1] = ne - 1;
    for (int i = 0; i < s; ++i) { d->letam[i] = i; d->letap[ne - s + i] = ne - s + i; }
    for (int i = s; i < ne; ++i) { d->letam[i] = i - s; d->letap[i - s] = i; }
    for (int i = 0; i < s * s; ++i) { d->lzetam[i] = i; d->lzetap[ne - s * s + i] = ne - s * s + i; }
    for (int i = s * s; i < ne; ++i) { d->lzetam[i] = i - s * s; d->lzetap[i - s * s] = i; }

    /* boundary conditions, LULESH-OMP.cc:3153-3171 */
    for (int i = 0; i < s; ++i) {
        const int pinc = i * s * s, rinc = i * s;
        for (int j = 0; j < s; ++j) {
            d->elem_bc[pinc + j * s] |= BC_XI_M_SYMM;
            d->elem_bc[pinc + j * s + s - 1] |= BC_XI_P_FREE;
            d->elem_bc[pinc + j] |= BC_ETA_M_SYMM;
            d->elem_bc[pinc + j + s * s - s] |= BC_ETA_P_FREE;
            d->elem_bc[rinc + j] |= BC_ZETA_M_SYMM;
            d->elem_bc[rinc + j + ne - s * s] |= BC_ZETA_P_FREE;
        }
    }
    return d;
}

/* Face flags from node sets, as the reference's unstructured reader sets
 * them (reference/CUDA/lulesh-kepler-singlegpu/lulesh.cu:852-920): a face
 * whose four corners all carry the mark gets the face's SYMM flag (the
 * reader uses SYMM for its free-surface pass as well).  Corner bits 0-3 form
 * the zeta- face, 4-7 zeta+, {0,1,4,5} eta-, {2,3,6,7} eta+, {0,3,4,7} xi-,
 * {1,2,5,6} xi+. */
static void flag_faces(lo_domain *d, const unsigned char *mark)
{
    for (int k = 0; k < d->nelem; ++k) {
        int mask = 0;
        for (int c = 0; c < 8; ++c) mask |= (mark[d->nodelist[8 * k + c]] ? 1 : 0) << c;
        int *bc = &d->elem_bc[k];
        if ((mask & 0x0f) == 0x0f) *bc |= BC_ZETA_M_SYMM;
        if ((mask & 0xf0) == 0xf0) *bc |= BC_ZETA_P_SYMM;
        if ((mask & 0x33) == 0x33) *bc |= BC_ETA_M_SYMM;
        if ((mask & 0xcc) == 0xcc) *bc |= BC_ETA_P_SYMM;
        if ((mask & 0x99) == 0x99) *bc |= BC_XI_M_SYMM;
        if ((mask & 0x66) == 0x66) *bc |= BC_XI_P_SYMM;
    }
}

/* An unstructured mesh, set up as the reference's unstructured reader does
 * (lulesh.cu:733-923): LULESH 1.0 initial energy 3.948746e7 in the origin
 * element (the first flagged SYMM on its xi-, eta- and zeta- faces by the
 * symmetry pass; element 0 if none is) and dt0 = 1e-7. */
lo_domain *lo_create_mesh(const lo_mesh *m)
{
    if (!m || m->nelem < 1 || m->nnode < 1) return NULL;
    const int ne = m->nelem, nn = m->nnode;
    for (long i = 0; i < 8L * ne; ++i)
        if (m->nodelist[i] < 0 || m->nodelist[i] >= nn) return NULL;
    const int *nb[6] = {m->lxim, m->lxip, m->letam, m->letap, m->lzetam, m->lzetap};
    for (int f = 0; f < 6; ++f)
        for (int k = 0; k < ne; ++k)
            if (nb[f][k] < 0 || nb[f][k] >= ne) return NULL;
    const int *sets[4] = {m->symm_x, m->symm_y, m->symm_z, m->free_surf};
    const int counts[4] = {m->nsymm_x, m->nsymm_y, m->nsymm_z, m->nfree};
    for (int t = 0; t < 4; ++t)
        for (int i = 0; i < counts[t]; ++i)
            if (sets[t][i] < 0 || sets[t][i] >= nn) return NULL;

    lo_domain *d = alloc_domain(ne, nn, m->nsymm_x, m->nsymm_y, m->nsymm_z);
    d->s = 0;
    memcpy(d->x, m->x, sizeof(double) * (size_t)nn);
    memcpy(d->y, m->y, sizeof(double) * (size_t)nn);
    memcpy(d->z, m->z, sizeof(double) * (size_t)nn);
    memcpy(d->nodelist, m->nodelist, sizeof(int) * 8 * (size_t)ne);
    int *dst[6] = {d->lxim, d->lxip, d->letam, d->letap, d->lzetam, d->lzetap};
    for (int f = 0; f < 6; ++f) memcpy(dst[f], nb[f], sizeof(int) * (size_t)ne);
    memcpy(d->symm_x, m->symm_x, sizeof(int) * (size_t)m->nsymm_x);
    memcpy(d->symm_y, m->symm_y, sizeof(int) * (size_t)m->nsymm_y);
    memcpy(d->symm_z, m->symm_z, sizeof(int) * (size_t)m->nsymm_z);
    mesh_derived(d);

    unsigned char *mark = (unsigned char *)calloc((size_t)nn, 1);
    for (int t = 0; t < 3; ++t)
        for (int i = 0; i < counts[t]; ++i) mark[sets[t][i]] = 1;
    flag_faces(d, mark);
    d->origin = 0;
    for (int k = 0; k < ne; ++k)
        if (d->elem_bc[k] == (BC_XI_M_SYMM | BC_ETA_M_SYMM | BC_ZETA_M_SYMM)) { d->origin = k; break; }
    memset(mark, 0, (size_t)nn);
    for (int i = 0; i < m->nfree; ++i) mark[m->free_surf[i]] = 1;
    flag_faces(d, mark);
    free(mark);

    d->e[d->origin] = 3.948746e+7;
    d->deltatime = 1.0e-7;
    return d;
}

int lo_origin(lo_domain *d) { return d->origin; }

void lo_destroy(lo_domain *d)
{
    if (!d) return;
    double **dp[] = {&d->x, &d->y, &d->z, &d->xd, &d->yd, &d->zd, &d->xdd, &d->ydd, &d->zdd,
                     &d->fx, &d->fy, &d->fz, &d->nodal_mass, &d->e, &d->p, &d->q, &d->ql, &d->qq,
                     &d->v, &d->volo, &d->vnew, &d->delv, &d->vdov, &d->arealg, &d->ss,
                     &d->elem_mass, &d->determ, &d->delv_xi, &d->delv_eta, &d->delv_zeta,
                     &d->delx_xi, &d->delx_eta, &d->delx_zeta, &d->fx_elem, &d->fy_elem,
                     &d->fz_elem, &d->dvdx, &d->dvdy, &d->dvdz, &d->x8n, &d->y8n, &d->z8n};
    for (size_t i = 0; i < sizeof dp / sizeof dp[0]; ++i) free(*dp[i]);
    int **ip[] = {&d->nodelist, &d->lxim, &d->lxip, &d->letam, &d->letap, &d->lzetam, &d->lzetap,
                  &d->elem_bc, &d->node_elem_start, &d->node_elem_count, &d->node_elem_corner_list,
                  &d->symm_x, &d->symm_y, &d->symm_z};
    for (size_t i = 0; i < sizeof ip / sizeof ip[0]; ++i) free(*ip[i]);
    free(d);
}

lo_params *lo_params_of(lo_domain *d) { return &d->prm; }
int *lo_cycle(lo_domain *d) { return &d->cycle; }
int lo_size(lo_domain *d) { return d->s; }

double *lo_scalar(lo_domain *d, const char *name)
{
    if (!strcmp(name, "time")) return &d->time;
    if (!strcmp(name, "deltatime")) return &d->deltatime;
    if (!strcmp(name, "dtcourant")) return &d->dtcourant;
    if (!strcmp(name, "dthydro")) return &d->dthydro;
    return NULL;
}

double *lo_field(lo_domain *d, const char *name, long *len)
{
    const struct { const char *n; double *p; long l; } t[] = {
        {"x", d->x, d->nnode}, {"y", d->y, d->nnode}, {"z", d->z, d->nnode},
        {"xd", d->xd, d->nnode}, {"yd", d->yd, d->nnode}, {"zd", d->zd, d->nnode},
        {"xdd", d->xdd, d->nnode}, {"ydd", d->ydd, d->nnode}, {"zdd", d->zdd, d->nnode},
        {"fx", d->fx, d->nnode}, {"fy", d->fy, d->nnode}, {"fz", d->fz, d->nnode},
        {"nodalMass", d->nodal_mass, d->nnode},
        {"e", d->e, d->nelem}, {"p", d->p, d->nelem}, {"q", d->q, d->nelem},
        {"ql", d->ql, d->nelem}, {"qq", d->qq, d->nelem}, {"v", d->v, d->nelem},
        {"volo", d->volo, d->nelem}, {"vnew", d->vnew, d->nelem}, {"delv", d->delv, d->nelem},
        {"vdov", d->vdov, d->nelem}, {"arealg", d->arealg, d->nelem}, {"ss", d->ss, d->nelem},
        {"elemMass", d->elem_mass, d->nelem}, {"determ", d->determ, d->nelem},
        {"delv_xi", d->delv_xi, d->nelem}, {"delv_eta", d->delv_eta, d->nelem},
        {"delv_zeta", d->delv_zeta, d->nelem}, {"delx_xi", d->delx_xi, d->nelem},
        {"delx_eta", d->delx_eta, d->nelem}, {"delx_zeta", d->delx_zeta, d->nelem},
    };
    for (size_t i = 0; i < sizeof t / sizeof t[0]; ++i)
        if (!strcmp(name, t[i].n)) { if (len) *len = t[i].l; return t[i].p; }
    return NULL;
}

int *lo_ifield(lo_domain *d, const char *name, long *len)
{
    const struct { const char *n; int *p; long l; } t[] = {
        {"nodelist", d->nodelist, 8L * d->nelem},
        {"lxim", d->lxim, d->nelem}, {"lxip", d->lxip, d->nelem},
        {"letam", d->letam, d->nelem}, {"letap", d->letap, d->nelem},
        {"lzetam", d->lzetam, d->nelem}, {"lzetap", d->lzetap, d->nelem},
        {"elemBC", d->elem_bc, d->nelem},
        {"nodeElemStart", d->node_elem_start, d->nnode},
        {"nodeElemCount", d->node_elem_count, d->nnode},
        {"nodeElemCornerList", d->node_elem_corner_list, 8L * d->nelem},
        {"symmX", d->symm_x, d->nsymm_x}, {"symmY", d->symm_y, d->nsymm_y},
        {"symmZ", d->symm_z, d->nsymm_z},
    };
    for (size_t i = 0; i < sizeof t / sizeof t[0]; ++i)
        if (!strcmp(name, t[i].n)) { if (len) *len = t[i].l; return t[i].p; }
    return NULL;
}
