/*
 * lulesh_oracle.h -- CPU restatement of the LULESH 1.0 Lagrange leapfrog step.
 *
 * TEST INFRASTRUCTURE ONLY.  This oracle is the parity checker for the CUDA
 * library and the "port" CPU baseline.  Only tests/, __graft_entry__.smoke()
 * and bench.py's cpu_baseline / --impl reference legs may load it; the product
 * library never links it.
 *
 * The algorithm follows reference/C/LULESH-OMP.cc (tmcdonell/lulesh-accelerate)
 * phase by phase; each function in lulesh_oracle.c cites the lines it follows.
 * Error codes are the reference's own (LULESH-OMP.cc:82): VolumeError = -1,
 * QStopError = -2.  Where the reference calls exit(), the oracle returns the
 * code instead.
 *
 * Parity pin: tests/test_oracle_pin.py checks this oracle against (a) the
 * reference's published known-answer table (lulesh-ports.pdf Tab. 2, LULESH
 * 1.0 initialisation), (b) golden vectors produced by the unmodified
 * reference built from its own sources (oracle/ref_driver.cc), committed under
 * tests/golden/.
 */
#ifndef LULESH_ORACLE_H
#define LULESH_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

enum { LO_OK = 0, LO_VOLUME_ERROR = -1, LO_QSTOP_ERROR = -2 };

/* Initialisation flavours.  LO_INIT_V1: e(0) = 3.948746e7, dt0 = 1e-7
 * (LULESH-OMP.cc:3053, 3112).  LO_INIT_V2: e(0) = 3.948746e7*(s/45)^3 and
 * dt0 = 0.5*cbrt(volo(0))/sqrt(2*e0) (lulesh-2.0.3/lulesh-init.cc:171-182). */
enum { LO_INIT_V1 = 1, LO_INIT_V2 = 2 };

/* Scalar constants of the problem; defaults are LULESH-OMP.cc:3051-3087. */
typedef struct lo_params {
    double e_cut, p_cut, q_cut, v_cut, u_cut;
    double hgcoef, ss4o3, qstop, monoq_max_slope, monoq_limiter_mult;
    double qlc_monoq, qqc_monoq, qqc;
    double eosvmax, eosvmin, pmin, emin, dvovmax, refdens;
    double dtfixed, deltatimemultlb, deltatimemultub, dtmax, stoptime;
} lo_params;

typedef struct lo_domain lo_domain;

/* An unstructured hexahedral mesh (the reference's .lmesh contents): node
 * coordinates, 8 nodes per element in the reference's corner order, the six
 * face neighbours of each element (the element itself on a boundary), the
 * symmetry-plane node sets and the free-surface node set. */
typedef struct lo_mesh {
    int nelem, nnode;
    const double *x, *y, *z;
    const int *nodelist;
    const int *lxim, *lxip, *letam, *letap, *lzetam, *lzetap;
    const int *symm_x, *symm_y, *symm_z, *free_surf;
    int nsymm_x, nsymm_y, nsymm_z, nfree;
} lo_mesh;

void        lo_default_params(lo_params *p);
lo_domain  *lo_create(int s, int init_mode);
/* NULL for an empty mesh or an index out of range. */
lo_domain  *lo_create_mesh(const lo_mesh *m);
/* Element holding the initial energy (0 on the cube). */
int         lo_origin(lo_domain *d);
void        lo_destroy(lo_domain *d);
lo_params  *lo_params_of(lo_domain *d);

/* Field access by reference name ("x", "xd", "e", "delv_xi", "nodelist", ...).
 * Returns NULL for an unknown name.  *len receives the element count. */
double     *lo_field(lo_domain *d, const char *name, long *len);
int        *lo_ifield(lo_domain *d, const char *name, long *len);
/* Scalars: "time", "deltatime", "dtcourant", "dthydro". */
double     *lo_scalar(lo_domain *d, const char *name);
int        *lo_cycle(lo_domain *d);
int         lo_size(lo_domain *d);

/* One phase each, in the reference's call order. */
void        lo_time_increment(lo_domain *d);            /* LULESH-OMP.cc:557-604   */
int         lo_lagrange_nodal(lo_domain *d);            /* LULESH-OMP.cc:1685-1704 */
int         lo_lagrange_elements(lo_domain *d);         /* LULESH-OMP.cc:2784-2797 */
void        lo_time_constraints(lo_domain *d);          /* LULESH-OMP.cc:2935-2942 */
int         lo_lagrange_leapfrog(lo_domain *d);         /* LULESH-OMP.cc:2944-2958 */

/* The reference main loop (LULESH-OMP.cc:3179-3188): TimeIncrement then
 * LagrangeLeapFrog while time < stoptime, at most max_cycles cycles
 * (max_cycles <= 0: no cap).  *elapsed receives wall seconds of the loop. */
int         lo_run(lo_domain *d, int max_cycles, double *elapsed);

/* Plane-0 energy symmetry test (LULESH-OMP.cc:3197-3223). */
void        lo_symmetry(lo_domain *d, double *max_abs, double *total_abs, double *max_rel);

int         lo_num_threads(void);

#ifdef __cplusplus
}
#endif
#endif
