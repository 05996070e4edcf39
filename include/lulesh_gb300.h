/*
 * lulesh_gb300.h -- C ABI of the GB300-native LULESH Lagrange leapfrog step.
 *
 * This is the drop-in boundary for the hot path of tmcdonell/lulesh-accelerate:
 * the step API of src/LULESH.hs (lulesh :37-53, lagrangeLeapFrog :66-102,
 * timeIncrement :1166-1213) over the Domain record of src/Domain.hs:11-21,
 * with the semantics of the reference CPU implementation
 * reference/C/LULESH-OMP.cc.  The Haskell host binds it with
 * `foreign import ccall` in the same way src/VisIt.hs:71-86 binds
 * cbits/visit.cc:149-177 (one `double*` per structure-of-arrays component);
 * a C driver links it directly.  Nothing in these signatures is a C++, CUDA
 * or PyTorch type.
 *
 * Conventions
 *   - Node arrays have (s+1)^3 entries, element arrays s^3, both in the
 *     reference's linear order: node (plane*(s+1)+row)*(s+1)+col, element
 *     (plane*s+row)*s+col, col fastest (LULESH-OMP.cc:2996-3042).
 *   - Host arrays belong to the caller and are only read or written during
 *     the call (the touchArrayData idiom of src/VisIt.hs:43-48).
 *   - Device memory, the CUDA stream and the captured CUDA graphs belong to
 *     the context.  A context is used by one host thread at a time.
 *   - Every call returns LULESH_OK (0) or a negative status.  VolumeError and
 *     QStopError keep the reference's values (LULESH-OMP.cc:82); where the
 *     reference calls exit(), the library returns the code instead.
 *   - Calls that advance the state are ordered on the context's stream and
 *     return only after it has drained, so that their status is final.
 */
#ifndef LULESH_GB300_H
#define LULESH_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---------------------------------------------------- */
#define LULESH_OK            0
#define LULESH_VOLUME_ERROR (-1)   /* LULESH-OMP.cc:82 VolumeError */
#define LULESH_QSTOP_ERROR  (-2)   /* LULESH-OMP.cc:82 QStopError  */
#define LULESH_ERR_CUDA     (-3)   /* a CUDA call failed; see lulesh_last_error */
#define LULESH_ERR_TIMEOUT  (-4)   /* a run stopped short of stoptime: its cycle
                                      budget ran out, or the time step stopped
                                      being positive (the reference would loop
                                      forever); the state stays valid */
#define LULESH_ERR_ARG      (-5)   /* bad argument */

/* ---- precision of the element kernels -------------------------------- */
#define LULESH_PRECISION_FP64      0   /* plain FP64, the drop-in: FP64 state, node
                                          update, EOS and time constraints; element
                                          geometry and forces in double-float (pairs
                                          of FP32, ~48-bit significand) on the FP32
                                          pipe, held to the FP64 parity bar */
#define LULESH_PRECISION_SPLIT     1   /* FP32 geometry/forces/Q gradients, FP64 state */
#define LULESH_PRECISION_FP64_IEEE 2   /* every operation in IEEE FP64 */

/* ---- initial conditions of the Sedov problem ------------------------- */
#define LULESH_INIT_V1 1           /* e(0)=3.948746e7, dt0=1e-7 (LULESH-OMP.cc:3053,3112) */
#define LULESH_INIT_V2 2           /* e(0)=3.948746e7*(s/45)^3,
                                      dt0=0.5*cbrt(volo(0))/sqrt(2*e0)
                                      (lulesh-2.0.3/lulesh-init.cc:171-182) */

/* Problem constants: the Parameters record of src/Domain.hs:23-53 with the
 * values of the C reference (LULESH-OMP.cc:3051-3087). */
typedef struct lulesh_params {
    double e_cut, p_cut, q_cut, v_cut, u_cut;
    double hgcoef, ss4o3, qstop, monoq_max_slope, monoq_limiter_mult;
    double qlc_monoq, qqc_monoq, qqc;
    double eosvmax, eosvmin, pmin, emin, dvovmax, refdens;
    double dtfixed, deltatimemultlb, deltatimemultub, dtmax, stoptime;
} lulesh_params;

/* Scalar part of the Domain: the Scalar Time fields of src/Domain.hs:19-20
 * plus the constraint and cycle state of the C reference
 * (LULESH-OMP.cc:496-503). */
typedef struct lulesh_scalars {
    double time;
    double deltatime;
    double dtcourant;
    double dthydro;
    int cycle;
} lulesh_scalars;

/* Host description of a Sedov mesh.  Every pointer is caller-owned and may be
 * NULL (that array is then not produced).  Sizes: node arrays num_node,
 * element arrays num_elem, nodelist and node_elem_corner_list 8*num_elem. */
typedef struct lulesh_mesh_view {
    double *x, *y, *z;                       /* coordinates             */
    double *volo, *elem_mass, *nodal_mass;   /* reference volume, masses */
    int *nodelist;                           /* 8 node ids per element   */
    int *node_elem_start, *node_elem_count;  /* node -> corner index     */
    int *node_elem_corner_list;              /* entries 8*elem+corner    */
    int *lxim, *lxip, *letam, *letap, *lzetam, *lzetap;  /* face neighbours */
    int *elem_bc;                            /* boundary-condition bits  */
    double e0;                               /* out: energy of element 0 */
    double dt0;                              /* out: initial time step   */
} lulesh_mesh_view;

typedef struct lulesh_ctx lulesh_ctx;

/* Fill *p with the reference constants (LULESH-OMP.cc:3051-3087). */
void lulesh_default_params(lulesh_params *p);

/* Element and node counts of the s^3 mesh. */
int lulesh_mesh_sizes(int s, long *num_elem, long *num_node);

/* Build the Sedov cube on the host exactly as the reference's main() does
 * (LULESH-OMP.cc:2996-3171; node-to-corner lists as AllocateNodeElemIndexes
 * :209-268).  Needs no GPU. */
int lulesh_mesh_build(int s, int init_mode, lulesh_mesh_view *out);

/* Create a context for an s^3 Sedov problem on the current CUDA device,
 * build the mesh, upload it and set the initial state (replaces the
 * initialisation of LULESH-OMP.cc main() :2960-3171 and src/Main.hs:60-83).
 * params may be NULL for the reference constants. */
int lulesh_create(int s, int init_mode, int precision, const lulesh_params *params,
                  lulesh_ctx **out);
void lulesh_destroy(lulesh_ctx *ctx);

/* ---- unstructured meshes ----------------------------------------------
 * An arbitrary hexahedral mesh, as the reference's unstructured reader takes
 * it (reference/CUDA/lulesh-kepler-singlegpu/lulesh.cu:733-923, the "-u
 * file.lmesh" mode of its main(), :3324-3328, :3479-3494).  All arrays are
 * host memory, read during the call only:
 *   x, y, z [num_node]          initial node coordinates;
 *   nodelist [8*num_elem]       the 8 nodes of each element, element-major,
 *                               corners in the reference's order;
 *   lxim..lzetap [num_elem]     face neighbours (xi-, xi+, eta-, eta+, zeta-,
 *                               zeta+), the element itself on a boundary face;
 *   symm_x/y/z [num_symm_*]     nodes on the x, y, z symmetry planes, whose
 *                               x, y, z acceleration the step zeroes;
 *   free_surf [num_free_surf]   free-surface nodes.
 * Set-up follows the reader: a face whose four corners all lie in the union
 * of the symmetry sets, then a face whose four corners all lie in the free-
 * surface set, is flagged SYMM for the monotonic-Q limiter; the initial
 * energy 3.948746e7 goes to the origin element (the first one flagged SYMM
 * on exactly its xi-, eta- and zeta- faces by the symmetry pass; element 0 if
 * there is none) and the first time step is 1e-7 (LULESH 1.0).  Node-to-
 * corner lists, reference volumes and masses are built as on the cube. */
typedef struct lulesh_unstructured_mesh {
    long num_elem, num_node;
    const double *x, *y, *z;
    const int *nodelist;
    const int *lxim, *lxip, *letam, *letap, *lzetam, *lzetap;
    const int *symm_x, *symm_y, *symm_z, *free_surf;
    long num_symm_x, num_symm_y, num_symm_z, num_free_surf;
} lulesh_unstructured_mesh;

/* A context for an unstructured mesh.  LULESH_ERR_ARG (nothing allocated)
 * for an empty mesh, more than 2^28-1 elements, an index out of range, or a
 * node that belongs to no element. */
int lulesh_create_unstructured(const lulesh_unstructured_mesh *mesh, int precision,
                               const lulesh_params *params, lulesh_ctx **out);

/* Read a .lmesh text file (numElem numNode; numNode coordinate triples; 8
 * node indices per element; 6 face neighbours per element; then the
 * symmetry X, Y, Z and free-surface node sets, each a count followed by its
 * node indices) and create a context for it.  Where the reference exits
 * with LFileError on a file it cannot read, this returns LULESH_ERR_ARG. */
int lulesh_create_lmesh(const char *path, int precision, const lulesh_params *params,
                        lulesh_ctx **out);

/* The element holding the initial energy (0 on the cube); its energy is what
 * lulesh_origin_energy reports (the reference's domain->octantCorner,
 * lulesh.cu:3540-3542). */
int lulesh_origin_element(lulesh_ctx *ctx, long *elem);

/* Message of the last failing call on this context (static storage when ctx
 * is NULL). */
const char *lulesh_last_error(const lulesh_ctx *ctx);

/* ---- the Domain record (src/Domain.hs:11-21) ------------------------- */
/* Upload / download the evolving state: position (x,y,z), velocity
 * (xd,yd,zd), energy, pressure, viscosity, relative volume, sound speed
 * and the two Scalar Time fields.  Any array pointer may be NULL to skip it. */
int lulesh_upload_domain(lulesh_ctx *ctx,
                         const double *x, const double *y, const double *z,
                         const double *xd, const double *yd, const double *zd,
                         const double *e, const double *p, const double *q,
                         const double *v, const double *ss,
                         double time, double deltatime);
int lulesh_download_domain(lulesh_ctx *ctx,
                           double *x, double *y, double *z,
                           double *xd, double *yd, double *zd,
                           double *e, double *p, double *q,
                           double *v, double *ss,
                           double *time, double *deltatime);

/* Scalars, including dtcourant/dthydro/cycle (checkpoint/restart). */
int lulesh_get_scalars(lulesh_ctx *ctx, lulesh_scalars *out);
int lulesh_set_scalars(lulesh_ctx *ctx, const lulesh_scalars *in);

/* Any named field, by the reference's accessor name (LULESH-OMP.cc:278-389):
 * nodal "x" "y" "z" "xd" "yd" "zd" "fx" "fy" "fz" "nodalMass"; element "e"
 * "p" "q" "ql" "qq" "v" "volo" "vnew" "delv" "vdov" "arealg" "ss" "elemMass"
 * "delv_xi" "delv_eta" "delv_zeta" "delx_xi" "delx_eta" "delx_zeta".
 * n must equal the field's length.  "fx/fy/fz" hold the nodal forces of the
 * last LagrangeNodal only when the context keeps them (lulesh_keep_forces). */
int lulesh_get_field(lulesh_ctx *ctx, const char *name, double *host, long n);
int lulesh_set_field(lulesh_ctx *ctx, const char *name, const double *host, long n);
int lulesh_keep_forces(lulesh_ctx *ctx, int keep);
/* Change problem constants (e.g. qstop) of an existing context. */
int lulesh_set_params(lulesh_ctx *ctx, const lulesh_params *params);
int lulesh_get_params(lulesh_ctx *ctx, lulesh_params *params);

/* ---- LULESH 2.0 regions ------------------------------------------------
 * lulesh_set_regions splits the elements into num_regions material regions
 * as LULESH 2.0 does on one rank (Domain::CreateRegionIndexSets,
 * lulesh-2.0.3/lulesh-init.cc:377-486, its -r/-b/-c options
 * lulesh-util.cc:95-136): runs of consecutive elements, each run's region
 * drawn with weight (r+1)^balance from the C library generator seeded with
 * 0, run lengths from the reference's bin table.  Every region is the same
 * material, so results do not change; what changes is the work: the EOS of
 * an element in region r (0-based) is evaluated 1, 1+cost or 10*(1+cost)
 * times (ApplyMaterialPropertiesForElems, lulesh.cc:2410-2424).
 * num_regions = 0 removes the regions (one EOS evaluation per element, the
 * LULESH 1.0 / LULESH-OMP.cc behaviour and the default).  LULESH_ERR_ARG for
 * negative arguments, cost > 100 or weights that overflow an int.
 * lulesh_get_regions writes each element's region number (1..num_regions;
 * all 1 without regions) into reg_num_list [num_elem] (regNumList). */
int lulesh_set_regions(lulesh_ctx *ctx, int num_regions, int balance, int cost);
int lulesh_get_regions(lulesh_ctx *ctx, int *reg_num_list);
/* The same assignment on the host, without a context: region numbers of
 * num_elem elements into reg_num_list [num_elem]. */
int lulesh_region_numbers(long num_elem, int num_regions, int balance, int *reg_num_list);

/* ---- the step API ---------------------------------------------------- */
int lulesh_time_increment(lulesh_ctx *ctx);        /* TimeIncrement      LULESH-OMP.cc:557-604;
                                                      returns without waiting for the GPU (it has
                                                      no error exit of its own)                */
int lulesh_lagrange_nodal(lulesh_ctx *ctx);        /* LagrangeNodal      LULESH-OMP.cc:1685-1704 */
int lulesh_lagrange_elements(lulesh_ctx *ctx);     /* LagrangeElements   LULESH-OMP.cc:2784-2797 */
int lulesh_calc_time_constraints(lulesh_ctx *ctx); /* CalcTimeConstraintsForElems :2935-2942   */
int lulesh_lagrange_leapfrog(lulesh_ctx *ctx);     /* LagrangeLeapFrog   LULESH-OMP.cc:2944-2958;
                                                      lagrangeLeapFrog   src/LULESH.hs:66-102     */

/* The reference's main loop (LULESH-OMP.cc:3179-3188; src/Main.hs:90-108):
 * while (time < stoptime) { TimeIncrement; LagrangeLeapFrog }, at most
 * max_cycles cycles.  The loop runs on the device inside one CUDA graph; the
 * host does not wait per cycle.  A device loop always ends: max_cycles <= 0
 * (or above the budget) means LULESH_RUN_CYCLE_BUDGET cycles, and a run that
 * stops before stoptime without reaching the caller's own max_cycles -- the
 * budget ran out, or the time step is no longer positive -- returns
 * LULESH_ERR_TIMEOUT with the state intact (a further call continues). */
#define LULESH_RUN_CYCLE_BUDGET (1 << 20)
int lulesh_run(lulesh_ctx *ctx, int max_cycles, int *cycles_done);

/* Result checks of LULESH-OMP.cc:3197-3223 / src/Main.hs:132-156.  The
 * plane-0 symmetry test needs the cube: LULESH_ERR_ARG on an unstructured
 * mesh. */
int lulesh_origin_energy(lulesh_ctx *ctx, double *e0);
int lulesh_symmetry(lulesh_ctx *ctx, double *max_abs_diff, double *total_abs_diff,
                    double *max_rel_diff);

/* ---- visualisation output --------------------------------------------
 * The reference writes each step for VisIt with Silo (writeDomain,
 * cbits/visit.cc:149-177, bound at src/VisIt.hs:71-86): mesh connectivity and
 * coordinates with the time and cycle, the zone fields e, p, v, q and the
 * node fields xd, yd, zd and speed.  Silo is not available here, so the same
 * content goes to a raw structure-of-arrays file ("LULESHD1": a header with
 * s, elements, nodes, step and time, then named, typed, counted sections;
 * the layout is spelled out in csrc/output.cpp).  The file name is
 * printf(basename, step) as in the reference, with at most one %d conversion
 * allowed.  lulesh_write_domain has the reference's argument list (host
 * arrays of the s^3 cube, num_elem = s) and needs no GPU;
 * lulesh_dump_domain writes a context's current state, cube or unstructured.
 * LULESH_ERR_ARG for a bad pattern, size or file. */
int lulesh_write_domain(const char *basename, int num_elem, int step, double time,
                        const double *x, const double *y, const double *z,
                        const double *xd, const double *yd, const double *zd,
                        const double *e, const double *p, const double *v, const double *q);
int lulesh_dump_domain(lulesh_ctx *ctx, const char *basename, int step);

/* Sizes of this context's mesh (s = 0 for an unstructured mesh). */
int lulesh_sizes(lulesh_ctx *ctx, int *s, long *num_elem, long *num_node);

/* The context's cudaStream_t (as void*), for callers that time or order
 * their own work against the library. */
void *lulesh_stream(lulesh_ctx *ctx);

/* Number of kernels this context has launched so far (graph replays count
 * each kernel node).  Lets a caller check that the GPU path ran. */
long long lulesh_kernel_launches(lulesh_ctx *ctx);

/* ---- measurement helpers (no counterpart in the reference) ----------- */
/* The same loop as lulesh_run, launched kernel by kernel with a CUDA event
 * between kernels and one host synchronisation per cycle.  kernel_ms[i]
 * receives the summed device time of kernel i over all cycles, in the order
 * time increment, element force, node update, element kinematics, element
 * material, constraint publication (LULESH_NUM_TIMED_KERNELS entries). */
#define LULESH_NUM_TIMED_KERNELS 6
int lulesh_run_profiled(lulesh_ctx *ctx, int max_cycles, int *cycles_done, double *kernel_ms);

/* Measured FP64 fused-multiply-add throughput of the current device in
 * TFLOP/s (2 flops per FMA), from a register-only kernel. */
int lulesh_probe_fp64_peak(double *tflops);

/* Issue rates of the current device, in operations per SM per clock at its
 * maximum clock: rates[0] FP32 FMA, rates[1] FP64 FMA, rates[2] FP64->FP32
 * conversion (each paired with one FP64 add), rates[3] FP64 division. */
int lulesh_probe_pipe_rates(double *rates);

/* Accuracy of the library's own FP64 root and reciprocal functions against
 * CUDA's, over 2^20 arguments spread over [2^-140, 2^140]: the largest
 * relative difference of errs[0] the inverse cube root (hourglass
 * coefficient) from rcbrt, errs[1] x*rsqrt(x) (sound speed) from sqrt,
 * errs[2] the reciprocal (compressions, Q limiter) from __drcp_rn, errs[3]
 * the quotient (strain rate, density, hydro constraint) from a / x. */
int lulesh_probe_math(double errs[4]);

/* ---- LagrangeNodal without allocation ---------------------------------
 * No counterpart in the reference: an addition for callers that cannot
 * allocate GPU memory themselves -- code whose device memory is handed out by
 * a host framework's own pool or arena, or that must not call the allocator
 * while its work is in flight.  Everything else in this header allocates
 * inside lulesh_create; this call allocates nothing.
 *
 * It performs LagrangeNodal (LULESH-OMP.cc:1685-1704) -- the same kernels as
 * lulesh_lagrange_nodal -- on arrays the caller owns, all DEVICE pointers in
 * the reference's layout: nodelist [8E]; node_elem_start, node_elem_count [N]
 * and node_elem_corner_list [8E] (entries 8*elem+corner,
 * AllocateNodeElemIndexes :209-268); symm_x/y/z [num_symm] (the symmetry
 * node sets, :3114-3125); volo, elem_mass, p, q, v, ss [E]; nodal_mass [N].
 * x, y, z, xd, yd, zd [N] are read and updated in place; fx, fy, fz [N]
 * receive the nodal forces when all three are non-NULL.  deltatime is the
 * step's time increment; params supplies u_cut and hgcoef.  stream is a
 * cudaStream_t (NULL: the default stream); the call returns after that stream
 * has drained, with LULESH_OK, LULESH_VOLUME_ERROR, or LULESH_ERR_ARG
 * (message on stderr) for a mesh over the limit or malformed tables: an index
 * out of range, or node-to-corner lists that are not the reference's map
 * (packed from 0 to 8E, node n's list holding only corners on node n, each
 * list increasing).  On LULESH_ERR_ARG the state arrays are left unchanged.
 *
 * Its working memory (per-corner forces, node-to-corner slots, the
 * symmetry-plane mask, error words) is one fixed device array compiled into
 * the library: at most 65,536 elements and 131,072 nodes, 14.6 MiB that every
 * GPU on which this call is used keeps until the process exits.  All calls
 * share that array, so calls that overlap on the GPU race; order them on one
 * stream.  Every call looks up the array's device address on the calling
 * thread's current device (a host-side lookup, no allocation); the first call
 * on a device also loads the library's device code there. */
int lulesh_lagrange_nodal_noalloc(
    int num_elem, int num_node, double deltatime, const lulesh_params *params,
    const int *nodelist, const int *node_elem_start, const int *node_elem_count,
    const int *node_elem_corner_list, const int *symm_x, const int *symm_y, const int *symm_z,
    int num_symm, const double *volo, const double *elem_mass, const double *nodal_mass,
    const double *p, const double *q, const double *v, const double *ss,
    double *x, double *y, double *z, double *xd, double *yd, double *zd,
    double *fx, double *fy, double *fz, void *stream);

/* ---- batched ensembles -------------------------------------------------
 * Many independent Sedov problems of uneven size advanced together on one
 * GPU, each with its own time, time step and stop time (the reference runs
 * one problem per process; its MPI variants decompose one problem, they do
 * not batch several).  Instance i has edge length sizes[i] and initial
 * energy e0(s_i) * e0_scale[i] (e0_scale may be NULL for 1.0); with
 * LULESH_INIT_V2 its initial time step is 0.5*cbrt(volo0)/sqrt(2*e0) of the
 * scaled energy.  Every instance's arithmetic is exactly that of a
 * single-instance context with the same initial state.  The batch runs as
 * one CUDA graph; in split precision per size class of instance (s <= 24,
 * s <= 48, larger) each step kernel has its own launch shape and the classes
 * run as parallel branches, in FP64 all instances form one class. */
typedef struct lulesh_batch lulesh_batch;

int lulesh_batch_create(int n, const int *sizes, const double *e0_scale, int init_mode, int precision,
                        const lulesh_params *params, lulesh_batch **out);
void lulesh_batch_destroy(lulesh_batch *b);
const char *lulesh_batch_last_error(const lulesh_batch *b);

/* Run every instance until its time reaches stoptime (the main loop of
 * LULESH-OMP.cc:3179-3188 per instance), at most max_cycles cycles each
 * (<= 0: LULESH_RUN_CYCLE_BUDGET).  *cycles_done receives the largest
 * per-instance count.  LULESH_ERR_TIMEOUT when an instance without an error
 * stopped short of stoptime and of the caller's max_cycles (lulesh_run's
 * rule); an instance's own error is its status in lulesh_batch_instance. */
int lulesh_batch_run(lulesh_batch *b, int max_cycles, int *cycles_done);

/* Counts; the per-instance state and status (LULESH_OK, LULESH_VOLUME_ERROR
 * or LULESH_QSTOP_ERROR) and fields (the names of lulesh_get_field: "x" "y"
 * "z" "xd" "yd" "zd" "e" "p" "q" "v" "ss" "vdov" "arealg" "volo" "elemMass"
 * "nodalMass"). */
int lulesh_batch_size(lulesh_batch *b, int *n, long *total_elements, long *total_nodes);
int lulesh_batch_instance(lulesh_batch *b, int i, lulesh_scalars *out, double *origin_energy, int *status);
int lulesh_batch_get_field(lulesh_batch *b, int i, const char *name, double *host, long n);
/* Sum over instances of elements x cycles done by the last lulesh_batch_run
 * or lulesh_batch_run_retuned call. */
int lulesh_batch_zone_cycles(lulesh_batch *b, double *zone_cycles);

/* Choose threads per block (64/128/256, i.e. 4/2/1 elements per thread of a
 * 256-element tile) and resident blocks per SM (1/2/4/8 and the most that
 * fit) of each step kernel per size class by timing the candidates on this
 * batch, whose state is restored afterwards; in split precision, for a
 * class whose instances are all cubes with s >= 64, also the staging depth
 * of the force kernel: its corners gathered from global memory (0), or
 * tiles of 2 or 4 element rows x 64 columns staged in shared memory (blocks
 * of 128 or 256 threads).
 * Choices are cached in the JSON file cache_path (keyed by GPU model, SM
 * count, precision, class, kernel; NULL: no cache); retune != 0 ignores
 * cached entries. */
int lulesh_batch_autotune(lulesh_batch *b, const char *cache_path, int retune);

/* lulesh_batch_run in chunks of at most chunk cycles; after a chunk, when the
 * elements of the instances still running have fallen below fraction
 * (0 < fraction < 1) of those the launch shapes were last tuned for, the
 * shapes are re-timed on the running set (lulesh_batch_autotune, not
 * cached) and the graph rebuilt.  Results are those of lulesh_batch_run:
 * the launch shapes change no element's arithmetic.  *cycles_done: the
 * largest per-instance count; *retunes: how many re-tunings ran. */
int lulesh_batch_run_retuned(lulesh_batch *b, int chunk, double fraction, int max_cycles, int *cycles_done,
                             int *retunes);
int lulesh_batch_tuning(lulesh_batch *b, int size_class, int kernel, int *block, int *grid);
/* The staging depth in use for a class's kernel: element rows per staged
 * tile, 0 for gathered corners (always 0 but for the split force kernel). */
int lulesh_batch_staging(lulesh_batch *b, int size_class, int kernel, int *rows);
/* Set a class's kernel launch shape by hand: threads per block (a multiple
 * of 32, at most 256), resident blocks per SM of the persistent grid
 * (>= 1, capped at what fits), staging depth rows (0; or 2 or 4 for the
 * split force kernel of a class that can be staged, block then ignored).
 * The shapes change no element's arithmetic. */
int lulesh_batch_set_tuning(lulesh_batch *b, int size_class, int kernel, int block, int blocks_per_sm, int rows);

void *lulesh_batch_stream(lulesh_batch *b);
long long lulesh_batch_kernel_launches(lulesh_batch *b);

#ifdef __cplusplus
}
#endif
#endif
