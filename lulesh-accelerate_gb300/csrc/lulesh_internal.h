// lulesh_internal.h -- definitions shared by the host code and the kernels.
#pragma once

#include "../../include/lulesh_gb300.h"

#include <cstdint>
#include <vector_types.h>
#include <string>
#include <vector>

namespace lulesh {

// Largest edge length: 8*s^3 corner indices must fit an int32
// (Index_t is int in the reference, LULESH-OMP.cc:93).
constexpr int kMaxEdge = 640;

// Element boundary-condition bits (LULESH-OMP.cc:231-253).
enum : int {
    BC_XI_M = 0x003, BC_XI_M_SYMM = 0x001, BC_XI_M_FREE = 0x002,
    BC_XI_P = 0x00c, BC_XI_P_SYMM = 0x004, BC_XI_P_FREE = 0x008,
    BC_ETA_M = 0x030, BC_ETA_M_SYMM = 0x010, BC_ETA_M_FREE = 0x020,
    BC_ETA_P = 0x0c0, BC_ETA_P_SYMM = 0x040, BC_ETA_P_FREE = 0x080,
    BC_ZETA_M = 0x300, BC_ZETA_M_SYMM = 0x100, BC_ZETA_M_FREE = 0x200,
    BC_ZETA_P = 0xc00, BC_ZETA_P_SYMM = 0x400, BC_ZETA_P_FREE = 0x800,
};

// Error words written by the kernels, in the reference's program order
// within one cycle; the first non-zero word decides the status.
enum ErrSite : int {
    ERR_K1_DETERM = 0,   // IntegrateStressForElems determ <= 0   (LULESH-OMP.cc:1579-1584)
    ERR_K1_VOLUME = 1,   // CalcHourglassControlForElems v <= 0   (:1541-1543)
    ERR_K3_VNEW = 2,     // CalcLagrangeElements vnew <= 0        (:2026-2029)
    ERR_K3_QSTOP = 3,    // CalcQForElems q > qstop              (:2369-2381)
    ERR_K3_MATV = 4,     // ApplyMaterialPropertiesForElems v<=0  (:2750-2752)
    ERR_NUM = 5
};

// Device-resident scalar state of one problem instance.
struct DevScalars {
    double time, deltatime, dtcourant, dthydro;
    int cycle;
    int err_any;                         // OR of err[]
    int err[ERR_NUM];                    // first offending element + 1, 0 = none
    int run_cycles;                      // cycles done by the current lulesh_run
    int run_max;                         // its cap (<= 0: none)
    int geo_valid;                       // Dom::geo holds the current positions' geometry
    int elem_begin;                      // first element of the instance (batches)
    int edge;                            // its edge length s, a structured cube (batches; 0 otherwise)
    int node_begin;                      // its first node (batches)
    unsigned long long courant_key;      // order-preserving keys of the
    unsigned long long hydro_key;        // constraint minima (see keys below)
};

// Host copy of the mesh (built in mesh.cpp).
struct HostMesh {
    int s = 0;
    long ne = 0, nn = 0;
    std::vector<double> x, y, z, volo, elem_mass, nodal_mass;
    std::vector<int> nodelist, node_elem_start, node_elem_count, node_elem_corner_list;
    std::vector<int> lxim, lxip, letam, letap, lzetam, lzetap, elem_bc;
    std::vector<unsigned char> node_bc;  // bit0 x=0, bit1 y=0, bit2 z=0 plane
    double e0 = 0.0, dt0 = 0.0;
    long origin = 0;                     // element holding e0
    void build(int s, int init_mode);
    // LULESH_OK, or LULESH_ERR_ARG with a message in *err
    int build_unstructured(const lulesh_unstructured_mesh &u, std::string *err);

  private:
    void derive();                       // corner lists, volumes, masses
};

// The numbers of a .lmesh file; the arrays back a lulesh_unstructured_mesh.
struct LmeshFile {
    lulesh_unstructured_mesh view{};
    std::vector<double> x, y, z;
    std::vector<int> nodelist, nb[6], sets[4];
    int read(const char *path, std::string *err);
};

double host_elem_volume(const double x[8], const double y[8], const double z[8]);
// LULESH 2.0 region numbers (1..nr) of ne elements and the EOS repetitions
// of region r (0-based)
void region_numbers(long ne, int nr, int balance, std::vector<int> &reg);
int region_reps(int r, int nr, int cost);
// The visualisation dump (output.cpp): fields in the reference's writeDomain
// order x y z xd yd zd e p v q; LULESH_OK or LULESH_ERR_ARG with *err set.
int write_domain_file(const char *basename, int s, long ne, long nn, const int *nodelist, int step,
                      double time, const double *const fields[10], std::string *err);
// The message lulesh_last_error(NULL) returns.
void set_last_error(const std::string &msg);
void default_params(lulesh_params *p);

// Arithmetic of the kernels of a context whose state is FP64 (Dom::df):
//   kArithDF64   element geometry and forces in double-float pairs on the
//                FP32 pipe (step_df.cu; LULESH_PRECISION_FP64), corner forces
//                and the geometry cache stored as float2 pairs
//   kArithIEEE   every operation in IEEE FP64 (step_fp64.cu's element
//                kernels; LULESH_PRECISION_FP64_IEEE)
enum : int { kArithIEEE = 0, kArithDF64 = 1 };
inline int arith_of(int precision)
{
    return precision == LULESH_PRECISION_FP64 ? kArithDF64 : kArithIEEE;
}

// Everything one kernel launch needs, passed by value.
// Words per element of the FP64 path's geometry cache (Dom::geo).
constexpr int kGeoWords = 39;

struct Dom {
    int s, ne, nn;
    int keep;                            // bit0: store nodal forces, bit1: store ql/qq
    // mesh (read-only)
    const int *nodelist;                 // [8*ne] element-major, as the reference
    const int *corner_start;             // [nn+1]
    const int *corner_list;              // [8*ne] corner-major slots c*ne+e
    const unsigned char *node_bc;        // [nn]
    const int *lxim, *lxip, *letam, *letap, *lzetam, *lzetap, *elem_bc;
    // LULESH 2.0 regions (null without): the material kernel visits elements
    // in mat_order (grouped by cost) and evaluates the EOS reps[k] times
    const int *mat_order, *reps;
    // threads per block of the element and node kernels (0: kBlockElem /
    // kBlockNode); smaller on small meshes so that the blocks spread over
    // every SM
    int eblock, nblock;
    // arithmetic of the FP64-state kernels (kArith*; arith_of)
    int df;
    const double *volo, *elem_mass, *nodal_mass;
    // nodal state
    double *x, *y, *z, *xd, *yd, *zd;
    double *fx, *fy, *fz;                // only when keep & 1
    // element state
    double *e, *p, *q, *v, *ss;
    double *vnew, *delv, *vdov, *arealg, *ql, *qq;
    double *delv_xi, *delv_eta, *delv_zeta, *delx_xi, *delx_eta, *delx_zeta;
    // corner forces, corner-major [8*ne]: each corner's stress plus
    // hourglass force (the reference sums the two parts over the node's
    // corners separately and then adds the sums; adding them per corner
    // first differs only by rounding)
    double *fcx, *fcy, *fcz;
    // split precision: FP32 corner forces (corner-major [8*ne]), hi/lo
    // float pairs of the FP64 positions and velocities [nn], reciprocal
    // nodal masses [nn], FP32 monotonic-Q gradients [6][ne] in the order
    // delv_xi, delv_eta, delv_zeta, delx_xi, delx_eta, delx_zeta
    float *f32x, *f32y, *f32z;
    float2 *xs, *ys, *zs, *xds, *yds, *zds;
    double *inv_mass;
    double *inv_volo;                    // [ne] 1/volo (the element kernels need it)
    // FP64 path: element geometry of the current positions, left by the
    // kinematics kernel for the next cycle's force kernel (the positions do
    // not change between the two): the Walsh modes M1..M7 (21 words) and the
    // six shared cross products (18 words), [kGeoWords][ne]; valid while
    // DevScalars::geo_valid is set.  Null: not kept.  With df set each word
    // is a double-float pair (float2) instead of a double, and so are the
    // corner forces fcx/fcy/fcz.
    double *geo;
    float *gq;
    DevScalars *sc;
    const int *gate;                     // host-driven run loop: cycle runs while *gate != 0
    lulesh_params prm;
};

// ---- batched ensembles -------------------------------------------------
// Many independent Sedov instances share flat arrays: each instance's nodes
// and elements occupy a range that starts on a multiple of kTile, so every
// tile of kTile elements (or nodes) belongs to exactly one instance.  Tiles
// are grouped into size classes, each with its own launch shape.
constexpr int kTile = 256;
constexpr int kMaxClasses = 3;
constexpr int kBatchKernels = 4;   // force, node update, kinematics, material

struct BatchView {
    int n_inst, n_classes, n_etiles, n_ntiles;
    const int *etile_inst, *ntile_inst;          // instance of each tile
    const int *etile_class, *ntile_class;        // size class of each tile
    const int *inst_elem_end, *inst_node_end;    // one past the instance's last element / node
    const int *eclass_off, *nclass_off;          // start of each class's active list
    int *active_etiles, *active_ntiles;          // active tiles, grouped by class
    // counts[c] / counts[kMaxClasses + c]: active element / node tiles of
    // class c; counts[2*kMaxClasses]: rebuild the lists; [2*kMaxClasses+1]:
    // instances still running
    int *counts;
    unsigned char *inst_active;
};

// Launch shape of a batched kernel: threads per block, persistent grid, and
// for the split force kernel of a class of structured cubes the staging
// depth -- 0 gathers every element's corners from global memory, 2 or 4
// stages tiles of that many element rows x kTileCols columns in shared
// memory (block = rows x kTileCols threads).
struct LaunchCfg {
    int block, grid;
    int stage = 0;
};

// The staged tiles of one size class of a split batch whose instances are
// all structured cubes wide enough for a tile row (s >= kTileCols): the
// class's instances in order, with their edge lengths, first element and
// node in the flat arrays, and tile_begin[j] the first tile of instance j
// (n + 1 entries; the tile count per instance depends on the rows per
// tile, so there is one StagedClass per depth).
struct StagedClass {
    int n;
    const int *inst, *s;
    const int *elem_base, *node_base;
    const long long *tile_begin;
};

}  // namespace lulesh
