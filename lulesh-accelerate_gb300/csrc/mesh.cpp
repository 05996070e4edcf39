// mesh.cpp -- host construction of the Sedov problem.
//
// Builds what the reference's main() builds before its time loop
// (reference/C/LULESH-OMP.cc:2960-3171): coordinates, hexahedron
// connectivity, node-to-corner lists (AllocateNodeElemIndexes :209-268),
// reference volumes and masses, face neighbours, boundary-condition bits and
// the initial energy / time step -- on the s^3 cube, or on an unstructured
// mesh as the reference's unstructured reader sets it up
// (reference/CUDA/lulesh-kepler-singlegpu/lulesh.cu:733-923).  Compiled with
// -ffp-contract=off so that the floating-point results are the reference's
// on every host architecture.
#include "lulesh_internal.h"

#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

namespace lulesh {

// CalcElemVolume (LULESH-OMP.cc:1706-1790), same association as the
// reference, for the host set-up.
double host_elem_volume(const double x[8], const double y[8], const double z[8])
{
    const double twelveth = 1.0 / 12.0;
    const double dx61 = x[6] - x[1], dy61 = y[6] - y[1], dz61 = z[6] - z[1];
    const double dx70 = x[7] - x[0], dy70 = y[7] - y[0], dz70 = z[7] - z[0];
    const double dx63 = x[6] - x[3], dy63 = y[6] - y[3], dz63 = z[6] - z[3];
    const double dx20 = x[2] - x[0], dy20 = y[2] - y[0], dz20 = z[2] - z[0];
    const double dx50 = x[5] - x[0], dy50 = y[5] - y[0], dz50 = z[5] - z[0];
    const double dx64 = x[6] - x[4], dy64 = y[6] - y[4], dz64 = z[6] - z[4];
    const double dx31 = x[3] - x[1], dy31 = y[3] - y[1], dz31 = z[3] - z[1];
    const double dx72 = x[7] - x[2], dy72 = y[7] - y[2], dz72 = z[7] - z[2];
    const double dx43 = x[4] - x[3], dy43 = y[4] - y[3], dz43 = z[4] - z[3];
    const double dx57 = x[5] - x[7], dy57 = y[5] - y[7], dz57 = z[5] - z[7];
    const double dx14 = x[1] - x[4], dy14 = y[1] - y[4], dz14 = z[1] - z[4];
    const double dx25 = x[2] - x[5], dy25 = y[2] - y[5], dz25 = z[2] - z[5];
    auto triple = [](double x1, double y1, double z1, double x2, double y2, double z2,
                     double x3, double y3, double z3) {
        return x1 * (y2 * z3 - z2 * y3) + x2 * (z1 * y3 - y1 * z3) + x3 * (y1 * z2 - z1 * y2);
    };
    double vol = triple(dx31 + dx72, dx63, dx20, dy31 + dy72, dy63, dy20, dz31 + dz72, dz63, dz20) +
                 triple(dx43 + dx57, dx64, dx70, dy43 + dy57, dy64, dy70, dz43 + dz57, dz64, dz70) +
                 triple(dx14 + dx25, dx61, dx50, dy14 + dy25, dy61, dy50, dz14 + dz25, dz61, dz50);
    return vol * twelveth;
}

void default_params(lulesh_params *p)
{
    std::memset(p, 0, sizeof *p);
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

// Node-to-corner lists in (element, corner) order, reference volumes and the
// element and nodal masses of a filled-in nodelist.
void HostMesh::derive()
{
    // node -> corner lists in (element, corner) order: a counting sort.
    node_elem_count.assign(nn, 0);
    node_elem_start.assign(nn, 0);
    node_elem_corner_list.assign(8 * ne, 0);
    for (long i = 0; i < 8 * ne; ++i) node_elem_count[nodelist[i]]++;
    for (long i = 1; i < nn; ++i) node_elem_start[i] = node_elem_start[i - 1] + node_elem_count[i - 1];
    std::vector<int> fill(nn, 0);
    for (long i = 0; i < ne; ++i)
        for (int j = 0; j < 8; ++j) {
            const int m = nodelist[8 * i + j];
            node_elem_corner_list[node_elem_start[m] + fill[m]++] = int(8 * i + j);
        }

    volo.assign(ne, 0.0);
    elem_mass.assign(ne, 0.0);
    nodal_mass.assign(nn, 0.0);
    for (long i = 0; i < ne; ++i) {
        double xl[8], yl[8], zl[8];
        for (int k = 0; k < 8; ++k) {
            const int g = nodelist[8 * i + k];
            xl[k] = x[g];
            yl[k] = y[g];
            zl[k] = z[g];
        }
        const double vol = host_elem_volume(xl, yl, zl);
        volo[i] = vol;
        elem_mass[i] = vol;
        for (int k = 0; k < 8; ++k) nodal_mass[nodelist[8 * i + k]] += vol / 8.0;
    }
}

void HostMesh::build(int s_, int init_mode)
{
    s = s_;
    const int en = s + 1;
    ne = (long)s * s * s;
    nn = (long)en * en * en;

    x.assign(nn, 0.0);
    y.assign(nn, 0.0);
    z.assign(nn, 0.0);
    long n = 0;
    for (int pl = 0; pl < en; ++pl)
        for (int row = 0; row < en; ++row)
            for (int col = 0; col < en; ++col, ++n) {
                // LULESH-OMP.cc:3001-3014: 1.125*(i)/s, exactly 0 on the first plane
                x[n] = col ? 1.125 * double(col) / double(s) : 0.0;
                y[n] = row ? 1.125 * double(row) / double(s) : 0.0;
                z[n] = pl ? 1.125 * double(pl) / double(s) : 0.0;
            }

    nodelist.assign(8 * ne, 0);
    long e = 0;
    for (int pl = 0; pl < s; ++pl)
        for (int row = 0; row < s; ++row)
            for (int col = 0; col < s; ++col, ++e) {
                const int n0 = (pl * en + row) * en + col;
                int *l = &nodelist[8 * e];
                l[0] = n0;
                l[1] = n0 + 1;
                l[2] = n0 + en + 1;
                l[3] = n0 + en;
                l[4] = n0 + en * en;
                l[5] = n0 + en * en + 1;
                l[6] = n0 + en * en + en + 1;
                l[7] = n0 + en * en + en;
            }

    derive();

    origin = 0;
    if (init_mode == LULESH_INIT_V2) {
        // lulesh-2.0.3/lulesh-init.cc:171-182
        const double ebase = 3.948746e+7;
        const double scale = double(s) / 45.0;
        e0 = ebase * scale * scale * scale;
        dt0 = (.5 * std::cbrt(volo[0])) / std::sqrt(2.0 * e0);
    } else {
        e0 = 3.948746e+7;   // LULESH-OMP.cc:3112
        dt0 = 1.0e-7;       // LULESH-OMP.cc:3053
    }

    // symmetry-plane node sets (LULESH-OMP.cc:3114-3125) as a per-node mask
    node_bc.assign(nn, 0);
    for (int i = 0; i < en; ++i)
        for (int j = 0; j < en; ++j) {
            node_bc[i * en * en + j * en] |= 1;  // symmX: x = 0 plane
            node_bc[i * en * en + j] |= 2;       // symmY: y = 0 plane
            node_bc[i * en + j] |= 4;            // symmZ: z = 0 plane
        }

    // face neighbours (LULESH-OMP.cc:3127-3151)
    lxim.assign(ne, 0); lxip.assign(ne, 0);
    letam.assign(ne, 0); letap.assign(ne, 0);
    lzetam.assign(ne, 0); lzetap.assign(ne, 0);
    lxim[0] = 0;
    for (long i = 1; i < ne; ++i) { lxim[i] = int(i - 1); lxip[i - 1] = int(i); }
    lxip[ne - 1] = int(ne - 1);
    for (long i = 0; i < s; ++i) { letam[i] = int(i); letap[ne - s + i] = int(ne - s + i); }
    for (long i = s; i < ne; ++i) { letam[i] = int(i - s); letap[i - s] = int(i); }
    const long s2 = (long)s * s;
    for (long i = 0; i < s2; ++i) { lzetam[i] = int(i); lzetap[ne - s2 + i] = int(ne - s2 + i); }
    for (long i = s2; i < ne; ++i) { lzetam[i] = int(i - s2); lzetap[i - s2] = int(i); }

    // boundary-condition bits (LULESH-OMP.cc:3153-3171)
    elem_bc.assign(ne, 0);
    for (long i = 0; i < s; ++i) {
        const long pinc = i * s2, rinc = i * s;
        for (long j = 0; j < s; ++j) {
            elem_bc[pinc + j * s] |= BC_XI_M_SYMM;
            elem_bc[pinc + j * s + s - 1] |= BC_XI_P_FREE;
            elem_bc[pinc + j] |= BC_ETA_M_SYMM;
            elem_bc[pinc + j + s2 - s] |= BC_ETA_P_FREE;
            elem_bc[rinc + j] |= BC_ZETA_M_SYMM;
            elem_bc[rinc + j + ne - s2] |= BC_ZETA_P_FREE;
        }
    }
}

// Face flags of the reference's unstructured reader (lulesh.cu:852-920): a
// face whose four corners all carry the mark is flagged SYMM -- in the
// free-surface pass as well.  Corner bits 0-3 form the zeta- face, 4-7
// zeta+, {0,1,4,5} eta-, {2,3,6,7} eta+, {0,3,4,7} xi-, {1,2,5,6} xi+.
static void flag_faces(const std::vector<int> &nodelist, const std::vector<unsigned char> &mark,
                       std::vector<int> &elem_bc)
{
    const long ne = (long)elem_bc.size();
    for (long k = 0; k < ne; ++k) {
        int mask = 0;
        for (int c = 0; c < 8; ++c) mask |= (mark[nodelist[8 * k + c]] ? 1 : 0) << c;
        int &bc = elem_bc[k];
        if ((mask & 0x0f) == 0x0f) bc |= BC_ZETA_M_SYMM;
        if ((mask & 0xf0) == 0xf0) bc |= BC_ZETA_P_SYMM;
        if ((mask & 0x33) == 0x33) bc |= BC_ETA_M_SYMM;
        if ((mask & 0xcc) == 0xcc) bc |= BC_ETA_P_SYMM;
        if ((mask & 0x99) == 0x99) bc |= BC_XI_M_SYMM;
        if ((mask & 0x66) == 0x66) bc |= BC_XI_P_SYMM;
    }
}

int HostMesh::build_unstructured(const lulesh_unstructured_mesh &u, std::string *err)
{
    auto bad = [&](const std::string &m) {
        if (err) *err = "unstructured mesh: " + m;
        return LULESH_ERR_ARG;
    };
    if (u.num_elem < 1 || u.num_node < 1) return bad("empty mesh");
    if (u.num_elem > (1L << 28) - 1 || u.num_node > (1L << 31) - 1) return bad("too many elements or nodes");
    if (!u.x || !u.y || !u.z || !u.nodelist || !u.lxim || !u.lxip || !u.letam || !u.letap || !u.lzetam ||
        !u.lzetap)
        return bad("NULL array");
    const long NE = u.num_elem, NN = u.num_node;
    const int *sets[4] = {u.symm_x, u.symm_y, u.symm_z, u.free_surf};
    const long counts[4] = {u.num_symm_x, u.num_symm_y, u.num_symm_z, u.num_free_surf};
    for (int t = 0; t < 4; ++t) {
        if (counts[t] < 0 || (counts[t] > 0 && !sets[t])) return bad("bad node set");
        for (long i = 0; i < counts[t]; ++i)
            if (sets[t][i] < 0 || sets[t][i] >= NN) return bad("node set index out of range");
    }
    for (long i = 0; i < 8 * NE; ++i)
        if (u.nodelist[i] < 0 || u.nodelist[i] >= NN) return bad("nodelist index out of range");
    const int *nb[6] = {u.lxim, u.lxip, u.letam, u.letap, u.lzetam, u.lzetap};
    for (int f = 0; f < 6; ++f)
        for (long k = 0; k < NE; ++k)
            if (nb[f][k] < 0 || nb[f][k] >= NE) return bad("face neighbour out of range");
    {
        std::vector<unsigned char> used(NN, 0);
        for (long i = 0; i < 8 * NE; ++i) used[u.nodelist[i]] = 1;
        for (long n = 0; n < NN; ++n)
            if (!used[n]) return bad("node " + std::to_string(n) + " belongs to no element");
    }

    s = 0;
    ne = NE;
    nn = NN;
    x.assign(u.x, u.x + NN);
    y.assign(u.y, u.y + NN);
    z.assign(u.z, u.z + NN);
    nodelist.assign(u.nodelist, u.nodelist + 8 * NE);
    lxim.assign(u.lxim, u.lxim + NE);
    lxip.assign(u.lxip, u.lxip + NE);
    letam.assign(u.letam, u.letam + NE);
    letap.assign(u.letap, u.letap + NE);
    lzetam.assign(u.lzetam, u.lzetam + NE);
    lzetap.assign(u.lzetap, u.lzetap + NE);
    derive();

    // the symmetry node sets (lulesh.cu:810-838) as a per-node mask
    node_bc.assign(NN, 0);
    for (int t = 0; t < 3; ++t)
        for (long i = 0; i < counts[t]; ++i) node_bc[sets[t][i]] |= (unsigned char)(1 << t);

    elem_bc.assign(NE, 0);
    std::vector<unsigned char> mark(NN, 0);
    for (long n = 0; n < NN; ++n) mark[n] = node_bc[n] ? 1 : 0;
    flag_faces(nodelist, mark, elem_bc);
    origin = 0;
    for (long k = 0; k < NE; ++k)
        if (elem_bc[k] == (BC_XI_M_SYMM | BC_ETA_M_SYMM | BC_ZETA_M_SYMM)) {
            origin = k;
            break;
        }
    std::fill(mark.begin(), mark.end(), 0);
    for (long i = 0; i < counts[3]; ++i) mark[sets[3][i]] = 1;
    flag_faces(nodelist, mark, elem_bc);

    e0 = 3.948746e+7;   // lulesh.cu:923
    dt0 = 1.0e-7;       // lulesh.cu:999
    return LULESH_OK;
}

// A whitespace-separated .lmesh file (the reader of lulesh.cu:733-850).
int LmeshFile::read(const char *path, std::string *err)
{
    auto bad = [&](const std::string &m) {
        if (err) *err = std::string("lmesh ") + (path ? path : "(null)") + ": " + m;
        return LULESH_ERR_ARG;
    };
    if (!path) return bad("no path");
    FILE *f = std::fopen(path, "rb");
    if (!f) return bad(std::string("cannot open: ") + std::strerror(errno));
    std::string text;
    char buf[1 << 16];
    size_t got;
    while ((got = std::fread(buf, 1, sizeof buf, f)) > 0) text.append(buf, got);
    std::fclose(f);

    const char *p = text.c_str();
    bool ok = true;
    auto next_long = [&]() -> long {
        char *end;
        const long v = std::strtol(p, &end, 10);
        if (end == p) ok = false;
        p = end;
        return v;
    };
    auto next_double = [&]() -> double {
        char *end;
        const double v = std::strtod(p, &end);
        if (end == p) ok = false;
        p = end;
        return v;
    };
    const long NE = next_long(), NN = next_long();
    if (!ok || NE < 1 || NN < 1 || NE > (1L << 28) - 1 || NN > (1L << 31) - 1) return bad("bad header");
    // each number takes at least two characters: refuse sizes the file cannot hold
    if ((double)text.size() < 2.0 * (3.0 * NN + 14.0 * NE)) return bad("file shorter than its header says");
    x.resize(NN);
    y.resize(NN);
    z.resize(NN);
    for (long i = 0; i < NN && ok; ++i) {
        x[i] = next_double();
        y[i] = next_double();
        z[i] = next_double();
    }
    nodelist.resize(8 * NE);
    for (long i = 0; i < 8 * NE && ok; ++i) nodelist[i] = (int)next_long();
    for (int f = 0; f < 6; ++f) nb[f].resize(NE);
    for (long k = 0; k < NE && ok; ++k)
        for (int f = 0; f < 6; ++f) nb[f][k] = (int)next_long();
    for (int t = 0; t < 4 && ok; ++t) {
        const long n = next_long();
        if (!ok || n < 0 || n > NN) return bad("bad node-set size");
        sets[t].resize(n);
        for (long i = 0; i < n && ok; ++i) sets[t][i] = (int)next_long();
    }
    if (!ok) return bad("truncated or malformed");
    view = lulesh_unstructured_mesh{};
    view.num_elem = NE;
    view.num_node = NN;
    view.x = x.data();
    view.y = y.data();
    view.z = z.data();
    view.nodelist = nodelist.data();
    view.lxim = nb[0].data();
    view.lxip = nb[1].data();
    view.letam = nb[2].data();
    view.letap = nb[3].data();
    view.lzetam = nb[4].data();
    view.lzetap = nb[5].data();
    view.symm_x = sets[0].data();
    view.symm_y = sets[1].data();
    view.symm_z = sets[2].data();
    view.free_surf = sets[3].data();
    view.num_symm_x = (long)sets[0].size();
    view.num_symm_y = (long)sets[1].size();
    view.num_symm_z = (long)sets[2].size();
    view.num_free_surf = (long)sets[3].size();
    return LULESH_OK;
}

}  // namespace lulesh

extern "C" {

void lulesh_default_params(lulesh_params *p)
{
    if (p) lulesh::default_params(p);
}

int lulesh_mesh_sizes(int s, long *num_elem, long *num_node)
{
    if (s < 1 || s > lulesh::kMaxEdge) return LULESH_ERR_ARG;
    if (num_elem) *num_elem = (long)s * s * s;
    if (num_node) *num_node = (long)(s + 1) * (s + 1) * (s + 1);
    return LULESH_OK;
}

int lulesh_region_numbers(long num_elem, int num_regions, int balance, int *reg_num_list)
{
    if (num_elem < 0 || num_regions < 1 || balance < 0 || (num_elem > 0 && !reg_num_list)) return LULESH_ERR_ARG;
    double weights = 0.0;
    for (int i = 0; i < num_regions; ++i) weights += std::pow(double(i + 1), double(balance));
    if (weights > 2147483647.0) return LULESH_ERR_ARG;
    std::vector<int> reg;
    lulesh::region_numbers(num_elem, num_regions, balance, reg);
    std::memcpy(reg_num_list, reg.data(), reg.size() * sizeof(int));
    return LULESH_OK;
}

int lulesh_mesh_build(int s, int init_mode, lulesh_mesh_view *out)
{
    if (!out || s < 1 || s > lulesh::kMaxEdge) return LULESH_ERR_ARG;
    if (init_mode != LULESH_INIT_V1 && init_mode != LULESH_INIT_V2) return LULESH_ERR_ARG;
    lulesh::HostMesh m;
    m.build(s, init_mode);
    auto put_d = [](double *dst, const std::vector<double> &src) {
        if (dst) std::memcpy(dst, src.data(), src.size() * sizeof(double));
    };
    auto put_i = [](int *dst, const std::vector<int> &src) {
        if (dst) std::memcpy(dst, src.data(), src.size() * sizeof(int));
    };
    put_d(out->x, m.x);
    put_d(out->y, m.y);
    put_d(out->z, m.z);
    put_d(out->volo, m.volo);
    put_d(out->elem_mass, m.elem_mass);
    put_d(out->nodal_mass, m.nodal_mass);
    put_i(out->nodelist, m.nodelist);
    put_i(out->node_elem_start, m.node_elem_start);
    put_i(out->node_elem_count, m.node_elem_count);
    put_i(out->node_elem_corner_list, m.node_elem_corner_list);
    put_i(out->lxim, m.lxim);
    put_i(out->lxip, m.lxip);
    put_i(out->letam, m.letam);
    put_i(out->letap, m.letap);
    put_i(out->lzetam, m.lzetam);
    put_i(out->lzetap, m.lzetap);
    put_i(out->elem_bc, m.elem_bc);
    out->e0 = m.e0;
    out->dt0 = m.dt0;
    return LULESH_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------
// LULESH 2.0 regions
// ---------------------------------------------------------------------
namespace lulesh {

namespace {

// The C library generator the reference seeds with srand(0) (glibc's
// additive feedback generator: 34 words seeded by the Park-Miller LCG
// x' = 16807 x mod (2^31 - 1), then r[i] = r[i-31] + r[i-3] mod 2^32 with
// the first 310 outputs discarded, each output r >> 1).  Restated so that
// the assignment does not depend on the host's rand() state.
class CRand {
  public:
    explicit CRand(unsigned seed)
    {
        int32_t r = seed ? (int32_t)seed : 1;
        w_[0] = (uint32_t)r;
        for (int i = 1; i < 31; ++i) {
            const int32_t hi = r / 127773, lo = r % 127773;
            r = 16807 * lo - 2836 * hi;
            if (r < 0) r += 2147483647;
            w_[i] = (uint32_t)r;
        }
        for (int i = 31; i < 34; ++i) w_[i] = w_[i - 31];
        n_ = 34;
        for (int i = 34; i < 344; ++i) step();
    }
    int next() { return (int)(step() >> 1); }

  private:
    uint32_t step()
    {
        // ring of the last 34 words: r[n] = r[n-31] + r[n-3]
        const uint32_t v = w_[(n_ - 31) % 34] + w_[(n_ - 3) % 34];
        w_[n_ % 34] = v;
        ++n_;
        return v;
    }
    uint32_t w_[34];
    long n_;
};

}  // namespace

// Region number (1..nr) of each element, as CreateRegionIndexSets
// (lulesh-2.0.3/lulesh-init.cc:377-486) assigns them on one rank: runs of
// consecutive elements, each run's region drawn with weight (r+1)^balance
// and never the previous run's region, each run's length drawn from the
// reference's bin table.
void region_numbers(long ne, int nr, int balance, std::vector<int> &reg)
{
    reg.assign(ne, 1);
    if (nr <= 1) return;
    CRand rnd(0);
    std::vector<int> bin_end(nr);
    int denom = 0;
    for (int i = 0; i < nr; ++i) {
        denom += (int)std::pow((double)(i + 1), (double)balance);
        bin_end[i] = denom;
    }
    auto pick = [&]() {
        const int v = rnd.next() % denom;
        int i = 0;
        while (v >= bin_end[i]) ++i;
        return i % nr + 1;
    };
    long next = 0;
    int last = -1;
    while (next < ne) {
        int region = pick();
        while (region == last) region = pick();
        const int bin = rnd.next() % 1000;
        long len;
        if (bin < 773) len = rnd.next() % 15 + 1;
        else if (bin < 937) len = rnd.next() % 16 + 16;
        else if (bin < 970) len = rnd.next() % 32 + 32;
        else if (bin < 974) len = rnd.next() % 64 + 64;
        else if (bin < 978) len = rnd.next() % 128 + 128;
        else if (bin < 981) len = rnd.next() % 256 + 256;
        else len = rnd.next() % 1537 + 512;
        for (const long end = next + len; next < end && next < ne; ++next) reg[next] = region;
        last = region;
    }
}

// EOS evaluations per element of region r (0-based) of nr
// (ApplyMaterialPropertiesForElems, lulesh-2.0.3/lulesh.cc:2410-2424).
int region_reps(int r, int nr, int cost)
{
    if (r < nr / 2) return 1;
    if (r < nr - (nr + 15) / 20) return 1 + cost;
    return 10 * (1 + cost);
}

}  // namespace lulesh
