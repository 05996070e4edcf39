/*
 * ref_driver.cc -- drives the UNMODIFIED reference implementation
 * (reference/C/LULESH-OMP.cc) from a driver of our own.
 *
 * TEST INFRASTRUCTURE ONLY: used to pin the oracle restatement and as the
 * "reference" CPU baseline.  The reference source is compiled as part of this
 * translation unit (its main() renamed by the preprocessor), so the step
 * functions that run are the reference's own: TimeIncrement (:557),
 * LagrangeNodal (:1685), LagrangeElements (:2784),
 * CalcTimeConstraintsForElems (:2935), LagrangeLeapFrog (:2944).
 *
 * What this driver adds, outside the reference's step code:
 *   - the mesh set-up of the reference's main() (:2960-3171), restated, with
 *     a choice of LULESH 1.0 (e0 = 3.948746e7, dt0 = 1e-7) or LULESH 2.0
 *     initial energy and time step (lulesh-2.0.3/lulesh-init.cc:171-182);
 *   - an unstructured mesh read from a .lmesh file (-u FILE), set up as the
 *     reference's unstructured reader does
 *     (reference/CUDA/lulesh-kepler-singlegpu/lulesh.cu:733-923, restated);
 *   - an energy factor (--efactor F) that multiplies the LULESH 2.0 initial
 *     energy before dt0 is formed from it, as the seeded ensembles draw it;
 *   - a cycle cap, full-precision JSON output and binary state dumps;
 *   - the whole-problem results of the final state (total energy, largest
 *     nodal speed, viscosity-weighted shock radius; the definitions of the
 *     package's sedov_metrics), so long runs need no state dump.
 *
 * Usage: lulesh_ref S [--init v1|v2] [--efactor F] [--cycles N] [--warmup W]
 *                     [--dump FILE] [--phase-dump FILE CYCLE]
 *        lulesh_ref -u FILE.lmesh [--cycles N] [--warmup W] [--dump FILE]
 *                     [--phase-dump FILE CYCLE]
 * (--warmup W: the first W cycles run before the timer starts; they count
 * towards --cycles.)
 */
#ifndef LULESH_OMP_SOURCE
#error "define LULESH_OMP_SOURCE as the quoted path of LULESH-OMP.cc"
#endif

#define main lulesh_omp_reference_main
#include LULESH_OMP_SOURCE
#undef main

#include <string.h>
#include <string>

namespace {

struct Field { const char *name; bool node; Real_t &(Domain::*get)(Index_t); };

const Field kFields[] = {
    {"x", true, &Domain::x},   {"y", true, &Domain::y},   {"z", true, &Domain::z},
    {"xd", true, &Domain::xd}, {"yd", true, &Domain::yd}, {"zd", true, &Domain::zd},
    {"fx", true, &Domain::fx}, {"fy", true, &Domain::fy}, {"fz", true, &Domain::fz},
    {"e", false, &Domain::e},  {"p", false, &Domain::p},  {"q", false, &Domain::q},
    {"ql", false, &Domain::ql}, {"qq", false, &Domain::qq}, {"v", false, &Domain::v},
    {"vnew", false, &Domain::vnew}, {"delv", false, &Domain::delv},
    {"vdov", false, &Domain::vdov}, {"arealg", false, &Domain::arealg},
    {"ss", false, &Domain::ss},
    {"delv_xi", false, &Domain::delv_xi}, {"delv_eta", false, &Domain::delv_eta},
    {"delv_zeta", false, &Domain::delv_zeta}, {"delx_xi", false, &Domain::delx_xi},
    {"delx_eta", false, &Domain::delx_eta}, {"delx_zeta", false, &Domain::delx_zeta},
};

/* Binary record: "LREF" tag, int32 stage, int32 s, 6 doubles of scalars
 * (time, deltatime, dtcourant, dthydro, cycle, 0), int32 field count, then
 * per field: 16-byte name, int64 length, doubles. */
void dump(FILE *f, int stage)
{
    const int s = domain.sizeX();
    const int nfields = (int)(sizeof kFields / sizeof kFields[0]);
    fwrite("LREF", 1, 4, f);
    fwrite(&stage, 4, 1, f);
    fwrite(&s, 4, 1, f);
    double sc[6] = {domain.time(), domain.deltatime(), domain.dtcourant(), domain.dthydro(),
                    (double)domain.cycle(), 0.0};
    fwrite(sc, 8, 6, f);
    fwrite(&nfields, 4, 1, f);
    for (int k = 0; k < nfields; ++k) {
        char name[16] = {0};
        strncpy(name, kFields[k].name, 15);
        fwrite(name, 1, 16, f);
        const long long n = kFields[k].node ? domain.numNode() : domain.numElem();
        fwrite(&n, 8, 1, f);
        for (long long i = 0; i < n; ++i) {
            double v = (domain.*kFields[k].get)((Index_t)i);
            fwrite(&v, 8, 1, f);
        }
    }
}

/* Mesh and state set-up: the reference main() :2960-3171 restated. */
void setup(Index_t edgeElems, bool v2, Real_t efactor)
{
    const Index_t edgeNodes = edgeElems + 1;
    domain.sizeX() = edgeElems;
    domain.sizeY() = edgeElems;
    domain.sizeZ() = edgeElems;
    domain.numElem() = edgeElems * edgeElems * edgeElems;
    domain.numNode() = edgeNodes * edgeNodes * edgeNodes;
    const Index_t domElems = domain.numElem();

    domain.AllocateElemPersistent(domain.numElem());
    domain.AllocateElemTemporary(domain.numElem());
    domain.AllocateNodalPersistent(domain.numNode());
    domain.AllocateNodesets(edgeNodes * edgeNodes);

    Index_t nidx = 0;
    for (Index_t plane = 0; plane < edgeNodes; ++plane)
        for (Index_t row = 0; row < edgeNodes; ++row)
            for (Index_t col = 0; col < edgeNodes; ++col) {
                domain.x(nidx) = col ? Real_t(1.125) * Real_t(col) / Real_t(edgeElems) : Real_t(0.);
                domain.y(nidx) = row ? Real_t(1.125) * Real_t(row) / Real_t(edgeElems) : Real_t(0.);
                domain.z(nidx) = plane ? Real_t(1.125) * Real_t(plane) / Real_t(edgeElems) : Real_t(0.);
                ++nidx;
            }

    Index_t zidx = 0;
    for (Index_t plane = 0; plane < edgeElems; ++plane)
        for (Index_t row = 0; row < edgeElems; ++row)
            for (Index_t col = 0; col < edgeElems; ++col) {
                const Index_t n0 = (plane * edgeNodes + row) * edgeNodes + col;
                Index_t *l = domain.nodelist(zidx++);
                l[0] = n0;
                l[1] = n0 + 1;
                l[2] = n0 + edgeNodes + 1;
                l[3] = n0 + edgeNodes;
                l[4] = n0 + edgeNodes * edgeNodes;
                l[5] = n0 + edgeNodes * edgeNodes + 1;
                l[6] = n0 + edgeNodes * edgeNodes + edgeNodes + 1;
                l[7] = n0 + edgeNodes * edgeNodes + edgeNodes;
            }

    domain.AllocateNodeElemIndexes();
    for (Index_t i = 0; i < domElems; ++i) domain.matElemlist(i) = i;

    domain.dtfixed() = Real_t(-1.0e-7);
    domain.deltatime() = Real_t(1.0e-7);
    domain.deltatimemultlb() = Real_t(1.1);
    domain.deltatimemultub() = Real_t(1.2);
    domain.stoptime() = Real_t(1.0e-2);
    domain.dtcourant() = Real_t(1.0e+20);
    domain.dthydro() = Real_t(1.0e+20);
    domain.dtmax() = Real_t(1.0e-2);
    domain.time() = Real_t(0.);
    domain.cycle() = 0;
    domain.e_cut() = Real_t(1.0e-7);
    domain.p_cut() = Real_t(1.0e-7);
    domain.q_cut() = Real_t(1.0e-7);
    domain.u_cut() = Real_t(1.0e-7);
    domain.v_cut() = Real_t(1.0e-10);
    domain.hgcoef() = Real_t(3.0);
    domain.ss4o3() = Real_t(4.0) / Real_t(3.0);
    domain.qstop() = Real_t(1.0e+12);
    domain.monoq_max_slope() = Real_t(1.0);
    domain.monoq_limiter_mult() = Real_t(2.0);
    domain.qlc_monoq() = Real_t(0.5);
    domain.qqc_monoq() = Real_t(2.0) / Real_t(3.0);
    domain.qqc() = Real_t(2.0);
    domain.pmin() = Real_t(0.);
    domain.emin() = Real_t(-1.0e+15);
    domain.dvovmax() = Real_t(0.1);
    domain.eosvmax() = Real_t(1.0e+9);
    domain.eosvmin() = Real_t(1.0e-9);
    domain.refdens() = Real_t(1.0);

    for (Index_t i = 0; i < domElems; ++i) {
        Real_t xl[8], yl[8], zl[8];
        Index_t *nl = domain.nodelist(i);
        for (int k = 0; k < 8; ++k) {
            xl[k] = domain.x(nl[k]);
            yl[k] = domain.y(nl[k]);
            zl[k] = domain.z(nl[k]);
        }
        const Real_t volume = CalcElemVolume(xl, yl, zl);
        domain.volo(i) = volume;
        domain.elemMass(i) = volume;
        for (int k = 0; k < 8; ++k) domain.nodalMass(nl[k]) += volume / Real_t(8.0);
    }

    if (v2) {
        const Real_t ebase = Real_t(3.948746e+7);
        const Real_t scale = Real_t(edgeElems) / Real_t(45.0);
        const Real_t einit = ebase * scale * scale * scale * efactor;
        domain.e(0) = einit;
        domain.deltatime() = (Real_t(.5) * cbrt(domain.volo(0))) / sqrt(Real_t(2.0) * einit);
    } else {
        domain.e(0) = Real_t(3.948746e+7);
    }

    nidx = 0;
    for (Index_t i = 0; i < edgeNodes; ++i) {
        const Index_t planeInc = i * edgeNodes * edgeNodes, rowInc = i * edgeNodes;
        for (Index_t j = 0; j < edgeNodes; ++j) {
            domain.symmX(nidx) = planeInc + j * edgeNodes;
            domain.symmY(nidx) = planeInc + j;
            domain.symmZ(nidx) = rowInc + j;
            ++nidx;
        }
    }

    domain.lxim(0) = 0;
    for (Index_t i = 1; i < domElems; ++i) { domain.lxim(i) = i - 1; domain.lxip(i - 1) = i; }
    domain.lxip(domElems - 1) = domElems - 1;
    for (Index_t i = 0; i < edgeElems; ++i) {
        domain.letam(i) = i;
        domain.letap(domElems - edgeElems + i) = domElems - edgeElems + i;
    }
    for (Index_t i = edgeElems; i < domElems; ++i) {
        domain.letam(i) = i - edgeElems;
        domain.letap(i - edgeElems) = i;
    }
    for (Index_t i = 0; i < edgeElems * edgeElems; ++i) {
        domain.lzetam(i) = i;
        domain.lzetap(domElems - edgeElems * edgeElems + i) = domElems - edgeElems * edgeElems + i;
    }
    for (Index_t i = edgeElems * edgeElems; i < domElems; ++i) {
        domain.lzetam(i) = i - edgeElems * edgeElems;
        domain.lzetap(i - edgeElems * edgeElems) = i;
    }

    for (Index_t i = 0; i < domElems; ++i) domain.elemBC(i) = 0;
    for (Index_t i = 0; i < edgeElems; ++i) {
        const Index_t planeInc = i * edgeElems * edgeElems, rowInc = i * edgeElems;
        for (Index_t j = 0; j < edgeElems; ++j) {
            domain.elemBC(planeInc + j * edgeElems) |= XI_M_SYMM;
            domain.elemBC(planeInc + j * edgeElems + edgeElems - 1) |= XI_P_FREE;
            domain.elemBC(planeInc + j) |= ETA_M_SYMM;
            domain.elemBC(planeInc + j + edgeElems * edgeElems - edgeElems) |= ETA_P_FREE;
            domain.elemBC(rowInc + j) |= ZETA_M_SYMM;
            domain.elemBC(rowInc + j + domElems - edgeElems * edgeElems) |= ZETA_P_FREE;
        }
    }
}

/* Parameters of LULESH-OMP.cc:3051-3087 (both mesh kinds). */
void set_params()
{
    domain.dtfixed() = Real_t(-1.0e-7);
    domain.deltatime() = Real_t(1.0e-7);
    domain.deltatimemultlb() = Real_t(1.1);
    domain.deltatimemultub() = Real_t(1.2);
    domain.stoptime() = Real_t(1.0e-2);
    domain.dtcourant() = Real_t(1.0e+20);
    domain.dthydro() = Real_t(1.0e+20);
    domain.dtmax() = Real_t(1.0e-2);
    domain.time() = Real_t(0.);
    domain.cycle() = 0;
    domain.e_cut() = Real_t(1.0e-7);
    domain.p_cut() = Real_t(1.0e-7);
    domain.q_cut() = Real_t(1.0e-7);
    domain.u_cut() = Real_t(1.0e-7);
    domain.v_cut() = Real_t(1.0e-10);
    domain.hgcoef() = Real_t(3.0);
    domain.ss4o3() = Real_t(4.0) / Real_t(3.0);
    domain.qstop() = Real_t(1.0e+12);
    domain.monoq_max_slope() = Real_t(1.0);
    domain.monoq_limiter_mult() = Real_t(2.0);
    domain.qlc_monoq() = Real_t(0.5);
    domain.qqc_monoq() = Real_t(2.0) / Real_t(3.0);
    domain.qqc() = Real_t(2.0);
    domain.pmin() = Real_t(0.);
    domain.emin() = Real_t(-1.0e+15);
    domain.dvovmax() = Real_t(0.1);
    domain.eosvmax() = Real_t(1.0e+9);
    domain.eosvmin() = Real_t(1.0e-9);
    domain.refdens() = Real_t(1.0);
}

/* Unstructured set-up from a .lmesh file.  The file holds, as whitespace-
 * separated numbers: numElem numNode; numNode coordinate triples; 8 node
 * indices per element; 6 face neighbours per element (xi-, xi+, eta-, eta+,
 * zeta-, zeta+); then four node sets, each a count and its indices:
 * symmetry X, Y, Z and the free surface.
 *
 * The reference's step applies its symmetry sets over (sizeX+1)^2 entries
 * (ApplyAccelerationBoundaryConditionsForNodes, LULESH-OMP.cc:1626-1645), so
 * sizeX is chosen to make (sizeX+1)^2 cover the largest set and each set is
 * padded by repeating its last node (zeroing the same acceleration twice is
 * harmless).  Element face flags follow the reference's unstructured reader:
 * a face whose four corners all lie in the union of the symmetry sets, and
 * then a face whose four corners all lie in the free-surface set, is marked
 * SYMM; the origin element is the first one flagged SYMM on its xi-, eta- and
 * zeta- faces by the first pass. */
Index_t setup_unstructured(const char *path)
{
    FILE *fp = fopen(path, "r");
    if (!fp) { fprintf(stderr, "could not open %s\n", path); exit(2); }
    auto rd_i = [&](void) { int v; if (fscanf(fp, "%d", &v) != 1) { fprintf(stderr, "bad lmesh %s\n", path); exit(2); } return v; };
    auto rd_d = [&](void) { double v; if (fscanf(fp, "%lf", &v) != 1) { fprintf(stderr, "bad lmesh %s\n", path); exit(2); } return v; };
    const Index_t ne = rd_i(), nn = rd_i();
    domain.numElem() = ne;
    domain.numNode() = nn;
    domain.AllocateElemPersistent(ne);
    domain.AllocateElemTemporary(ne);
    domain.AllocateNodalPersistent(nn);
    for (Index_t i = 0; i < nn; ++i) {
        domain.x(i) = Real_t(rd_d());
        domain.y(i) = Real_t(rd_d());
        domain.z(i) = Real_t(rd_d());
    }
    for (Index_t k = 0; k < ne; ++k) {
        Index_t *l = domain.nodelist(k);
        for (int c = 0; c < 8; ++c) l[c] = rd_i();
    }
    for (Index_t k = 0; k < ne; ++k) {
        domain.lxim(k) = rd_i();  domain.lxip(k) = rd_i();
        domain.letam(k) = rd_i(); domain.letap(k) = rd_i();
        domain.lzetam(k) = rd_i(); domain.lzetap(k) = rd_i();
    }
    std::vector<Index_t> sets[4];
    for (int t = 0; t < 4; ++t) {
        const int n = rd_i();
        sets[t].resize(n);
        for (int i = 0; i < n; ++i) sets[t][i] = rd_i();
    }
    fclose(fp);

    size_t most = 1;
    for (int t = 0; t < 3; ++t) {
        if (sets[t].empty()) { fprintf(stderr, "empty symmetry set in %s\n", path); exit(2); }
        most = std::max(most, sets[t].size());
    }
    Index_t side = 1;
    while (size_t(side) * size_t(side) < most) ++side;
    domain.sizeX() = domain.sizeY() = domain.sizeZ() = side - 1;
    domain.AllocateNodesets(size_t(side) * size_t(side));
    for (size_t i = 0; i < size_t(side) * size_t(side); ++i) {
        domain.symmX(i) = sets[0][std::min(i, sets[0].size() - 1)];
        domain.symmY(i) = sets[1][std::min(i, sets[1].size() - 1)];
        domain.symmZ(i) = sets[2][std::min(i, sets[2].size() - 1)];
    }

    domain.AllocateNodeElemIndexes();
    for (Index_t i = 0; i < ne; ++i) domain.matElemlist(i) = i;
    set_params();

    for (Index_t i = 0; i < ne; ++i) {
        Real_t xl[8], yl[8], zl[8];
        Index_t *nl = domain.nodelist(i);
        for (int k = 0; k < 8; ++k) {
            xl[k] = domain.x(nl[k]);
            yl[k] = domain.y(nl[k]);
            zl[k] = domain.z(nl[k]);
        }
        const Real_t volume = CalcElemVolume(xl, yl, zl);
        domain.volo(i) = volume;
        domain.elemMass(i) = volume;
        for (int k = 0; k < 8; ++k) domain.nodalMass(nl[k]) += volume / Real_t(8.0);
    }

    /* face flags from the corner masks: bits 0-3 are the zeta- face,
     * 4-7 zeta+, {0,1,4,5} eta-, {2,3,6,7} eta+, {0,3,4,7} xi-, {1,2,5,6} xi+ */
    auto flag_faces = [&](const std::vector<char> &on) {
        for (Index_t k = 0; k < ne; ++k) {
            const Index_t *l = domain.nodelist(k);
            int mask = 0;
            for (int c = 0; c < 8; ++c) mask |= (on[l[c]] ? 1 : 0) << c;
            Int_t &bc = domain.elemBC(k);
            if ((mask & 0x0f) == 0x0f) bc |= ZETA_M_SYMM;
            if ((mask & 0xf0) == 0xf0) bc |= ZETA_P_SYMM;
            if ((mask & 0x33) == 0x33) bc |= ETA_M_SYMM;
            if ((mask & 0xcc) == 0xcc) bc |= ETA_P_SYMM;
            if ((mask & 0x99) == 0x99) bc |= XI_M_SYMM;
            if ((mask & 0x66) == 0x66) bc |= XI_P_SYMM;
        }
    };
    for (Index_t k = 0; k < ne; ++k) domain.elemBC(k) = 0;
    std::vector<char> on(nn, 0);
    for (int t = 0; t < 3; ++t)
        for (Index_t n : sets[t]) on[n] = 1;
    flag_faces(on);
    Index_t origin = 0;
    for (Index_t k = 0; k < ne; ++k)
        if (domain.elemBC(k) == (XI_M_SYMM | ETA_M_SYMM | ZETA_M_SYMM)) { origin = k; break; }
    std::fill(on.begin(), on.end(), 0);
    for (Index_t n : sets[3]) on[n] = 1;
    flag_faces(on);

    domain.e(origin) = Real_t(3.948746e+7);
    return origin;
}

/* Whole-problem results of the current state: internal plus kinetic energy
 * sum(e m_elem) + sum(m_node |v|^2)/2, the largest nodal speed, and the
 * mean radius of the element centroids weighted by q m_elem (q is non-zero
 * only in the compression zone, so the mean follows the shock front). */
struct Metrics { double total_energy, max_velocity, shock_radius; };

Metrics metrics()
{
    double eint = 0.0, ekin = 0.0, vmax2 = 0.0, wr = 0.0, w = 0.0;
    for (Index_t n = 0; n < domain.numNode(); ++n) {
        const double v2 = double(domain.xd(n)) * domain.xd(n) + double(domain.yd(n)) * domain.yd(n) +
                          double(domain.zd(n)) * domain.zd(n);
        ekin += 0.5 * domain.nodalMass(n) * v2;
        if (v2 > vmax2) vmax2 = v2;
    }
    for (Index_t k = 0; k < domain.numElem(); ++k) {
        eint += double(domain.e(k)) * domain.elemMass(k);
        const Index_t *l = domain.nodelist(k);
        double cx = 0.0, cy = 0.0, cz = 0.0;
        for (int c = 0; c < 8; ++c) { cx += domain.x(l[c]); cy += domain.y(l[c]); cz += domain.z(l[c]); }
        cx /= 8.0; cy /= 8.0; cz /= 8.0;
        const double qm = double(domain.q(k)) * domain.elemMass(k);
        wr += sqrt(cx * cx + cy * cy + cz * cz) * qm;
        w += qm;
    }
    Metrics m;
    m.total_energy = eint + ekin;
    m.max_velocity = sqrt(vmax2);
    m.shock_radius = w > 0.0 ? wr / w : 0.0;
    return m;
}

}  // namespace

int main(int argc, char *argv[])
{
    if (argc < 2) {
        fprintf(stderr, "usage: %s S [--init v1|v2] [--cycles N] [--dump FILE] "
                        "[--phase-dump FILE CYCLE]\n", argv[0]);
        return 2;
    }
    const bool unstructured = !strcmp(argv[1], "-u");
    if (unstructured && argc < 3) return 2;
    const int s = unstructured ? 0 : atoi(argv[1]);
    bool v2 = true;
    int max_cycles = 0, phase_cycle = -1, warmup = 0;
    Real_t efactor = Real_t(1.0);
    const char *dump_path = NULL, *phase_path = NULL;
    for (int i = unstructured ? 3 : 2; i < argc; ++i) {
        if (!strcmp(argv[i], "--init") && i + 1 < argc) v2 = strcmp(argv[++i], "v1") != 0;
        else if (!strcmp(argv[i], "--cycles") && i + 1 < argc) max_cycles = atoi(argv[++i]);
        else if (!strcmp(argv[i], "--efactor") && i + 1 < argc) efactor = Real_t(strtod(argv[++i], NULL));
        else if (!strcmp(argv[i], "--warmup") && i + 1 < argc) warmup = atoi(argv[++i]);
        else if (!strcmp(argv[i], "--dump") && i + 1 < argc) dump_path = argv[++i];
        else if (!strcmp(argv[i], "--phase-dump") && i + 2 < argc) {
            phase_path = argv[++i];
            phase_cycle = atoi(argv[++i]);
        } else {
            fprintf(stderr, "unknown argument %s\n", argv[i]);
            return 2;
        }
    }
    Index_t origin = 0;
    if (unstructured) {
        origin = setup_unstructured(argv[2]);
        v2 = false;
    } else {
        if (s < 1 || !(efactor > Real_t(0.))) return 2;
        setup(s, v2, efactor);
    }

    FILE *pf = phase_path ? fopen(phase_path, "wb") : NULL;
    timeval start, end;
    gettimeofday(&start, NULL);
    int n = 0;
    while (domain.time() < domain.stoptime() && (max_cycles <= 0 || n < max_cycles)) {
        if (n == warmup && warmup > 0) gettimeofday(&start, NULL);
        if (pf && n == phase_cycle) {
            /* one cycle split into its phases, a state record after each */
            dump(pf, 0);
            TimeIncrement();
            dump(pf, 1);
            LagrangeNodal();
            dump(pf, 2);
            LagrangeElements();
            dump(pf, 3);
            CalcTimeConstraintsForElems();
            dump(pf, 4);
        } else {
            TimeIncrement();
            LagrangeLeapFrog();
        }
        ++n;
    }
    gettimeofday(&end, NULL);
    if (pf) fclose(pf);
    const double elapsed = double(end.tv_sec - start.tv_sec) + double(end.tv_usec - start.tv_usec) * 1e-6;

    Real_t MaxAbsDiff = 0.0, TotalAbsDiff = 0.0, MaxRelDiff = 0.0;
    for (Index_t j = 0; j < s; ++j)
        for (Index_t k = j + 1; k < s; ++k) {
            const Real_t a = FABS(domain.e(j * s + k) - domain.e(k * s + j));
            TotalAbsDiff += a;
            if (MaxAbsDiff < a) MaxAbsDiff = a;
            const Real_t r = a / domain.e(k * s + j);
            if (MaxRelDiff < r) MaxRelDiff = r;
        }
    const Metrics mt = metrics();
    if (dump_path) {
        FILE *f = fopen(dump_path, "wb");
        if (f) { dump(f, 9); fclose(f); }
    }
    const int timed = n > warmup ? n - warmup : n;
    const double zc = double(domain.numElem()) * double(timed);
    printf("{\"s\": %d, \"init\": \"%s\", \"origin_elem\": %d, \"num_elem\": %d, \"cycles\": %d, \"origin_energy\": %.17e, "
           "\"time\": %.17e, \"deltatime\": %.17e, \"dtcourant\": %.17e, \"dthydro\": %.17e, "
           "\"max_abs_diff\": %.17e, \"total_abs_diff\": %.17e, \"max_rel_diff\": %.17e, "
           "\"total_energy\": %.17e, \"max_velocity\": %.17e, \"shock_radius\": %.17e, "
           "\"elapsed_s\": %.6f, \"timed_cycles\": %d, \"threads\": %d, \"mzone_cycles_per_s\": %.6f}\n",
           s, v2 ? "v2" : "v1", int(origin), int(domain.numElem()), domain.cycle(), double(domain.e(origin)), double(domain.time()),
           double(domain.deltatime()), double(domain.dtcourant()), double(domain.dthydro()),
           double(MaxAbsDiff), double(TotalAbsDiff), double(MaxRelDiff),
           mt.total_energy, mt.max_velocity, mt.shock_radius, elapsed, timed,
           omp_get_max_threads(), elapsed > 0 ? zc / elapsed * 1e-6 : 0.0);
    return 0;
}
