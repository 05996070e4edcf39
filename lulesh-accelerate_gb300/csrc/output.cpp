// output.cpp -- the visualisation dump of a step's state, on the host.
//
// The reference writes every step for VisIt through the Silo library
// (cbits/visit.cc:149-177, bound by src/VisIt.hs:22-86 and called each step
// by src/Main.hs:85-100 when an output path is given): the hexahedral mesh
// (connectivity and node coordinates, with the time and cycle), the zone
// fields e, p, v, q and the node fields xd, yd, zd and speed = |v|.  Silo is
// not available here, so the same content goes to a raw structure-of-arrays
// file that any reader can map:
//
//   char[8]  "LULESHD1"
//   int32    edge elements s (0 for an unstructured mesh), elements E,
//            nodes N, step
//   float64  time
//   int32    number of sections, then per section:
//            char[16] name, int32 type (0 int32, 1 float64),
//            int32 centring (0 zone, 1 node, 2 mesh), int64 count, the data
//
// with sections connectivity (int32, 8 per element, the reference's corner
// order), X, Y, Z, xd, yd, zd, speed (node) and e, p, v, q (zone), all in the
// host's byte order.  The file name is the caller's pattern formatted with
// the step, as the reference's printf(basename, step) does; only one %d-style
// conversion (with an optional zero flag and width) or none is accepted.
#include "lulesh_internal.h"

#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

namespace lulesh {
namespace {

// printf(pattern, step) for patterns holding at most one %d (flags "0" and a
// width allowed) and "%%"; false for anything else.
bool format_name(const char *pattern, int step, std::string *out)
{
    std::string name;
    int conversions = 0;
    for (const char *p = pattern; *p; ++p) {
        if (*p != '%') {
            name += *p;
            continue;
        }
        if (p[1] == '%') {
            name += '%';
            ++p;
            continue;
        }
        const char *q = p + 1;
        bool zero = false;
        if (*q == '0') { zero = true; ++q; }
        int width = 0;
        while (*q >= '0' && *q <= '9' && width < 100) width = width * 10 + (*q++ - '0');
        if (*q != 'd' || ++conversions > 1 || width >= 100) return false;
        char buf[128];
        std::snprintf(buf, sizeof buf, zero ? "%0*d" : "%*d", width, step);
        name += buf;
        p = q;
    }
    *out = name;
    return true;
}

struct Section {
    const char *name;
    int type, centring;
    long long count;
    const void *data;
};

int write_file(const std::string &path, int s, long ne, long nn, int step, double time,
               const std::vector<Section> &sections, std::string *err)
{
    FILE *f = std::fopen(path.c_str(), "wb");
    if (!f) {
        *err = "cannot create " + path;
        return LULESH_ERR_ARG;
    }
    const int head[4] = {s, (int)ne, (int)nn, step};
    const int nsec = (int)sections.size();
    bool ok = std::fwrite("LULESHD1", 1, 8, f) == 8 && std::fwrite(head, sizeof(int), 4, f) == 4 &&
              std::fwrite(&time, sizeof(double), 1, f) == 1 && std::fwrite(&nsec, sizeof(int), 1, f) == 1;
    for (const Section &sec : sections) {
        char name[16] = {0};
        std::strncpy(name, sec.name, 15);
        const int meta[2] = {sec.type, sec.centring};
        const size_t width = sec.type == 0 ? sizeof(int) : sizeof(double);
        ok = ok && std::fwrite(name, 1, 16, f) == 16 && std::fwrite(meta, sizeof(int), 2, f) == 2 &&
             std::fwrite(&sec.count, sizeof(long long), 1, f) == 1 &&
             std::fwrite(sec.data, width, (size_t)sec.count, f) == (size_t)sec.count;
    }
    ok = (std::fclose(f) == 0) && ok;
    if (!ok) {
        *err = "write failed: " + path;
        return LULESH_ERR_ARG;
    }
    return LULESH_OK;
}

}  // namespace

int write_domain_file(const char *basename, int s, long ne, long nn, const int *nodelist, int step,
                      double time, const double *const fields[10], std::string *err)
{
    std::string path;
    if (!basename || !format_name(basename, step, &path)) {
        *err = "file name pattern must hold at most one %d conversion";
        return LULESH_ERR_ARG;
    }
    for (int i = 0; i < 10; ++i)
        if (!fields[i]) {
            *err = "NULL field array";
            return LULESH_ERR_ARG;
        }
    // x y z xd yd zd e p v q, as the reference's argument list
    std::vector<double> speed(nn);
    for (long i = 0; i < nn; ++i) {
        const double a = fields[3][i], b = fields[4][i], c = fields[5][i];
        speed[i] = std::sqrt(a * a + b * b + c * c);
    }
    const std::vector<Section> sections = {
        {"connectivity", 0, 2, 8LL * ne, nodelist},
        {"X", 1, 1, nn, fields[0]}, {"Y", 1, 1, nn, fields[1]}, {"Z", 1, 1, nn, fields[2]},
        {"e", 1, 0, ne, fields[6]}, {"p", 1, 0, ne, fields[7]}, {"v", 1, 0, ne, fields[8]},
        {"q", 1, 0, ne, fields[9]},
        {"xd", 1, 1, nn, fields[3]}, {"yd", 1, 1, nn, fields[4]}, {"zd", 1, 1, nn, fields[5]},
        {"speed", 1, 1, nn, speed.data()},
    };
    return write_file(path, s, ne, nn, step, time, sections, err);
}

}  // namespace lulesh

extern "C" int lulesh_write_domain(const char *basename, int num_elem, int step, double time, const double *x,
                                   const double *y, const double *z, const double *xd, const double *yd,
                                   const double *zd, const double *e, const double *p, const double *v,
                                   const double *q)
{
    std::string err;
    if (num_elem < 1 || num_elem > lulesh::kMaxEdge) {
        lulesh::set_last_error("lulesh_write_domain: bad edge size");
        return LULESH_ERR_ARG;
    }
    // the cube's connectivity (LULESH-OMP.cc:3020-3042; cbits/visit.cc
    // regenerates the same lists)
    const long s = num_elem, en = s + 1, ne = s * s * s, nn = en * en * en;
    std::vector<int> nodelist(8 * ne);
    long k = 0;
    for (long pl = 0; pl < s; ++pl)
        for (long row = 0; row < s; ++row)
            for (long col = 0; col < s; ++col, ++k) {
                const int n0 = (int)((pl * en + row) * en + col);
                int *l = &nodelist[8 * k];
                l[0] = n0;
                l[1] = n0 + 1;
                l[2] = n0 + (int)en + 1;
                l[3] = n0 + (int)en;
                l[4] = n0 + (int)(en * en);
                l[5] = n0 + (int)(en * en) + 1;
                l[6] = n0 + (int)(en * en + en) + 1;
                l[7] = n0 + (int)(en * en + en);
            }
    const double *fields[10] = {x, y, z, xd, yd, zd, e, p, v, q};
    const int rc = lulesh::write_domain_file(basename, num_elem, ne, nn, nodelist.data(), step, time, fields, &err);
    if (rc) lulesh::set_last_error("lulesh_write_domain: " + err);
    return rc;
}
