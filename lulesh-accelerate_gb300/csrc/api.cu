// api.cu -- the C ABI (include/lulesh_gb300.h): contexts, device memory,
// the captured run-loop graph and the step entry points.
#include "lulesh_internal.h"
#include "kernels.h"

#include <cuda_runtime.h>

#include <cstdio>
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

using namespace lulesh;

struct lulesh_ctx {
    int s = 0;
    long ne = 0, nn = 0;
    int precision = LULESH_PRECISION_FP64;
    int device = 0;
    cudaStream_t stream = nullptr;
    Dom dom{};
    std::vector<void *> allocs;
    DevScalars *h_sc = nullptr;      // pinned mirror for scalar reads
    int *d_active = nullptr;         // run-loop gate
    int *d_max_cycles = nullptr;
    int *h_stage = nullptr;          // pinned staging ints
    // run loop
    cudaGraphExec_t run_exec = nullptr;
    int run_mode = 0;                // 0 not built, 1 conditional while node, 2 host-driven chunks
    cudaGraphExec_t chunk_exec = nullptr;
    int status = LULESH_OK;          // sticky step error
    long long launches = 0;
    long origin = 0;                 // element holding the initial energy
    std::vector<int> regions;        // LULESH 2.0 region number per element (empty: none)
    int *d_mat_order = nullptr, *d_reps = nullptr;
    std::string err;
};

namespace {

constexpr int kChunkCycles = 16;     // cycles per graph in the host-driven fallback
thread_local std::string g_err;

}  // namespace

void lulesh::set_last_error(const std::string &msg) { g_err = msg; }

namespace {

int fail(lulesh_ctx *c, int code, const std::string &msg)
{
    if (c) c->err = msg;
    else g_err = msg;
    return code;
}

#define CK(call)                                                                          \
    do {                                                                                  \
        cudaError_t e_ = (call);                                                          \
        if (e_ != cudaSuccess)                                                            \
            return fail(ctx, LULESH_ERR_CUDA,                                             \
                        std::string(#call) + ": " + cudaGetErrorString(e_));              \
    } while (0)

template <typename T>
int dalloc(lulesh_ctx *ctx, T **p, size_t n)
{
    void *q = nullptr;
    if (n == 0) n = 1;
    cudaError_t e = cudaMalloc(&q, n * sizeof(T));
    if (e != cudaSuccess)
        return fail(ctx, LULESH_ERR_CUDA, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    ctx->allocs.push_back(q);
    *p = static_cast<T *>(q);
    return LULESH_OK;
}

struct FieldRef {
    const char *name;
    double *Dom::*member;
    bool node;
};

const FieldRef kFields[] = {
    {"x", &Dom::x, true},   {"y", &Dom::y, true},   {"z", &Dom::z, true},
    {"xd", &Dom::xd, true}, {"yd", &Dom::yd, true}, {"zd", &Dom::zd, true},
    {"fx", &Dom::fx, true}, {"fy", &Dom::fy, true}, {"fz", &Dom::fz, true},
    {"e", &Dom::e, false},  {"p", &Dom::p, false},  {"q", &Dom::q, false},
    {"ql", &Dom::ql, false}, {"qq", &Dom::qq, false}, {"v", &Dom::v, false},
    {"vnew", &Dom::vnew, false}, {"delv", &Dom::delv, false}, {"vdov", &Dom::vdov, false},
    {"arealg", &Dom::arealg, false}, {"ss", &Dom::ss, false},
    {"delv_xi", &Dom::delv_xi, false}, {"delv_eta", &Dom::delv_eta, false},
    {"delv_zeta", &Dom::delv_zeta, false}, {"delx_xi", &Dom::delx_xi, false},
    {"delx_eta", &Dom::delx_eta, false}, {"delx_zeta", &Dom::delx_zeta, false},
};

// Read-only mesh fields reachable by name.
double *const_field(lulesh_ctx *ctx, const char *name, bool *node)
{
    if (!strcmp(name, "volo")) { *node = false; return const_cast<double *>(ctx->dom.volo); }
    if (!strcmp(name, "elemMass")) { *node = false; return const_cast<double *>(ctx->dom.elem_mass); }
    if (!strcmp(name, "nodalMass")) { *node = true; return const_cast<double *>(ctx->dom.nodal_mass); }
    return nullptr;
}

double *find_field(lulesh_ctx *ctx, const char *name, bool *node, bool *writable)
{
    for (const FieldRef &f : kFields)
        if (!strcmp(name, f.name)) {
            *node = f.node;
            *writable = true;
            return ctx->dom.*(f.member);
        }
    *writable = false;
    return const_field(ctx, name, node);
}

// Status of the step after the stream drained: the first error site in
// program order wins (see ErrSite).
int read_status(lulesh_ctx *ctx)
{
    CK(cudaMemcpyAsync(ctx->h_sc, ctx->dom.sc, sizeof(DevScalars), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    if (ctx->h_sc->err_any) {
        static const int code[ERR_NUM] = {LULESH_VOLUME_ERROR, LULESH_VOLUME_ERROR, LULESH_VOLUME_ERROR,
                                          LULESH_QSTOP_ERROR, LULESH_VOLUME_ERROR};
        static const char *what[ERR_NUM] = {"IntegrateStressForElems: determ <= 0",
                                            "CalcHourglassControlForElems: v <= 0",
                                            "CalcLagrangeElements: vnew <= 0",
                                            "CalcQForElems: q > qstop",
                                            "ApplyMaterialPropertiesForElems: v <= 0"};
        for (int i = 0; i < ERR_NUM; ++i)
            if (ctx->h_sc->err[i]) {
                ctx->status = code[i];
                char buf[160];
                snprintf(buf, sizeof buf, "%s (element %d, cycle %d)", what[i], ctx->h_sc->err[i] - 1,
                         ctx->h_sc->cycle);
                ctx->err = buf;
                return code[i];
            }
    }
    return LULESH_OK;
}

// A run loop that ended with time < stoptime although the caller's own cap
// was not reached: the cycle budget ran out, or the time step stopped being
// positive.  Reported, not sticky: the state is valid and a further run
// continues from it.  Reads the scalars read_status just fetched.
int short_of_stoptime(lulesh_ctx *ctx, int max_cycles, int done)
{
    const DevScalars *h = ctx->h_sc;
    if (!(h->time < ctx->dom.prm.stoptime)) return LULESH_OK;
    if (max_cycles > 0 && max_cycles <= kRunCycleLimit && done >= max_cycles) return LULESH_OK;
    char buf[200];
    snprintf(buf, sizeof buf, "run stopped at time %.17g < stoptime %.17g after %d cycles: %s", h->time,
             ctx->dom.prm.stoptime, done,
             h->deltatime > 0.0 ? "the cycle budget (LULESH_RUN_CYCLE_BUDGET) ran out"
                                : "the time step is no longer positive");
    ctx->err = buf;
    return LULESH_ERR_TIMEOUT;
}

int check_launch(lulesh_ctx *ctx)
{
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(ctx, LULESH_ERR_CUDA, std::string("kernel launch: ") + cudaGetErrorString(e));
    return LULESH_OK;
}

int clear_errors(lulesh_ctx *ctx)
{
    DevScalars *h = ctx->h_sc;
    CK(cudaMemcpyAsync(h, ctx->dom.sc, sizeof(DevScalars), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    h->err_any = 0;
    for (int i = 0; i < ERR_NUM; ++i) h->err[i] = 0;
    h->geo_valid = 0;   // the host may have replaced positions
    CK(cudaMemcpyAsync(ctx->dom.sc, h, sizeof(DevScalars), cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    ctx->status = LULESH_OK;
    return LULESH_OK;
}

int upload(lulesh_ctx *ctx, double *dst, const double *src, long n)
{
    if (!src) return LULESH_OK;
    CK(cudaMemcpyAsync(dst, src, n * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    return LULESH_OK;
}

int download(lulesh_ctx *ctx, double *dst, const double *src, long n)
{
    if (!dst) return LULESH_OK;
    CK(cudaMemcpyAsync(dst, src, n * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    return LULESH_OK;
}

bool is_split(const lulesh_ctx *ctx) { return ctx->precision == LULESH_PRECISION_SPLIT; }

// After the host replaced FP64 node state, refresh the split path's hi/lo
// copies (a no-op for the FP64 path).
int refresh_split(lulesh_ctx *ctx)
{
    if (!is_split(ctx)) return LULESH_OK;
    launch_split_sync(ctx->dom, ctx->stream);
    int rc = check_launch(ctx);
    if (rc) return rc;
    CK(cudaStreamSynchronize(ctx->stream));
    return LULESH_OK;
}

void nodal(lulesh_ctx *ctx, const Dom &d)
{
    if (is_split(ctx)) launch_lagrange_nodal_split(d, ctx->stream);
    else launch_lagrange_nodal(d, ctx->stream);
}

void elements(lulesh_ctx *ctx, const Dom &d, bool with_constraints)
{
    if (is_split(ctx)) launch_lagrange_elements_split(d, ctx->stream, with_constraints);
    else launch_lagrange_elements(d, ctx->stream, with_constraints);
}

void run_body(lulesh_ctx *ctx, const Dom &d, cudaGraphConditionalHandle h)
{
    if (is_split(ctx)) launch_run_body_split(d, ctx->stream, h, ctx->d_active);
    else launch_run_body(d, ctx->stream, h, ctx->d_active);
}

// Build the run-loop graph: prologue -> while(cond) { one cycle }.  Falls
// back to a host-driven graph of kChunkCycles gated cycles when conditional
// nodes are not available.
int build_run_graph(lulesh_ctx *ctx)
{
    if (ctx->run_mode) return LULESH_OK;
    cudaGraph_t g = nullptr;
    cudaGraphConditionalHandle h = 0;
    bool ok = cudaGraphCreate(&g, 0) == cudaSuccess &&
              cudaGraphConditionalHandleCreate(&h, g, 0, 0) == cudaSuccess;
    if (ok) {
        // prologue, captured into g
        ok = cudaStreamBeginCaptureToGraph(ctx->stream, g, nullptr, nullptr, 0,
                                           cudaStreamCaptureModeThreadLocal) == cudaSuccess;
        if (ok) {
            launch_run_prologue(ctx->dom, ctx->stream, ctx->d_max_cycles, h, ctx->d_active);
            ok = cudaStreamEndCapture(ctx->stream, &g) == cudaSuccess;
        }
        size_t nnodes = 0;
        cudaGraphNode_t prologue = nullptr;
        if (ok) ok = cudaGraphGetNodes(g, nullptr, &nnodes) == cudaSuccess && nnodes == 1;
        if (ok) ok = cudaGraphGetNodes(g, &prologue, &nnodes) == cudaSuccess;
        cudaGraphNodeParams cp = {cudaGraphNodeTypeConditional};
        cp.conditional.handle = h;
        cp.conditional.type = cudaGraphCondTypeWhile;
        cp.conditional.size = 1;
        cudaGraphNode_t cnode = nullptr;
        if (ok) ok = cudaGraphAddNode(&cnode, g, &prologue, nullptr, 1, &cp) == cudaSuccess;
        if (ok) {
            cudaGraph_t body = cp.conditional.phGraph_out[0];
            ok = cudaStreamBeginCaptureToGraph(ctx->stream, body, nullptr, nullptr, 0,
                                               cudaStreamCaptureModeThreadLocal) == cudaSuccess;
            if (ok) {
                Dom d = ctx->dom;
                d.gate = nullptr;
                run_body(ctx, d, h);
                cudaGraph_t out = nullptr;
                ok = cudaStreamEndCapture(ctx->stream, &out) == cudaSuccess;
            }
        }
        if (ok) ok = cudaGraphInstantiate(&ctx->run_exec, g, 0) == cudaSuccess;
    }
    if (g) cudaGraphDestroy(g);
    if (ok) {
        ctx->run_mode = 1;
        return LULESH_OK;
    }
    // conditional nodes unavailable: clear the sticky error and capture the
    // gated fallback
    cudaGetLastError();
    cudaStreamCaptureStatus cs;
    if (cudaStreamIsCapturing(ctx->stream, &cs) == cudaSuccess && cs != cudaStreamCaptureStatusNone) {
        cudaGraph_t junk = nullptr;
        cudaStreamEndCapture(ctx->stream, &junk);
        if (junk) cudaGraphDestroy(junk);
    }
    cudaGetLastError();
    cudaGraph_t cg = nullptr;
    CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    Dom d = ctx->dom;
    d.gate = ctx->d_active;
    for (int i = 0; i < kChunkCycles; ++i) run_body(ctx, d, 0);
    CK(cudaStreamEndCapture(ctx->stream, &cg));
    cudaError_t e = cudaGraphInstantiate(&ctx->chunk_exec, cg, 0);
    cudaGraphDestroy(cg);
    if (e != cudaSuccess) return fail(ctx, LULESH_ERR_CUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e));
    ctx->run_mode = 2;
    return LULESH_OK;
}

}  // namespace

extern "C" {

const char *lulesh_last_error(const lulesh_ctx *ctx)
{
    return ctx ? ctx->err.c_str() : g_err.c_str();
}

void lulesh_destroy(lulesh_ctx *ctx)
{
    if (!ctx) return;
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    if (ctx->run_exec) cudaGraphExecDestroy(ctx->run_exec);
    if (ctx->chunk_exec) cudaGraphExecDestroy(ctx->chunk_exec);
    for (void *p : ctx->allocs) cudaFree(p);
    if (ctx->h_sc) cudaFreeHost(ctx->h_sc);
    if (ctx->h_stage) cudaFreeHost(ctx->h_stage);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
}

}  // extern "C"

namespace {

// A context for a built host mesh: device arrays, initial state, stream.
int create_from_mesh(const HostMesh &m, int precision, const lulesh_params *params, lulesh_ctx **out)
{
    const int s = m.s;
    *out = nullptr;
    lulesh_ctx *ctx = new lulesh_ctx;
    int rc = LULESH_OK;
    auto bail = [&](int code) { g_err = ctx->err; lulesh_destroy(ctx); return code; };

    ctx->s = s;
    ctx->origin = m.origin;
    ctx->ne = m.ne;
    ctx->nn = m.nn;
    ctx->precision = precision;
    if (cudaGetDevice(&ctx->device) != cudaSuccess ||
        cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess) {
        ctx->err = std::string("no usable CUDA device: ") + cudaGetErrorString(cudaGetLastError());
        return bail(LULESH_ERR_CUDA);
    }
    if (cudaMallocHost(&ctx->h_sc, sizeof(DevScalars)) != cudaSuccess ||
        cudaMallocHost(&ctx->h_stage, 16 * sizeof(int)) != cudaSuccess) {
        ctx->err = "cudaMallocHost failed";
        return bail(LULESH_ERR_CUDA);
    }

    Dom &d = ctx->dom;
    d.s = s;
    d.ne = (int)m.ne;
    d.nn = (int)m.nn;
    d.keep = 0;
    if (params) d.prm = *params;
    else default_params(&d.prm);
    {
        int sms = 0;
        if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device) != cudaSuccess || sms < 1)
            sms = 1;
        choose_blocks(d, sms);
    }
    const size_t ne = m.ne, nn = m.nn;

    int *nodelist, *cstart, *clist, *lxim, *lxip, *letam, *letap, *lzetam, *lzetap, *ebc;
    unsigned char *nbc;
    double *volo, *emass, *nmass;
#define A(p, n) if ((rc = dalloc(ctx, &(p), (n))) != LULESH_OK) return bail(rc)
    A(nodelist, 8 * ne); A(cstart, nn + 1); A(clist, 8 * ne); A(nbc, nn);
    A(lxim, ne); A(lxip, ne); A(letam, ne); A(letap, ne); A(lzetam, ne); A(lzetap, ne); A(ebc, ne);
    A(volo, ne); A(emass, ne); A(nmass, nn);
    A(d.x, nn); A(d.y, nn); A(d.z, nn); A(d.xd, nn); A(d.yd, nn); A(d.zd, nn);
    A(d.fx, nn); A(d.fy, nn); A(d.fz, nn);
    A(d.e, ne); A(d.p, ne); A(d.q, ne); A(d.v, ne); A(d.ss, ne);
    A(d.vnew, ne); A(d.delv, ne); A(d.vdov, ne); A(d.arealg, ne); A(d.ql, ne); A(d.qq, ne);
    A(d.delv_xi, ne); A(d.delv_eta, ne); A(d.delv_zeta, ne);
    A(d.delx_xi, ne); A(d.delx_eta, ne); A(d.delx_zeta, ne);
    d.df = arith_of(precision);
    if (precision != LULESH_PRECISION_SPLIT) {
        A(d.fcx, 8 * ne); A(d.fcy, 8 * ne); A(d.fcz, 8 * ne);
        A(d.geo, (size_t)kGeoWords * ne);
    } else {
        A(d.f32x, 8 * ne); A(d.f32y, 8 * ne); A(d.f32z, 8 * ne);
        A(d.xs, nn); A(d.ys, nn); A(d.zs, nn); A(d.xds, nn); A(d.yds, nn); A(d.zds, nn);
        A(d.gq, 6 * ne);
    }
    A(d.inv_mass, nn); A(d.inv_volo, ne);
    A(d.sc, 1); A(ctx->d_active, 1); A(ctx->d_max_cycles, 1);
#undef A
    d.nodelist = nodelist;
    d.corner_start = cstart;
    d.corner_list = clist;
    d.node_bc = nbc;
    d.lxim = lxim; d.lxip = lxip; d.letam = letam; d.letap = letap; d.lzetam = lzetam; d.lzetap = lzetap;
    d.elem_bc = ebc;
    d.volo = volo; d.elem_mass = emass; d.nodal_mass = nmass;
    d.gate = nullptr;

    // node -> corner slots, translated from the reference's 8*elem+corner
    // numbering to the corner-major slot corner*ne + elem
    std::vector<int> start(nn + 1), slots(8 * ne);
    for (size_t i = 0; i < nn; ++i) start[i] = m.node_elem_start[i];
    start[nn] = (int)(8 * ne);
    for (size_t i = 0; i < 8 * ne; ++i) {
        const int k = m.node_elem_corner_list[i];
        slots[i] = (k & 7) * (int)ne + (k >> 3);
    }
    std::vector<double> zeros(ne, 0.0), ones(ne, 1.0), e(ne, 0.0), inv_mass(nn);
    for (size_t i = 0; i < nn; ++i) inv_mass[i] = 1.0 / m.nodal_mass[i];
    std::vector<double> inv_volo(ne);
    for (size_t i = 0; i < ne; ++i) inv_volo[i] = 1.0 / m.volo[i];
    e[m.origin] = m.e0;
    cudaStream_t st = ctx->stream;
    auto up = [&](void *dst, const void *src, size_t bytes) {
        return cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, st) == cudaSuccess;
    };
    bool ok = up(nodelist, m.nodelist.data(), 8 * ne * 4) && up(cstart, start.data(), (nn + 1) * 4) &&
              up(clist, slots.data(), 8 * ne * 4) && up(nbc, m.node_bc.data(), nn) &&
              up(lxim, m.lxim.data(), ne * 4) && up(lxip, m.lxip.data(), ne * 4) &&
              up(letam, m.letam.data(), ne * 4) && up(letap, m.letap.data(), ne * 4) &&
              up(lzetam, m.lzetam.data(), ne * 4) && up(lzetap, m.lzetap.data(), ne * 4) &&
              up(ebc, m.elem_bc.data(), ne * 4) && up(volo, m.volo.data(), ne * 8) &&
              up(emass, m.elem_mass.data(), ne * 8) && up(nmass, m.nodal_mass.data(), nn * 8) && up(d.inv_mass, inv_mass.data(), nn * 8) && up(d.inv_volo, inv_volo.data(), ne * 8) &&
              up(d.x, m.x.data(), nn * 8) && up(d.y, m.y.data(), nn * 8) && up(d.z, m.z.data(), nn * 8) &&
              up(d.e, e.data(), ne * 8) && up(d.v, ones.data(), ne * 8);
    ok = ok && cudaMemsetAsync(d.xd, 0, nn * 8, st) == cudaSuccess &&
         cudaMemsetAsync(d.yd, 0, nn * 8, st) == cudaSuccess &&
         cudaMemsetAsync(d.zd, 0, nn * 8, st) == cudaSuccess &&
         cudaMemsetAsync(d.fx, 0, nn * 8, st) == cudaSuccess &&
         cudaMemsetAsync(d.fy, 0, nn * 8, st) == cudaSuccess &&
         cudaMemsetAsync(d.fz, 0, nn * 8, st) == cudaSuccess;
    for (double *f : {d.p, d.q, d.ss, d.vnew, d.delv, d.vdov, d.arealg, d.ql, d.qq, d.delv_xi, d.delv_eta,
                      d.delv_zeta, d.delx_xi, d.delx_eta, d.delx_zeta})
        ok = ok && cudaMemsetAsync(f, 0, ne * 8, st) == cudaSuccess;
    DevScalars *h = ctx->h_sc;
    memset(h, 0, sizeof *h);
    h->time = 0.0;
    h->deltatime = m.dt0;
    h->dtcourant = 1.0e+20;
    h->dthydro = 1.0e+20;
    h->cycle = 0;
    h->courant_key = ~0ULL;
    h->hydro_key = ~0ULL;
    ok = ok && up(d.sc, h, sizeof *h);
    if (ok && precision == LULESH_PRECISION_SPLIT) {
        launch_split_sync(d, st);
        ok = cudaGetLastError() == cudaSuccess;
    }
    ok = ok && cudaStreamSynchronize(st) == cudaSuccess;
    if (!ok) {
        ctx->err = std::string("lulesh_create upload: ") + cudaGetErrorString(cudaGetLastError());
        return bail(LULESH_ERR_CUDA);
    }
    *out = ctx;
    return LULESH_OK;
}

int check_precision(int precision, const char *who)
{
    if (precision != LULESH_PRECISION_FP64 && precision != LULESH_PRECISION_SPLIT &&
        precision != LULESH_PRECISION_FP64_IEEE)
        return fail(nullptr, LULESH_ERR_ARG, std::string(who) + ": unknown precision");
    return LULESH_OK;
}

}  // namespace

extern "C" {

int lulesh_create(int s, int init_mode, int precision, const lulesh_params *params, lulesh_ctx **out)
{
    if (!out || s < 1 || s > kMaxEdge) return fail(nullptr, LULESH_ERR_ARG, "lulesh_create: bad size or output pointer");
    if (init_mode != LULESH_INIT_V1 && init_mode != LULESH_INIT_V2)
        return fail(nullptr, LULESH_ERR_ARG, "lulesh_create: init_mode must be LULESH_INIT_V1 or LULESH_INIT_V2");
    if (int rc = check_precision(precision, "lulesh_create")) return rc;
    HostMesh m;
    m.build(s, init_mode);
    return create_from_mesh(m, precision, params, out);
}

int lulesh_create_unstructured(const lulesh_unstructured_mesh *mesh, int precision, const lulesh_params *params,
                               lulesh_ctx **out)
{
    if (!out || !mesh) return fail(nullptr, LULESH_ERR_ARG, "lulesh_create_unstructured: NULL argument");
    *out = nullptr;
    if (int rc = check_precision(precision, "lulesh_create_unstructured")) return rc;
    HostMesh m;
    std::string err;
    if (m.build_unstructured(*mesh, &err) != LULESH_OK) return fail(nullptr, LULESH_ERR_ARG, err);
    return create_from_mesh(m, precision, params, out);
}

int lulesh_create_lmesh(const char *path, int precision, const lulesh_params *params, lulesh_ctx **out)
{
    if (!out) return fail(nullptr, LULESH_ERR_ARG, "lulesh_create_lmesh: NULL output pointer");
    *out = nullptr;
    if (int rc = check_precision(precision, "lulesh_create_lmesh")) return rc;
    LmeshFile f;
    std::string err;
    if (f.read(path, &err) != LULESH_OK) return fail(nullptr, LULESH_ERR_ARG, err);
    return lulesh_create_unstructured(&f.view, precision, params, out);
}

int lulesh_dump_domain(lulesh_ctx *ctx, const char *basename, int step)
{
    if (!ctx) return LULESH_ERR_ARG;
    const size_t ne = ctx->ne, nn = ctx->nn;
    std::vector<double> node(6 * nn), elem(4 * ne);
    std::vector<int> nodelist(8 * ne);
    const Dom &d = ctx->dom;
    double *const ndst[6] = {d.x, d.y, d.z, d.xd, d.yd, d.zd};
    double *const edst[4] = {d.e, d.p, d.v, d.q};
    for (int i = 0; i < 6; ++i)
        CK(cudaMemcpyAsync(node.data() + i * nn, ndst[i], nn * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    for (int i = 0; i < 4; ++i)
        CK(cudaMemcpyAsync(elem.data() + i * ne, edst[i], ne * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaMemcpyAsync(nodelist.data(), d.nodelist, 8 * ne * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaMemcpyAsync(ctx->h_sc, d.sc, sizeof(DevScalars), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    const double *fields[10] = {node.data(), node.data() + nn, node.data() + 2 * nn, node.data() + 3 * nn,
                                node.data() + 4 * nn, node.data() + 5 * nn, elem.data(), elem.data() + ne,
                                elem.data() + 2 * ne, elem.data() + 3 * ne};
    std::string err;
    const int rc = write_domain_file(basename, ctx->s, (long)ne, (long)nn, nodelist.data(), step, ctx->h_sc->time,
                                     fields, &err);
    return rc ? fail(ctx, rc, "lulesh_dump_domain: " + err) : LULESH_OK;
}

int lulesh_origin_element(lulesh_ctx *ctx, long *elem)
{
    if (!ctx || !elem) return LULESH_ERR_ARG;
    *elem = ctx->origin;
    return LULESH_OK;
}

int lulesh_sizes(lulesh_ctx *ctx, int *s, long *num_elem, long *num_node)
{
    if (!ctx) return LULESH_ERR_ARG;
    if (s) *s = ctx->s;
    if (num_elem) *num_elem = ctx->ne;
    if (num_node) *num_node = ctx->nn;
    return LULESH_OK;
}

void *lulesh_stream(lulesh_ctx *ctx) { return ctx ? (void *)ctx->stream : nullptr; }

long long lulesh_kernel_launches(lulesh_ctx *ctx) { return ctx ? ctx->launches : 0; }

int lulesh_keep_forces(lulesh_ctx *ctx, int keep)
{
    if (!ctx) return LULESH_ERR_ARG;
    ctx->dom.keep = keep ? 3 : 0;
    // the run graph bakes in the kernel arguments: rebuild on next run
    if (ctx->run_exec) { cudaGraphExecDestroy(ctx->run_exec); ctx->run_exec = nullptr; }
    if (ctx->chunk_exec) { cudaGraphExecDestroy(ctx->chunk_exec); ctx->chunk_exec = nullptr; }
    ctx->run_mode = 0;
    return LULESH_OK;
}

int lulesh_set_regions(lulesh_ctx *ctx, int num_regions, int balance, int cost)
{
    if (!ctx) return LULESH_ERR_ARG;
    if (num_regions < 0 || balance < 0 || cost < 0 || cost > 100)
        return fail(ctx, LULESH_ERR_ARG, "lulesh_set_regions: need num_regions >= 0, balance >= 0, 0 <= cost <= 100");
    double weights = 0.0;
    for (int i = 0; i < num_regions; ++i) weights += std::pow(double(i + 1), double(balance));
    if (weights > 2147483647.0) return fail(ctx, LULESH_ERR_ARG, "lulesh_set_regions: region weights overflow int");
    // the run graph bakes in the kernel arguments: rebuild on next run
    if (ctx->run_exec) { cudaGraphExecDestroy(ctx->run_exec); ctx->run_exec = nullptr; }
    if (ctx->chunk_exec) { cudaGraphExecDestroy(ctx->chunk_exec); ctx->chunk_exec = nullptr; }
    ctx->run_mode = 0;
    if (num_regions == 0) {
        ctx->regions.clear();
        ctx->dom.mat_order = nullptr;
        ctx->dom.reps = nullptr;
        return LULESH_OK;
    }
    const long ne = ctx->ne;
    region_numbers(ne, num_regions, balance, ctx->regions);
    std::vector<int> reps(ne), order(ne);
    for (long k = 0; k < ne; ++k) {
        reps[k] = region_reps(ctx->regions[k] - 1, num_regions, cost);
        order[k] = (int)k;
    }
    // costliest elements first, element order within a cost: warps see one
    // repetition count and the longest ones start earliest
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return reps[a] > reps[b]; });
    int rc;
    if (!ctx->d_mat_order && (rc = dalloc(ctx, &ctx->d_mat_order, ne)) != LULESH_OK) return rc;
    if (!ctx->d_reps && (rc = dalloc(ctx, &ctx->d_reps, ne)) != LULESH_OK) return rc;
    CK(cudaMemcpyAsync(ctx->d_mat_order, order.data(), ne * sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(ctx->d_reps, reps.data(), ne * sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    ctx->dom.mat_order = ctx->d_mat_order;
    ctx->dom.reps = ctx->d_reps;
    return LULESH_OK;
}

int lulesh_get_regions(lulesh_ctx *ctx, int *reg_num_list)
{
    if (!ctx || !reg_num_list) return LULESH_ERR_ARG;
    for (long k = 0; k < ctx->ne; ++k) reg_num_list[k] = ctx->regions.empty() ? 1 : ctx->regions[k];
    return LULESH_OK;
}

int lulesh_set_params(lulesh_ctx *ctx, const lulesh_params *params)
{
    if (!ctx || !params) return LULESH_ERR_ARG;
    ctx->dom.prm = *params;
    if (ctx->run_exec) { cudaGraphExecDestroy(ctx->run_exec); ctx->run_exec = nullptr; }
    if (ctx->chunk_exec) { cudaGraphExecDestroy(ctx->chunk_exec); ctx->chunk_exec = nullptr; }
    ctx->run_mode = 0;
    return LULESH_OK;
}

int lulesh_get_params(lulesh_ctx *ctx, lulesh_params *params)
{
    if (!ctx || !params) return LULESH_ERR_ARG;
    *params = ctx->dom.prm;
    return LULESH_OK;
}

int lulesh_upload_domain(lulesh_ctx *ctx, const double *x, const double *y, const double *z,
                         const double *xd, const double *yd, const double *zd, const double *e,
                         const double *p, const double *q, const double *v, const double *ss,
                         double time, double deltatime)
{
    if (!ctx) return LULESH_ERR_ARG;
    Dom &d = ctx->dom;
    int rc;
    const long nn = ctx->nn, ne = ctx->ne;
    if ((rc = upload(ctx, d.x, x, nn)) || (rc = upload(ctx, d.y, y, nn)) || (rc = upload(ctx, d.z, z, nn)) ||
        (rc = upload(ctx, d.xd, xd, nn)) || (rc = upload(ctx, d.yd, yd, nn)) || (rc = upload(ctx, d.zd, zd, nn)) ||
        (rc = upload(ctx, d.e, e, ne)) || (rc = upload(ctx, d.p, p, ne)) || (rc = upload(ctx, d.q, q, ne)) ||
        (rc = upload(ctx, d.v, v, ne)) || (rc = upload(ctx, d.ss, ss, ne)))
        return rc;
    CK(cudaMemcpyAsync(ctx->h_sc, d.sc, sizeof(DevScalars), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    ctx->h_sc->time = time;
    ctx->h_sc->deltatime = deltatime;
    ctx->h_sc->err_any = 0;
    for (int i = 0; i < ERR_NUM; ++i) ctx->h_sc->err[i] = 0;
    ctx->h_sc->geo_valid = 0;   // new positions: the geometry cache is stale
    CK(cudaMemcpyAsync(d.sc, ctx->h_sc, sizeof(DevScalars), cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    ctx->status = LULESH_OK;
    return refresh_split(ctx);
}

int lulesh_download_domain(lulesh_ctx *ctx, double *x, double *y, double *z, double *xd, double *yd,
                           double *zd, double *e, double *p, double *q, double *v, double *ss,
                           double *time, double *deltatime)
{
    if (!ctx) return LULESH_ERR_ARG;
    Dom &d = ctx->dom;
    int rc;
    const long nn = ctx->nn, ne = ctx->ne;
    if ((rc = download(ctx, x, d.x, nn)) || (rc = download(ctx, y, d.y, nn)) || (rc = download(ctx, z, d.z, nn)) ||
        (rc = download(ctx, xd, d.xd, nn)) || (rc = download(ctx, yd, d.yd, nn)) ||
        (rc = download(ctx, zd, d.zd, nn)) || (rc = download(ctx, e, d.e, ne)) ||
        (rc = download(ctx, p, d.p, ne)) || (rc = download(ctx, q, d.q, ne)) ||
        (rc = download(ctx, v, d.v, ne)) || (rc = download(ctx, ss, d.ss, ne)))
        return rc;
    CK(cudaMemcpyAsync(ctx->h_sc, d.sc, sizeof(DevScalars), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    if (time) *time = ctx->h_sc->time;
    if (deltatime) *deltatime = ctx->h_sc->deltatime;
    return LULESH_OK;
}

int lulesh_get_scalars(lulesh_ctx *ctx, lulesh_scalars *out)
{
    if (!ctx || !out) return LULESH_ERR_ARG;
    CK(cudaMemcpyAsync(ctx->h_sc, ctx->dom.sc, sizeof(DevScalars), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    out->time = ctx->h_sc->time;
    out->deltatime = ctx->h_sc->deltatime;
    out->dtcourant = ctx->h_sc->dtcourant;
    out->dthydro = ctx->h_sc->dthydro;
    out->cycle = ctx->h_sc->cycle;
    return LULESH_OK;
}

int lulesh_set_scalars(lulesh_ctx *ctx, const lulesh_scalars *in)
{
    if (!ctx || !in) return LULESH_ERR_ARG;
    CK(cudaMemcpyAsync(ctx->h_sc, ctx->dom.sc, sizeof(DevScalars), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    DevScalars *h = ctx->h_sc;
    h->time = in->time;
    h->deltatime = in->deltatime;
    h->dtcourant = in->dtcourant;
    h->dthydro = in->dthydro;
    h->cycle = in->cycle;
    h->err_any = 0;
    for (int i = 0; i < ERR_NUM; ++i) h->err[i] = 0;
    h->courant_key = ~0ULL;
    h->hydro_key = ~0ULL;
    CK(cudaMemcpyAsync(ctx->dom.sc, h, sizeof(DevScalars), cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    ctx->status = LULESH_OK;
    return LULESH_OK;
}

int lulesh_get_field(lulesh_ctx *ctx, const char *name, double *host, long n)
{
    if (!ctx || !name || !host) return LULESH_ERR_ARG;
    bool node = false, writable = false;
    double *f = find_field(ctx, name, &node, &writable);
    if (!f) return fail(ctx, LULESH_ERR_ARG, std::string("unknown field ") + name);
    if (n != (node ? ctx->nn : ctx->ne)) return fail(ctx, LULESH_ERR_ARG, std::string("wrong length for field ") + name);
    if (is_split(ctx)) {
        // the split path keeps the monotonic-Q gradients in FP32
        static const char *gnames[6] = {"delv_xi", "delv_eta", "delv_zeta", "delx_xi", "delx_eta", "delx_zeta"};
        for (int g = 0; g < 6; ++g)
            if (!strcmp(name, gnames[g])) {
                std::vector<float> tmp((size_t)n);
                CK(cudaMemcpyAsync(tmp.data(), ctx->dom.gq + (size_t)g * ctx->ne, n * sizeof(float),
                                   cudaMemcpyDeviceToHost, ctx->stream));
                CK(cudaStreamSynchronize(ctx->stream));
                for (long i = 0; i < n; ++i) host[i] = tmp[(size_t)i];
                return LULESH_OK;
            }
    }
    CK(cudaMemcpyAsync(host, f, n * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return LULESH_OK;
}

int lulesh_set_field(lulesh_ctx *ctx, const char *name, const double *host, long n)
{
    if (!ctx || !name || !host) return LULESH_ERR_ARG;
    bool node = false, writable = false;
    double *f = find_field(ctx, name, &node, &writable);
    if (!f) return fail(ctx, LULESH_ERR_ARG, std::string("unknown field ") + name);
    if (n != (node ? ctx->nn : ctx->ne)) return fail(ctx, LULESH_ERR_ARG, std::string("wrong length for field ") + name);
    CK(cudaMemcpyAsync(f, host, n * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    int rc = clear_errors(ctx);
    return rc ? rc : refresh_split(ctx);
}

int lulesh_time_increment(lulesh_ctx *ctx)
{
    if (!ctx) return LULESH_ERR_ARG;
    if (ctx->status) return ctx->status;
    launch_time_increment(ctx->dom, ctx->stream);
    ctx->launches += 1;
    // TimeIncrement has no error exit of its own and every other call reads
    // the status when it returns, so this one does not wait for the GPU
    return check_launch(ctx);
}

int lulesh_lagrange_nodal(lulesh_ctx *ctx)
{
    if (!ctx) return LULESH_ERR_ARG;
    if (ctx->status) return ctx->status;
    nodal(ctx, ctx->dom);
    ctx->launches += 2;
    int rc = check_launch(ctx);
    return rc ? rc : read_status(ctx);
}

int lulesh_lagrange_elements(lulesh_ctx *ctx)
{
    if (!ctx) return LULESH_ERR_ARG;
    if (ctx->status) return ctx->status;
    elements(ctx, ctx->dom, false);
    ctx->launches += 2;
    int rc = check_launch(ctx);
    return rc ? rc : read_status(ctx);
}

int lulesh_calc_time_constraints(lulesh_ctx *ctx)
{
    if (!ctx) return LULESH_ERR_ARG;
    if (ctx->status) return ctx->status;
    launch_time_constraints(ctx->dom, ctx->stream);
    ctx->launches += 2;
    int rc = check_launch(ctx);
    return rc ? rc : read_status(ctx);
}

int lulesh_lagrange_leapfrog(lulesh_ctx *ctx)
{
    if (!ctx) return LULESH_ERR_ARG;
    if (ctx->status) return ctx->status;
    nodal(ctx, ctx->dom);
    elements(ctx, ctx->dom, true);
    launch_finalize(ctx->dom, ctx->stream);
    ctx->launches += 5;
    int rc = check_launch(ctx);
    return rc ? rc : read_status(ctx);
}

int lulesh_run(lulesh_ctx *ctx, int max_cycles, int *cycles_done)
{
    if (!ctx) return LULESH_ERR_ARG;
    if (cycles_done) *cycles_done = 0;
    if (ctx->status) return ctx->status;
    int rc = build_run_graph(ctx);
    if (rc) return rc;
    ctx->h_stage[0] = max_cycles;
    CK(cudaMemcpyAsync(ctx->d_max_cycles, ctx->h_stage, sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
    if (ctx->run_mode == 1) {
        CK(cudaGraphLaunch(ctx->run_exec, ctx->stream));
    } else {
        launch_run_prologue(ctx->dom, ctx->stream, ctx->d_max_cycles, 0, ctx->d_active);
        if ((rc = check_launch(ctx))) return rc;
        for (;;) {
            CK(cudaGraphLaunch(ctx->chunk_exec, ctx->stream));
            CK(cudaMemcpyAsync(ctx->h_stage + 1, ctx->d_active, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
            CK(cudaStreamSynchronize(ctx->stream));
            if (!ctx->h_stage[1]) break;
        }
    }
    rc = read_status(ctx);
    const int done = ctx->h_sc->run_cycles;
    if (cycles_done) *cycles_done = done;
    ctx->launches += 1 + (long long)done * kernels_per_cycle();
    return rc ? rc : short_of_stoptime(ctx, max_cycles, done);
}

int lulesh_run_profiled(lulesh_ctx *ctx, int max_cycles, int *cycles_done, double *kernel_ms)
{
    if (!ctx) return LULESH_ERR_ARG;
    if (cycles_done) *cycles_done = 0;
    if (kernel_ms)
        for (int i = 0; i < kTimedKernels; ++i) kernel_ms[i] = 0.0;
    if (ctx->status) return ctx->status;
    cudaEvent_t ev[kTimedKernels + 1];
    for (auto &e : ev) CK(cudaEventCreate(&e));
    const int cap = (max_cycles > 0 && max_cycles < kRunCycleLimit) ? max_cycles : kRunCycleLimit;
    int done = 0, rc = LULESH_OK;
    Dom d = ctx->dom;
    d.gate = nullptr;
    for (;;) {
        if ((rc = read_status(ctx))) break;
        const DevScalars *h = ctx->h_sc;
        if (!(h->time < d.prm.stoptime) || !(h->deltatime > 0.0) || done >= cap) break;
        if (is_split(ctx)) launch_cycle_timed_split(d, ctx->stream, ev);
        else launch_cycle_timed(d, ctx->stream, ev);
        if ((rc = check_launch(ctx))) break;
        CK(cudaEventSynchronize(ev[kTimedKernels]));
        for (int i = 0; i < kTimedKernels && kernel_ms; ++i) {
            float ms = 0.f;
            CK(cudaEventElapsedTime(&ms, ev[i], ev[i + 1]));
            kernel_ms[i] += ms;
        }
        ++done;
        ctx->launches += kTimedKernels;
    }
    for (auto &e : ev) cudaEventDestroy(e);
    if (!rc) rc = read_status(ctx);
    if (cycles_done) *cycles_done = done;
    return rc ? rc : short_of_stoptime(ctx, max_cycles, done);
}

int lulesh_probe_fp64_peak(double *tflops)
{
    lulesh_ctx *ctx = nullptr;
    if (!tflops) return LULESH_ERR_ARG;
    int dev = 0, sms = 0;
    CK(cudaGetDevice(&dev));
    CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    double *out = nullptr;
    CK(cudaMalloc(&out, sizeof(double)));
    cudaStream_t st;
    CK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    cudaEvent_t a, b;
    CK(cudaEventCreate(&a));
    CK(cudaEventCreate(&b));
    const int threads = 256, blocks = sms * 8, iters = 4096;
    launch_fp64_probe(out, blocks, threads, iters, st);   // warm-up
    CK(cudaEventRecord(a, st));
    launch_fp64_probe(out, blocks, threads, iters, st);
    CK(cudaEventRecord(b, st));
    CK(cudaEventSynchronize(b));
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, a, b));
    *tflops = 2.0 * 8.0 * (double)iters * threads * blocks / (ms * 1e-3) * 1e-12;
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaStreamDestroy(st);
    cudaFree(out);
    return LULESH_OK;
}

int lulesh_probe_math(double errs[4])
{
    if (!errs) return LULESH_ERR_ARG;
    unsigned long long *keys = nullptr, h[4] = {0, 0, 0, 0};
    cudaStream_t st = nullptr;
    const int n = 1 << 20;
    if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess ||
        cudaMalloc(&keys, sizeof h) != cudaSuccess) {
        if (st) cudaStreamDestroy(st);
        return fail(nullptr, LULESH_ERR_CUDA, "lulesh_probe_math: no usable CUDA device");
    }
    cudaError_t e = cudaMemsetAsync(keys, 0, sizeof h, st);
    if (e == cudaSuccess) {
        launch_math_probe(keys, n, st);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(h, keys, sizeof h, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaFree(keys);
    cudaStreamDestroy(st);
    if (e != cudaSuccess) return fail(nullptr, LULESH_ERR_CUDA, std::string("lulesh_probe_math: ") + cudaGetErrorString(e));
    for (int i = 0; i < 4; ++i) std::memcpy(&errs[i], &h[i], sizeof(double));
    return LULESH_OK;
}

int lulesh_probe_pipe_rates(double *rates)
{
    lulesh_ctx *ctx = nullptr;
    if (!rates) return LULESH_ERR_ARG;
    int dev = 0, sms = 0, clk_khz = 0;
    CK(cudaGetDevice(&dev));
    CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    CK(cudaDeviceGetAttribute(&clk_khz, cudaDevAttrClockRate, dev));
    const int threads = 256, blocks = sms * 8;
    float *out = nullptr;
    CK(cudaMalloc(&out, sizeof(float) * threads * blocks));
    double *dout = nullptr;
    CK(cudaMalloc(&dout, sizeof(double)));
    cudaStream_t st;
    CK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    cudaEvent_t a, b;
    CK(cudaEventCreate(&a));
    CK(cudaEventCreate(&b));
    // ops per thread of each probe: FFMA, DFMA, D2F (+DADD), DDIV
    const int iters[4] = {4096, 1024, 1024, 64};
    const double ops[4] = {8.0 * 4096, 8.0 * 1024, 8.0 * 1024, 4.0 * 64};
    for (int w = 0; w < 4; ++w) {
        for (int rep = 0; rep < 2; ++rep) {     // the first launch warms up
            CK(cudaEventRecord(a, st));
            if (w == 1) launch_fp64_probe(dout, blocks, threads, iters[w], st);
            else launch_rate_probe(w == 0 ? 0 : (w == 2 ? 1 : 2), out, blocks, threads, iters[w], st);
            CK(cudaEventRecord(b, st));
        }
        CK(cudaEventSynchronize(b));
        float ms = 0.f;
        CK(cudaEventElapsedTime(&ms, a, b));
        // operations per SM per clock at the nominal maximum clock
        rates[w] = ops[w] * threads * blocks / (ms * 1e-3) / ((double)clk_khz * 1e3) / sms;
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaStreamDestroy(st);
    cudaFree(out);
    cudaFree(dout);
    return LULESH_OK;
}

int lulesh_origin_energy(lulesh_ctx *ctx, double *e0)
{
    if (!ctx || !e0) return LULESH_ERR_ARG;
    CK(cudaMemcpyAsync(ctx->h_sc, ctx->dom.e + ctx->origin, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    memcpy(e0, ctx->h_sc, sizeof(double));
    return LULESH_OK;
}

int lulesh_symmetry(lulesh_ctx *ctx, double *max_abs_diff, double *total_abs_diff, double *max_rel_diff)
{
    if (!ctx) return LULESH_ERR_ARG;
    const int s = ctx->s;
    if (s < 1) return fail(ctx, LULESH_ERR_ARG, "lulesh_symmetry: the plane-0 test needs the cube mesh");
    std::vector<double> plane((size_t)s * s);
    CK(cudaMemcpyAsync(plane.data(), ctx->dom.e, plane.size() * sizeof(double), cudaMemcpyDeviceToHost,
                       ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    double ma = 0.0, ta = 0.0, mr = 0.0;
    for (int j = 0; j < s; ++j)
        for (int k = j + 1; k < s; ++k) {
            const double a = std::fabs(plane[(size_t)j * s + k] - plane[(size_t)k * s + j]);
            ta += a;
            if (ma < a) ma = a;
            const double r = a / plane[(size_t)k * s + j];
            if (mr < r) mr = r;
        }
    if (max_abs_diff) *max_abs_diff = ma;
    if (total_abs_diff) *total_abs_diff = ta;
    if (max_rel_diff) *max_rel_diff = mr;
    return LULESH_OK;
}

}  // extern "C"
