// batch.cu -- batched ensembles: many independent Sedov instances of uneven
// size advanced together, each with its own time, time step and stop time.
//
// Layout.  The instances' nodes and elements are concatenated into flat
// arrays; every instance's range starts on a multiple of kTile, so a tile of
// kTile elements (or nodes) belongs to one instance.  Connectivity is
// rewritten to global indices at upload (nodelist, face neighbours, the
// node-to-corner slots corner*E_total + element), so the per-element and
// per-node bodies of the single-instance step run unchanged; only the scalar
// block they read and write (time step, error words, constraint minima) is
// the instance's own.
//
// Execution.  One cycle is: a per-instance TimeIncrement; the four step
// kernels, each a persistent kernel per size class walking that class's list
// of active tiles (each class's chain of four is one parallel graph branch);
// a per-instance epilogue that publishes the constraint minima, counts the
// cycle and retires instances that reached their stop time; and a compaction
// of the active-tile lists when an instance retired.  The whole run is one
// CUDA graph with a conditional WHILE node that loops while any instance is
// active -- no host synchronisation per cycle.
//
// Launch shapes (threads per block = kTile / elements per thread, resident
// blocks per SM of the persistent grid, and for the split force kernel of a
// class of structured cubes the staging depth: gathered corners, or tiles of
// two or four element rows staged in shared memory) are chosen per size
// class and kernel by lulesh_batch_autotune, which times the candidates on
// the batch itself, restores its state, and caches the choice per GPU model.
#include "lulesh_internal.h"
#include "kernels.h"
#include "common.cuh"
#include "tile.cuh"

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

using namespace lulesh;

struct lulesh_batch {
    int n = 0;
    int precision = LULESH_PRECISION_FP64;
    std::vector<int> s;
    std::vector<long> eoff, noff, ne_i, nn_i;
    long ne_tot = 0, nn_tot = 0;
    std::vector<int> inst_class;
    int class_etiles[kMaxClasses] = {0, 0, 0};
    int class_ntiles[kMaxClasses] = {0, 0, 0};
    LaunchCfg cfg[kMaxClasses][kBatchKernels];
    // staged tiles of the split force kernel, per class, for tiles of 2 and
    // of 4 element rows (n == 0: the class cannot be staged)
    StagedClass staged[kMaxClasses][2] = {};
    int sms = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t side[kMaxClasses] = {nullptr, nullptr, nullptr};
    cudaEvent_t ev_fork = nullptr, ev_join[kMaxClasses] = {nullptr, nullptr, nullptr};
    Dom dom{};
    BatchView bv{};
    std::vector<void *> allocs;
    int *d_max = nullptr;
    int *h_stage = nullptr;
    DevScalars *h_sc = nullptr;     // pinned, n entries
    cudaGraphExec_t run_exec = nullptr;
    long long launches = 0;
    int kernels_per_cycle = 0;
    bool tuned = false;
    double last_zc = 0.0;   // elements x cycles of the last run call
    std::string err;
};

namespace lulesh {
namespace {

thread_local std::string g_batch_err;

int bfail(lulesh_batch *b, int code, const std::string &msg)
{
    if (b) b->err = msg;
    else g_batch_err = msg;
    return code;
}

#define BCK(call)                                                                           \
    do {                                                                                    \
        cudaError_t e_ = (call);                                                            \
        if (e_ != cudaSuccess)                                                              \
            return bfail(b, LULESH_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

template <typename T>
int balloc(lulesh_batch *b, T **p, size_t n)
{
    void *q = nullptr;
    cudaError_t e = cudaMalloc(&q, (n ? n : 1) * sizeof(T));
    if (e != cudaSuccess) return bfail(b, LULESH_ERR_CUDA, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    b->allocs.push_back(q);
    *p = static_cast<T *>(q);
    return LULESH_OK;
}

// Size class of an instance by edge length.  Split-precision batches use
// three classes, whose chains of four kernels run as parallel graph
// branches: their kernels lean on different units (the force kernel on FP32
// issue and latency, kinematics on FP64, the node update on HBM), and
// overlapping one class's force with another's kinematics ran the 528-
// instance split ensemble 2.8 % faster than one chain.  In plain FP64 every
// kernel is bound by the FP64 pipe, so there is nothing to overlap: FP64
// batches keep all instances in one class (one chain of persistent kernels
// over every running instance's tiles), which ran the 64-instance FP64
// ensemble 2.4 % faster than three classes, whose persistent grids crowded
// one another once the small instances had retired.
int size_class(int s, int precision)
{
    if (precision != LULESH_PRECISION_SPLIT) return 0;
    return s <= 24 ? 0 : (s <= 48 ? 1 : 2);
}

long round_tile(long n) { return (n + kTile - 1) / kTile * kTile; }

// ---- control kernels ---------------------------------------------------

__global__ void kb_geo_invalidate(DevScalars *sc, int n)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) sc[i].geo_valid = 0;
}

__global__ void kb_time_increment(const __grid_constant__ Dom d, const __grid_constant__ BatchView b)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= b.n_inst || !b.inst_active[i]) return;
    DevScalars *sc = d.sc + i;
    if (sc->err_any) return;
    time_increment(sc, d.prm);
}

// One block: reset the per-instance run counters, decide which instances
// run at all, ask for a full rebuild of the active-tile lists.
__global__ void kb_prologue(const __grid_constant__ Dom d, const __grid_constant__ BatchView b,
                            const int *max_cycles, cudaGraphConditionalHandle h)
{
    __shared__ int any;
    if (threadIdx.x == 0) any = 0;
    __syncthreads();
    for (int i = threadIdx.x; i < b.n_inst; i += blockDim.x) {
        DevScalars *sc = d.sc + i;
        sc->run_cycles = 0;
        sc->run_max = *max_cycles;
        const unsigned go = run_continue(sc, d.prm);
        b.inst_active[i] = (unsigned char)go;
        if (go) any = 1;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int c = 0; c < 2 * kMaxClasses; ++c) b.counts[c] = 0;
        b.counts[2 * kMaxClasses] = 1;
        b.counts[2 * kMaxClasses + 1] = any;
        if (h) cudaGraphSetConditional(h, any);
    }
}

// One block: publish each running instance's constraint minima, count its
// cycle, retire it when it reached its stop time (or failed), and set the
// loop condition.
__global__ void kb_epilogue(const __grid_constant__ Dom d, const __grid_constant__ BatchView b,
                            cudaGraphConditionalHandle h)
{
    __shared__ int any, changed;
    if (threadIdx.x == 0) {
        any = 0;
        changed = 0;
    }
    __syncthreads();
    for (int i = threadIdx.x; i < b.n_inst; i += blockDim.x) {
        if (!b.inst_active[i]) continue;
        DevScalars *sc = d.sc + i;
        finalize_constraints(sc);
        sc->run_cycles++;
        if (run_continue(sc, d.prm)) {
            any = 1;
        } else {
            b.inst_active[i] = 0;
            changed = 1;
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        if (changed)
            for (int c = 0; c < 2 * kMaxClasses; ++c) b.counts[c] = 0;
        b.counts[2 * kMaxClasses] = changed;
        b.counts[2 * kMaxClasses + 1] = any;
        if (h) cudaGraphSetConditional(h, any);
    }
}

// Rebuild the active-tile lists (only after an instance retired).  The
// order inside a list does not matter: every tile's work is independent and
// the constraint reduction is an order-free minimum.
__global__ void kb_compact(const __grid_constant__ BatchView b)
{
    if (!b.counts[2 * kMaxClasses]) return;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < b.n_etiles && b.inst_active[b.etile_inst[t]]) {
        const int c = b.etile_class[t];
        const int slot = atomicAdd(&b.counts[c], 1);
        b.active_etiles[b.eclass_off[c] + slot] = t;
    }
    if (t < b.n_ntiles && b.inst_active[b.ntile_inst[t]]) {
        const int c = b.ntile_class[t];
        const int slot = atomicAdd(&b.counts[kMaxClasses + c], 1);
        b.active_ntiles[b.nclass_off[c] + slot] = t;
    }
}

// ---- host helpers ------------------------------------------------------

// Staging depths of the split force kernel (element rows per staged tile).
const int kStageRows[2] = {2, 4};
int stage_index(int rows) { return rows == 4 ? 1 : 0; }
bool can_stage(const lulesh_batch *b, int cls)
{
    return b->precision == LULESH_PRECISION_SPLIT && b->staged[cls][0].n > 0;
}

void launch_kernel(lulesh_batch *b, int kernel, int cls, cudaStream_t st)
{
    const LaunchCfg cfg = b->cfg[cls][kernel];
    if (b->precision == LULESH_PRECISION_SPLIT && kernel == 0 && cfg.stage > 0 && can_stage(b, cls))
        launch_batch_force_split_staged(b->dom, b->bv, b->staged[cls][stage_index(cfg.stage)], cfg.stage, cfg, st);
    else if (b->precision == LULESH_PRECISION_SPLIT) launch_batch_kernel_split(b->dom, b->bv, st, kernel, cls, cfg);
    else launch_batch_kernel_fp64(b->dom, b->bv, st, kernel, cls, cfg);
}

// Staged tiles of the split force kernel over all of a class's instances.
long long staged_tiles(const lulesh_batch *b, int cls, int rows)
{
    long long t = 0;
    for (int i = 0; i < b->n; ++i)
        if (b->inst_class[i] == cls) t += rows == 4 ? TileShape<4>::tiles(b->s[i]) : TileShape<2>::tiles(b->s[i]);
    return t;
}

int max_blocks(lulesh_batch *b, int kernel, int block)
{
    return b->precision == LULESH_PRECISION_SPLIT ? batch_max_blocks_split(kernel, block)
                                                  : batch_max_blocks_fp64(kernel, block, b->dom.df);
}

unsigned compact_blocks(const lulesh_batch *b)
{
    const long t = std::max(b->bv.n_etiles, b->bv.n_ntiles);
    return (unsigned)((t + 255) / 256);
}

// One cycle on b->stream; each size class runs its four kernels as one
// parallel branch (fork/join through events, which stream capture turns into
// graph edges).
void launch_cycle(lulesh_batch *b, cudaGraphConditionalHandle h)
{
    cudaStream_t st = b->stream;
    kb_time_increment<<<(b->n + 127) / 128, 128, 0, st>>>(b->dom, b->bv);
    // Instances never interact, so each size class runs its whole chain of
    // four phases on its own branch: a class that finishes a phase goes on
    // to its next one while the others are still busy, instead of waiting
    // at a join after every phase.  The branches join before the epilogue.
    int first = -1;
    for (int c = 0; c < kMaxClasses; ++c)
        if (b->class_etiles[c] > 0 || b->class_ntiles[c] > 0) {
            first = c;
            break;
        }
    cudaEventRecord(b->ev_fork, st);
    for (int c = 0; c < kMaxClasses; ++c) {
        if (b->class_etiles[c] == 0 && b->class_ntiles[c] == 0) continue;
        cudaStream_t sc = c == first ? st : b->side[c];
        if (c != first) cudaStreamWaitEvent(sc, b->ev_fork, 0);
        for (int k = 0; k < kBatchKernels; ++k)
            if ((k == 1 ? b->class_ntiles[c] : b->class_etiles[c]) > 0) launch_kernel(b, k, c, sc);
        if (c != first) {
            cudaEventRecord(b->ev_join[c], sc);
            cudaStreamWaitEvent(st, b->ev_join[c], 0);
        }
    }
    kb_epilogue<<<1, 1024, 0, st>>>(b->dom, b->bv, h);
    kb_compact<<<compact_blocks(b), 256, 0, st>>>(b->bv);
}

int count_kernels_per_cycle(const lulesh_batch *b)
{
    int n = 3;   // time increment, epilogue, compaction
    for (int k = 0; k < kBatchKernels; ++k)
        for (int c = 0; c < kMaxClasses; ++c) n += (k == 1 ? b->class_ntiles[c] : b->class_etiles[c]) > 0;
    return n;
}

void destroy_graph(lulesh_batch *b)
{
    if (b->run_exec) cudaGraphExecDestroy(b->run_exec);
    b->run_exec = nullptr;
}

int build_graph(lulesh_batch *b)
{
    if (b->run_exec) return LULESH_OK;
    cudaGraph_t g = nullptr;
    cudaGraphConditionalHandle h = 0;
    BCK(cudaGraphCreate(&g, 0));
    cudaError_t e = cudaGraphConditionalHandleCreate(&h, g, 0, 0);
    if (e == cudaSuccess) e = cudaStreamBeginCaptureToGraph(b->stream, g, nullptr, nullptr, 0,
                                                             cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
        kb_prologue<<<1, 1024, 0, b->stream>>>(b->dom, b->bv, b->d_max, h);
        kb_compact<<<compact_blocks(b), 256, 0, b->stream>>>(b->bv);
        e = cudaStreamEndCapture(b->stream, &g);
    }
    // the last node of the prologue part is the compaction
    cudaGraphNode_t tail = nullptr;
    if (e == cudaSuccess) {
        size_t nn = 0;
        e = cudaGraphGetNodes(g, nullptr, &nn);
        std::vector<cudaGraphNode_t> nodes(nn);
        if (e == cudaSuccess) e = cudaGraphGetNodes(g, nodes.data(), &nn);
        for (size_t i = 0; e == cudaSuccess && i < nn; ++i) {
            size_t ndep = 0;
            e = cudaGraphNodeGetDependentNodes(nodes[i], nullptr, nullptr, &ndep);
            if (e == cudaSuccess && ndep == 0) tail = nodes[i];
        }
    }
    cudaGraphNodeParams cp = {cudaGraphNodeTypeConditional};
    cp.conditional.handle = h;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t cnode = nullptr;
    if (e == cudaSuccess && tail) e = cudaGraphAddNode(&cnode, g, &tail, nullptr, 1, &cp);
    if (e == cudaSuccess) {
        cudaGraph_t body = cp.conditional.phGraph_out[0];
        e = cudaStreamBeginCaptureToGraph(b->stream, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess) {
            launch_cycle(b, h);
            cudaGraph_t out = nullptr;
            e = cudaStreamEndCapture(b->stream, &out);
        }
    }
    if (e == cudaSuccess) e = cudaGraphInstantiate(&b->run_exec, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return bfail(b, LULESH_ERR_CUDA, std::string("batch run graph: ") + cudaGetErrorString(e));
    }
    b->kernels_per_cycle = count_kernels_per_cycle(b);
    return LULESH_OK;
}

void default_cfg(lulesh_batch *b)
{
    for (int c = 0; c < kMaxClasses; ++c)
        for (int k = 0; k < kBatchKernels; ++k) {
            const int tiles = k == 1 ? b->class_ntiles[c] : b->class_etiles[c];
            const int per_sm = std::max(1, max_blocks(b, k, 128));
            b->cfg[c][k] = {128, std::max(1, std::min(tiles, b->sms * per_sm))};
        }
}

const char *kKernelNames[kBatchKernels] = {"elem_force", "node_update", "elem_kinematics", "elem_material"};

std::string tune_key(const lulesh_batch *b, int cls, int kernel)
{
    cudaDeviceProp prop;
    int dev = 0;
    cudaGetDevice(&dev);
    cudaGetDeviceProperties(&prop, dev);
    std::ostringstream o;
    o << prop.name << "|sm" << prop.multiProcessorCount << "|"
      << (b->precision == LULESH_PRECISION_SPLIT ? "split" : (b->dom.df == kArithDF64 ? "fp64" : "fp64ieee")) << "|class" << cls << "|"
      << kKernelNames[kernel];
    return o.str();
}

// The cache is a flat JSON object {"key": [block, blocks_per_sm, stage], ...}
// (stage: element rows per staged tile, 0 for gathered corners; entries
// without it read as 0).
struct TuneEntry {
    int block, per_sm, stage;
};
std::map<std::string, TuneEntry> read_cache(const char *path)
{
    std::map<std::string, TuneEntry> m;
    std::ifstream f(path);
    if (!f) return m;
    std::stringstream ss;
    ss << f.rdbuf();
    const std::string t = ss.str();
    size_t p = 0;
    while ((p = t.find('"', p)) != std::string::npos) {
        const size_t q = t.find('"', p + 1);
        if (q == std::string::npos) break;
        const std::string key = t.substr(p + 1, q - p - 1);
        const size_t lb = t.find('[', q), rb = t.find(']', q);
        if (lb == std::string::npos || rb == std::string::npos) break;
        int a = 0, c = 0, st = 0;
        const int got = sscanf(t.c_str() + lb + 1, "%d , %d , %d", &a, &c, &st);
        if (got >= 2) m[key] = {a, c, got == 3 ? st : 0};
        p = rb + 1;
    }
    return m;
}

void write_cache(const char *path, const std::map<std::string, TuneEntry> &m)
{
    std::ofstream f(path);
    f << "{\n";
    size_t i = 0;
    for (const auto &kv : m)
        f << "  \"" << kv.first << "\": [" << kv.second.block << ", " << kv.second.per_sm << ", "
          << kv.second.stage << "]" << (++i < m.size() ? ",\n" : "\n");
    f << "}\n";
}

}  // namespace
}  // namespace lulesh

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
extern "C" {

const char *lulesh_batch_last_error(const lulesh_batch *b) { return b ? b->err.c_str() : g_batch_err.c_str(); }

void lulesh_batch_destroy(lulesh_batch *b)
{
    if (!b) return;
    if (b->stream) cudaStreamSynchronize(b->stream);
    destroy_graph(b);
    for (void *p : b->allocs) cudaFree(p);
    for (int c = 0; c < kMaxClasses; ++c) {
        if (b->side[c]) cudaStreamDestroy(b->side[c]);
        if (b->ev_join[c]) cudaEventDestroy(b->ev_join[c]);
    }
    if (b->ev_fork) cudaEventDestroy(b->ev_fork);
    if (b->h_sc) cudaFreeHost(b->h_sc);
    if (b->h_stage) cudaFreeHost(b->h_stage);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
}

int lulesh_batch_create(int n, const int *sizes, const double *e0_scale, int init_mode, int precision,
                        const lulesh_params *params, lulesh_batch **out)
{
    if (!out || n < 1 || !sizes) return bfail(nullptr, LULESH_ERR_ARG, "lulesh_batch_create: bad arguments");
    if (init_mode != LULESH_INIT_V1 && init_mode != LULESH_INIT_V2)
        return bfail(nullptr, LULESH_ERR_ARG, "lulesh_batch_create: bad init_mode");
    if (precision != LULESH_PRECISION_FP64 && precision != LULESH_PRECISION_SPLIT &&
        precision != LULESH_PRECISION_FP64_IEEE)
        return bfail(nullptr, LULESH_ERR_ARG, "lulesh_batch_create: bad precision");
    long ne_sum = 0;
    for (int i = 0; i < n; ++i) {
        if (sizes[i] < 1 || sizes[i] > kMaxEdge) return bfail(nullptr, LULESH_ERR_ARG, "lulesh_batch_create: bad size");
        if (e0_scale && !(e0_scale[i] > 0.0)) return bfail(nullptr, LULESH_ERR_ARG, "lulesh_batch_create: e0 scale must be > 0");
        ne_sum += round_tile((long)sizes[i] * sizes[i] * sizes[i]);
    }
    if (8 * ne_sum >= (1L << 31)) return bfail(nullptr, LULESH_ERR_ARG, "lulesh_batch_create: ensemble too large for 32-bit corner indices");
    *out = nullptr;
    lulesh_batch *b = new lulesh_batch;
    auto bail = [&](int code) { g_batch_err = b->err; lulesh_batch_destroy(b); return code; };
    b->n = n;
    b->precision = precision;
    b->s.assign(sizes, sizes + n);

    // offsets and tiles
    b->eoff.resize(n); b->noff.resize(n); b->ne_i.resize(n); b->nn_i.resize(n); b->inst_class.resize(n);
    long eo = 0, no = 0;
    for (int i = 0; i < n; ++i) {
        const long s = sizes[i];
        b->ne_i[i] = s * s * s;
        b->nn_i[i] = (s + 1) * (s + 1) * (s + 1);
        b->eoff[i] = eo;
        b->noff[i] = no;
        eo += round_tile(b->ne_i[i]);
        no += round_tile(b->nn_i[i]);
        b->inst_class[i] = size_class(sizes[i], precision);
    }
    b->ne_tot = eo;
    b->nn_tot = no;
    const long net = eo / kTile, nnt = no / kTile;
    std::vector<int> etile_inst(net), ntile_inst(nnt), etile_class(net), ntile_class(nnt);
    for (int i = 0; i < n; ++i) {
        for (long t = b->eoff[i] / kTile; t < (b->eoff[i] + round_tile(b->ne_i[i])) / kTile; ++t) {
            etile_inst[t] = i;
            etile_class[t] = b->inst_class[i];
            b->class_etiles[b->inst_class[i]]++;
        }
        for (long t = b->noff[i] / kTile; t < (b->noff[i] + round_tile(b->nn_i[i])) / kTile; ++t) {
            ntile_inst[t] = i;
            ntile_class[t] = b->inst_class[i];
            b->class_ntiles[b->inst_class[i]]++;
        }
    }
    int eclass_off[kMaxClasses], nclass_off[kMaxClasses];
    for (int c = 0, ea = 0, na = 0; c < kMaxClasses; ++c) {
        eclass_off[c] = ea;
        nclass_off[c] = na;
        ea += b->class_etiles[c];
        na += b->class_ntiles[c];
    }

    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
        cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess) {
        b->err = std::string("no usable CUDA device: ") + cudaGetErrorString(cudaGetLastError());
        return bail(LULESH_ERR_CUDA);
    }
    for (int c = 0; c < kMaxClasses; ++c)
        if (cudaStreamCreateWithFlags(&b->side[c], cudaStreamNonBlocking) != cudaSuccess ||
            cudaEventCreateWithFlags(&b->ev_join[c], cudaEventDisableTiming) != cudaSuccess) {
            b->err = "stream/event creation failed";
            return bail(LULESH_ERR_CUDA);
        }
    if (cudaEventCreateWithFlags(&b->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaMallocHost(&b->h_sc, sizeof(DevScalars) * n) != cudaSuccess ||
        cudaMallocHost(&b->h_stage, 16 * sizeof(int)) != cudaSuccess) {
        b->err = "event / pinned allocation failed";
        return bail(LULESH_ERR_CUDA);
    }

    Dom &d = b->dom;
    d.s = 0;
    d.ne = (int)b->ne_tot;
    d.nn = (int)b->nn_tot;
    d.keep = 0;
    if (params) d.prm = *params;
    else default_params(&d.prm);
    const size_t ne = b->ne_tot, nn = b->nn_tot;
    int rc;
    int *nodelist, *cstart, *clist, *lxim, *lxip, *letam, *letap, *lzetam, *lzetap, *ebc;
    unsigned char *nbc;
    double *volo, *emass, *nmass;
#define A(p, cnt) if ((rc = balloc(b, &(p), (cnt))) != LULESH_OK) return bail(rc)
    A(nodelist, 8 * ne); A(cstart, nn + 1); A(clist, 8 * ne); A(nbc, nn);
    A(lxim, ne); A(lxip, ne); A(letam, ne); A(letap, ne); A(lzetam, ne); A(lzetap, ne); A(ebc, ne);
    A(volo, ne); A(emass, ne); A(nmass, nn);
    A(d.x, nn); A(d.y, nn); A(d.z, nn); A(d.xd, nn); A(d.yd, nn); A(d.zd, nn);
    A(d.e, ne); A(d.p, ne); A(d.q, ne); A(d.v, ne); A(d.ss, ne);
    A(d.vnew, ne); A(d.delv, ne); A(d.vdov, ne); A(d.arealg, ne);
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
    A(d.sc, (size_t)n); A(b->d_max, 1);
    int *etile_inst_d, *ntile_inst_d, *etile_class_d, *ntile_class_d, *iee, *ine, *eco, *nco;
    A(etile_inst_d, net); A(ntile_inst_d, nnt); A(etile_class_d, net); A(ntile_class_d, nnt);
    A(iee, n); A(ine, n); A(eco, kMaxClasses); A(nco, kMaxClasses);
    A(b->bv.active_etiles, net); A(b->bv.active_ntiles, nnt); A(b->bv.counts, 2 * kMaxClasses + 2);
    A(b->bv.inst_active, n);
    d.nodelist = nodelist; d.corner_start = cstart; d.corner_list = clist; d.node_bc = nbc;
    d.lxim = lxim; d.lxip = lxip; d.letam = letam; d.letap = letap; d.lzetam = lzetam; d.lzetap = lzetap;
    d.elem_bc = ebc; d.volo = volo; d.elem_mass = emass; d.nodal_mass = nmass;
    d.ql = nullptr; d.qq = nullptr; d.fx = nullptr; d.fy = nullptr; d.fz = nullptr;
    d.gate = nullptr;

    BatchView &bv = b->bv;
    bv.n_inst = n;
    bv.n_classes = kMaxClasses;
    bv.n_etiles = (int)net;
    bv.n_ntiles = (int)nnt;
    bv.etile_inst = etile_inst_d; bv.ntile_inst = ntile_inst_d;
    bv.etile_class = etile_class_d; bv.ntile_class = ntile_class_d;
    bv.inst_elem_end = iee; bv.inst_node_end = ine;
    bv.eclass_off = eco; bv.nclass_off = nco;

    // host images of the flat arrays, instance by instance
    cudaStream_t st = b->stream;
    bool ok = true;
    auto up = [&](void *dst, const void *src, size_t bytes) {
        ok = ok && cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, st) == cudaSuccess;
    };
    std::vector<int> start(nn + 1, 0), iee_h(n), ine_h(n);
    std::vector<double> fill_one;
    long cpos = 0;   // corner-list position: instances contiguous, no padding
    for (int i = 0; i < n; ++i) {
        HostMesh m;
        m.build(sizes[i], init_mode);
        const double f = e0_scale ? e0_scale[i] : 1.0;
        const double e0 = m.e0 * f;
        const double dt0 = init_mode == LULESH_INIT_V2 ? (.5 * std::cbrt(m.volo[0])) / std::sqrt(2.0 * e0) : m.dt0;
        const long eo_i = b->eoff[i], no_i = b->noff[i], nei = b->ne_i[i], nni = b->nn_i[i];
        std::vector<int> nl(8 * nei), slots(8 * nei), lx[6];
        for (long k = 0; k < 8 * nei; ++k) {
            nl[k] = (int)(m.nodelist[k] + no_i);
            const int c = m.node_elem_corner_list[k];
            slots[k] = (int)((c & 7) * (long)ne + eo_i + (c >> 3));
        }
        const std::vector<int> *src[6] = {&m.lxim, &m.lxip, &m.letam, &m.letap, &m.lzetam, &m.lzetap};
        int *dst[6] = {lxim, lxip, letam, letap, lzetam, lzetap};
        for (int j = 0; j < 6; ++j) {
            lx[j].resize(nei);
            for (long k = 0; k < nei; ++k) lx[j][k] = (int)((*src[j])[k] + eo_i);
            up(dst[j] + eo_i, lx[j].data(), nei * 4);
        }
        for (long k = 0; k < nni; ++k) start[no_i + k] = (int)(cpos + m.node_elem_start[k]);
        for (long k = nni; k < round_tile(nni); ++k) start[no_i + k] = (int)(cpos + 8 * nei);
        std::vector<double> e(nei, 0.0), one(nei, 1.0);
        e[0] = e0;
        up(nodelist + 8 * eo_i, nl.data(), 8 * nei * 4);
        up(clist + cpos, slots.data(), 8 * nei * 4);
        up(nbc + no_i, m.node_bc.data(), nni);
        up(ebc + eo_i, m.elem_bc.data(), nei * 4);
        up(volo + eo_i, m.volo.data(), nei * 8);
        up(emass + eo_i, m.elem_mass.data(), nei * 8);
        up(nmass + no_i, m.nodal_mass.data(), nni * 8);
        std::vector<double> im(nni);
        for (long k2 = 0; k2 < nni; ++k2) im[k2] = 1.0 / m.nodal_mass[k2];
        up(d.inv_mass + no_i, im.data(), nni * 8);
        std::vector<double> iv(nei);
        for (long k2 = 0; k2 < nei; ++k2) iv[k2] = 1.0 / m.volo[k2];
        up(d.inv_volo + eo_i, iv.data(), nei * 8);
        up(d.x + no_i, m.x.data(), nni * 8);
        up(d.y + no_i, m.y.data(), nni * 8);
        up(d.z + no_i, m.z.data(), nni * 8);
        up(d.e + eo_i, e.data(), nei * 8);
        up(d.v + eo_i, one.data(), nei * 8);
        cudaStreamSynchronize(st);   // the host vectors above go out of scope
        DevScalars &h = b->h_sc[i];
        memset(&h, 0, sizeof h);
        h.deltatime = dt0;
        h.dtcourant = 1.0e+20;
        h.dthydro = 1.0e+20;
        h.courant_key = ~0ULL;
        h.hydro_key = ~0ULL;
        h.elem_begin = (int)eo_i;
        h.edge = sizes[i];
        h.node_begin = (int)no_i;
        iee_h[i] = (int)(eo_i + nei);
        ine_h[i] = (int)(no_i + nni);
        cpos += 8 * nei;
    }
    start[nn] = (int)cpos;
    // padded node tails after the last instance keep empty corner ranges
    up(cstart, start.data(), (nn + 1) * 4);
    up(d.sc, b->h_sc, sizeof(DevScalars) * n);
    up(etile_inst_d, etile_inst.data(), net * 4);
    up(ntile_inst_d, ntile_inst.data(), nnt * 4);
    up(etile_class_d, etile_class.data(), net * 4);
    up(ntile_class_d, ntile_class.data(), nnt * 4);
    up(iee, iee_h.data(), n * 4);
    up(ine, ine_h.data(), n * 4);
    up(eco, eclass_off, sizeof eclass_off);
    up(nco, nclass_off, sizeof nclass_off);
    // padding entries of the mass arrays are read by whole-array kernels
    // (the split path's reciprocal masses): give them unit values
    {
        std::vector<double> ones(std::max(ne, nn), 1.0);
        for (int i = 0; i < n; ++i) {
            const long etail = round_tile(b->ne_i[i]) - b->ne_i[i], ntail = round_tile(b->nn_i[i]) - b->nn_i[i];
            if (etail) {
                up(volo + b->eoff[i] + b->ne_i[i], ones.data(), etail * 8);
                up(emass + b->eoff[i] + b->ne_i[i], ones.data(), etail * 8);
                up(d.inv_volo + b->eoff[i] + b->ne_i[i], ones.data(), etail * 8);
            }
            if (ntail) {
                up(nmass + b->noff[i] + b->nn_i[i], ones.data(), ntail * 8);
                up(d.inv_mass + b->noff[i] + b->nn_i[i], ones.data(), ntail * 8);
            }
        }
        cudaStreamSynchronize(st);
    }
    for (double *f : {d.xd, d.yd, d.zd}) ok = ok && cudaMemsetAsync(f, 0, nn * 8, st) == cudaSuccess;
    for (double *f : {d.p, d.q, d.ss, d.vnew, d.delv, d.vdov, d.arealg, d.delv_xi, d.delv_eta, d.delv_zeta,
                      d.delx_xi, d.delx_eta, d.delx_zeta})
        ok = ok && cudaMemsetAsync(f, 0, ne * 8, st) == cudaSuccess;
    ok = ok && cudaMemsetAsync(b->bv.counts, 0, (2 * kMaxClasses + 2) * 4, st) == cudaSuccess;
    if (ok && precision == LULESH_PRECISION_SPLIT) {
        launch_split_sync(d, st);
        ok = cudaGetLastError() == cudaSuccess;
    }
    ok = ok && cudaStreamSynchronize(st) == cudaSuccess;
    if (!ok) {
        b->err = std::string("lulesh_batch_create upload: ") + cudaGetErrorString(cudaGetLastError());
        return bail(LULESH_ERR_CUDA);
    }
    // the staged tiles of the split force kernel, for every class whose
    // instances are all cubes of at least one tile row's width
    if (precision == LULESH_PRECISION_SPLIT) {
        for (int c = 0; c < kMaxClasses; ++c) {
            std::vector<int> inst, sz, eb, nb;
            bool all = true;
            for (int i = 0; i < n; ++i)
                if (b->inst_class[i] == c) {
                    all = all && sizes[i] >= kTileCols;
                    inst.push_back(i);
                    sz.push_back(sizes[i]);
                    eb.push_back((int)b->eoff[i]);
                    nb.push_back((int)b->noff[i]);
                }
            if (inst.empty() || !all) continue;
            const int m = (int)inst.size();
            int *d_inst, *d_s, *d_eb, *d_nb;
            A(d_inst, m); A(d_s, m); A(d_eb, m); A(d_nb, m);
            ok = cudaMemcpy(d_inst, inst.data(), m * 4, cudaMemcpyHostToDevice) == cudaSuccess &&
                 cudaMemcpy(d_s, sz.data(), m * 4, cudaMemcpyHostToDevice) == cudaSuccess &&
                 cudaMemcpy(d_eb, eb.data(), m * 4, cudaMemcpyHostToDevice) == cudaSuccess &&
                 cudaMemcpy(d_nb, nb.data(), m * 4, cudaMemcpyHostToDevice) == cudaSuccess;
            for (int r = 0; ok && r < 2; ++r) {
                std::vector<long long> begin(m + 1, 0);
                for (int j = 0; j < m; ++j)
                    begin[j + 1] = begin[j] + (kStageRows[r] == 4 ? TileShape<4>::tiles(sz[j]) : TileShape<2>::tiles(sz[j]));
                long long *d_begin;
                A(d_begin, m + 1);
                ok = cudaMemcpy(d_begin, begin.data(), (m + 1) * sizeof(long long), cudaMemcpyHostToDevice) == cudaSuccess;
                b->staged[c][r] = {m, d_inst, d_s, d_eb, d_nb, d_begin};
            }
            if (!ok) {
                b->err = std::string("lulesh_batch_create staged tiles: ") + cudaGetErrorString(cudaGetLastError());
                return bail(LULESH_ERR_CUDA);
            }
        }
    }
#undef A
    default_cfg(b);
    *out = b;
    return LULESH_OK;
}

int lulesh_batch_run(lulesh_batch *b, int max_cycles, int *cycles_done)
{
    if (!b) return LULESH_ERR_ARG;
    if (cycles_done) *cycles_done = 0;
    int rc = build_graph(b);
    if (rc) return rc;
    b->h_stage[0] = max_cycles;
    BCK(cudaMemcpyAsync(b->d_max, b->h_stage, sizeof(int), cudaMemcpyHostToDevice, b->stream));
    BCK(cudaGraphLaunch(b->run_exec, b->stream));
    BCK(cudaMemcpyAsync(b->h_sc, b->dom.sc, sizeof(DevScalars) * b->n, cudaMemcpyDeviceToHost, b->stream));
    BCK(cudaStreamSynchronize(b->stream));
    int most = 0;
    long long total = 0;
    b->last_zc = 0.0;
    for (int i = 0; i < b->n; ++i) {
        most = std::max(most, b->h_sc[i].run_cycles);
        total += b->h_sc[i].run_cycles;
        b->last_zc += (double)b->ne_i[i] * b->h_sc[i].run_cycles;
    }
    if (cycles_done) *cycles_done = most;
    // time increment, epilogue and compaction run every cycle; each step
    // kernel once per class per cycle
    b->launches += 2 + (long long)most * b->kernels_per_cycle;
    (void)total;
    // an instance that stopped short of its stop time without an error and
    // without reaching the caller's cap ran out of cycle budget (or of
    // positive time step): lulesh_run's LULESH_ERR_TIMEOUT
    for (int i = 0; i < b->n; ++i) {
        const DevScalars &h = b->h_sc[i];
        if (h.err_any || !(h.time < b->dom.prm.stoptime)) continue;
        if (max_cycles > 0 && max_cycles <= kRunCycleLimit && h.run_cycles >= max_cycles) continue;
        return bfail(b, LULESH_ERR_TIMEOUT,
                     "lulesh_batch_run: instance " + std::to_string(i) + " stopped short of stoptime (" +
                         (h.deltatime > 0.0 ? "cycle budget ran out" : "time step no longer positive") + ")");
    }
    return LULESH_OK;
}

int lulesh_batch_run_retuned(lulesh_batch *b, int chunk, double fraction, int max_cycles, int *cycles_done,
                             int *retunes)
{
    if (!b || chunk < 1 || !(fraction > 0.0 && fraction < 1.0)) return LULESH_ERR_ARG;
    if (cycles_done) *cycles_done = 0;
    if (retunes) *retunes = 0;
    // elements of the instances still running (the host copy of the scalars
    // is current after every run call)
    auto running = [&]() {
        long m = 0;
        for (int i = 0; i < b->n; ++i) {
            const DevScalars &h = b->h_sc[i];
            if (!h.err_any && h.time < b->dom.prm.stoptime && h.deltatime > 0.0) m += b->ne_i[i];
        }
        return m;
    };
    BCK(cudaMemcpyAsync(b->h_sc, b->dom.sc, sizeof(DevScalars) * b->n, cudaMemcpyDeviceToHost, b->stream));
    BCK(cudaStreamSynchronize(b->stream));
    long tuned_for = running();
    std::vector<long long> done_i(b->n, 0);
    long long total = 0;
    int n_retunes = 0;
    double zc = 0.0;
    for (;;) {
        int cap = chunk;
        if (max_cycles > 0) cap = (int)std::min<long long>(chunk, max_cycles - total);
        int most = 0;
        int rc = lulesh_batch_run(b, cap, &most);
        for (int i = 0; i < b->n; ++i) done_i[i] += b->h_sc[i].run_cycles;
        total += most;
        zc += b->last_zc;
        b->last_zc = zc;
        if (rc) return rc;
        const long now = running();
        if (now == 0 || most == 0 || (max_cycles > 0 && total >= max_cycles)) break;
        if (now < fraction * tuned_for) {
            // the running set shrank: re-time the launch shapes on it (not
            // cached: they belong to this part of this run) and rebuild the
            // graph
            if ((rc = lulesh_batch_autotune(b, nullptr, 1))) return rc;
            tuned_for = now;
            ++n_retunes;
        }
    }
    if (cycles_done) *cycles_done = (int)*std::max_element(done_i.begin(), done_i.end());
    if (retunes) *retunes = n_retunes;
    return LULESH_OK;
}

int lulesh_batch_size(lulesh_batch *b, int *n, long *total_elements, long *total_nodes)
{
    if (!b) return LULESH_ERR_ARG;
    if (n) *n = b->n;
    long te = 0, tn = 0;
    for (int i = 0; i < b->n; ++i) { te += b->ne_i[i]; tn += b->nn_i[i]; }
    if (total_elements) *total_elements = te;
    if (total_nodes) *total_nodes = tn;
    return LULESH_OK;
}

int lulesh_batch_instance(lulesh_batch *b, int i, lulesh_scalars *out, double *origin_energy, int *status)
{
    if (!b || i < 0 || i >= b->n) return LULESH_ERR_ARG;
    DevScalars h;
    BCK(cudaMemcpyAsync(&h, b->dom.sc + i, sizeof h, cudaMemcpyDeviceToHost, b->stream));
    double e0 = 0.0;
    BCK(cudaMemcpyAsync(&e0, b->dom.e + b->eoff[i], sizeof e0, cudaMemcpyDeviceToHost, b->stream));
    BCK(cudaStreamSynchronize(b->stream));
    if (out) {
        out->time = h.time;
        out->deltatime = h.deltatime;
        out->dtcourant = h.dtcourant;
        out->dthydro = h.dthydro;
        out->cycle = h.cycle;
    }
    if (origin_energy) *origin_energy = e0;
    if (status) {
        *status = LULESH_OK;
        static const int code[ERR_NUM] = {LULESH_VOLUME_ERROR, LULESH_VOLUME_ERROR, LULESH_VOLUME_ERROR,
                                          LULESH_QSTOP_ERROR, LULESH_VOLUME_ERROR};
        for (int k = 0; k < ERR_NUM; ++k)
            if (h.err[k]) { *status = code[k]; break; }
    }
    return LULESH_OK;
}

int lulesh_batch_get_field(lulesh_batch *b, int i, const char *name, double *host, long n)
{
    if (!b || i < 0 || i >= b->n || !name || !host) return LULESH_ERR_ARG;
    const Dom &d = b->dom;
    const struct { const char *nm; double *p; bool node; } t[] = {
        {"x", d.x, true}, {"y", d.y, true}, {"z", d.z, true}, {"xd", d.xd, true}, {"yd", d.yd, true},
        {"zd", d.zd, true}, {"e", d.e, false}, {"p", d.p, false}, {"q", d.q, false}, {"v", d.v, false},
        {"ss", d.ss, false}, {"vdov", d.vdov, false}, {"arealg", d.arealg, false},
        {"volo", const_cast<double *>(d.volo), false}, {"elemMass", const_cast<double *>(d.elem_mass), false},
        {"nodalMass", const_cast<double *>(d.nodal_mass), true}};
    for (const auto &f : t)
        if (!strcmp(f.nm, name)) {
            const long len = f.node ? b->nn_i[i] : b->ne_i[i];
            if (n != len) return bfail(b, LULESH_ERR_ARG, std::string("wrong length for field ") + name);
            const long off = f.node ? b->noff[i] : b->eoff[i];
            BCK(cudaMemcpyAsync(host, f.p + off, n * sizeof(double), cudaMemcpyDeviceToHost, b->stream));
            BCK(cudaStreamSynchronize(b->stream));
            return LULESH_OK;
        }
    return bfail(b, LULESH_ERR_ARG, std::string("unknown field ") + name);
}

int lulesh_batch_zone_cycles(lulesh_batch *b, double *zone_cycles)
{
    if (!b || !zone_cycles) return LULESH_ERR_ARG;
    *zone_cycles = b->last_zc;
    return LULESH_OK;
}

void *lulesh_batch_stream(lulesh_batch *b) { return b ? (void *)b->stream : nullptr; }

long long lulesh_batch_kernel_launches(lulesh_batch *b) { return b ? b->launches : 0; }

int lulesh_batch_tuning(lulesh_batch *b, int cls, int kernel, int *block, int *grid)
{
    if (!b || cls < 0 || cls >= kMaxClasses || kernel < 0 || kernel >= kBatchKernels) return LULESH_ERR_ARG;
    if (block) *block = b->cfg[cls][kernel].block;
    if (grid) *grid = b->cfg[cls][kernel].grid;
    return LULESH_OK;
}

int lulesh_batch_staging(lulesh_batch *b, int cls, int kernel, int *rows)
{
    if (!b || !rows || cls < 0 || cls >= kMaxClasses || kernel < 0 || kernel >= kBatchKernels) return LULESH_ERR_ARG;
    *rows = b->cfg[cls][kernel].stage;
    return LULESH_OK;
}

int lulesh_batch_set_tuning(lulesh_batch *b, int cls, int kernel, int block, int blocks_per_sm, int rows)
{
    if (!b || cls < 0 || cls >= kMaxClasses || kernel < 0 || kernel >= kBatchKernels || blocks_per_sm < 1)
        return bfail(b, LULESH_ERR_ARG, "lulesh_batch_set_tuning: bad arguments");
    const int tiles = kernel == 1 ? b->class_ntiles[cls] : b->class_etiles[cls];
    if (rows != 0) {
        if (kernel != 0 || (rows != 2 && rows != 4) || !can_stage(b, cls))
            return bfail(b, LULESH_ERR_ARG, "lulesh_batch_set_tuning: this class's kernel cannot be staged that deep");
        const int per_sm = std::max(1, std::min(blocks_per_sm, batch_max_blocks_split_staged(rows)));
        b->cfg[cls][kernel] = {rows * kTileCols,
                               (int)std::max(1LL, std::min(staged_tiles(b, cls, rows), (long long)b->sms * per_sm)), rows};
    } else {
        if (block < 32 || block > 256 || block % 32)
            return bfail(b, LULESH_ERR_ARG, "lulesh_batch_set_tuning: block must be a multiple of 32 up to 256");
        const int fit = max_blocks(b, kernel, block);
        if (fit < 1) return bfail(b, LULESH_ERR_ARG, "lulesh_batch_set_tuning: no block of that size fits on an SM");
        const int per_sm = std::min(blocks_per_sm, fit);
        b->cfg[cls][kernel] = {block, std::max(1, std::min(std::max(tiles, 1), b->sms * per_sm))};
    }
    destroy_graph(b);   // the run graph bakes in the launch shapes
    return LULESH_OK;
}

int lulesh_batch_autotune(lulesh_batch *b, const char *cache_path, int retune)
{
    if (!b) return LULESH_ERR_ARG;
    std::map<std::string, TuneEntry> cache;
    if (cache_path) cache = read_cache(cache_path);
    bool need = false;
    for (int c = 0; c < kMaxClasses; ++c)
        for (int k = 0; k < kBatchKernels; ++k) {
            const int tiles = k == 1 ? b->class_ntiles[c] : b->class_etiles[c];
            if (!tiles) continue;
            auto it = cache.find(tune_key(b, c, k));
            if (it == cache.end() || retune) { need = true; continue; }
            const TuneEntry &te = it->second;
            if (k == 0 && (te.stage == 2 || te.stage == 4) && can_stage(b, c)) {
                const int per_sm = std::max(1, std::min(te.per_sm, batch_max_blocks_split_staged(te.stage)));
                b->cfg[c][k] = {te.stage * kTileCols,
                                (int)std::max(1LL, std::min(staged_tiles(b, c, te.stage), (long long)b->sms * per_sm)),
                                te.stage};
            } else {
                const int per_sm = std::max(1, std::min(te.per_sm, max_blocks(b, k, te.block)));
                b->cfg[c][k] = {te.block, std::max(1, std::min(tiles, b->sms * per_sm))};
            }
        }
    if (need) {
        // snapshot the evolving state; tuning runs real kernels on it
        const Dom &d = b->dom;
        const size_t ne = b->ne_tot, nn = b->nn_tot;
        double *node_f[6] = {d.x, d.y, d.z, d.xd, d.yd, d.zd};
        double *elem_f[5] = {d.e, d.p, d.q, d.v, d.ss};
        std::vector<void *> snap;
        auto cleanup = [&]() { for (void *p : snap) cudaFree(p); };
        for (int j = 0; j < 11; ++j) {
            void *p = nullptr;
            const size_t bytes = (j < 6 ? nn : ne) * sizeof(double);
            if (cudaMalloc(&p, bytes) != cudaSuccess) { cleanup(); return bfail(b, LULESH_ERR_CUDA, "autotune snapshot allocation failed"); }
            snap.push_back(p);
            cudaMemcpyAsync(p, j < 6 ? node_f[j] : elem_f[j - 6], bytes, cudaMemcpyDeviceToDevice, b->stream);
        }
        void *ssnap = nullptr;
        if (cudaMalloc(&ssnap, sizeof(DevScalars) * b->n) != cudaSuccess) { cleanup(); return bfail(b, LULESH_ERR_CUDA, "autotune snapshot allocation failed"); }
        snap.push_back(ssnap);
        cudaMemcpyAsync(ssnap, d.sc, sizeof(DevScalars) * b->n, cudaMemcpyDeviceToDevice, b->stream);

        // active lists for the current state
        b->h_stage[0] = 0;
        cudaMemcpyAsync(b->d_max, b->h_stage, sizeof(int), cudaMemcpyHostToDevice, b->stream);
        kb_prologue<<<1, 1024, 0, b->stream>>>(b->dom, b->bv, b->d_max, 0);
        kb_compact<<<compact_blocks(b), 256, 0, b->stream>>>(b->bv);
        cudaEvent_t e0, e1;
        cudaEventCreate(&e0);
        cudaEventCreate(&e1);
        const int blocks[3] = {64, 128, 256};
        const int depths[4] = {1, 2, 4, 8};
        for (int c = 0; c < kMaxClasses; ++c)
            for (int k = 0; k < kBatchKernels; ++k) {
                const int tiles = k == 1 ? b->class_ntiles[c] : b->class_etiles[c];
                if (!tiles) continue;
                float best = 1e30f;
                LaunchCfg best_cfg = b->cfg[c][k];
                int best_depth = 1;
                auto try_cfg = [&](LaunchCfg cfg, int dp) {
                    b->cfg[c][k] = cfg;
                    float t = 1e30f;
                    for (int r = 0; r < 3; ++r) {
                        cudaEventRecord(e0, b->stream);
                        launch_kernel(b, k, c, b->stream);
                        cudaEventRecord(e1, b->stream);
                        cudaEventSynchronize(e1);
                        float ms = 0.f;
                        cudaEventElapsedTime(&ms, e0, e1);
                        t = std::min(t, ms);
                    }
                    if (t < best) {
                        best = t;
                        best_cfg = cfg;
                        best_depth = dp;
                    }
                };
                // resident blocks per SM: 1, 2, 4, 8 and the most that fit
                // (three 128-thread blocks of the 168-register force body,
                // for instance, which no power of two reaches)
                auto per_sm_candidates = [&](int cap) {
                    std::vector<int> v;
                    for (int dp : depths)
                        if (dp <= cap) v.push_back(dp);
                    if (cap >= 1 && std::find(v.begin(), v.end(), cap) == v.end()) v.push_back(cap);
                    return v;
                };
                for (int bs : blocks)
                    for (int dp : per_sm_candidates(max_blocks(b, k, bs)))
                        try_cfg({bs, std::max(1, std::min(tiles, b->sms * dp))}, dp);
                // the split force kernel of a class of structured cubes: the
                // staged tiles, two or four element rows deep
                if (k == 0 && can_stage(b, c))
                    for (int rows : kStageRows) {
                        const long long st_tiles = staged_tiles(b, c, rows);
                        for (int dp : per_sm_candidates(batch_max_blocks_split_staged(rows)))
                            try_cfg({rows * kTileCols, (int)std::max(1LL, std::min(st_tiles, (long long)b->sms * dp)), rows},
                                    dp);
                    }
                b->cfg[c][k] = best_cfg;
                cache[tune_key(b, c, k)] = {best_cfg.block, best_depth, best_cfg.stage};
            }
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        // restore
        for (int j = 0; j < 11; ++j)
            cudaMemcpyAsync(j < 6 ? node_f[j] : elem_f[j - 6], snap[j], (j < 6 ? nn : ne) * sizeof(double),
                            cudaMemcpyDeviceToDevice, b->stream);
        cudaMemcpyAsync(d.sc, ssnap, sizeof(DevScalars) * b->n, cudaMemcpyDeviceToDevice, b->stream);
        // the tuning runs rewrote the geometry cache from positions that are
        // now restored: mark it stale
        kb_geo_invalidate<<<(b->n + 127) / 128, 128, 0, b->stream>>>(d.sc, b->n);
        if (b->precision == LULESH_PRECISION_SPLIT) launch_split_sync(b->dom, b->stream);
        cudaError_t e = cudaStreamSynchronize(b->stream);
        cleanup();
        if (e != cudaSuccess) return bfail(b, LULESH_ERR_CUDA, std::string("autotune: ") + cudaGetErrorString(e));
        if (cache_path) write_cache(cache_path, cache);
    }
    destroy_graph(b);   // the run graph bakes in the launch shapes
    b->tuned = true;
    return LULESH_OK;
}

}  // extern "C"
