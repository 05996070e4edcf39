// noalloc.cu -- LagrangeNodal on caller-owned device arrays, allocating nothing.
//
// Some callers cannot allocate GPU memory: code that runs inside a memory
// pool or arena owned by someone else (a host framework that hands out only
// the arrays of its own data structures), code that must not touch the
// allocator between two synchronisation points, or drivers that budget every
// byte of device memory up front.  lulesh_lagrange_nodal_noalloc serves them:
// the caller passes every input and output as a device pointer, and the one
// piece of working memory the step needs -- the per-corner forces between the
// element kernel and the node gather, plus the node-to-corner slot table, the
// symmetry-plane mask and the error words -- lives in the file-scope device
// array below, of a fixed size that is part of the library image.
//
// Consequences a caller must know:
//   - every GPU on which this entry point is used holds kScratchBytes of
//     device memory for the array until the process exits;
//   - all calls share the one array, so calls that overlap on the GPU (two
//     streams, or two host threads) race: order them on one stream;
//   - every call looks up the array's device address (cudaGetSymbolAddress,
//     a host-side lookup that allocates nothing) with the calling thread's
//     current device, so the address is never stale, whichever context is
//     current; the first call on a device also loads the library's device
//     code, and with it the array, onto that device;
//   - the call reads its status back and waits for its stream before it
//     returns.
#include "lulesh_internal.h"
#include "kernels.h"

#include <cuda_runtime.h>

#include <cstdio>

namespace lulesh {
namespace {

// Largest mesh the fixed array serves.
constexpr long kNoAllocMaxElem = 1L << 16;   // 65,536 elements (a 40^3 cube fits)
constexpr long kNoAllocMaxNode = 1L << 17;   // 131,072 nodes

// Layout of the array, in bytes from its start (each part 256-aligned):
//   DevScalars | corner forces 3 x 8*E doubles | slot table 8*E ints |
//   corner starts (N+1) ints | node mask N bytes
constexpr size_t align256(size_t b) { return (b + 255) & ~size_t(255); }
constexpr size_t kOffScalars = 0;
constexpr size_t kOffForces = align256(sizeof(DevScalars));
constexpr size_t kOffSlots = kOffForces + align256(3 * 8 * kNoAllocMaxElem * sizeof(double));
constexpr size_t kOffStart = kOffSlots + align256(8 * kNoAllocMaxElem * sizeof(int));
constexpr size_t kOffMask = kOffStart + align256((kNoAllocMaxNode + 1) * sizeof(int));
constexpr size_t kScratchBytes = kOffMask + align256(kNoAllocMaxNode);

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

// Messages go to stderr: this entry point reports through its status code
// only (it has no context whose lulesh_last_error could carry them).
int noalloc_fail(int code, const char *msg)
{
    fprintf(stderr, "lulesh_lagrange_nodal_noalloc: %s\n", msg);
    return code;
}

// err_any value that marks malformed input; the step kernels then do nothing.
constexpr int kBadInput = 2;

// Per-call preparation, after the scalar block was zeroed: set the time
// step, check the caller's mesh tables, translate the reference's
// node-to-corner list (entries 8*elem+corner) into corner-major slots, close
// the start table and clear the node mask.
//
// The tables must describe the reference's node-to-corner map
// (AllocateNodeElemIndexes, LULESH-OMP.cc:209-268): every nodelist entry and
// corner-list entry in range; node n's list is corner_list[start[n] ..
// start[n] + count[n]), the lists packed back to back from 0 to 8E; every
// entry of node n's list a corner whose nodelist entry is n; and each list
// strictly increasing, as the reference builds it.  Together these make the
// lists a permutation of the 8E corners, so the gather sums every corner
// force exactly once.  A table that breaks any of them marks kBadInput and
// the step kernels then read nothing through it.
__global__ void k_noalloc_prepare(DevScalars *sc, double deltatime, const int *nodelist,
                                  const int *corner_list_ref, int *slots, const int *start_ref,
                                  const int *count_ref, int *start, unsigned char *mask, int ne, int nn)
{
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const long nc = 8L * ne;
    if (i == 0) {
        sc->deltatime = deltatime;
        const long end = (long)start_ref[nn - 1] + count_ref[nn - 1];
        start[nn] = (int)end;
        if (end != nc || start_ref[0] != 0) sc->err_any = kBadInput;
    }
    if (i < nc) {
        const int k = corner_list_ref[i];
        const int n = nodelist[i];
        if (k < 0 || k >= nc || n < 0 || n >= nn) {
            sc->err_any = kBadInput;
            slots[i] = 0;
        } else {
            slots[i] = (k & 7) * ne + (k >> 3);
        }
    }
    if (i < nn) {
        const int st = start_ref[i], cnt = count_ref[i];
        bool bad = st < 0 || cnt < 0 || (long)st + cnt > nc;
        if (!bad && i + 1 < nn) bad = (long)st + cnt != (long)start_ref[i + 1];
        // the node's own list: in range, its corners on this node, increasing
        for (int j = 0, prev = -1; !bad && j < cnt; ++j) {
            const int k = corner_list_ref[st + j];
            bad = k <= prev || k >= nc || nodelist[k] != (int)i;
            prev = k;
        }
        if (bad) sc->err_any = kBadInput;
        start[i] = st;
        mask[i] = 0;
    }
}

// Symmetry-plane node sets (the reference's symmX/symmY/symmZ) into the mask.
__global__ void k_noalloc_mask(DevScalars *sc, unsigned char *mask, const int *symm_x,
                               const int *symm_y, const int *symm_z, int nsymm, int nn)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nsymm) return;
    // the three sets share the nodes on the coordinate axes: combine bits
    // with atomics on the 32-bit word that holds the node's byte
    auto set_bit = [&](int node, unsigned bit) {
        if (node < 0 || node >= nn) {
            sc->err_any = kBadInput;
            return;
        }
        unsigned *word = reinterpret_cast<unsigned *>(mask + (node & ~3));
        atomicOr(word, bit << (8 * (node & 3)));
    };
    set_bit(symm_x[i], 1u);
    set_bit(symm_y[i], 2u);
    set_bit(symm_z[i], 4u);
}

}  // namespace
}  // namespace lulesh

using namespace lulesh;

extern "C" int lulesh_lagrange_nodal_noalloc(
    int num_elem, int num_node, double deltatime, const lulesh_params *params,
    const int *nodelist, const int *node_elem_start, const int *node_elem_count,
    const int *node_elem_corner_list, const int *symm_x, const int *symm_y, const int *symm_z,
    int num_symm, const double *volo, const double *elem_mass, const double *nodal_mass,
    const double *p, const double *q, const double *v, const double *ss,
    double *x, double *y, double *z, double *xd, double *yd, double *zd,
    double *fx, double *fy, double *fz, void *stream)
{
    if (num_elem < 1 || num_node < 1 || num_symm < 0)
        return noalloc_fail(LULESH_ERR_ARG, "empty mesh");
    if (num_elem > kNoAllocMaxElem || num_node > kNoAllocMaxNode) {
        char buf[200];
        snprintf(buf, sizeof buf,
                 "mesh of %d elements / %d nodes exceeds the fixed working array "
                 "(at most %ld elements and %ld nodes)",
                 num_elem, num_node, kNoAllocMaxElem, kNoAllocMaxNode);
        return noalloc_fail(LULESH_ERR_ARG, buf);
    }
    if (!params || !nodelist || !node_elem_start || !node_elem_count || !node_elem_corner_list ||
        !volo || !elem_mass || !nodal_mass || !p || !q || !v || !ss || !x || !y || !z || !xd ||
        !yd || !zd || (num_symm > 0 && (!symm_x || !symm_y || !symm_z)))
        return noalloc_fail(LULESH_ERR_ARG, "missing array");
    const bool keep = fx && fy && fz;

    // the array's device address on the current device and context (its
    // host-side name is only a stand-in); looked up on every call, so a
    // reset device or another context never leaves a stale address behind
    void *ptr = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
    if (e != cudaSuccess) return noalloc_fail(LULESH_ERR_CUDA, cudaGetErrorString(e));
    unsigned char *base = static_cast<unsigned char *>(ptr);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const size_t ne = (size_t)num_elem;

    Dom d{};
    d.s = 0;
    d.ne = num_elem;
    d.nn = num_node;
    d.keep = keep ? 1 : 0;
    d.df = arith_of(LULESH_PRECISION_FP64);   // the plain path's arithmetic
    d.nodelist = nodelist;
    d.corner_start = reinterpret_cast<const int *>(base + kOffStart);
    d.corner_list = reinterpret_cast<const int *>(base + kOffSlots);
    d.node_bc = base + kOffMask;
    d.volo = volo;
    d.elem_mass = elem_mass;
    d.nodal_mass = nodal_mass;
    d.x = x; d.y = y; d.z = z;
    d.xd = xd; d.yd = yd; d.zd = zd;
    d.fx = fx; d.fy = fy; d.fz = fz;
    d.p = const_cast<double *>(p);
    d.q = const_cast<double *>(q);
    d.v = const_cast<double *>(v);
    d.ss = const_cast<double *>(ss);
    double *forces = reinterpret_cast<double *>(base + kOffForces);
    d.fcx = forces;
    d.fcy = forces + 8 * ne;
    d.fcz = forces + 16 * ne;
    d.sc = reinterpret_cast<DevScalars *>(base + kOffScalars);
    d.gate = nullptr;
    d.prm = *params;

    // the array keeps the previous call's contents: zero the scalar block
    // (error words), everything else is rewritten below before it is read
    e = cudaMemsetAsync(d.sc, 0, sizeof(DevScalars), st);
    if (e != cudaSuccess) return noalloc_fail(LULESH_ERR_CUDA, cudaGetErrorString(e));
    const long work = 8L * num_elem > num_node ? 8L * num_elem : num_node;
    k_noalloc_prepare<<<(unsigned)((work + 255) / 256), 256, 0, st>>>(
        d.sc, deltatime, nodelist, node_elem_corner_list, const_cast<int *>(d.corner_list),
        node_elem_start, node_elem_count, const_cast<int *>(d.corner_start),
        const_cast<unsigned char *>(d.node_bc), num_elem, num_node);
    if (num_symm > 0)
        k_noalloc_mask<<<(num_symm + 255) / 256, 256, 0, st>>>(
            d.sc, const_cast<unsigned char *>(d.node_bc), symm_x, symm_y, symm_z, num_symm, num_node);
    launch_lagrange_nodal(d, st);
    e = cudaGetLastError();
    if (e != cudaSuccess) return noalloc_fail(LULESH_ERR_CUDA, cudaGetErrorString(e));

    DevScalars h;
    e = cudaMemcpyAsync(&h, d.sc, sizeof h, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return noalloc_fail(LULESH_ERR_CUDA, cudaGetErrorString(e));
    if (h.err_any == kBadInput)
        return noalloc_fail(LULESH_ERR_ARG,
                            "malformed mesh tables (an index out of range, or node-to-corner lists "
                            "that are not the reference's packed, increasing map)");
    if (h.err[ERR_K1_DETERM] || h.err[ERR_K1_VOLUME]) return LULESH_VOLUME_ERROR;
    return LULESH_OK;
}
