// batch_kernels.cuh -- persistent kernels over the active tiles of one size
// class of a batched ensemble.  Each block walks the class's active-tile list
// with a grid stride; a tile is kTile consecutive elements (nodes) of one
// instance, processed blockDim at a time (kTile / blockDim elements per
// thread).  The per-element work is the single-instance body, given the
// instance's scalar block.
#pragma once

#include "common.cuh"

namespace lulesh {

template <void (*Body)(const Dom &, int, DevScalars *)>
__global__ void kb_elem(const __grid_constant__ Dom d, const __grid_constant__ BatchView b, int cls)
{
    const int n_act = b.counts[cls];
    const int *list = b.active_etiles + b.eclass_off[cls];
    for (int i = blockIdx.x; i < n_act; i += gridDim.x) {
        const int t = list[i];
        const int inst = b.etile_inst[t];
        DevScalars *sc = d.sc + inst;
        if (sc->err_any) continue;
        const int end = min(b.inst_elem_end[inst], (t + 1) * kTile);
        for (int k = t * kTile + threadIdx.x; k < end; k += blockDim.x) Body(d, k, sc);
    }
}

template <void (*Body)(const Dom &, int, const DevScalars *)>
__global__ void kb_node(const __grid_constant__ Dom d, const __grid_constant__ BatchView b, int cls)
{
    const int n_act = b.counts[kMaxClasses + cls];
    const int *list = b.active_ntiles + b.nclass_off[cls];
    for (int i = blockIdx.x; i < n_act; i += gridDim.x) {
        const int t = list[i];
        const int inst = b.ntile_inst[t];
        const DevScalars *sc = d.sc + inst;
        if (sc->err_any) continue;
        const int end = min(b.inst_node_end[inst], (t + 1) * kTile);
        for (int n = t * kTile + threadIdx.x; n < end; n += blockDim.x) Body(d, n, sc);
    }
}

// The material kernel also reduces the instance's constraint keys: one
// block minimum per tile (every thread reaches the barrier; the trip counts
// are uniform over the block).
template <void (*Body)(const Dom &, int, DevScalars *, unsigned long long &, unsigned long long &)>
__global__ void kb_material(const __grid_constant__ Dom d, const __grid_constant__ BatchView b, int cls)
{
    const int n_act = b.counts[cls];
    const int *list = b.active_etiles + b.eclass_off[cls];
    for (int i = blockIdx.x; i < n_act; i += gridDim.x) {
        const int t = list[i];
        const int inst = b.etile_inst[t];
        DevScalars *sc = d.sc + inst;
        const bool live = sc->err_any == 0;
        const int end = min(b.inst_elem_end[inst], (t + 1) * kTile);
        unsigned long long kc = ~0ULL, kh = ~0ULL;
        for (int j = 0; j < kTile; j += blockDim.x) {
            const int k = t * kTile + j + threadIdx.x;
            unsigned long long c = ~0ULL, h = ~0ULL;
            if (live && k < end) Body(d, k, sc, c, h);
            kc = c < kc ? c : kc;
            kh = h < kh ? h : kh;
        }
        block_min_publish(kc, kh, sc);
        __syncthreads();   // the shared staging of block_min_publish is reused next tile
    }
}

}  // namespace lulesh
