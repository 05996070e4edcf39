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
__device__ __forceinline__ void kb_elem_tiles(const Dom &d, const BatchView &b, int cls)
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

// The material kernel also reduces the instance's constraint keys: one
// block minimum per tile (every thread reaches the barrier; the trip counts
// are uniform over the block).
template <void (*Body)(const Dom &, int, DevScalars *, unsigned long long &, unsigned long long &)>
__device__ __forceinline__ void kb_material_tiles(const Dom &d, const BatchView &b, int cls)
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

template <void (*Body)(const Dom &, int, DevScalars *)>
__global__ void kb_elem(const __grid_constant__ Dom d, const __grid_constant__ BatchView b, int cls)
{
    kb_elem_tiles<Body>(d, b, cls);
}

template <void (*Body)(const Dom &, int, DevScalars *, unsigned long long &, unsigned long long &)>
__global__ void kb_material(const __grid_constant__ Dom d, const __grid_constant__ BatchView b, int cls)
{
    kb_material_tiles<Body>(d, b, cls);
}

// Register-capped variants for the kinematics and material bodies, which
// wait on their gathers: blocks of up to kBatchMaxBlock threads (the
// autotuner's largest), kMinBlocks of them resident per SM, so 4 -> 64
// registers, 3 -> 85 and 2 -> 128.  The material bodies of both arithmetics
// run at 64 (as the single-instance material kernels do).  On the
// 528-instance split ensemble (kinematics at 128 registers instead of 134,
// material at 64 instead of 77) this took 36.7 s to 30.2 s; capping the
// force body as well (64 or 85 registers, with spills) lost 5 %.
constexpr int kBatchMaxBlock = 256;

template <void (*Body)(const Dom &, int, DevScalars *), int kMinBlocks>
__global__ void __launch_bounds__(kBatchMaxBlock, kMinBlocks)
    kb_elem_capped(const __grid_constant__ Dom d, const __grid_constant__ BatchView b, int cls)
{
    kb_elem_tiles<Body>(d, b, cls);
}

template <void (*Body)(const Dom &, int, DevScalars *, unsigned long long &, unsigned long long &),
          int kMinBlocks>
__global__ void __launch_bounds__(kBatchMaxBlock, kMinBlocks)
    kb_material_capped(const __grid_constant__ Dom d, const __grid_constant__ BatchView b, int cls)
{
    kb_material_tiles<Body>(d, b, cls);
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
        // the instance's positions move: its geometry cache goes stale
        if (d.geo && threadIdx.x == 0) d.sc[inst].geo_valid = 0;
        const int end = min(b.inst_node_end[inst], (t + 1) * kTile);
        for (int n = t * kTile + threadIdx.x; n < end; n += blockDim.x) Body(d, n, sc);
    }
}

}  // namespace lulesh
