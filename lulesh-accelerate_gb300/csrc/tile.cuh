// tile.cuh -- staging of a structured cube's corner nodes in shared memory.
//
// On the s^3 cube (the reference's node and element numbering: element
// (plane, row, col) = (plane s + row) s + col, its corner 0 at node
// (plane (s+1) + row)(s+1) + col), an element kernel's block covers
// kRows x kCols elements of one plane.  Their corners are the
// 2 x (kRows+1) x (kCols+1) nodes of the tile, which the block loads once
// into shared memory, coalesced along the rows, instead of gathering eight
// corners per element from global memory.  The element arithmetic is
// unchanged, so a tiled kernel gives the same bits as the gathering one.
//
// A cube may be one instance of a batched ensemble: its elements and nodes
// then start at offsets into the ensemble's flat arrays (elem_base,
// node_base), and tile t is the t-th tile of that instance.
#pragma once

#include "common.cuh"

namespace lulesh {

constexpr int kTileCols = 64;

// The tile of a block: plane p, first element row r0 and column c0.
struct TileCoord {
    int p, r0, c0;
};

template <int ROWS>
struct TileShape {
    static constexpr int kRows = ROWS;
    static constexpr int kCols = kTileCols;
    static constexpr int kNodeCols = kCols + 1, kNodeRows = ROWS + 1;
    static constexpr int kNodes = 2 * kNodeRows * kNodeCols;
    static constexpr int kThreads = ROWS * kCols;

    // Tiles of an s^3 cube.
    static __host__ __device__ long tiles(int s)
    {
        return (long)s * ((s + ROWS - 1) / ROWS) * ((s + kCols - 1) / kCols);
    }

    // Tile t of the cube.
    static __device__ TileCoord coord(int s, long t)
    {
        const int nbc = (s + kCols - 1) / kCols, nbr = (s + ROWS - 1) / ROWS;
        const int cb = (int)(t % nbc), rb = (int)((t / nbc) % nbr), p = (int)(t / ((long)nbc * nbr));
        return {p, rb * ROWS, cb * kCols};
    }

    // This thread's element of the tile (numbered within its cube): false
    // when the tile reaches past the cube's edge.
    static __device__ bool element(int s, TileCoord t, int &k, int &rr, int &cc)
    {
        rr = threadIdx.x / kCols;
        cc = threadIdx.x % kCols;
        const int r = t.r0 + rr, c = t.c0 + cc;
        if (rr >= ROWS || r >= s || c >= s) return false;
        k = (t.p * s + r) * s + c;
        return true;
    }

    // The places of an element's corners in the tile, in the reference's
    // corner order (LULESH-OMP.cc:3023-3040).
    static __device__ void corners(int rr, int cc, int li[8])
    {
        const int b = rr * kNodeCols + cc, up = kNodeRows * kNodeCols;
        li[0] = b;
        li[1] = b + 1;
        li[2] = b + kNodeCols + 1;
        li[3] = b + kNodeCols;
        li[4] = b + up;
        li[5] = b + up + 1;
        li[6] = b + up + kNodeCols + 1;
        li[7] = b + up + kNodeCols;
    }

    // Fields lo..hi-1 of the tile's nodes into tile[f * kNodes + i]; get(f)
    // is field f's global array, node_base the cube's first node in it.
    // Every thread of the block takes part.
    template <typename T, class Get>
    static __device__ void load(T *tile, int s, TileCoord t, long node_base, int lo, int hi, Get get)
    {
        const int en = s + 1;
        for (int i = threadIdx.x; i < kNodes; i += blockDim.x) {
            const int dc = i % kNodeCols, dr = (i / kNodeCols) % kNodeRows;
            const int dp = i / (kNodeCols * kNodeRows);
            const int r = t.r0 + dr, c = t.c0 + dc;
            if (r > s || c > s) continue;
            const long n = node_base + ((long)(t.p + dp) * en + r) * en + c;
            for (int f = lo; f < hi; ++f) tile[f * kNodes + i] = __ldg(get(f) + n);
        }
    }
};

// The single-instance staged kernels' tile: 2 x 64 elements.
using SoloTile = TileShape<2>;

}  // namespace lulesh
