// tile.cuh -- staging of a structured cube's corner nodes in shared memory.
//
// On the s^3 cube (the reference's node and element numbering: element
// (plane, row, col) = (plane s + row) s + col, its corner 0 at node
// (plane (s+1) + row)(s+1) + col), an element kernel's block covers
// kTileRows x kTileCols elements of one plane.  Their corners are the
// 2 x (kTileRows+1) x (kTileCols+1) nodes of the tile, which the block loads
// once into shared memory, coalesced along the rows, instead of gathering
// eight corners per element from global memory.  The element arithmetic is
// unchanged, so a tiled kernel gives the same bits as the gathering one.
#pragma once

#include "common.cuh"

namespace lulesh {

constexpr int kTileCols = 64, kTileRows = 2;
constexpr int kTileNodeCols = kTileCols + 1, kTileNodeRows = kTileRows + 1;
constexpr int kTileNodes = 2 * kTileNodeRows * kTileNodeCols;
constexpr int kTileThreads = kTileRows * kTileCols;

// Blocks of a tiled launch over the s^3 cube.
inline long tile_blocks(int s)
{
    return (long)s * ((s + kTileRows - 1) / kTileRows) * ((s + kTileCols - 1) / kTileCols);
}

// The tile of this block: plane p, first element row r0 and column c0.
struct TileCoord {
    int p, r0, c0;
};
__device__ __forceinline__ TileCoord tile_coord(int s)
{
    const int nbc = (s + kTileCols - 1) / kTileCols, nbr = (s + kTileRows - 1) / kTileRows;
    const int cb = blockIdx.x % nbc, rb = (blockIdx.x / nbc) % nbr, p = blockIdx.x / (nbc * nbr);
    return {p, rb * kTileRows, cb * kTileCols};
}

// This thread's element: false when the tile reaches past the cube's edge.
__device__ __forceinline__ bool tile_element(int s, TileCoord t, int &k, int &rr, int &cc)
{
    rr = threadIdx.x / kTileCols;
    cc = threadIdx.x % kTileCols;
    const int r = t.r0 + rr, c = t.c0 + cc;
    if (rr >= kTileRows || r >= s || c >= s) return false;
    k = (t.p * s + r) * s + c;
    return true;
}

// The places of an element's corners in the tile, in the reference's corner
// order (LULESH-OMP.cc:3023-3040).
__device__ __forceinline__ void tile_corners(int rr, int cc, int li[8])
{
    const int b = rr * kTileNodeCols + cc, up = kTileNodeRows * kTileNodeCols;
    li[0] = b;
    li[1] = b + 1;
    li[2] = b + kTileNodeCols + 1;
    li[3] = b + kTileNodeCols;
    li[4] = b + up;
    li[5] = b + up + 1;
    li[6] = b + up + kTileNodeCols + 1;
    li[7] = b + up + kTileNodeCols;
}

// Fields lo..hi-1 of the tile's nodes into tile[f * kTileNodes + i]; get(f)
// is field f's global array.  Every thread of the block takes part.
template <typename T, class Get>
__device__ __forceinline__ void load_tile(T *tile, int s, TileCoord t, int lo, int hi, Get get)
{
    const int en = s + 1;
    for (int i = threadIdx.x; i < kTileNodes; i += blockDim.x) {
        const int dc = i % kTileNodeCols, dr = (i / kTileNodeCols) % kTileNodeRows;
        const int dp = i / (kTileNodeCols * kTileNodeRows);
        const int r = t.r0 + dr, c = t.c0 + dc;
        if (r > s || c > s) continue;
        const long n = ((long)(t.p + dp) * en + r) * en + c;
        for (int f = lo; f < hi; ++f) tile[f * kTileNodes + i] = __ldg(get(f) + n);
    }
}

}  // namespace lulesh
