"""The staged-tile index arithmetic of csrc/tile.cuh (TileShape<ROWS>)
restated in numpy (CPU): for cube edges around and above the tile width and
both staging depths, the tiles cover every element of the cube exactly once,
every node a tile loads lies inside the cube, and each element's eight
corner slots in the tile hold exactly its eight corner nodes of the
reference's numbering (LULESH-OMP.cc:3023-3040).  This checks the arithmetic
before any kernel runs it; the GPU tests compare the staged kernels' results
with the gathering ones."""
from __future__ import annotations

import numpy as np
import pytest

COLS = 64


def tiles(s, rows):
    return s * ((s + rows - 1) // rows) * ((s + COLS - 1) // COLS)


def coord(s, rows, t):
    nbc, nbr = (s + COLS - 1) // COLS, (s + rows - 1) // rows
    return t // (nbc * nbr), ((t // nbc) % nbr) * rows, (t % nbc) * COLS


def element(s, rows, p, r0, c0, tid):
    rr, cc = tid // COLS, tid % COLS
    r, c = r0 + rr, c0 + cc
    ok = (rr < rows) & (r < s) & (c < s)
    return ok, (p * s + r) * s + c, rr, cc


def tile_nodes(s, rows, p, r0, c0):
    """Global node of each tile slot (-1 where the slot is past the edge)."""
    ncol, nrow = COLS + 1, rows + 1
    i = np.arange(2 * nrow * ncol)
    dc, dr, dp = i % ncol, (i // ncol) % nrow, i // (ncol * nrow)
    r, c = r0 + dr, c0 + dc
    en = s + 1
    n = ((p + dp) * en + r) * en + c
    return np.where((r > s) | (c > s), -1, n)


def corners(rows, rr, cc):
    ncol, up = COLS + 1, (rows + 1) * (COLS + 1)
    b = rr * ncol + cc
    return np.stack([b, b + 1, b + ncol + 1, b + ncol, b + up, b + up + 1, b + up + ncol + 1, b + up + ncol], -1)


def reference_corners(s, k):
    en = s + 1
    p, rem = divmod(k, s * s)
    r, c = divmod(rem, s)
    n0 = (p * en + r) * en + c
    return np.stack([n0, n0 + 1, n0 + en + 1, n0 + en,
                     n0 + en * en, n0 + en * en + 1, n0 + en * en + en + 1, n0 + en * en + en], -1)


@pytest.mark.parametrize("rows", [2, 4])
@pytest.mark.parametrize("s", [64, 65, 70, 96, 131])
def test_tiles_cover_the_cube(s, rows):
    seen = np.zeros(s ** 3, dtype=np.int64)
    tid = np.arange(rows * COLS)
    nn = (s + 1) ** 3
    for t in range(tiles(s, rows)):
        p, r0, c0 = coord(s, rows, t)
        assert 0 <= p < s
        nodes = tile_nodes(s, rows, p, r0, c0)
        assert nodes.max() < nn
        ok, k, rr, cc = element(s, rows, p, r0, c0, tid)
        k, rr, cc = k[ok], rr[ok], cc[ok]
        np.add.at(seen, k, 1)
        slots = corners(rows, rr, cc)
        got = nodes[slots]
        assert np.all(got >= 0)
        assert np.array_equal(got, reference_corners(s, k))
    assert np.all(seen == 1)
