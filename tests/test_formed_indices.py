"""Indices the kernels form arithmetically instead of loading, restated in
numpy (CPU) and checked against the host mesh the reference's set-up
builds:

* the material kernels' face neighbours on the structured cube
  (``face_neighbours`` in csrc/common.cuh): k -+ 1, k -+ s, k -+ s^2 equal
  the mesh's lxim..lzetap on every face without a boundary flag -- the only
  faces whose neighbour the monotonic limiter reads;
* the batched staged force kernel's walk over a class's tiles
  (``kb_force_split_staged``): the binary search over the instances' first
  tiles puts every tile in the instance that owns it, and the tiles of all
  instances are visited once each."""
from __future__ import annotations

import numpy as np
import pytest

# elem_bc fields of the six faces (LULESH-OMP.cc:532-554): any bit set in a
# face's field means the face is a boundary (symmetry or free)
XI_M, XI_P = 0x003, 0x00C
ETA_M, ETA_P = 0x030, 0x0C0
ZETA_M, ZETA_P = 0x300, 0xC00


@pytest.mark.parametrize("s", [1, 2, 3, 6, 9])
def test_face_neighbours_on_interior_faces(pkg, s):
    m = pkg.mesh_build(s, pkg.INIT_V2)
    k = np.arange(s ** 3)
    bc = m["elem_bc"]
    for name, mask, formed in (("lxim", XI_M, k - 1), ("lxip", XI_P, k + 1),
                               ("letam", ETA_M, k - s), ("letap", ETA_P, k + s),
                               ("lzetam", ZETA_M, k - s * s), ("lzetap", ZETA_P, k + s * s)):
        interior = (bc & mask) == 0
        assert np.array_equal(m[name][interior], formed[interior]), name
        # a boundary face always carries a flag: the formed index is never read there
        edge = {"lxim": k % s == 0, "lxip": k % s == s - 1, "letam": (k // s) % s == 0,
                "letap": (k // s) % s == s - 1, "lzetam": k // (s * s) == 0, "lzetap": k // (s * s) == s - 1}[name]
        assert np.all((bc & mask)[edge] != 0), name


def tiles(s, rows, cols=64):
    return s * ((s + rows - 1) // rows) * ((s + cols - 1) // cols)


@pytest.mark.parametrize("rows", [2, 4])
def test_staged_tile_walk(rows):
    sizes = [64, 65, 70, 96, 64, 131]
    begin = np.concatenate([[0], np.cumsum([tiles(s, rows) for s in sizes])])
    total = begin[-1]
    seen = np.zeros(total, dtype=np.int64)
    for t in range(total):
        lo, hi = 0, len(sizes) - 1          # the kernel's search, as written there
        while lo < hi:
            mid = (lo + hi + 1) // 2
            if begin[mid] <= t:
                lo = mid
            else:
                hi = mid - 1
        assert begin[lo] <= t < begin[lo + 1]
        local = t - begin[lo]
        assert 0 <= local < tiles(sizes[lo], rows)
        seen[t] += 1
    assert np.all(seen == 1)
