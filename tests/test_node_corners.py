"""The node-to-corner order of the structured cube, formed arithmetically by
the node update kernels (``for_node_corners`` in csrc/common.cuh), restated
here (CPU) and checked against the host mesh's node-to-corner lists, which
follow the reference's AllocateNodeElemIndexes (LULESH-OMP.cc:209-268):
every node's corners, in the same order (the order in which the node's
force sum is accumulated)."""
from __future__ import annotations

import numpy as np
import pytest

# corner of an element at offset (dp, dr, dc) from its first node, in the
# reference's corner order (LULESH-OMP.cc:3023-3040)
CORNER_OF = [[[0, 1], [3, 2]], [[4, 5], [7, 6]]]


def node_corners(s, n):
    """8 * element + corner of node n's corners, as the kernels form them."""
    en = s + 1
    c, r, p = n % en, (n // en) % en, n // (en * en)
    out = []
    for dp in (1, 0):
        for dr in (1, 0):
            for dc in (1, 0):
                ep, er, ec = p - dp, r - dr, c - dc
                if not (0 <= ep < s and 0 <= er < s and 0 <= ec < s):
                    continue
                e = (ep * s + er) * s + ec
                out.append(8 * e + CORNER_OF[dp][dr][dc])
    return out


@pytest.mark.parametrize("s", [1, 2, 3, 5, 8])
def test_arithmetic_corners_are_the_reference_lists(pkg, s):
    m = pkg.mesh_build(s, pkg.INIT_V2)
    start, count, lst = m["node_elem_start"], m["node_elem_count"], m["node_elem_corner_list"]
    for n in range((s + 1) ** 3):
        want = list(lst[start[n]:start[n] + count[n]])
        assert node_corners(s, n) == want, n
