"""LULESH 2.0 regions on the GPU: the per-region EOS repetitions change the
work, never the results, as in the reference (lulesh-2.0.3/lulesh.cc:
2410-2424 repeats an evaluation whose inputs do not change)."""
from __future__ import annotations

import json

import numpy as np
import pytest

from conftest import GOLDEN, find_run

pytestmark = pytest.mark.gpu

REGIONS = json.loads((GOLDEN / "regions.json").read_text())
FIELDS = ("x", "y", "z", "xd", "yd", "zd", "e", "p", "q", "v", "ss")


def _expand(runs):
    return np.concatenate([np.full(n, r, dtype=np.int32) for r, n in runs])


@pytest.mark.parametrize("precision", ["FP64", "SPLIT"])
def test_regions_leave_results_bitwise_unchanged(pkg, precision):
    prec = getattr(pkg, precision)
    n = 150
    with pkg.Lulesh(20, pkg.INIT_V2, prec) as a, pkg.Lulesh(20, pkg.INIT_V2, prec) as b:
        b.set_regions(21, 2, 3)               # rep 1, 4 and 40 evaluations
        assert a.run(n) == n and b.run(n) == n
        for k in FIELDS:
            np.testing.assert_array_equal(a.get_field(k), b.get_field(k), err_msg=k)
        sa, sb = a.scalars, b.scalars
        assert (sa.deltatime, sa.dtcourant, sa.dthydro) == (sb.deltatime, sb.dtcourant, sb.dthydro)


def test_default_regions_reproduce_reference_answer(pkg, answers):
    ref = find_run(answers, 30, "v2", 0)
    with pkg.Lulesh(30, pkg.INIT_V2) as g:
        g.set_regions(11, 1, 1)
        case = next(c for c in REGIONS["assignments"] if (c["s"], c["num_regions"], c["balance"]) == (30, 11, 1))
        np.testing.assert_array_equal(g.regions(), _expand(case["runs"]))
        assert g.run() == ref["cycles"]
        e0 = g.origin_energy()
        assert abs(e0 - ref["origin_energy"]) <= 1e-10 * ref["origin_energy"]
        ma, ta, mr = g.symmetry()
        assert mr <= max(1e-10, 10 * ref["max_rel_diff"])


def test_regions_removed_and_bad_arguments(pkg):
    with pkg.Lulesh(6, pkg.INIT_V2) as g:
        g.set_regions(11, 1, 1)
        assert g.regions().max() == 11
        g.set_regions(0)
        assert (g.regions() == 1).all()
        for bad in ((-1, 1, 1), (11, -1, 1), (11, 1, 101), (11, 1, -2)):
            with pytest.raises(pkg.LuleshError) as e:
                g.set_regions(*bad)
            assert e.value.code == pkg.ERR_ARG
        assert g.run(10) == 10


def test_regions_with_the_step_calls(pkg):
    """Regions apply to the per-call step API as to the run graph."""
    with pkg.Lulesh(10, pkg.INIT_V2) as a, pkg.Lulesh(10, pkg.INIT_V2) as b:
        b.set_regions(11, 1, 1)
        for _ in range(40):
            a.time_increment(); a.lagrange_leapfrog()
            b.time_increment(); b.lagrange_leapfrog()
        for k in FIELDS:
            np.testing.assert_array_equal(a.get_field(k), b.get_field(k), err_msg=k)
