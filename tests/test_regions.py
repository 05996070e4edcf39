"""LULESH 2.0 regions on the CPU: the library's restatement of the region
assignment against the unmodified reference's (lulesh-2.0.3,
Domain::CreateRegionIndexSets), and the reference's own answers, which
regions do not change."""
from __future__ import annotations

import json

import numpy as np
import pytest

from conftest import GOLDEN, find_run

REGIONS = json.loads((GOLDEN / "regions.json").read_text())


def _expand(runs):
    return np.concatenate([np.full(n, r, dtype=np.int32) for r, n in runs])


@pytest.mark.parametrize("case", REGIONS["assignments"], ids=lambda c: f"s{c['s']}-r{c['num_regions']}-b{c['balance']}")
def test_assignment_matches_reference(pkg, case):
    ref = _expand(case["runs"])
    got = pkg.region_numbers(len(ref), case["num_regions"], case["balance"])
    np.testing.assert_array_equal(got, ref)


def test_single_region(pkg):
    assert (pkg.region_numbers(1000, 1, 1) == 1).all()


@pytest.mark.parametrize("args", [(100, 0, 1), (100, 11, -1), (100, 40, 7)])
def test_bad_region_arguments(pkg, args):
    with pytest.raises(pkg.LuleshError) as e:
        pkg.region_numbers(*args)
    assert e.value.code == pkg.ERR_ARG


def test_regions_do_not_change_the_reference_answer(answers):
    base = find_run(answers, 30, "v2", 0)
    for a in REGIONS["answers"]:
        assert a["cycles"] == base["cycles"]
        assert a["origin_energy_printed"] == float(f"{base['origin_energy']:.6e}")
