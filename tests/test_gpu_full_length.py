"""The headline configurations at their full length, against the reference.

The fixture ``tests/golden/reference_runs.json`` holds the unmodified
reference step's (reference/C/LULESH-OMP.cc, LULESH 2.0 initial conditions)
answers, made by ``tests/golden/make_reference_runs.py``:

* s=192 after exactly 500 cycles (the plain FP64 and split-precision
  headline runs): cycle count, time, origin energy, the plane-0 symmetry of
  LULESH-OMP.cc:3197-3223, and the whole-problem results (total energy,
  largest nodal speed, viscosity-weighted shock radius);
* every instance of the seeded FP64 ensemble (64 instances, s in 16..64) and
  of the seeded split ensemble (512 instances, s in 8..48, and its s=96
  instances), each run to t = 1e-2 from its scaled initial energy.

Bars: plain FP64 reproduces the cycle count, the origin energy within 1e-10
and the time within 1e-12 (relative); split precision keeps every result
within 1e-6 of the reference.
"""
from __future__ import annotations

import json

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

FP64_ENERGY_TOL = 1e-10
FP64_TIME_TOL = 1e-12
FP64_RESULT_TOL = 1e-10   # total energy, max |v|, shock radius
SPLIT_TOL = 1e-6
# Plane-0 symmetry at s=192 after 500 cycles.  The reference's own
# MaxRelDiff there is 7.4e-12, one realisation of FP64 rounding noise in the
# elements just ahead of the shock front, whose energies are tiny; the
# library's all-IEEE-FP64 kernels (the same quantities through the Walsh-mode
# formulas) measure 1.7e-10 on the same problem, the default double-float
# kernels 2.6e-10.  The bar is 1e-9: symmetric to rounding noise at this
# size, for both arithmetics.
S192_SYMM_BAR = 1e-9


@pytest.fixture(scope="module")
def ref_runs():
    p = GOLDEN / "reference_runs.json"
    if not p.exists():
        pytest.skip("tests/golden/reference_runs.json is absent")
    return json.loads(p.read_text())


@pytest.fixture(scope="module")
def ensembles():
    return json.loads((GOLDEN / "ensembles.json").read_text())


@pytest.fixture(scope="module")
def mesh192(pkg):
    return pkg.mesh_build(192, pkg.INIT_V2)


def _headline(pkg, mesh, precision, ref):
    with pkg.Lulesh(192, pkg.INIT_V2, precision) as g:
        n = g.run(ref["cycles"])
        got = pkg.sedov_metrics(g, mesh)
        sc = g.scalars
        sym = g.symmetry()
    return n, sc, got, sym


@pytest.mark.parametrize("arith", ["fp64", "fp64_ieee"])
def test_fp64_s192_500_cycles_matches_reference(pkg, ref_runs, mesh192, arith):
    ref = ref_runs["s192_c500"]
    assert ref["cycles"] == 500
    prec = {"fp64": pkg.FP64, "fp64_ieee": pkg.FP64_IEEE}[arith]
    n, sc, got, sym = _headline(pkg, mesh192, prec, ref)
    assert n == sc.cycle == 500
    assert abs(sc.time - ref["time"]) <= FP64_TIME_TOL * ref["time"]
    assert abs(sc.deltatime - ref["deltatime"]) <= FP64_TIME_TOL * ref["deltatime"]
    err = pkg.relative_errors(got, {k: ref[k] for k in got})
    assert err["origin_energy"] <= FP64_ENERGY_TOL, err
    for k in ("total_energy", "max_velocity", "shock_radius"):
        assert err[k] <= FP64_RESULT_TOL, (k, err)
    # the reference's symmetry test
    assert sym[2] <= S192_SYMM_BAR, (sym, ref["max_rel_diff"])


def test_split_s192_500_cycles_within_bar(pkg, ref_runs, mesh192):
    ref = ref_runs["s192_c500"]
    n, sc, got, _ = _headline(pkg, mesh192, pkg.SPLIT, ref)
    assert n == 500
    err = pkg.relative_errors(got, {k: ref[k] for k in got})
    for k, e in err.items():
        assert e <= SPLIT_TOL, (k, err)
    assert abs(sc.time - ref["time"]) <= SPLIT_TOL * ref["time"]


def _run_ensemble(pkg, ens, name, precision):
    sizes, scale = ens[name]["sizes"], ens[name]["e0_scale"]
    with pkg.Batch(sizes, scale, pkg.INIT_V2, precision) as b:
        b.run()
        return [b.instance(i) for i in range(b.n)]


def test_fp64_ensemble_every_instance_matches_reference(pkg, ref_runs, ensembles):
    """Config 3: 64 instances in one FP64 batch; each against the reference's
    own run of it."""
    refs = ref_runs.get("c3", [])
    if len(refs) < len(ensembles["c3"]["sizes"]):
        pytest.skip("the c3 reference answers are incomplete")
    final = _run_ensemble(pkg, ensembles, "c3", pkg.FP64)
    bad = []
    for r in refs:
        sc, e0, status = final[r["index"]]
        assert status == pkg.OK
        err = abs(e0 - r["origin_energy"]) / abs(r["origin_energy"])
        if sc.cycle != r["cycles"] or err > FP64_ENERGY_TOL or \
                abs(sc.time - r["time"]) > FP64_TIME_TOL * r["time"]:
            bad.append((r["index"], r["s"], sc.cycle, r["cycles"], err))
    assert not bad, bad


def test_split_ensemble_every_instance_within_bar(pkg, ref_runs, ensembles):
    """Config 4: 528 instances in one split-precision batch; every instance
    the reference ran keeps its origin energy within 1e-6 of the reference."""
    refs = ref_runs.get("c4", [])
    small = sum(1 for s in ensembles["c4"]["sizes"] if s <= 48)
    if len([r for r in refs if r["s"] <= 48]) < small:
        pytest.skip("the c4 reference answers are incomplete")
    final = _run_ensemble(pkg, ensembles, "c4", pkg.SPLIT)
    errs = []
    for r in refs:
        sc, e0, status = final[r["index"]]
        assert status == pkg.OK
        errs.append((abs(e0 - r["origin_energy"]) / abs(r["origin_energy"]), r["index"], r["s"]))
    worst = max(errs)
    assert worst[0] <= SPLIT_TOL, worst
    assert np.median([e for e, _, _ in errs]) < SPLIT_TOL / 10
