"""Pin the oracle restatement before trusting it as the checker.

(a) against the reference's published known answers (lulesh-ports.pdf
section 6.2, Tab. 2, LULESH 1.0 initialisation), and
(b) against golden vectors produced by the unmodified reference step
functions (tests/golden/make_golden.py): full-run answers and the state
after every phase of one cycle.

The oracle and the reference build are both compiled with
-ffp-contract=off, so on the same machine class they agree bit for bit.
"""
from __future__ import annotations

import platform

import numpy as np
import pytest

from conftest import find_run, load_phases, rel_err

# bitwise on the machine that generated the fixtures; last-place slack on
# other hosts (libm's cbrt may round differently)
EXACT = platform.machine() in ("x86_64", "AMD64")
TOL = 0.0 if EXACT else 1e-13


def _close(a, b, tol=TOL):
    if tol == 0.0:
        return np.array_equal(np.asarray(a), np.asarray(b))
    return rel_err(a, b) <= tol


@pytest.mark.parametrize("s", [5, 10])
def test_published_table_v1(orc, answers, s):
    o = orc.Oracle(s, orc.INIT_V1)
    rc, _ = o.run()
    assert rc == 0
    cycles, energy = answers["published_v1"][str(s)]
    assert o.cycle == cycles
    # the table prints 7 significant digits
    assert float(f"{o.field('e')[0]:.6e}") == energy


@pytest.mark.parametrize("s,init,cap", [(1, "v1", 0), (2, "v1", 0), (3, "v1", 0), (1, "v2", 0),
                                        (2, "v2", 0), (3, "v2", 0),
                                        (5, "v1", 0), (10, "v1", 0), (4, "v2", 0), (5, "v2", 0),
                                        (8, "v2", 0), (10, "v2", 0), (16, "v2", 0), (30, "v2", 100),
                                        (30, "v2", 0)])
def test_oracle_matches_reference_runs(orc, answers, s, init, cap):
    ref = find_run(answers, s, init, cap)
    o = orc.Oracle(s, orc.INIT_V1 if init == "v1" else orc.INIT_V2)
    rc, _ = o.run(cap)
    assert rc == 0
    assert o.cycle == ref["cycles"]
    assert _close(o.field("e")[0], ref["origin_energy"])
    for k in ("time", "deltatime", "dtcourant", "dthydro"):
        assert _close(o.scalar(k), ref[k]), k
    ma, ta, mr = o.symmetry()
    assert _close(ma, ref["max_abs_diff"], max(TOL, 1e-9))
    assert _close(mr, ref["max_rel_diff"], max(TOL, 1e-9))


def test_reference_reproduces_published_table(answers):
    """The reference build itself reproduces Tab. 2 (s = 5, 10, 45)."""
    for s in (5, 10, 45):
        ref = find_run(answers, s, "v1", 0)
        cycles, energy = answers["published_v1"][str(s)]
        assert ref["cycles"] == cycles
        assert float(f"{ref['origin_energy']:.6e}") == energy


STAGE_FIELDS = {
    "lagrange_nodal": ("x", "y", "z", "xd", "yd", "zd", "fx", "fy", "fz"),
    "lagrange_elements": ("e", "p", "q", "ql", "qq", "v", "vnew", "delv", "vdov", "arealg", "ss",
                          "delv_xi", "delv_eta", "delv_zeta", "delx_xi", "delx_eta", "delx_zeta"),
}


@pytest.mark.parametrize("s,cyc", [(5, 0), (6, 40), (10, 150)])
def test_oracle_phases_match_reference(orc, s, cyc):
    st = load_phases(s, cyc)
    o = orc.Oracle(s, orc.INIT_V2)
    if cyc:
        rc, _ = o.run(cyc)
        assert rc == 0
    for k in ("x", "xd", "e", "p", "q", "v", "ss"):
        assert _close(o.field(k), st["start"][k]), k
    o.time_increment()
    for k in ("time", "deltatime"):
        assert _close(o.scalar(k), st["time_increment"][k]), k
    assert o.lagrange_nodal() == 0
    for k in STAGE_FIELDS["lagrange_nodal"]:
        assert _close(o.field(k), st["lagrange_nodal"][k]), k
    assert o.lagrange_elements() == 0
    for k in STAGE_FIELDS["lagrange_elements"]:
        assert _close(o.field(k), st["lagrange_elements"][k]), k
    o.time_constraints()
    for k in ("dtcourant", "dthydro"):
        assert _close(o.scalar(k), st["time_constraints"][k]), k


def test_oracle_error_codes(orc):
    """VolumeError / QStopError (LULESH-OMP.cc:82) are returned, not exit()ed."""
    o = orc.Oracle(5, orc.INIT_V2)
    o.params.qstop = 1e-30
    rc, _ = o.run(20)
    assert rc == orc.QSTOP_ERROR
    o = orc.Oracle(5, orc.INIT_V2)
    x = o.field("x")
    x[0] = 10.0            # fold element 0 inside out
    rc, _ = o.run(1)
    assert rc == orc.VOLUME_ERROR
