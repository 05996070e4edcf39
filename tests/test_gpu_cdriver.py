"""The C ABI from C: the driver in driver/lulesh_gb300_main.c links the
library through include/lulesh_gb300.h only and prints the reference's
result lines."""
from __future__ import annotations

import json
import subprocess

import pytest

from conftest import ROOT, find_run

pytestmark = pytest.mark.gpu

EXE = ROOT / "lulesh-accelerate_gb300" / "lulesh_gb300_main"


def _run(*args):
    r = subprocess.run([str(EXE), *map(str, args)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    return r.stdout, json.loads(r.stdout.strip().splitlines()[-1])


@pytest.mark.parametrize("mode", [[], ["--calls"]])
def test_c_driver_reproduces_published_table(pkg, answers, mode):
    out, res = _run(10, "--init", "v1", *mode)
    assert "Iteration count     =  593" in out
    assert "Final Origin Energy = 5.174622e+05" in out
    assert res["cycles"] == 593


def test_c_driver_sedov30(pkg, answers):
    ref = find_run(answers, 30, "v2", 0)
    _, res = _run(30)
    assert res["cycles"] == ref["cycles"]
    assert abs(res["origin_energy"] - ref["origin_energy"]) <= 1e-10 * ref["origin_energy"]
