"""Shared fixtures.  GPU tests carry ``@pytest.mark.gpu``; the rest run on CPU."""
from __future__ import annotations

import json
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
GOLDEN = ROOT / "tests" / "golden"
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300)")
    config.addinivalue_line("markers", "slow: long-running")


@pytest.fixture(scope="session")
def pkg():
    import __graft_entry__ as ge

    ge._load_build_module().build()
    return ge.load_package()


@pytest.fixture(scope="session")
def orc():
    import oracle

    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def answers():
    return json.loads((GOLDEN / "known_answers.json").read_text())


def find_run(answers, s, init, cap=0):
    for r in answers["runs"]:
        if r["s"] == s and r["init"] == init and r["cap"] == cap:
            return r
    raise KeyError((s, init, cap))


def load_phases(s, cyc, mesh=None):
    z = np.load(GOLDEN / (f"phases_{mesh}_c{cyc}.npz" if mesh else f"phases_s{s}_c{cyc}.npz"))
    stages = {}
    for key in z.files:
        st, name = key.split("/")
        stages.setdefault(st, {})[name] = z[key]
    return stages


def rel_err(a, b, scale=0.0):
    """max |a-b| / max(max |b|, scale) (0 when both are zero).

    ``scale`` is the natural magnitude of a field that is a difference of
    larger quantities (delv = vnew - v is compared on the scale of vnew)."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    scale = max(np.max(np.abs(b)) if b.size else 0.0, scale)
    d = np.max(np.abs(a - b)) if b.size else 0.0
    return 0.0 if d == 0.0 else d / max(scale, 1e-300)
