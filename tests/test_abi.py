"""The C ABI on CPU: the library loads, exports every declared symbol, builds
the host mesh exactly as the reference does, and refuses to run without a
GPU (there is no CPU fallback)."""
from __future__ import annotations

import ctypes as C
import re

import numpy as np
import pytest

from conftest import ROOT


def declared_functions():
    text = (ROOT / "include" / "lulesh_gb300.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(lulesh_[a-z0-9_]+)\s*\(", text)))


def test_every_declared_symbol_is_exported(pkg):
    lib = pkg.load_library()
    names = declared_functions()
    assert len(names) >= 25
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_default_params_are_the_reference_constants(pkg, orc):
    p = pkg.default_parameters()
    o = orc.Oracle(4)
    ref = o.params
    for name, _ in pkg.Parameters._fields_:
        assert getattr(p, name) == getattr(ref, name), name


@pytest.mark.parametrize("s,init", [(1, 2), (3, 1), (7, 2), (12, 2)])
def test_host_mesh_matches_reference_setup(pkg, orc, s, init):
    m = pkg.mesh_build(s, init)
    o = orc.Oracle(s, init)
    pairs = {"x": "x", "y": "y", "z": "z", "volo": "volo", "elem_mass": "elemMass",
             "nodal_mass": "nodalMass", "nodelist": "nodelist", "node_elem_start": "nodeElemStart",
             "node_elem_count": "nodeElemCount", "node_elem_corner_list": "nodeElemCornerList",
             "lxim": "lxim", "lxip": "lxip", "letam": "letam", "letap": "letap", "lzetam": "lzetam",
             "lzetap": "lzetap", "elem_bc": "elemBC"}
    for mine, ref in pairs.items():
        assert np.array_equal(m[mine], o.field(ref)), mine
    assert m["e0"] == o.field("e")[0]
    assert m["dt0"] == o.scalar("deltatime")


def test_bad_sizes_are_rejected(pkg):
    with pytest.raises(pkg.LuleshError) as ei:
        pkg.mesh_sizes(0)
    assert ei.value.code == pkg.ERR_ARG
    with pytest.raises(pkg.LuleshError):
        pkg.mesh_sizes(100000)
    assert pkg.mesh_sizes(192) == (192 ** 3, 193 ** 3)


def _have_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.mark.skipif(_have_gpu(), reason="checks the no-GPU behaviour")
def test_create_fails_loudly_without_gpu(pkg):
    with pytest.raises(pkg.LuleshError) as ei:
        pkg.Lulesh(4)
    assert ei.value.code == pkg.ERR_CUDA


def test_ensemble_fixture_is_the_seeded_draw(pkg):
    """tests/golden/ensembles.json holds the seeded draws of the batched
    configurations (c3: 64 instances s in 16..64, seed 0; c4: 512 in 8..48
    plus 16 at s=96, seed 1; energy factors log-uniform in [0.5, 2])."""
    import json

    fx = json.loads((ROOT / "tests" / "golden" / "ensembles.json").read_text())
    s3, f3 = pkg.ensemble(0, 64, 16, 64)
    assert fx["c3"]["sizes"] == s3.tolist() and fx["c3"]["e0_scale"] == f3.tolist()
    s4, f4 = pkg.ensemble(1, 512, 8, 48, (96,) * 16)
    assert fx["c4"]["sizes"] == s4.tolist() and fx["c4"]["e0_scale"] == f4.tolist()
    assert all(16 <= s <= 64 for s in s3) and all(0.5 <= f <= 2.0 for f in f3)
    assert s4[-16:].tolist() == [96] * 16 and all(8 <= s <= 48 for s in s4[:512])
