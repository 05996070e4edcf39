"""Unstructured meshes on the CPU: the oracle against the reference's own
results on the reference's .lmesh inputs, and the library's mesh reader and
argument checks (which run before any device call)."""
from __future__ import annotations

import ctypes as C
import gzip
import json

import numpy as np
import pytest

from conftest import GOLDEN

UNSTRUCTURED = json.loads((GOLDEN / "unstructured.json").read_text())
# xyz.asc prints 10 decimals: half a unit of the last place, plus room for the
# last bits of two FP64 runs that sum node forces in different orders
PRINTED = 0.5e-10 + 1e-13


def mesh_of(orc, name):
    return orc.read_lmesh(GOLDEN / f"{name}.lmesh.gz")


def plain_lmesh(tmp_path, name):
    p = tmp_path / f"{name}.lmesh"
    p.write_bytes(gzip.decompress((GOLDEN / f"{name}.lmesh.gz").read_bytes()))
    return p


@pytest.mark.parametrize("name,ne,nn", [("sedov15oct", 875, 1126), ("sedov21oct", 31408, 34446)])
def test_lmesh_contents(orc, name, ne, nn):
    m = mesh_of(orc, name)
    assert (m["nelem"], m["nnode"]) == (ne, nn)
    assert m["nodelist"].shape == (8 * ne,) and m["nodelist"].min() >= 0 and m["nodelist"].max() < nn
    for k in ("lxim", "lxip", "letam", "letap", "lzetam", "lzetap"):
        assert m[k].min() >= 0 and m[k].max() < ne
    assert all(len(m[k]) > 0 for k in ("symm_x", "symm_y", "symm_z", "free_surf"))


def test_oracle_matches_reference_sedov15oct(orc):
    ref = UNSTRUCTURED["meshes"]["sedov15oct"]
    o = orc.Oracle.from_mesh(mesh_of(orc, "sedov15oct"))
    assert o.origin == ref["origin_elem"]
    rc, _ = o.run()
    assert rc == 0
    assert o.cycle == ref["cycles"]
    assert o.field("e")[o.origin] == ref["origin_energy"]           # bit for bit
    for k in ("deltatime", "dtcourant", "dthydro"):
        assert o.scalar(k) == ref[k]


def test_oracle_phases_sedov15oct(orc):
    z = np.load(GOLDEN / "phases_sedov15oct_c80.npz")
    o = orc.Oracle.from_mesh(mesh_of(orc, "sedov15oct"))
    assert o.run(80)[0] == 0
    stages = [("start", None), ("time_increment", o.time_increment), ("lagrange_nodal", o.lagrange_nodal),
              ("lagrange_elements", o.lagrange_elements), ("time_constraints", o.time_constraints)]
    for st, fn in stages:
        if fn is not None:
            assert (fn() or 0) == 0
        for k in ("x", "y", "z", "xd", "yd", "zd", "e", "p", "q", "v", "ss", "vdov", "arealg"):
            np.testing.assert_array_equal(o.field(k), z[f"{st}/{k}"], err_msg=f"{st}/{k}")
        assert o.scalar("deltatime") == z[f"{st}/deltatime"]


def test_reference_reproduces_published_solution():
    """The reference's own run on sedov21oct wrote xyz.asc (10 decimals); the
    reference's step functions on our set-up of that mesh agree with it to
    the printed precision."""
    r = UNSTRUCTURED["meshes"]["sedov21oct"]
    assert r["kepler_max_abs_diff"] <= PRINTED
    np.testing.assert_allclose(np.array(r["ref_sample"]), np.array(r["kepler_sample"]), rtol=0, atol=PRINTED)


def test_oracle_sedov21oct_against_published_solution(orc):
    r = UNSTRUCTURED["meshes"]["sedov21oct"]
    o = orc.Oracle.from_mesh(mesh_of(orc, "sedov21oct"))
    assert o.run()[0] == 0
    assert o.cycle == r["cycles"]
    assert o.field("e")[o.origin] == r["origin_energy"]
    idx = np.array(r["sample_nodes"])
    got = np.stack([o.field(k)[idx] for k in ("x", "y", "z")], 1)
    np.testing.assert_array_equal(got, np.array(r["ref_sample"]))
    np.testing.assert_allclose(got, np.array(r["kepler_sample"]), rtol=0, atol=PRINTED)


def test_oracle_rejects_bad_mesh(orc):
    m = mesh_of(orc, "sedov15oct")
    m["nodelist"] = m["nodelist"].copy()
    m["nodelist"][5] = m["nnode"]
    with pytest.raises(ValueError):
        orc.Oracle.from_mesh(m)


# ---- the library's reader and checks, before any device call -----------------

def _create(pkg, mesh):
    try:
        return pkg.Lulesh.from_mesh(mesh), None
    except pkg.LuleshError as e:
        return None, e


@pytest.mark.parametrize("break_it,needle", [
    (lambda m: m["nodelist"].__setitem__(3, -1), "nodelist index out of range"),
    (lambda m: m["lxip"].__setitem__(7, 875), "face neighbour out of range"),
    (lambda m: m["symm_y"].__setitem__(0, 1126), "node set index out of range"),
    (lambda m: m["free_surf"].__setitem__(0, -5), "node set index out of range"),
])
def test_library_rejects_bad_mesh(pkg, orc, break_it, needle):
    m = mesh_of(orc, "sedov15oct")
    m = {k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in m.items()}
    break_it(m)
    ctx, err = _create(pkg, m)
    assert ctx is None and err.code == pkg.ERR_ARG and needle in str(err)


def test_library_rejects_orphan_node(pkg, orc):
    m = mesh_of(orc, "sedov15oct")
    m = dict(m)
    for k in ("x", "y", "z"):
        m[k] = np.append(m[k], 9.0)
    _, err = _create(pkg, m)
    assert err.code == pkg.ERR_ARG and "belongs to no element" in str(err)


def test_library_lmesh_reader(pkg, tmp_path):
    good = plain_lmesh(tmp_path, "sedov15oct")
    with pytest.raises(pkg.LuleshError) as e:
        pkg.Lulesh.from_lmesh(tmp_path / "missing.lmesh")
    assert e.value.code == pkg.ERR_ARG and "cannot open" in str(e.value)
    trunc = tmp_path / "trunc.lmesh"
    trunc.write_bytes(good.read_bytes()[: len(good.read_bytes()) // 2])
    with pytest.raises(pkg.LuleshError) as e:
        pkg.Lulesh.from_lmesh(trunc)
    assert e.value.code == pkg.ERR_ARG
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except ImportError:
        has_gpu = False
    if not has_gpu:
        # the file parses and passes the checks; only the device is missing
        with pytest.raises(pkg.LuleshError) as e:
            pkg.Lulesh.from_lmesh(good)
        assert e.value.code == pkg.ERR_CUDA


def test_unstructured_symbols_exported(pkg):
    lib = C.CDLL(str(pkg.library_path()))
    for name in ("lulesh_create_unstructured", "lulesh_create_lmesh", "lulesh_origin_element"):
        assert hasattr(lib, name)
