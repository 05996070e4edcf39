"""The visualisation dump on the host (no GPU): lulesh_write_domain takes
the reference's writeDomain arguments (cbits/visit.cc:149-177) and writes
the same content -- connectivity, coordinates, time and cycle, e p v q,
xd yd zd and speed -- as a raw structure-of-arrays file."""
from __future__ import annotations

import numpy as np
import pytest


def _fields(pkg, s, seed=0):
    rng = np.random.default_rng(seed)
    ne, nn = pkg.mesh_sizes(s)
    return {k: rng.normal(size=nn if k in ("x", "y", "z", "xd", "yd", "zd") else ne)
            for k in ("x", "y", "z", "xd", "yd", "zd", "e", "p", "v", "q")}


def test_write_and_read_back(pkg, tmp_path):
    s = 3
    f = _fields(pkg, s)
    pkg.write_domain(tmp_path / "sedov_%04d.lgb", s, 17, 2.5e-3, f)
    d = pkg.read_domain_file(tmp_path / "sedov_0017.lgb")
    assert (d["s"], d["num_elem"], d["num_node"], d["step"], d["time"]) == (3, 27, 64, 17, 2.5e-3)
    np.testing.assert_array_equal(d["connectivity"], pkg.mesh_build(s, pkg.INIT_V2)["nodelist"])
    for mine, k in (("X", "x"), ("Y", "y"), ("Z", "z"), ("xd", "xd"), ("yd", "yd"), ("zd", "zd"),
                    ("e", "e"), ("p", "p"), ("v", "v"), ("q", "q")):
        np.testing.assert_array_equal(d[mine], f[k])
    np.testing.assert_allclose(d["speed"], np.sqrt(f["xd"] ** 2 + f["yd"] ** 2 + f["zd"] ** 2), rtol=1e-15)


@pytest.mark.parametrize("pattern", ["out_%s", "out_%d_%d", "out_%x", "out_%100d"])
def test_bad_patterns_are_rejected(pkg, tmp_path, pattern):
    with pytest.raises(pkg.LuleshError) as e:
        pkg.write_domain(tmp_path / pattern, 2, 0, 0.0, _fields(pkg, 2))
    assert e.value.code == pkg.ERR_ARG


def test_plain_name_and_percent(pkg, tmp_path):
    pkg.write_domain(tmp_path / "final%%.lgb", 2, 5, 0.0, _fields(pkg, 2))
    assert pkg.read_domain_file(tmp_path / "final%.lgb")["step"] == 5
