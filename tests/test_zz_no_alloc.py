"""The allocation-free LagrangeNodal entry point against the ordinary one.

lulesh_lagrange_nodal_noalloc exists for callers that cannot allocate GPU
memory themselves -- code whose device arrays come from a host framework's
own pool, or that must not call the allocator while work is in flight.  It
keeps its working memory in one fixed device array inside the library.  This
test calls it through the C ABI on device arrays the test owns and compares
its positions, velocities and nodal forces with lulesh_lagrange_nodal on the
same state, for two calls in a row: the second call finds the first call's
leftovers in the shared array and must not be affected by them.

The file is named so that pytest collects it last.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu

TOL = 1e-12   # the per-phase tolerance of the parity tests (same kernels; the context divides
              # by precomputed reciprocal masses where this call divides: within an ulp)


def _symm_sets(s):
    """The reference's symmetry node sets (LULESH-OMP.cc:3114-3125)."""
    en = s + 1
    i, j = np.meshgrid(np.arange(en), np.arange(en), indexing="ij")
    sx = (i * en * en + j * en).ravel()
    sy = (i * en * en + j).ravel()
    sz = (i * en + j).ravel()
    return [a.astype(np.int32) for a in (sx, sy, sz)]


def test_noalloc_nodal_matches_context_path(pkg):
    torch = pytest.importorskip("torch")
    lib = pkg.load_library()
    fn = lib.lulesh_lagrange_nodal_noalloc
    fn.restype = C.c_int
    fn.argtypes = ([C.c_int, C.c_int, C.c_double, C.POINTER(pkg.Parameters)] + [C.c_void_p] * 7 +
                   [C.c_int] + [C.c_void_p] * 16 + [C.c_void_p])

    s = 9
    dev = torch.device("cuda", 0)
    mesh = pkg.mesh_build(s, pkg.INIT_V2)
    ne, nn = pkg.mesh_sizes(s)
    params = pkg.default_parameters()

    def d(a, dtype=torch.float64):
        return torch.as_tensor(np.ascontiguousarray(a)).to(dev, dtype)

    sx, sy, sz = _symm_sets(s)
    const = {k: d(mesh[k], torch.int32) for k in
             ("nodelist", "node_elem_start", "node_elem_count", "node_elem_corner_list")}
    const.update({k: d(mesh[k]) for k in ("volo", "elem_mass", "nodal_mass")})
    symm = [d(a, torch.int32) for a in (sx, sy, sz)]

    with pkg.Lulesh(s, pkg.INIT_V2) as g:
        g.keep_forces(True)
        g.run(25)
        for call in range(2):
            # the state LagrangeNodal starts from, after this cycle's TimeIncrement
            g.time_increment()
            dt = g.scalars.deltatime
            state = {k: d(g.get_field(k)) for k in ("x", "y", "z", "xd", "yd", "zd", "p", "q", "v", "ss")}
            out_f = [torch.zeros(nn, dtype=torch.float64, device=dev) for _ in range(3)]

            g.lagrange_nodal()   # the ordinary entry point, on the context's own memory
            want = {k: g.get_field(k) for k in ("x", "y", "z", "xd", "yd", "zd", "fx", "fy", "fz")}

            stream = torch.cuda.current_stream(dev)
            rc = fn(ne, nn, dt, C.byref(params),
                    const["nodelist"].data_ptr(), const["node_elem_start"].data_ptr(),
                    const["node_elem_count"].data_ptr(), const["node_elem_corner_list"].data_ptr(),
                    symm[0].data_ptr(), symm[1].data_ptr(), symm[2].data_ptr(), len(sx),
                    const["volo"].data_ptr(), const["elem_mass"].data_ptr(), const["nodal_mass"].data_ptr(),
                    state["p"].data_ptr(), state["q"].data_ptr(), state["v"].data_ptr(), state["ss"].data_ptr(),
                    state["x"].data_ptr(), state["y"].data_ptr(), state["z"].data_ptr(),
                    state["xd"].data_ptr(), state["yd"].data_ptr(), state["zd"].data_ptr(),
                    out_f[0].data_ptr(), out_f[1].data_ptr(), out_f[2].data_ptr(),
                    C.c_void_p(stream.cuda_stream))
            assert rc == pkg.OK, rc
            torch.cuda.synchronize(dev)
            got = {k: state[k].cpu().numpy() for k in ("x", "y", "z", "xd", "yd", "zd")}
            got.update({k: f.cpu().numpy() for k, f in zip(("fx", "fy", "fz"), out_f)})
            for k in want:
                err = rel_err(got[k], want[k])
                assert err <= TOL, (call, k, err)
            # advance the context to the next cycle's start
            g.lagrange_elements()
            g.calc_time_constraints()


def _bind(pkg):
    fn = pkg.load_library().lulesh_lagrange_nodal_noalloc
    fn.restype = C.c_int
    fn.argtypes = ([C.c_int, C.c_int, C.c_double, C.POINTER(pkg.Parameters)] + [C.c_void_p] * 7 +
                   [C.c_int] + [C.c_void_p] * 16 + [C.c_void_p])
    return fn


def _call_fresh(pkg, s, edit=None):
    """One call on the initial s^3 Sedov state after ``edit(arrays)`` changed
    the host arrays; returns the status and the state before/after."""
    torch = pytest.importorskip("torch")
    fn = _bind(pkg)
    dev = torch.device("cuda", 0)
    mesh = pkg.mesh_build(s, pkg.INIT_V2)
    ne, nn = pkg.mesh_sizes(s)
    sx, sy, sz = _symm_sets(s)
    host = {k: np.array(mesh[k], dtype=np.int32) for k in
            ("nodelist", "node_elem_start", "node_elem_count", "node_elem_corner_list")}
    host.update({k: np.array(mesh[k], dtype=np.float64) for k in ("volo", "elem_mass", "nodal_mass")})
    host.update({"sx": sx, "sy": sy, "sz": sz})
    host.update({k: np.array(mesh[k], dtype=np.float64) for k in ("x", "y", "z")})
    host.update({k: np.zeros(nn) for k in ("xd", "yd", "zd")})
    host.update({"p": np.zeros(ne), "q": np.zeros(ne), "v": np.ones(ne), "ss": np.zeros(ne)})
    host["xd"][nn - 1] = 1.0   # some motion, so that an unchanged state says something
    if edit is not None:
        edit(host)
    dv = {k: torch.as_tensor(np.ascontiguousarray(a)).to(dev) for k, a in host.items()}
    f = [torch.zeros(nn, dtype=torch.float64, device=dev) for _ in range(3)]
    params = pkg.default_parameters()
    ptr = {k: t.data_ptr() for k, t in dv.items()}
    rc = fn(ne, nn, 1e-7, C.byref(params), ptr["nodelist"], ptr["node_elem_start"],
            ptr["node_elem_count"], ptr["node_elem_corner_list"], ptr["sx"], ptr["sy"], ptr["sz"],
            len(sx), ptr["volo"], ptr["elem_mass"], ptr["nodal_mass"], ptr["p"], ptr["q"], ptr["v"],
            ptr["ss"], ptr["x"], ptr["y"], ptr["z"], ptr["xd"], ptr["yd"], ptr["zd"],
            f[0].data_ptr(), f[1].data_ptr(), f[2].data_ptr(), None)
    torch.cuda.synchronize(dev)
    after = {k: dv[k].cpu().numpy() for k in ("x", "y", "z", "xd", "yd", "zd")}
    return rc, host, after


def test_noalloc_good_tables_step(pkg):
    rc, before, after = _call_fresh(pkg, 3)
    assert rc == pkg.OK
    # the moving node moved
    assert after["x"][-1] != before["x"][-1]


@pytest.mark.parametrize("case", ["corner_out_of_range", "start_count_gap", "corner_of_other_node",
                                  "corner_repeated", "nodelist_out_of_range"])
def test_noalloc_rejects_malformed_tables(pkg, case):
    """Tables that are in bounds but do not describe the reference's
    node-to-corner map are refused before any step kernel reads through them:
    the call returns LULESH_ERR_ARG and leaves the state as it was."""
    s = 3
    ne = s ** 3

    def edit(h):
        cl, st, cnt = h["node_elem_corner_list"], h["node_elem_start"], h["node_elem_count"]
        if case == "corner_out_of_range":
            cl[5] = 8 * ne
        elif case == "start_count_gap":
            # node 1's list starts one slot late: the lists no longer pack
            st[1] += 1
            cnt[1] -= 1
        elif case == "corner_of_other_node":
            # node 0's single corner swapped for one of node 1's
            cl[st[0]], cl[st[1]] = cl[st[1]], cl[st[0]]
        elif case == "corner_repeated":
            # a corner listed twice by its node, another of its corners dropped
            n = int(np.argmax(cnt))
            cl[st[n] + 1] = cl[st[n]]
        elif case == "nodelist_out_of_range":
            h["nodelist"][7] = -1

    rc, before, after = _call_fresh(pkg, s, edit)
    assert rc == pkg.ERR_ARG, rc
    for k in after:
        np.testing.assert_array_equal(after[k], before[k], err_msg=k)


def test_noalloc_volume_error(pkg):
    """A relative volume of 0 is the reference's VolumeError
    (CalcHourglassControlForElems, LULESH-OMP.cc:1541-1543); the nodes do not
    move."""
    def edit(h):
        h["v"][4] = 0.0

    rc, before, after = _call_fresh(pkg, 3, edit)
    assert rc == pkg.VOLUME_ERROR, rc
    for k in after:
        np.testing.assert_array_equal(after[k], before[k], err_msg=k)


def test_noalloc_rejects_oversized_mesh(pkg):
    torch = pytest.importorskip("torch")
    lib = pkg.load_library()
    fn = lib.lulesh_lagrange_nodal_noalloc
    fn.restype = C.c_int
    params = pkg.default_parameters()
    dummy = torch.zeros(8, dtype=torch.float64, device="cuda")
    p = C.c_void_p(dummy.data_ptr())
    rc = fn(C.c_int(41 ** 3), C.c_int(42 ** 3), C.c_double(1e-7), C.byref(params),
            *([p] * 7), C.c_int(0), *([p] * 16), C.c_void_p(0))
    assert rc == pkg.ERR_ARG
