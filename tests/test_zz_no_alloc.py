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
