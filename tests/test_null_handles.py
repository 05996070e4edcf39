"""Every call that takes a context or batch handle answers LULESH_ERR_ARG
for a NULL handle (or a NULL output pointer) instead of faulting, and the
query calls return neutral values; none of this needs a GPU."""
from __future__ import annotations

import ctypes as C

import pytest

ERR_ARG = -5

# name -> argument list after the NULL handle
CTX_CALLS = {
    "lulesh_origin_element": [None],
    "lulesh_upload_domain": [None] * 11 + [C.c_double(0.0), C.c_double(0.0)],
    "lulesh_download_domain": [None] * 13,
    "lulesh_get_scalars": [None],
    "lulesh_set_scalars": [None],
    "lulesh_get_field": [b"x", None, C.c_long(0)],
    "lulesh_set_field": [b"x", None, C.c_long(0)],
    "lulesh_keep_forces": [1],
    "lulesh_set_params": [None],
    "lulesh_get_params": [None],
    "lulesh_set_regions": [11, 1, 1],
    "lulesh_get_regions": [None],
    "lulesh_time_increment": [],
    "lulesh_lagrange_nodal": [],
    "lulesh_lagrange_elements": [],
    "lulesh_calc_time_constraints": [],
    "lulesh_lagrange_leapfrog": [],
    "lulesh_run": [0, None],
    "lulesh_origin_energy": [None],
    "lulesh_symmetry": [None, None, None],
    "lulesh_dump_domain": [b"x", 0],
    "lulesh_sizes": [None, None, None],
    "lulesh_run_profiled": [0, None, None],
}
BATCH_CALLS = {
    "lulesh_batch_run": [0, None],
    "lulesh_batch_size": [None, None, None],
    "lulesh_batch_instance": [0, None, None, None],
    "lulesh_batch_get_field": [0, b"x", None, C.c_long(0)],
    "lulesh_batch_zone_cycles": [None],
    "lulesh_batch_autotune": [None, 0],
    "lulesh_batch_tuning": [0, 0, None, None],
}


def _lib(pkg):
    return C.CDLL(str(pkg.library_path()))


@pytest.mark.parametrize("name", sorted(CTX_CALLS))
def test_null_context(pkg, name):
    fn = getattr(_lib(pkg), name)
    fn.restype = C.c_int
    assert fn(None, *CTX_CALLS[name]) == ERR_ARG


@pytest.mark.parametrize("name", sorted(BATCH_CALLS))
def test_null_batch(pkg, name):
    fn = getattr(_lib(pkg), name)
    fn.restype = C.c_int
    assert fn(None, *BATCH_CALLS[name]) == ERR_ARG


def test_null_queries_and_destroy(pkg):
    lib = _lib(pkg)
    lib.lulesh_stream.restype = C.c_void_p
    lib.lulesh_kernel_launches.restype = C.c_longlong
    lib.lulesh_batch_stream.restype = C.c_void_p
    lib.lulesh_batch_kernel_launches.restype = C.c_longlong
    assert lib.lulesh_stream(None) is None
    assert lib.lulesh_kernel_launches(None) == 0
    assert lib.lulesh_batch_stream(None) is None
    assert lib.lulesh_batch_kernel_launches(None) == 0
    lib.lulesh_destroy(None)
    lib.lulesh_batch_destroy(None)
    lib.lulesh_last_error.restype = C.c_char_p
    assert isinstance(lib.lulesh_last_error(None), bytes)


def test_null_outputs_of_context_free_calls(pkg):
    lib = _lib(pkg)
    assert lib.lulesh_mesh_build(4, 2, None) == ERR_ARG
    assert lib.lulesh_create(4, 2, 0, None, None) == ERR_ARG
    assert lib.lulesh_create_unstructured(None, 0, None, None) == ERR_ARG
    assert lib.lulesh_create_lmesh(b"x", 0, None, None) == ERR_ARG
    assert lib.lulesh_probe_math(None) == ERR_ARG
