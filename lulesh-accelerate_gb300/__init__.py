"""GB300-native LULESH Lagrange leapfrog step: Python host interface.

A thin ctypes layer over the C ABI of ``liblulesh_gb300.so``
(``include/lulesh_gb300.h``).  It mirrors the reference's step API:

* :class:`Parameters` -- the ``Parameters`` record (src/Domain.hs:23-82) with
  the C reference's constants (reference/C/LULESH-OMP.cc:3051-3087);
* :class:`Domain` -- the ``Domain`` record (src/Domain.hs:11-21): position,
  velocity, energy, pressure, viscosity, relative volume, sound speed, time
  and time step;
* :class:`Lulesh` -- one problem on the GPU with ``time_increment``
  (TimeIncrement, LULESH-OMP.cc:557-604), ``lagrange_leapfrog``
  (LagrangeLeapFrog, :2944-2958) and its phases, and ``run`` (the main loop,
  :3179-3188);
* :func:`lulesh` -- the functional step of src/LULESH.hs:37-53 over host
  arrays.

Errors of the physics raise :class:`VolumeError` / :class:`QStopError`
(the reference's exit codes -1 / -2, LULESH-OMP.cc:82).  There is no CPU
fallback: without the built library or a CUDA device every call raises.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

__all__ = [
    "Parameters", "Domain", "Scalars", "Lulesh", "lulesh", "library_path", "load_library",
    "LuleshError", "VolumeError", "QStopError", "mesh_build", "mesh_sizes", "default_parameters",
    "INIT_V1", "INIT_V2", "FP64", "SPLIT", "sedov_metrics", "relative_errors", "probe_fp64_peak",
    "Batch", "ensemble",
]

_PKG = Path(__file__).resolve().parent
LIB_NAME = "liblulesh_gb300.so"

OK, VOLUME_ERROR, QSTOP_ERROR, ERR_CUDA, ERR_TIMEOUT, ERR_ARG = 0, -1, -2, -3, -4, -5
FP64, SPLIT, FP64_IEEE = 0, 1, 2
RUN_CYCLE_BUDGET = 1 << 20   # LULESH_RUN_CYCLE_BUDGET: cycles of a run given no cap
INIT_V1, INIT_V2 = 1, 2


class LuleshError(RuntimeError):
    """A failing call of the library; ``code`` is its status."""

    def __init__(self, code: int, message: str):
        super().__init__(f"[{code}] {message}")
        self.code = code


class VolumeError(LuleshError):
    """An element volume became non-positive (reference exit code -1)."""


class QStopError(LuleshError):
    """Artificial viscosity exceeded qstop (reference exit code -2)."""


class RunTimeout(LuleshError):
    """A run stopped short of stoptime: its cycle budget
    (``RUN_CYCLE_BUDGET`` when no cap is given) ran out, or the time step
    stopped being positive.  The state stays valid."""


class Parameters(C.Structure):
    """``lulesh_params``: the constants of src/Domain.hs:23-53."""

    _fields_ = [(n, C.c_double) for n in (
        "e_cut", "p_cut", "q_cut", "v_cut", "u_cut",
        "hgcoef", "ss4o3", "qstop", "monoq_max_slope", "monoq_limiter_mult",
        "qlc_monoq", "qqc_monoq", "qqc",
        "eosvmax", "eosvmin", "pmin", "emin", "dvovmax", "refdens",
        "dtfixed", "deltatimemultlb", "deltatimemultub", "dtmax", "stoptime")]

    def as_dict(self) -> dict:
        return {n: getattr(self, n) for n, _ in self._fields_}


class Scalars(C.Structure):
    """``lulesh_scalars``: time, time step, constraint state and cycle."""

    _fields_ = [("time", C.c_double), ("deltatime", C.c_double), ("dtcourant", C.c_double),
                ("dthydro", C.c_double), ("cycle", C.c_int)]


_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


class MeshView(C.Structure):
    _fields_ = [("x", _dp), ("y", _dp), ("z", _dp), ("volo", _dp), ("elem_mass", _dp),
                ("nodal_mass", _dp), ("nodelist", _ip), ("node_elem_start", _ip),
                ("node_elem_count", _ip), ("node_elem_corner_list", _ip),
                ("lxim", _ip), ("lxip", _ip), ("letam", _ip), ("letap", _ip),
                ("lzetam", _ip), ("lzetap", _ip), ("elem_bc", _ip),
                ("e0", C.c_double), ("dt0", C.c_double)]


class UnstructuredMesh(C.Structure):
    """``lulesh_unstructured_mesh``: host arrays of an arbitrary hex mesh."""

    _fields_ = [("num_elem", C.c_long), ("num_node", C.c_long),
                ("x", _dp), ("y", _dp), ("z", _dp), ("nodelist", _ip)] + \
               [(n, _ip) for n in ("lxim", "lxip", "letam", "letap", "lzetam", "lzetap",
                                   "symm_x", "symm_y", "symm_z", "free_surf")] + \
               [(n, C.c_long) for n in ("num_symm_x", "num_symm_y", "num_symm_z", "num_free_surf")]


MESH_ARRAYS = ("x", "y", "z", "nodelist", "lxim", "lxip", "letam", "letap", "lzetam", "lzetap",
               "symm_x", "symm_y", "symm_z", "free_surf")


_SIGNATURES = {
    "lulesh_default_params": (None, [C.POINTER(Parameters)]),
    "lulesh_mesh_sizes": (C.c_int, [C.c_int, C.POINTER(C.c_long), C.POINTER(C.c_long)]),
    "lulesh_mesh_build": (C.c_int, [C.c_int, C.c_int, C.POINTER(MeshView)]),
    "lulesh_create": (C.c_int, [C.c_int, C.c_int, C.c_int, C.POINTER(Parameters), C.POINTER(C.c_void_p)]),
    "lulesh_create_unstructured": (C.c_int, [C.POINTER(UnstructuredMesh), C.c_int, C.POINTER(Parameters),
                                             C.POINTER(C.c_void_p)]),
    "lulesh_create_lmesh": (C.c_int, [C.c_char_p, C.c_int, C.POINTER(Parameters), C.POINTER(C.c_void_p)]),
    "lulesh_origin_element": (C.c_int, [C.c_void_p, C.POINTER(C.c_long)]),
    "lulesh_write_domain": (C.c_int, [C.c_char_p, C.c_int, C.c_int, C.c_double] + [_dp] * 10),
    "lulesh_dump_domain": (C.c_int, [C.c_void_p, C.c_char_p, C.c_int]),
    "lulesh_set_regions": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int]),
    "lulesh_get_regions": (C.c_int, [C.c_void_p, _ip]),
    "lulesh_region_numbers": (C.c_int, [C.c_long, C.c_int, C.c_int, _ip]),
    "lulesh_destroy": (None, [C.c_void_p]),
    "lulesh_last_error": (C.c_char_p, [C.c_void_p]),
    "lulesh_upload_domain": (C.c_int, [C.c_void_p] + [_dp] * 11 + [C.c_double, C.c_double]),
    "lulesh_download_domain": (C.c_int, [C.c_void_p] + [_dp] * 13),
    "lulesh_get_scalars": (C.c_int, [C.c_void_p, C.POINTER(Scalars)]),
    "lulesh_set_scalars": (C.c_int, [C.c_void_p, C.POINTER(Scalars)]),
    "lulesh_get_field": (C.c_int, [C.c_void_p, C.c_char_p, _dp, C.c_long]),
    "lulesh_set_field": (C.c_int, [C.c_void_p, C.c_char_p, _dp, C.c_long]),
    "lulesh_keep_forces": (C.c_int, [C.c_void_p, C.c_int]),
    "lulesh_set_params": (C.c_int, [C.c_void_p, C.POINTER(Parameters)]),
    "lulesh_get_params": (C.c_int, [C.c_void_p, C.POINTER(Parameters)]),
    "lulesh_time_increment": (C.c_int, [C.c_void_p]),
    "lulesh_lagrange_nodal": (C.c_int, [C.c_void_p]),
    "lulesh_lagrange_elements": (C.c_int, [C.c_void_p]),
    "lulesh_calc_time_constraints": (C.c_int, [C.c_void_p]),
    "lulesh_lagrange_leapfrog": (C.c_int, [C.c_void_p]),
    "lulesh_run": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_int)]),
    "lulesh_origin_energy": (C.c_int, [C.c_void_p, _dp]),
    "lulesh_symmetry": (C.c_int, [C.c_void_p, _dp, _dp, _dp]),
    "lulesh_sizes": (C.c_int, [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_long), C.POINTER(C.c_long)]),
    "lulesh_stream": (C.c_void_p, [C.c_void_p]),
    "lulesh_kernel_launches": (C.c_longlong, [C.c_void_p]),
    "lulesh_run_profiled": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_int), _dp]),
    "lulesh_probe_fp64_peak": (C.c_int, [_dp]),
    "lulesh_probe_pipe_rates": (C.c_int, [_dp]),
    "lulesh_probe_math": (C.c_int, [_dp]),
    "lulesh_batch_create": (C.c_int, [C.c_int, _ip, _dp, C.c_int, C.c_int, C.POINTER(Parameters),
                                      C.POINTER(C.c_void_p)]),
    "lulesh_batch_destroy": (None, [C.c_void_p]),
    "lulesh_batch_last_error": (C.c_char_p, [C.c_void_p]),
    "lulesh_batch_run": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_int)]),
    "lulesh_batch_size": (C.c_int, [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_long), C.POINTER(C.c_long)]),
    "lulesh_batch_instance": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(Scalars), _dp, C.POINTER(C.c_int)]),
    "lulesh_batch_get_field": (C.c_int, [C.c_void_p, C.c_int, C.c_char_p, _dp, C.c_long]),
    "lulesh_batch_zone_cycles": (C.c_int, [C.c_void_p, _dp]),
    "lulesh_batch_autotune": (C.c_int, [C.c_void_p, C.c_char_p, C.c_int]),
    "lulesh_batch_run_retuned": (C.c_int, [C.c_void_p, C.c_int, C.c_double, C.c_int, C.POINTER(C.c_int),
                                           C.POINTER(C.c_int)]),
    "lulesh_batch_tuning": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "lulesh_batch_staging": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.POINTER(C.c_int)]),
    "lulesh_batch_set_tuning": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int]),
    "lulesh_batch_stream": (C.c_void_p, [C.c_void_p]),
    "lulesh_batch_kernel_launches": (C.c_longlong, [C.c_void_p]),
}

TIMED_KERNELS = ("time_increment", "elem_force", "node_update", "elem_kinematics",
                 "elem_material", "finalize")

_lib = None


def library_path() -> Path:
    return Path(os.environ.get("LULESH_GB300_LIB", _PKG / LIB_NAME))


def load_library():
    """Load ``liblulesh_gb300.so`` (built by ``build.py``); raise if absent."""
    global _lib
    if _lib is None:
        path = library_path()
        if not path.exists():
            raise LuleshError(ERR_ARG, f"{path} is not built: run lulesh-accelerate_gb300/build.py")
        lib = C.CDLL(str(path))
        for name, (res, args) in _SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


def _ptr(a: np.ndarray | None, ctype=C.c_double):
    if a is None:
        return None
    return a.ctypes.data_as(C.POINTER(ctype))


def _check(rc: int, handle=None):
    if rc == OK:
        return
    msg = load_library().lulesh_last_error(handle).decode(errors="replace")
    if rc == VOLUME_ERROR:
        raise VolumeError(rc, msg)
    if rc == QSTOP_ERROR:
        raise QStopError(rc, msg)
    if rc == ERR_TIMEOUT:
        raise RunTimeout(rc, msg)
    raise LuleshError(rc, msg)


def default_parameters() -> Parameters:
    p = Parameters()
    load_library().lulesh_default_params(C.byref(p))
    return p


def write_domain(basename, s: int, step: int, time: float, fields: dict) -> None:
    """The reference's per-step visualisation write (cbits/visit.cc
    writeDomain) for host arrays of the s^3 cube; ``fields`` holds x, y, z,
    xd, yd, zd, e, p, v, q."""
    arrs = [np.ascontiguousarray(fields[k], dtype=np.float64)
            for k in ("x", "y", "z", "xd", "yd", "zd", "e", "p", "v", "q")]
    _check(load_library().lulesh_write_domain(os.fsencode(str(basename)), s, step, time, *[_ptr(a) for a in arrs]))


def read_domain_file(path) -> dict:
    """A file of ``lulesh_write_domain`` / ``lulesh_dump_domain``: header
    values (s, num_elem, num_node, step, time) and one array per section."""
    data = Path(path).read_bytes()
    if data[:8] != b"LULESHD1":
        raise ValueError(f"{path}: not a LULESHD1 file")
    s, ne, nn, step = np.frombuffer(data, np.int32, 4, 8)
    (time,) = np.frombuffer(data, np.float64, 1, 24)
    (nsec,) = np.frombuffer(data, np.int32, 1, 32)
    out = {"s": int(s), "num_elem": int(ne), "num_node": int(nn), "step": int(step), "time": float(time)}
    off = 36
    for _ in range(int(nsec)):
        name = data[off:off + 16].split(b"\0")[0].decode()
        typ, _centring = np.frombuffer(data, np.int32, 2, off + 16)
        (count,) = np.frombuffer(data, np.int64, 1, off + 24)
        dt = np.int32 if typ == 0 else np.float64
        out[name] = np.frombuffer(data, dt, int(count), off + 32).copy()
        off += 32 + int(count) * np.dtype(dt).itemsize
    return out


def region_numbers(num_elem: int, num_regions: int, balance: int = 1) -> np.ndarray:
    """LULESH 2.0's element-to-region assignment, computed on the host."""
    out = np.empty(num_elem, dtype=np.int32)
    _check(load_library().lulesh_region_numbers(num_elem, num_regions, balance, _ptr(out, C.c_int)))
    return out


def mesh_sizes(s: int) -> tuple[int, int]:
    ne, nn = C.c_long(), C.c_long()
    _check(load_library().lulesh_mesh_sizes(s, C.byref(ne), C.byref(nn)))
    return ne.value, nn.value


def mesh_build(s: int, init: int = INIT_V2) -> dict:
    """Host-built Sedov mesh (no GPU needed), as numpy arrays."""
    ne, nn = mesh_sizes(s)
    out = {k: np.zeros(nn) for k in ("x", "y", "z", "nodal_mass")}
    out.update({k: np.zeros(ne) for k in ("volo", "elem_mass")})
    out.update({k: np.zeros(8 * ne, np.int32) for k in ("nodelist", "node_elem_corner_list")})
    out.update({k: np.zeros(nn, np.int32) for k in ("node_elem_start", "node_elem_count")})
    out.update({k: np.zeros(ne, np.int32) for k in
                ("lxim", "lxip", "letam", "letap", "lzetam", "lzetap", "elem_bc")})
    mv = MeshView()
    for name, _ in MeshView._fields_:
        if name in out:
            setattr(mv, name, _ptr(out[name], C.c_int if out[name].dtype == np.int32 else C.c_double))
    _check(load_library().lulesh_mesh_build(s, init, C.byref(mv)))
    out["e0"], out["dt0"] = mv.e0, mv.dt0
    return out


@dataclass
class Domain:
    """The evolving state of src/Domain.hs:11-21, structure of arrays."""

    x: np.ndarray
    y: np.ndarray
    z: np.ndarray
    xd: np.ndarray
    yd: np.ndarray
    zd: np.ndarray
    e: np.ndarray
    p: np.ndarray
    q: np.ndarray
    v: np.ndarray
    ss: np.ndarray
    time: float = 0.0
    deltatime: float = 0.0

    NODE_FIELDS = ("x", "y", "z", "xd", "yd", "zd")
    ELEM_FIELDS = ("e", "p", "q", "v", "ss")

    @classmethod
    def empty(cls, ne: int, nn: int, pinned=None) -> "Domain":
        alloc = pinned or (lambda n: np.empty(n))
        return cls(**{k: alloc(nn) for k in cls.NODE_FIELDS}, **{k: alloc(ne) for k in cls.ELEM_FIELDS})

    def arrays(self):
        return [getattr(self, k) for k in self.NODE_FIELDS + self.ELEM_FIELDS]


NODE_FIELDS = {"x", "y", "z", "xd", "yd", "zd", "fx", "fy", "fz", "nodalMass"}


class Lulesh:
    """One Sedov problem resident on the current CUDA device.

    ``init`` is ``INIT_V1`` (LULESH 1.0 initial energy and time step) or
    ``INIT_V2`` (LULESH 2.0's scaled energy and analytic time step);
    ``precision`` is ``FP64`` (the drop-in) or ``SPLIT``.
    """

    def __init__(self, s: int, init: int = INIT_V2, precision: int = FP64,
                 params: Parameters | None = None, *, _handle: C.c_void_p | None = None):
        lib = load_library()
        if _handle is None:
            h = C.c_void_p()
            rc = lib.lulesh_create(s, init, precision, C.byref(params) if params is not None else None,
                                   C.byref(h))
            _check(rc)
        else:
            h = _handle
        self._h = h
        es, ne, nn = C.c_int(), C.c_long(), C.c_long()
        _check(lib.lulesh_sizes(h, C.byref(es), C.byref(ne), C.byref(nn)), h)
        self.s = es.value
        self.num_elem, self.num_node = ne.value, nn.value

    @classmethod
    def from_mesh(cls, mesh: dict, precision: int = FP64, params: Parameters | None = None) -> "Lulesh":
        """An unstructured problem from host arrays (keys of ``MESH_ARRAYS``;
        the reference's unstructured set-up, lulesh.cu:733-923)."""
        keep = {}
        m = UnstructuredMesh(num_elem=len(mesh["nodelist"]) // 8, num_node=len(mesh["x"]))
        for k in MESH_ARRAYS:
            dt = np.float64 if k in ("x", "y", "z") else np.int32
            a = np.ascontiguousarray(mesh[k], dtype=dt)
            keep[k] = a
            setattr(m, k, _ptr(a, C.c_double if dt is np.float64 else C.c_int))
        m.num_symm_x, m.num_symm_y, m.num_symm_z = (len(keep[k]) for k in ("symm_x", "symm_y", "symm_z"))
        m.num_free_surf = len(keep["free_surf"])
        h = C.c_void_p()
        rc = load_library().lulesh_create_unstructured(
            C.byref(m), precision, C.byref(params) if params is not None else None, C.byref(h))
        _check(rc)
        return cls(0, _handle=h)

    @classmethod
    def from_lmesh(cls, path, precision: int = FP64, params: Parameters | None = None) -> "Lulesh":
        """An unstructured problem read from a .lmesh text file by the library."""
        h = C.c_void_p()
        rc = load_library().lulesh_create_lmesh(
            os.fsencode(str(path)), precision, C.byref(params) if params is not None else None, C.byref(h))
        _check(rc)
        return cls(0, _handle=h)

    def set_regions(self, num_regions: int = 11, balance: int = 1, cost: int = 1) -> None:
        """LULESH 2.0 material regions (its -r/-b/-c options; defaults are its
        defaults).  Results do not change; the EOS of costly regions runs
        1+cost or 10*(1+cost) times.  ``num_regions=0`` removes them."""
        _check(load_library().lulesh_set_regions(self._h, num_regions, balance, cost), self._h)

    def regions(self) -> np.ndarray:
        """Region number (1-based) of every element."""
        out = np.empty(self.num_elem, dtype=np.int32)
        _check(load_library().lulesh_get_regions(self._h, _ptr(out, C.c_int)), self._h)
        return out

    def dump(self, basename, step: int) -> None:
        """Write the current state for visualisation (``read_domain_file``
        reads it back); ``basename`` may hold one %d for the step."""
        _check(load_library().lulesh_dump_domain(self._h, os.fsencode(str(basename)), step), self._h)

    @property
    def origin(self) -> int:
        """Element holding the initial energy (the reference's octantCorner)."""
        e = C.c_long()
        _check(load_library().lulesh_origin_element(self._h, C.byref(e)), self._h)
        return e.value

    # lifetime -----------------------------------------------------------
    def close(self):
        if getattr(self, "_h", None):
            load_library().lulesh_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # step API ------------------------------------------------------------
    def time_increment(self):
        _check(load_library().lulesh_time_increment(self._h), self._h)

    def lagrange_nodal(self):
        _check(load_library().lulesh_lagrange_nodal(self._h), self._h)

    def lagrange_elements(self):
        _check(load_library().lulesh_lagrange_elements(self._h), self._h)

    def calc_time_constraints(self):
        _check(load_library().lulesh_calc_time_constraints(self._h), self._h)

    def lagrange_leapfrog(self):
        _check(load_library().lulesh_lagrange_leapfrog(self._h), self._h)

    def run(self, max_cycles: int = 0) -> int:
        """The reference main loop; returns the number of cycles done."""
        n = C.c_int()
        _check(load_library().lulesh_run(self._h, max_cycles, C.byref(n)), self._h)
        return n.value

    def run_profiled(self, max_cycles: int = 0) -> tuple[int, dict]:
        """The main loop kernel by kernel; returns (cycles, summed ms per kernel)."""
        n = C.c_int()
        ms = np.zeros(len(TIMED_KERNELS))
        _check(load_library().lulesh_run_profiled(self._h, max_cycles, C.byref(n), _ptr(ms)), self._h)
        return n.value, dict(zip(TIMED_KERNELS, ms.tolist()))

    # state ---------------------------------------------------------------
    def _len(self, name: str) -> int:
        return self.num_node if name in NODE_FIELDS else self.num_elem

    def get_field(self, name: str) -> np.ndarray:
        out = np.empty(self._len(name))
        _check(load_library().lulesh_get_field(self._h, name.encode(), _ptr(out), out.size), self._h)
        return out

    def set_field(self, name: str, values) -> None:
        a = np.ascontiguousarray(values, dtype=np.float64)
        _check(load_library().lulesh_set_field(self._h, name.encode(), _ptr(a), a.size), self._h)

    def keep_forces(self, keep: bool = True):
        _check(load_library().lulesh_keep_forces(self._h, int(keep)), self._h)

    @property
    def params(self) -> Parameters:
        p = Parameters()
        _check(load_library().lulesh_get_params(self._h, C.byref(p)), self._h)
        return p

    @params.setter
    def params(self, p: Parameters):
        _check(load_library().lulesh_set_params(self._h, C.byref(p)), self._h)

    @property
    def scalars(self) -> Scalars:
        sc = Scalars()
        _check(load_library().lulesh_get_scalars(self._h, C.byref(sc)), self._h)
        return sc

    @scalars.setter
    def scalars(self, sc: Scalars):
        _check(load_library().lulesh_set_scalars(self._h, C.byref(sc)), self._h)

    def upload(self, dom: Domain):
        a = [np.ascontiguousarray(v, dtype=np.float64) for v in dom.arrays()]
        _check(load_library().lulesh_upload_domain(self._h, *[_ptr(v) for v in a],
                                                   float(dom.time), float(dom.deltatime)), self._h)

    def download(self, into: Domain | None = None) -> Domain:
        dom = into or Domain.empty(self.num_elem, self.num_node)
        t, dt = C.c_double(), C.c_double()
        _check(load_library().lulesh_download_domain(self._h, *[_ptr(v) for v in dom.arrays()],
                                                     C.byref(t), C.byref(dt)), self._h)
        dom.time, dom.deltatime = t.value, dt.value
        return dom

    def origin_energy(self) -> float:
        e = C.c_double()
        _check(load_library().lulesh_origin_energy(self._h, C.byref(e)), self._h)
        return e.value

    def symmetry(self) -> tuple[float, float, float]:
        """(MaxAbsDiff, TotalAbsDiff, MaxRelDiff) of energy plane 0."""
        a, t, r = C.c_double(), C.c_double(), C.c_double()
        _check(load_library().lulesh_symmetry(self._h, C.byref(a), C.byref(t), C.byref(r)), self._h)
        return a.value, t.value, r.value

    @property
    def stream(self) -> int:
        return load_library().lulesh_stream(self._h) or 0

    @property
    def kernel_launches(self) -> int:
        return load_library().lulesh_kernel_launches(self._h)


def _check_batch(rc: int, handle=None):
    if rc == OK:
        return
    msg = load_library().lulesh_batch_last_error(handle).decode(errors="replace")
    if rc == ERR_TIMEOUT:
        raise RunTimeout(rc, msg)
    raise LuleshError(rc, msg)


BATCH_KERNELS = ("elem_force", "node_update", "elem_kinematics", "elem_material")


class Batch:
    """An ensemble of independent Sedov problems advanced together on the GPU.

    ``sizes[i]`` is instance i's edge length and ``e0_scale[i]`` multiplies
    its initial energy.  Every instance runs to its own stop time with its
    own time step; its arithmetic is that of a single :class:`Lulesh` started
    from the same state.
    """

    def __init__(self, sizes, e0_scale=None, init: int = INIT_V2, precision: int = FP64,
                 params: Parameters | None = None):
        lib = load_library()
        self.sizes = np.ascontiguousarray(sizes, dtype=np.int32)
        scale = None if e0_scale is None else np.ascontiguousarray(e0_scale, dtype=np.float64)
        h = C.c_void_p()
        rc = lib.lulesh_batch_create(len(self.sizes), _ptr(self.sizes, C.c_int), _ptr(scale), init, precision,
                                     C.byref(params) if params is not None else None, C.byref(h))
        _check_batch(rc)
        self._h = h
        self.n = len(self.sizes)

    def close(self):
        if getattr(self, "_h", None):
            load_library().lulesh_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def run(self, max_cycles: int = 0) -> int:
        n = C.c_int()
        _check_batch(load_library().lulesh_batch_run(self._h, max_cycles, C.byref(n)), self._h)
        return n.value

    def instance(self, i: int) -> tuple[Scalars, float, int]:
        sc, e0, st = Scalars(), C.c_double(), C.c_int()
        _check_batch(load_library().lulesh_batch_instance(self._h, i, C.byref(sc), C.byref(e0), C.byref(st)),
                     self._h)
        return sc, e0.value, st.value

    def get_field(self, i: int, name: str) -> np.ndarray:
        s = int(self.sizes[i])
        n = (s + 1) ** 3 if name in NODE_FIELDS else s ** 3
        out = np.empty(n)
        _check_batch(load_library().lulesh_batch_get_field(self._h, i, name.encode(), _ptr(out), n), self._h)
        return out

    def zone_cycles(self) -> float:
        zc = C.c_double()
        _check_batch(load_library().lulesh_batch_zone_cycles(self._h, C.byref(zc)), self._h)
        return zc.value

    def run_retuned(self, chunk: int = 200, fraction: float = 0.5, max_cycles: int = 0) -> tuple[int, int]:
        """Run in chunks of cycles, re-tuning the launch shapes whenever the
        running instances' elements fall below ``fraction`` of those last
        tuned for; returns (largest per-instance cycle count, re-tunings)."""
        n, r = C.c_int(), C.c_int()
        _check_batch(load_library().lulesh_batch_run_retuned(self._h, chunk, fraction, max_cycles, C.byref(n),
                                                             C.byref(r)), self._h)
        return n.value, r.value

    def autotune(self, cache_path: str | None = None, retune: bool = False):
        path = None if cache_path is None else str(cache_path).encode()
        _check_batch(load_library().lulesh_batch_autotune(self._h, path, int(retune)), self._h)

    def tuning(self) -> dict:
        """Launch shape per class and kernel: threads per block, persistent
        grid, and the staging depth (element rows per staged tile, 0 for
        gathered corners)."""
        out = {}
        for cls in range(3):
            for k, name in enumerate(BATCH_KERNELS):
                b, g, r = C.c_int(), C.c_int(), C.c_int()
                load_library().lulesh_batch_tuning(self._h, cls, k, C.byref(b), C.byref(g))
                load_library().lulesh_batch_staging(self._h, cls, k, C.byref(r))
                out[f"class{cls}/{name}"] = {"block": b.value, "grid": g.value, "stage": r.value}
        return out

    def set_tuning(self, size_class: int, kernel: str, block: int = 128, blocks_per_sm: int = 4, rows: int = 0):
        """Set one kernel's launch shape by hand (see lulesh_batch_set_tuning)."""
        _check_batch(load_library().lulesh_batch_set_tuning(self._h, size_class, BATCH_KERNELS.index(kernel), block,
                                                            blocks_per_sm, rows), self._h)

    @property
    def stream(self) -> int:
        return load_library().lulesh_batch_stream(self._h) or 0

    @property
    def kernel_launches(self) -> int:
        return load_library().lulesh_batch_kernel_launches(self._h)


def ensemble(seed: int, n: int, lo: int, hi: int, extra_sizes=()) -> tuple[np.ndarray, np.ndarray]:
    """Seeded ensemble of Sedov instances: n sizes uniform in lo..hi, then the
    ``extra_sizes``, and one energy factor per instance, log-uniform in
    [0.5, 2] (sizes drawn first, then factors, from
    numpy.random.default_rng(seed))."""
    rng = np.random.default_rng(seed)
    sizes = np.concatenate([rng.integers(lo, hi + 1, n), np.asarray(extra_sizes, dtype=np.int64)])
    factors = np.exp(rng.uniform(np.log(0.5), np.log(2.0), len(sizes)))
    return sizes.astype(np.int32), factors


def sedov_metrics(ctx: "Lulesh", mesh: dict | None = None) -> dict:
    """Whole-problem results of a Sedov state, for comparing precisions.

    * ``origin_energy``: e of the origin element (the reference's printed
      result; element 0 on the cube);
    * ``total_energy``: internal plus kinetic energy,
      sum(e * elemMass) + sum(0.5 * nodalMass * |v|^2);
    * ``max_velocity``: largest nodal speed |v|;
    * ``shock_radius``: artificial-viscosity-weighted mean radius of the
      element centroids, sum(r q m) / sum(q m).  The monotonic q is non-zero
      only in the compression zone, so this follows the shock front and,
      unlike "radius of the element of largest pressure", varies smoothly.
      The reference defines no shock radius; this is this library's
      definition.
    """
    m = mesh if mesh is not None else mesh_build(ctx.s, INIT_V2)
    x, y, z = (ctx.get_field(k) for k in ("x", "y", "z"))
    xd, yd, zd = (ctx.get_field(k) for k in ("xd", "yd", "zd"))
    e, q = ctx.get_field("e"), ctx.get_field("q")
    speed2 = xd * xd + yd * yd + zd * zd
    nl = m["nodelist"].reshape(-1, 8)
    cx, cy, cz = x[nl].mean(axis=1), y[nl].mean(axis=1), z[nl].mean(axis=1)
    r = np.sqrt(cx * cx + cy * cy + cz * cz)
    w = q * m["elem_mass"]
    return {
        "origin_energy": float(e[ctx.origin]),
        "total_energy": float(np.sum(e * m["elem_mass"]) + 0.5 * np.sum(m["nodal_mass"] * speed2)),
        "max_velocity": float(np.sqrt(np.max(speed2))),
        "shock_radius": float(np.sum(r * w) / np.sum(w)) if np.sum(w) > 0 else 0.0,
    }


def relative_errors(got: dict, ref: dict) -> dict:
    return {k: abs(got[k] - ref[k]) / abs(ref[k]) if ref[k] else abs(got[k]) for k in ref}


def probe_fp64_peak() -> float:
    """Measured FP64 FMA throughput of the current device, TFLOP/s."""
    t = C.c_double()
    _check(load_library().lulesh_probe_fp64_peak(C.byref(t)))
    return t.value


def probe_math() -> dict:
    """Largest relative differences of the library's inverse cube root,
    square root, reciprocal and quotient from CUDA's rcbrt, sqrt, __drcp_rn
    and division."""
    e = np.zeros(4)
    _check(load_library().lulesh_probe_math(_ptr(e)))
    return dict(zip(("rcbrt", "sqrt", "rcp", "quot"), e.tolist()))


def probe_pipe_rates() -> dict:
    """Operations per SM per clock: FP32 FMA, FP64 FMA, FP64->FP32 conversion
    (paired with an FP64 add), FP64 division."""
    r = np.zeros(4)
    _check(load_library().lulesh_probe_pipe_rates(_ptr(r)))
    return dict(zip(("ffma", "dfma", "d2f_plus_dadd", "ddiv"), r.tolist()))


def lulesh(ctx: Lulesh, dom: Domain) -> Domain:
    """The functional step of src/LULESH.hs:37-53 over host arrays.

    Uploads ``dom``, advances one cycle in the C reference's order
    (TimeIncrement, then LagrangeLeapFrog) and returns the new state.  The
    reference volumes and masses (``v0``, ``mN0`` of the Haskell API) are the
    ones ``ctx`` was built with.
    """
    ctx.upload(dom)
    ctx.time_increment()
    ctx.lagrange_leapfrog()
    return ctx.download()
