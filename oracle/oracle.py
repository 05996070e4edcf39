"""ctypes binding of the oracle restatement (oracle/lulesh_oracle.c).

TEST INFRASTRUCTURE ONLY: the checker for the CUDA library's parity tests
and the source of the "port" CPU baseline.  Only tests/, the smoke check of
__graft_entry__ and bench.py's CPU-baseline legs import this module.
"""
from __future__ import annotations

import ctypes as C
import json
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "liboracle.so"
CLI = HERE / "_build" / "lulesh_oracle"
REF = HERE / "_ref" / "lulesh_ref"
REF_VERBATIM = HERE / "_ref" / "lulesh_omp_verbatim"

INIT_V1, INIT_V2 = 1, 2
OK, VOLUME_ERROR, QSTOP_ERROR = 0, -1, -2

NODE_FIELDS = ("x", "y", "z", "xd", "yd", "zd", "xdd", "ydd", "zdd", "fx", "fy", "fz", "nodalMass")
ELEM_FIELDS = ("e", "p", "q", "ql", "qq", "v", "volo", "vnew", "delv", "vdov", "arealg", "ss",
               "elemMass", "determ", "delv_xi", "delv_eta", "delv_zeta", "delx_xi", "delx_eta",
               "delx_zeta")
INT_FIELDS = ("nodelist", "lxim", "lxip", "letam", "letap", "lzetam", "lzetap", "elemBC",
              "nodeElemStart", "nodeElemCount", "nodeElemCornerList", "symmX", "symmY", "symmZ")


class Mesh(C.Structure):
    """lo_mesh: an unstructured hexahedral mesh."""
    _fields_ = [("nelem", C.c_int), ("nnode", C.c_int),
                ("x", C.POINTER(C.c_double)), ("y", C.POINTER(C.c_double)), ("z", C.POINTER(C.c_double)),
                ("nodelist", C.POINTER(C.c_int))] + \
               [(n, C.POINTER(C.c_int)) for n in ("lxim", "lxip", "letam", "letap", "lzetam", "lzetap",
                                                 "symm_x", "symm_y", "symm_z", "free_surf")] + \
               [(n, C.c_int) for n in ("nsymm_x", "nsymm_y", "nsymm_z", "nfree")]


def read_lmesh(path) -> dict:
    """The contents of a .lmesh file as numpy arrays.

    Layout (the reference's unstructured reader,
    reference/CUDA/lulesh-kepler-singlegpu/lulesh.cu:733-850): numElem numNode;
    numNode coordinate triples; 8 node indices per element; 6 face
    neighbours per element (xi-, xi+, eta-, eta+, zeta-, zeta+); then the
    symmetry X, Y, Z and free-surface node sets, each a count and indices.
    """
    import gzip
    raw = Path(path).read_bytes()
    if raw[:2] == b"\x1f\x8b":
        raw = gzip.decompress(raw)
    tok = raw.split()
    ne, nn = int(tok[0]), int(tok[1])
    off = 2
    xyz = np.array(tok[off:off + 3 * nn], dtype=np.float64).reshape(nn, 3)
    off += 3 * nn
    nodelist = np.array(tok[off:off + 8 * ne], dtype=np.int32)
    off += 8 * ne
    nb = np.array(tok[off:off + 6 * ne], dtype=np.int32).reshape(ne, 6)
    off += 6 * ne
    sets = []
    for _ in range(4):
        n = int(tok[off])
        sets.append(np.array(tok[off + 1:off + 1 + n], dtype=np.int32))
        off += 1 + n
    m = {"nelem": ne, "nnode": nn, "x": xyz[:, 0].copy(), "y": xyz[:, 1].copy(), "z": xyz[:, 2].copy(),
         "nodelist": nodelist, "symm_x": sets[0], "symm_y": sets[1], "symm_z": sets[2], "free_surf": sets[3]}
    for i, n in enumerate(("lxim", "lxip", "letam", "letap", "lzetam", "lzetap")):
        m[n] = np.ascontiguousarray(nb[:, i])
    return m


class Params(C.Structure):
    _fields_ = [(n, C.c_double) for n in (
        "e_cut", "p_cut", "q_cut", "v_cut", "u_cut",
        "hgcoef", "ss4o3", "qstop", "monoq_max_slope", "monoq_limiter_mult",
        "qlc_monoq", "qqc_monoq", "qqc",
        "eosvmax", "eosvmin", "pmin", "emin", "dvovmax", "refdens",
        "dtfixed", "deltatimemultlb", "deltatimemultub", "dtmax", "stoptime")]


def build() -> None:
    """Compile the restatement (and the reference build where possible)."""
    subprocess.run(["make", "-s", "-C", str(HERE)], check=True)


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not LIB.exists():
            build()
        L = C.CDLL(str(LIB))
        L.lo_create.restype = C.c_void_p
        L.lo_create.argtypes = [C.c_int, C.c_int]
        L.lo_create_mesh.restype = C.c_void_p
        L.lo_create_mesh.argtypes = [C.POINTER(Mesh)]
        L.lo_origin.restype = C.c_int
        L.lo_origin.argtypes = [C.c_void_p]
        L.lo_destroy.argtypes = [C.c_void_p]
        L.lo_params_of.restype = C.POINTER(Params)
        L.lo_params_of.argtypes = [C.c_void_p]
        L.lo_field.restype = C.POINTER(C.c_double)
        L.lo_field.argtypes = [C.c_void_p, C.c_char_p, C.POINTER(C.c_long)]
        L.lo_ifield.restype = C.POINTER(C.c_int)
        L.lo_ifield.argtypes = [C.c_void_p, C.c_char_p, C.POINTER(C.c_long)]
        L.lo_scalar.restype = C.POINTER(C.c_double)
        L.lo_scalar.argtypes = [C.c_void_p, C.c_char_p]
        L.lo_cycle.restype = C.POINTER(C.c_int)
        L.lo_cycle.argtypes = [C.c_void_p]
        for f in ("lo_lagrange_nodal", "lo_lagrange_elements", "lo_lagrange_leapfrog"):
            getattr(L, f).restype = C.c_int
            getattr(L, f).argtypes = [C.c_void_p]
        for f in ("lo_time_increment", "lo_time_constraints"):
            getattr(L, f).restype = None
            getattr(L, f).argtypes = [C.c_void_p]
        L.lo_run.restype = C.c_int
        L.lo_run.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_double)]
        L.lo_symmetry.argtypes = [C.c_void_p] + [C.POINTER(C.c_double)] * 3
        L.lo_num_threads.restype = C.c_int
        _lib = L
    return _lib


class Oracle:
    """One Sedov problem in the oracle; fields are live numpy views."""

    def __init__(self, s: int, init: int = INIT_V2, *, mesh: dict | None = None):
        if mesh is not None:
            self._keep = {k: np.ascontiguousarray(v, dtype=np.float64 if k in "xyz" else np.int32)
                          for k, v in mesh.items() if isinstance(v, np.ndarray)}
            m = Mesh(nelem=mesh["nelem"], nnode=mesh["nnode"])
            for k, v in self._keep.items():
                ct = C.c_double if v.dtype == np.float64 else C.c_int
                setattr(m, k, v.ctypes.data_as(C.POINTER(ct)))
            m.nsymm_x, m.nsymm_y, m.nsymm_z = (len(mesh[k]) for k in ("symm_x", "symm_y", "symm_z"))
            m.nfree = len(mesh["free_surf"])
            self._h = lib().lo_create_mesh(C.byref(m))
            if not self._h:
                raise ValueError("bad mesh")
            self.s = 0
            return
        self._h = lib().lo_create(s, init)
        if not self._h:
            raise ValueError(f"bad size {s}")
        self.s = s

    @classmethod
    def from_mesh(cls, mesh: dict) -> "Oracle":
        """An unstructured problem (read_lmesh's dictionary)."""
        return cls(0, mesh=mesh)

    @property
    def origin(self) -> int:
        return lib().lo_origin(self._h)

    def close(self):
        if self._h:
            lib().lo_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def field(self, name: str) -> np.ndarray:
        n = C.c_long()
        if name in INT_FIELDS:
            p = lib().lo_ifield(self._h, name.encode(), C.byref(n))
        else:
            p = lib().lo_field(self._h, name.encode(), C.byref(n))
        if not p:
            raise KeyError(name)
        return np.ctypeslib.as_array(p, shape=(n.value,))

    def scalar(self, name: str) -> float:
        return lib().lo_scalar(self._h, name.encode())[0]

    def set_scalar(self, name: str, value: float):
        lib().lo_scalar(self._h, name.encode())[0] = value

    @property
    def cycle(self) -> int:
        return lib().lo_cycle(self._h)[0]

    @cycle.setter
    def cycle(self, c: int):
        lib().lo_cycle(self._h)[0] = c

    @property
    def params(self) -> Params:
        return lib().lo_params_of(self._h).contents

    def time_increment(self):
        lib().lo_time_increment(self._h)

    def lagrange_nodal(self) -> int:
        return lib().lo_lagrange_nodal(self._h)

    def lagrange_elements(self) -> int:
        return lib().lo_lagrange_elements(self._h)

    def time_constraints(self):
        lib().lo_time_constraints(self._h)

    def lagrange_leapfrog(self) -> int:
        return lib().lo_lagrange_leapfrog(self._h)

    def run(self, max_cycles: int = 0) -> tuple[int, float]:
        el = C.c_double()
        rc = lib().lo_run(self._h, max_cycles, C.byref(el))
        return rc, el.value

    def symmetry(self) -> tuple[float, float, float]:
        a, t, r = C.c_double(), C.c_double(), C.c_double()
        lib().lo_symmetry(self._h, C.byref(a), C.byref(t), C.byref(r))
        return a.value, t.value, r.value


def run_cli(exe: Path, s: int, init: str = "v2", cycles: int = 0, threads: int | None = None,
            extra: list[str] | None = None, timeout: float | None = None) -> dict:
    """Run the oracle CLI or the reference build; return its JSON line."""
    env = dict(os.environ)
    if threads:
        env["OMP_NUM_THREADS"] = str(threads)
    cmd = [str(exe), str(s), "--init", init]
    if cycles:
        cmd += ["--cycles", str(cycles)]
    cmd += extra or []
    r = subprocess.run(cmd, capture_output=True, text=True, env=env, timeout=timeout, check=True)
    return json.loads(r.stdout.strip().splitlines()[-1])


def read_ref_dump(path: Path) -> list[dict]:
    """Records written by ref_driver.cc (--dump / --phase-dump)."""
    data = Path(path).read_bytes()
    out, off = [], 0
    while off < len(data):
        assert data[off:off + 4] == b"LREF", "bad record tag"
        stage, s = np.frombuffer(data, np.int32, 2, off + 4)
        sc = np.frombuffer(data, np.float64, 6, off + 12)
        (nf,) = np.frombuffer(data, np.int32, 1, off + 60)
        off += 64
        rec = {"stage": int(stage), "s": int(s), "time": sc[0], "deltatime": sc[1],
               "dtcourant": sc[2], "dthydro": sc[3], "cycle": int(sc[4])}
        for _ in range(nf):
            name = data[off:off + 16].split(b"\0")[0].decode()
            (n,) = np.frombuffer(data, np.int64, 1, off + 16)
            rec[name] = np.frombuffer(data, np.float64, int(n), off + 24).copy()
            off += 24 + 8 * int(n)
        out.append(rec)
    return out
