"""The Haskell side of the boundary (hs/LULESH/GB300.hs) against the C header.

There is no GHC toolchain here, so the module is not compiled; this test reads
every ``foreign import ccall`` in it and checks that the C function exists in
include/lulesh_gb300.h with the same number of arguments and matching types
(CInt = int, CLong = long, R = Double = double, Ptr/CString = a pointer,
IO () = void), and that the library exports it.
"""
from __future__ import annotations

import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
HS = ROOT / "hs" / "LULESH" / "GB300.hs"
HEADER = ROOT / "include" / "lulesh_gb300.h"


def header_prototypes() -> dict[str, tuple[str, list[str]]]:
    """name -> (return type, parameter types) of every function in the header."""
    text = re.sub(r"/\*.*?\*/", " ", HEADER.read_text(), flags=re.S)
    text = re.sub(r"#.*", " ", text)
    out = {}
    for m in re.finditer(r"([A-Za-z_][\w\s\*]*?)\b(lulesh_\w+)\s*\(([^;{]*?)\)\s*;", text, flags=re.S):
        ret, name, params = m.group(1).split()[-1:] and " ".join(m.group(1).split()), m.group(2), m.group(3)
        plist = [] if params.strip() in ("", "void") else [" ".join(p.split()) for p in params.split(",")]
        out[name] = (ret, plist)
    return out


def c_kind(decl: str) -> str:
    """'ptr', 'int', 'long', 'double' or 'void' of a C parameter/return type."""
    if "*" in decl or "[" in decl:
        return "ptr"
    words = decl.replace("const", " ").split()
    for kind in ("double", "long", "int", "void"):
        if kind in words:
            return kind
    raise AssertionError(f"unexpected C type {decl!r}")


def hs_kind(t: str) -> str:
    t = t.strip()
    if t.startswith("Ptr") or t == "CString":
        return "ptr"
    return {"CInt": "int", "CLong": "long", "R": "double", "Double": "double", "()": "void"}[t]


def hs_imports() -> list[tuple[str, list[str], str]]:
    text = HS.read_text()
    out = []
    for m in re.finditer(r'foreign import ccall (?:safe |unsafe )?"(\w+)"\s*\n\s*\w+\s*::(.*?)(?=\n\s*\n|\nforeign)',
                         text, flags=re.S):
        sig = re.sub(r"--[^\n]*", " ", m.group(2))
        parts = [p.strip() for p in sig.split("->")]
        ret = parts[-1]
        assert ret.startswith("IO "), (m.group(1), ret)
        out.append((m.group(1), parts[:-1], ret[3:].strip()))
    return out


def test_haskell_module_binds_the_step_api():
    names = {n for n, _, _ in hs_imports()}
    for need in ("lulesh_create", "lulesh_destroy", "lulesh_time_increment", "lulesh_lagrange_leapfrog",
                 "lulesh_run", "lulesh_upload_domain", "lulesh_download_domain", "lulesh_last_error"):
        assert need in names, need


@pytest.mark.parametrize("name,args,ret", hs_imports(), ids=lambda v: v if isinstance(v, str) else None)
def test_foreign_import_matches_header(name, args, ret):
    protos = header_prototypes()
    assert name in protos, f"{name} is not declared in {HEADER.name}"
    c_ret, c_params = protos[name]
    assert len(args) == len(c_params), (name, args, c_params)
    for i, (h, c) in enumerate(zip(args, c_params)):
        assert hs_kind(h) == c_kind(c), (name, i, h, c)
    assert hs_kind(ret) == c_kind(c_ret), (name, ret, c_ret)


def test_foreign_imports_are_exported(pkg):
    lib = pkg.load_library()
    for name, _, _ in hs_imports():
        assert hasattr(lib, name), name
