"""Build liblulesh_gb300.so in-tree for sm_103a (nvcc only, no cmake).

Each translation unit is compiled in parallel, then linked into
``lulesh-accelerate_gb300/liblulesh_gb300.so``.  Host code is compiled with
``-ffp-contract=off`` so that the host-side mesh set-up gives the same bits
on x86 and Arm hosts.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "liblulesh_gb300.so"
DRIVER = PKG / "lulesh_gb300_main"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ["-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
           "-Xcompiler", "-fPIC,-ffp-contract=off", "-I", str(PKG.parent / "include")]
SOURCES = ["api.cu", "step_fp64.cu", "step_df.cu", "step_split.cu", "batch.cu", "mesh.cpp", "noalloc.cu",
           "output.cpp"]


def nvcc() -> str:
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(exe).exists():
        raise RuntimeError("nvcc not found")
    return exe


def _compile(src: str, verbose: bool) -> Path:
    obj = BUILD / (src.replace(".", "_") + ".o")
    cmd = [nvcc(), *ARCH, *NVFLAGS, "-c", str(CSRC / src), "-o", str(obj)]
    if verbose:
        cmd[1:1] = ["-Xptxas", "-v"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    if verbose and r.stderr:
        sys.stderr.write(r.stderr)
    return obj


def build(verbose: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    deps = sorted(CSRC.glob("*")) + sorted((PKG / "driver").glob("*")) + [PKG.parent / "include" / "lulesh_gb300.h",
                                                                         Path(__file__)]
    if LIB.exists() and DRIVER.exists() and not verbose:
        newest = max(p.stat().st_mtime for p in deps)
        if LIB.stat().st_mtime > newest:
            return LIB
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), SOURCES))
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [nvcc(), *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    # the C host (driver/lulesh_gb300_main.c): links the library through its
    # C header only, as the reference's C driver would
    cc = shutil.which("gcc") or "cc"
    cmd = [cc, "-O2", "-std=c99", "-I", str(PKG.parent / "include"), str(PKG / "driver" / "lulesh_gb300_main.c"),
           "-L", str(PKG), "-llulesh_gb300", f"-Wl,-rpath,{PKG}", "-o", str(DRIVER)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"driver build failed:\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
