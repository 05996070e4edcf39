"""Generate the unstructured-mesh fixtures of tests/golden/ from the reference.

The reference's GPU driver runs the Sedov problem on unstructured meshes read
from .lmesh files (reference/CUDA/lulesh-kepler-singlegpu/lulesh.cu, "-u
file.lmesh"), and ships two of them with the solution file its run of the
larger one wrote (xyz.asc, node positions at t = 1e-2 with 10 decimals).
This script

* copies the two meshes, gzip-compressed, to ``sedov15oct.lmesh.gz`` and
  ``sedov21oct.lmesh.gz`` (input data of the reference's benchmark, needed
  where the reference tree is absent);
* runs ``oracle/_ref/lulesh_ref -u`` -- the unmodified LULESH-OMP.cc step
  functions on the mesh set up as the reference's unstructured reader does --
  on both meshes and records cycles, origin element and energy and the final
  time-step state in ``unstructured.json``;
* compares that run's final positions on sedov21oct with the reference's
  xyz.asc and records the largest difference, plus the positions of every
  97th node from both (``kepler_sample``, ``ref_sample``);
* writes the state before and after each phase of cycle 80 of sedov15oct to
  ``phases_sedov15oct_c80.npz``.

Needs the reference tree and its build (``make -C oracle``).
Usage: ``python tests/golden/make_unstructured.py [REFERENCE_ROOT]``; the
reference tree's root comes from the argument, else from the environment
variable ``REF_ROOT`` (the name ``oracle/Makefile`` uses), else
``/root/reference``.
"""
from __future__ import annotations

import gzip
import json
import os
import sys
import tempfile
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT / "oracle"))
import oracle  # noqa: E402

OUT = Path(__file__).resolve().parent
REF_ROOT = Path(sys.argv[1] if len(sys.argv) > 1 else os.environ.get("REF_ROOT", "/root/reference"))
KEPLER = REF_ROOT / "reference" / "CUDA" / "lulesh-kepler-singlegpu"
MESHES = ("sedov15oct", "sedov21oct")
PHASE_MESH, PHASE_CYCLE = "sedov15oct", 80
SAMPLE_STRIDE = 97
STAGES = ("start", "time_increment", "lagrange_nodal", "lagrange_elements", "time_constraints")


def run_ref(mesh: Path, extra: list[str]) -> dict:
    import subprocess
    r = subprocess.run([str(oracle.REF), "-u", str(mesh)] + extra, capture_output=True, text=True,
                       check=True, env={"OMP_NUM_THREADS": "8"})
    out = json.loads(r.stdout.strip().splitlines()[-1])
    for k in ("elapsed_s", "threads", "mzone_cycles_per_s", "timed_cycles", "s", "init",
              "max_abs_diff", "total_abs_diff", "max_rel_diff"):
        out.pop(k, None)
    return out


def main() -> None:
    if not oracle.REF.exists() or not KEPLER.exists():
        raise SystemExit("needs the reference tree and `make -C oracle`")
    res = {"source": "oracle/_ref/lulesh_ref -u (LULESH-OMP.cc step functions, unstructured set-up "
                     "of lulesh-kepler-singlegpu/lulesh.cu:733-923)", "meshes": {}}
    for name in MESHES:
        src = KEPLER / f"{name}.lmesh"
        (OUT / f"{name}.lmesh.gz").write_bytes(gzip.compress(src.read_bytes(), 9, mtime=0))
        with tempfile.TemporaryDirectory() as td:
            dump = Path(td) / "final.bin"
            r = run_ref(src, ["--dump", str(dump)])
            final = oracle.read_ref_dump(dump)[0]
        res["meshes"][name] = r
        print(f"{name}: {r['num_elem']} elements, {r['cycles']} cycles, origin {r['origin_elem']}, "
              f"e = {r['origin_energy']:.17e}")
        if name == "sedov21oct":
            tok = (KEPLER / "xyz.asc").read_text().split()
            kep = np.array(tok, dtype=np.float64).reshape(-1, 4)
            assert np.array_equal(kep[:, 0], np.arange(len(kep)))
            mine = np.stack([final["x"], final["y"], final["z"]], 1)
            diff = float(np.abs(mine - kep[:, 1:]).max())
            idx = np.arange(0, len(kep), SAMPLE_STRIDE)
            r["kepler_max_abs_diff"] = diff
            r["sample_nodes"] = idx.tolist()
            r["kepler_sample"] = kep[idx, 1:].tolist()
            r["ref_sample"] = mine[idx].tolist()
            print(f"  final positions vs xyz.asc: max |diff| = {diff:.3e} (10 printed decimals)")
    (OUT / "unstructured.json").write_text(json.dumps(res, indent=1) + "\n")

    with tempfile.TemporaryDirectory() as td:
        path = Path(td) / "phases.bin"
        run_ref(KEPLER / f"{PHASE_MESH}.lmesh",
                ["--cycles", str(PHASE_CYCLE + 1), "--phase-dump", str(path), str(PHASE_CYCLE)])
        recs = oracle.read_ref_dump(path)
    assert [r["stage"] for r in recs] == [0, 1, 2, 3, 4]
    arrays = {f"{st}/{k}": np.asarray(v) for st, rec in zip(STAGES, recs)
              for k, v in rec.items() if k not in ("stage", "s")}
    np.savez_compressed(OUT / f"phases_{PHASE_MESH}_c{PHASE_CYCLE}.npz", **arrays)
    print(f"phases {PHASE_MESH} cycle {PHASE_CYCLE}: {len(arrays)} arrays")


if __name__ == "__main__":
    main()
