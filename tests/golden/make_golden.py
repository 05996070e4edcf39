"""Generate the golden fixtures of tests/golden/ from the reference itself.

Runs ``oracle/_ref/lulesh_ref`` -- the unmodified reference/C/LULESH-OMP.cc
step functions driven by oracle/ref_driver.cc -- and records:

* ``known_answers.json``: cycle count, final origin energy (17 digits), time
  step state and the plane-0 symmetry statistics for a set of full and
  capped runs, plus the reference's published table (lulesh-ports.pdf,
  section 6.2, Tab. 2) for the LULESH 1.0 initialisation;
* ``phases_s<S>_c<C>.npz``: the state before and after each phase of cycle C
  (TimeIncrement, LagrangeNodal, LagrangeElements,
  CalcTimeConstraintsForElems) of an s=S problem with LULESH 2.0 initial
  conditions.

Needs the reference build (``make -C oracle`` where the reference tree is
available).  Usage: ``python tests/golden/make_golden.py``.
"""
from __future__ import annotations

import json
import sys
import tempfile
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT / "oracle"))
import oracle  # noqa: E402

OUT = Path(__file__).resolve().parent

# lulesh-ports.pdf section 6.2 "Correctness Checking", Tab. 2 (LULESH 1.0
# initialisation): problem size -> (iterations, final origin energy)
PUBLISHED_V1 = {5: (306, 1.670602e+05), 10: (593, 5.174622e+05), 45: (1495, 4.261463e+05),
                50: (1566, 4.052502e+05), 70: (1816, 3.453062e+05), 90: (2026, 3.063249e+05)}

RUNS = [  # (s, init, cycle cap or 0)
    (1, "v1", 0), (2, "v1", 0), (3, "v1", 0), (1, "v2", 0), (2, "v2", 0), (3, "v2", 0),
    (5, "v1", 0), (10, "v1", 0), (45, "v1", 0),
    (4, "v2", 0), (5, "v2", 0), (8, "v2", 0), (10, "v2", 0), (16, "v2", 0), (30, "v2", 0),
    (30, "v2", 100), (48, "v2", 40),
]

PHASES = [(5, 0), (6, 40), (10, 150)]
STAGES = ("start", "time_increment", "lagrange_nodal", "lagrange_elements", "time_constraints")


def main() -> None:
    if not oracle.REF.exists():
        raise SystemExit("reference build missing: run `make -C oracle` where the reference tree exists")
    answers = {"source": "oracle/_ref/lulesh_ref (reference/C/LULESH-OMP.cc step functions)",
               "published_v1": {str(k): list(v) for k, v in PUBLISHED_V1.items()}, "runs": []}
    for s, init, cap in RUNS:
        r = oracle.run_cli(oracle.REF, s, init, cap, threads=8)
        r["cap"] = cap
        for k in ("elapsed_s", "threads", "mzone_cycles_per_s"):
            r.pop(k, None)
        answers["runs"].append(r)
        print(f"s={s} {init} cap={cap}: {r['cycles']} cycles, e0={r['origin_energy']:.17e}")
    (OUT / "known_answers.json").write_text(json.dumps(answers, indent=1) + "\n")

    for s, cyc in PHASES:
        with tempfile.TemporaryDirectory() as td:
            path = Path(td) / "phases.bin"
            oracle.run_cli(oracle.REF, s, "v2", cyc + 1, threads=8,
                           extra=["--phase-dump", str(path), str(cyc)])
            recs = oracle.read_ref_dump(path)
        assert [r["stage"] for r in recs] == [0, 1, 2, 3, 4]
        arrays = {}
        for st, rec in zip(STAGES, recs):
            for k, v in rec.items():
                if k in ("stage", "s"):
                    continue
                arrays[f"{st}/{k}"] = np.asarray(v)
        np.savez_compressed(OUT / f"phases_s{s}_c{cyc}.npz", **arrays)
        print(f"phases s={s} cycle={cyc}: {len(arrays)} arrays")


if __name__ == "__main__":
    main()
