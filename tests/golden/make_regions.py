"""Generate the LULESH 2.0 region fixtures (``regions.json``) from the reference.

* ``assignments``: the element-to-region assignment of the unmodified
  reference (reference/C/lulesh-2.0.3, Domain::CreateRegionIndexSets,
  lulesh-init.cc:377-486) for several (s, regions, balance), printed by
  ``oracle/_ref/regions_dump`` as run lengths;
* ``answers``: the printed results of the unmodified LULESH 2.0 program
  (``oracle/_ref/lulesh2``) at s=30 with several -r/-b/-c options: regions
  change the work, not the answer.

Needs the reference tree and its build (``make -C oracle``).
Usage: ``python tests/golden/make_regions.py``.
"""
from __future__ import annotations

import json
import re
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT / "oracle"))
import oracle  # noqa: E402

OUT = Path(__file__).resolve().parent
DUMP = oracle.HERE / "_ref" / "regions_dump"
L2 = oracle.HERE / "_ref" / "lulesh2"
ASSIGN = [(6, 11, 1), (30, 11, 1), (30, 5, 2), (20, 21, 0), (45, 11, 1), (12, 2, 3)]
RUNS = [(30, 11, 1, 1), (30, 1, 1, 1), (30, 21, 2, 3)]


def main() -> None:
    if not DUMP.exists() or not L2.exists():
        raise SystemExit("needs the reference tree and `make -C oracle`")
    res = {"source": "reference/C/lulesh-2.0.3 (oracle/_ref/regions_dump, oracle/_ref/lulesh2)",
           "assignments": [], "answers": []}
    for s, nr, b in ASSIGN:
        out = subprocess.run([str(DUMP), str(s), str(nr), str(b)], capture_output=True, text=True, check=True)
        res["assignments"].append(json.loads(out.stdout))
        print(f"s={s} r={nr} b={b}: {len(res['assignments'][-1]['runs'])} runs")
    for s, nr, b, c in RUNS:
        out = subprocess.run([str(L2), "-s", str(s), "-r", str(nr), "-b", str(b), "-c", str(c)],
                             capture_output=True, text=True, check=True, env={"OMP_NUM_THREADS": "8"}).stdout
        cycles = int(re.search(r"Iteration count\s*=\s*(\d+)", out).group(1))
        energy = float(re.search(r"Final Origin Energy\s*=\s*(\S+)", out).group(1))
        res["answers"].append({"s": s, "num_regions": nr, "balance": b, "cost": c, "cycles": cycles,
                               "origin_energy_printed": energy})
        print(f"lulesh2 -s {s} -r {nr} -b {b} -c {c}: {cycles} cycles, {energy:.6e}")
    (OUT / "regions.json").write_text(json.dumps(res, separators=(",", ":")) + "\n")


if __name__ == "__main__":
    main()
