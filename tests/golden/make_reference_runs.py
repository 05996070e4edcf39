"""Reference answers for the full-length headline runs and the seeded ensembles.

Runs the unmodified reference step (oracle/_ref/lulesh_ref, built by
``make -C oracle`` from reference/C/LULESH-OMP.cc) and records, per run, the
cycle count, time, dt, origin energy, the plane-0 symmetry triple of
LULESH-OMP.cc:3197-3223 and the whole-problem results of the final state
(total energy, largest nodal speed, viscosity-weighted shock radius):

* ``s192_c500``: s=192, LULESH 2.0 initial conditions, 500 cycles (the
  plain FP64 and split-precision headline runs);
* ``c3``: the 64 instances of the seeded FP64 ensemble (s in 16..64), each
  to t = 1e-2 from its scaled initial energy;
* ``c4``: the 512 small instances of the seeded split ensemble (s in 8..48)
  and its s=96 instances, each to t = 1e-2.

The instances come from ``ensembles.json``.  The script is resumable: it
keeps what the output file already holds and runs only what is missing.

Usage: python tests/golden/make_reference_runs.py [--only s192|c3|c4|c4big]
           [--jobs N] [--big N] [--out FILE]
"""
import argparse
import json
import os
import subprocess
import sys
import time
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
REF = ROOT / "oracle" / "_ref" / "lulesh_ref"
KEEP = ("s", "num_elem", "cycles", "origin_energy", "time", "deltatime", "dtcourant", "dthydro",
        "max_abs_diff", "total_abs_diff", "max_rel_diff", "total_energy", "max_velocity", "shock_radius")


def run_ref(s, efactor=1.0, cycles=0, threads=1):
    cmd = [str(REF), str(s), "--init", "v2", "--efactor", repr(float(efactor))]
    if cycles:
        cmd += ["--cycles", str(cycles)]
    env = dict(os.environ, OMP_NUM_THREADS=str(threads))
    out = subprocess.run(cmd, check=True, capture_output=True, text=True, env=env).stdout
    rec = json.loads(out.strip().splitlines()[-1])
    res = {k: rec[k] for k in KEEP}
    res["efactor"] = float(efactor)
    return res


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--only", choices=("s192", "c3", "c4", "c4big"), action="append")
    ap.add_argument("--jobs", type=int, default=os.cpu_count())
    ap.add_argument("--big", type=int, default=16, help="how many of c4's s=96 instances")
    ap.add_argument("--out", default=str(HERE / "reference_runs.json"))
    args = ap.parse_args()
    if not REF.exists():
        sys.exit(f"{REF} is missing: run make -C oracle first")
    out = Path(args.out)
    data = json.loads(out.read_text()) if out.exists() else {}
    data["source"] = ("oracle/_ref/lulesh_ref: reference/C/LULESH-OMP.cc unmodified (TimeIncrement, "
                      "LagrangeLeapFrog) with LULESH 2.0 initial conditions (lulesh-2.0.3/lulesh-init.cc:171-182), "
                      "the initial energy times efactor; -O3 -ffp-contract=off; made by "
                      "tests/golden/make_reference_runs.py")
    ens = json.loads((HERE / "ensembles.json").read_text())
    what = args.only or ["s192", "c3", "c4", "c4big"]

    def save():
        tmp = out.with_suffix(".tmp")
        tmp.write_text(json.dumps(data, indent=1) + "\n")
        tmp.replace(out)

    if "s192" in what and "s192_c500" not in data:
        t0 = time.time()
        data["s192_c500"] = run_ref(192, 1.0, 500, threads=args.jobs)
        print(f"s192_c500 done in {time.time() - t0:.0f} s", flush=True)
        save()

    def ensemble(name, pick):
        sizes, factors = ens[name]["sizes"], ens[name]["e0_scale"]
        have = {r["index"]: r for r in data.get(name, [])}
        todo = [i for i in pick(sizes) if i not in have]
        # largest first so the pool drains evenly
        todo.sort(key=lambda i: -sizes[i])

        def one(i):
            r = run_ref(sizes[i], factors[i], 0, threads=1)
            r["index"] = i
            return r

        t0 = time.time()
        with ThreadPoolExecutor(args.jobs) as pool:
            for n, r in enumerate(pool.map(one, todo)):
                have[r["index"]] = r
                if n % 16 == 15 or n == len(todo) - 1:
                    data[name] = [have[i] for i in sorted(have)]
                    save()
                    print(f"{name}: {len(have)} instances ({time.time() - t0:.0f} s)", flush=True)

    if "c3" in what:
        ensemble("c3", lambda sz: range(len(sz)))
    if "c4" in what:
        ensemble("c4", lambda sz: [i for i, s in enumerate(sz) if s <= 48])
    if "c4big" in what:
        ensemble("c4", lambda sz: [i for i, s in enumerate(sz) if s > 48][: args.big])
    save()


if __name__ == "__main__":
    main()
