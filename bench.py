#!/usr/bin/env python3
"""Benchmark: LULESH Sedov blast, plain FP64 Lagrange leapfrog at s=192.

One "step" is one LULESH cycle (TimeIncrement + LagrangeLeapFrog) over the
s=192 mesh (7,077,888 elements, 7,189,057 nodes) with LULESH 2.0 initial
conditions.  The headline metric is zone-cycles per second (elements x
cycles / time), the reference's own figure of merit.

The plain path (LULESH_PRECISION_FP64) keeps its state, node update, EOS and
time constraints in FP64 and evaluates the element geometry and forces as
double-float pairs on the FP32 pipe; the same workload with every operation
in IEEE FP64 is the fp64_ieee leg.

Legs of the default run (one JSON line on rank 0):
  value        K cycles through the captured run-loop graph, state resident
               in HBM; CUDA events on the library's stream
  roofline     per-kernel device time of a kernel-by-kernel pass (CUDA
               events between launches) against the step's algorithmic
               bytes (K1/K2/K3); HBM peak from MEASURED_PEAKS.json; beside
               it the FP64 and FP32 issue rooflines that bind
  e2e          the same cycles through the public C ABI with host buffers:
               upload of the state from pinned memory, one
               lulesh_time_increment + lulesh_lagrange_leapfrog call per cycle
               with its status/scalar read-back, download of the final state;
               and a variant that copies the whole Domain every cycle
  accuracy     500 cycles from the initial state in each arithmetic, against
               the unmodified reference's own 500-cycle run
  fp64_ieee    the same workload, every operation in IEEE FP64
  cpu_baseline the reference CPU implementation on this host's cores, a
               bounded sample of the same workload
  split        the same workload in split precision
  batched      the seeded ensembles (64 FP64 instances; 528 split instances)
               against one-at-a-time runs and the reference's per-instance
               answers
  regions      LULESH 2.0 material regions with EOS cost (-r 11 -b 1 -c 1) on
               the same mesh, beside the unmodified LULESH 2.0 program

``--impl reference`` times only the reference CPU implementation (the
reference has no GPU path for this workload that runs on sm_103a).
Multi-GPU (torchrun): every rank runs an independent replica (the step has no
cross-instance exchange); ``value`` sums the replicas, timed by the slowest.
"""
from __future__ import annotations

import argparse
import json
import os
import re
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "Mzone-cycles/s: FP64 plain vs split-precision & batched, at ≤1e-6 origin-E err"
UNIT = "Mzone-cycles/s"
KERNELS = ("time_increment", "elem_force", "node_update", "elem_kinematics", "elem_material", "finalize")


# The step's compulsory DRAM traffic in its three-kernel form (8-byte doubles,
# 4-byte indices and floats, every array touched once):
#   K1 element forces: x..zd gathered (48/node), nodelist (32/elem),
#      p q v volo ss elemMass (48/elem) in; 24 corner forces out (192/elem,
#      96 in FP32)
#   K2 node update: start+count (8/node), corner list (32/elem), the corner
#      forces (192/elem, 96 in FP32), nodalMass (8/node), x..zd read and
#      written (96/node)
#   K3 element update: nodelist (32/elem), x..zd gathered (48/node), v volo
#      elemMass e p q (48/elem) in; e p q v ss (40/elem) out
# FP64: 616 E + 208 N bytes per cycle (827.3 per zone-cycle at s=192); split
# precision with FP32 corner forces: 424 E + 208 N (635.3).
SECTION8_KERNELS = {"elem_force": "K1", "node_update": "K2", "elem_kinematics": "K3", "elem_material": "K3"}


def step_bytes(ne: int, nn: int, precision: str = "fp64") -> dict:
    """Algorithmic bytes per cycle of K1, K2 and K3 (the step's compulsory
    traffic, independent of how this library splits and caches it)."""
    corner = 192 if precision == "fp64" else 96
    return {"K1": 48 * nn + (32 + 48 + corner) * ne,
            "K2": (8 + 8 + 96) * nn + (32 + corner) * ne,
            "K3": 48 * nn + (32 + 48 + 40) * ne}


def algorithmic_bytes(ne: int, nn: int, precision: str = "fp64") -> dict:
    """Compulsory DRAM bytes per launch of each of this library's kernels
    (8-byte doubles, 4-byte floats and indices, every array touched once),
    including what its own design adds to the step's traffic: the geometry
    cache, reciprocal masses and volumes, the Q gradients handed from the
    kinematics to the material kernel."""
    if precision == "split":
        return {
            "time_increment": 0,
            # hi/lo float pairs of x..zd gathered (48/node), nodelist (32),
            # p q v volo ss mass (48) in; FP32 corner forces (3 x 8 floats) out
            "elem_force": 48 * nn + (32 + 48 + 96) * ne,
            # slots (32/elem) + start (4/node), FP32 corner forces (96/elem),
            # 1/mass (8) + bc (1), x..zd read and written (96), hi/lo pairs out (48)
            "node_update": (4 + 8 + 1 + 96 + 48) * nn + (32 + 96) * ne,
            # nodelist, hi/lo pairs of x..zd gathered, 1/volo, v in; vnew delv
            # vdov arealg (FP64) and six FP32 Q gradients out
            "elem_kinematics": 48 * nn + (32 + 16 + 32 + 24) * ne,
            # bc + neighbour ids, FP32 gradients, vnew vdov delv arealg volo mass
            # q v e p in; p e q ss v out
            "elem_material": (4 + 24 + 24 + 80 + 40) * ne,
            "finalize": 0,
        }
    return {
        "time_increment": 0,
        # xd,yd,zd gathered (24/node), nodelist (32), the geometry cache the
        # kinematics kernel left (39 doubles), p q v volo ss mass (48) in;
        # corner forces (24 doubles, stress plus hourglass) out
        "elem_force": 24 * nn + (32 + 312 + 48 + 192) * ne,
        # corner slots (32/elem) + start (4/node), corner forces (192/elem),
        # 1/mass (8) + bc (1), x..zd read and written (96)
        "node_update": (4 + 8 + 1 + 96) * nn + (32 + 192) * ne,
        # nodelist, x..zd gathered, volo, 1/volo, v in; vnew delv arealg vdov
        # delv_* delx_* and the geometry cache (39 doubles) out
        "elem_kinematics": 48 * nn + (32 + 24 + 80 + 312) * ne,
        # bc + 6 neighbour ids, delv_* delx_*, vnew volo vdov delv mass q v e p
        # arealg in; p e q ss v out
        "elem_material": (4 + 24 + 48 + 80 + 40) * ne,
        "finalize": 0,
    }


def measured_peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        return {**json.loads(p.read_text()), "source": "measured"}
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "source": "fallback"}


class ClockSampler:
    """nvidia-smi clock/throttle samples while the timed region runs."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.path = Path(tempfile.mkstemp(prefix="clocks_", suffix=".csv")[1])

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=self.path.open("w"), stderr=subprocess.DEVNULL)
        except (FileNotFoundError, OSError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self) -> dict:
        rows = []
        for line in self.path.read_text().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                rows.append((float(f[1]), float(f[2]), f[5], f[6], f[7], f[8]))
            except ValueError:
                continue
        self.path.unlink(missing_ok=True)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        reasons = sorted({n for r in rows for n, v in zip(names, r[2:]) if v.lower() == "active"})
        return {"sm_mhz": statistics.median(r[0] for r in rows), "sm_max_mhz": max(r[1] for r in rows),
                "reasons": reasons, "samples": len(rows)}


def cpu_run(s: int, warmup: int, cycles: int, threads: int) -> dict:
    """Time the reference CPU implementation (built from its own sources by
    build()) or, where it could not be built, the oracle port."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle

    exe, kind = (oracle.REF, "reference") if oracle.REF.exists() else (oracle.CLI, "port")
    if not exe.exists():
        oracle.build()
        exe, kind = (oracle.REF, "reference") if oracle.REF.exists() else (oracle.CLI, "port")
    if kind == "reference":
        r = oracle.run_cli(exe, s, "v2", warmup + cycles, threads=threads, extra=["--warmup", str(warmup)])
    else:
        r = oracle.run_cli(exe, s, "v2", cycles, threads=threads, extra=["--warmup", str(warmup)])
    return {"value": r["mzone_cycles_per_s"], "unit": UNIT, "cores": r["threads"], "kind": kind,
            "elapsed_s": r["elapsed_s"], "cycles": r["timed_cycles"],
            "sample": f"s={s} LULESH 2.0 initial conditions, {r['timed_cycles']} cycles after "
                      f"{warmup} warm-up cycles, {r['threads']} OpenMP threads"}


def lulesh2_run(s: int, iters: int, regions: int, balance: int, cost: int, threads: int) -> dict | None:
    """The unmodified LULESH 2.0 program (regions and EOS cost), built from the
    reference's sources by build(); None where it could not be built."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle

    exe = oracle.HERE / "_ref" / "lulesh2"
    if not exe.exists():
        return None
    env = dict(os.environ, OMP_NUM_THREADS=str(threads))
    out = subprocess.run([str(exe), "-s", str(s), "-i", str(iters), "-r", str(regions), "-b", str(balance),
                          "-c", str(cost)], capture_output=True, text=True, env=env, check=True).stdout
    grind_us = float(re.search(r"Grind time \(us/z/c\)\s*=\s*(\S+)", out).group(1))
    return {"value": 1.0 / grind_us, "unit": UNIT, "cores": threads, "kind": "reference",
            "sample": f"lulesh-2.0.3 -s {s} -i {iters} -r {regions} -b {balance} -c {cost}, "
                      f"{threads} OpenMP threads (its grind time)"}


def regions_leg(pkg, args, timed, plain_value) -> dict:
    """LULESH 2.0 regions and EOS cost (-r 11 -b 1 -c 1, its defaults) on the
    headline mesh: same results, more EOS work in the costly regions."""
    nr, bal, cost = 11, 1, 1
    g = pkg.Lulesh(args.size, pkg.INIT_V2, pkg.FP64)
    g.set_regions(nr, bal, cost)
    reps = np.array([1 if r - 1 < nr // 2 else (1 + cost if r - 1 < nr - (nr + 15) // 20 else 10 * (1 + cost))
                     for r in range(1, nr + 1)])
    mean_rep = float(reps[g.regions() - 1].mean())
    ms, launches = timed(g, args.region_steps)
    value = g.num_elem * args.region_steps / (ms * 1e-3) * 1e-6
    g.close()
    return {"value": value, "unit": UNIT, "ms_per_step": ms / args.region_steps, "steps": args.region_steps,
            "regions": nr, "balance": bal, "cost": cost, "mean_eos_evaluations": mean_rep,
            "vs_plain_fp64": value / plain_value, "gpu_launches": launches}


def load_reference_runs() -> dict:
    """The unmodified reference's answers for the full-length runs and the
    seeded ensembles (tests/golden/reference_runs.json, made by
    tests/golden/make_reference_runs.py)."""
    p = ROOT / "tests" / "golden" / "reference_runs.json"
    return json.loads(p.read_text()) if p.exists() else {}


def accuracy_vs_reference(pkg, precision, mesh, ref: dict) -> dict:
    """The s=192 problem run from its initial state for the reference's own
    cycle count (500): relative errors of the four whole-problem results and
    of the time against the unmodified reference's run of the same cycles."""
    with pkg.Lulesh(ref["s"], pkg.INIT_V2, precision) as g:
        n = g.run(ref["cycles"])
        got = pkg.sedov_metrics(g, mesh)
        sc = g.scalars
        sym = g.symmetry()
    want = {k: ref[k] for k in ("origin_energy", "total_energy", "max_velocity", "shock_radius")}
    errs = pkg.relative_errors(got, want)
    errs["time"] = abs(sc.time - ref["time"]) / ref["time"]
    return {"cycles": n, "cycles_equal": n == ref["cycles"] and sc.cycle == ref["cycles"], "errors": errs,
            "plane0_max_rel_diff": sym[2], "reference_plane0_max_rel_diff": ref["max_rel_diff"],
            "reference": "tests/golden/reference_runs.json s192_c500 (LULESH-OMP.cc, 500 cycles)"}


SIZE_BANDS = ((1, 24), (25, 40), (41, 56), (57, 64), (65, 1 << 30))


def spread_order(n: int) -> list[int]:
    """0..n-1 visited middle first, then quarters, eighths, ...: a sample that
    stops early still spans the range."""
    order, seen, k = [], set(), 1
    while len(order) < n:
        for j in range(k):
            i = min(n - 1, int((2 * j + 1) * n / (2 * k)))
            if i not in seen:
                seen.add(i)
                order.append(i)
        k *= 2
    return order


def batch_legs(pkg, torch, args, barrier, max_over_ranks, ref_runs: dict) -> dict:
    """Configs 3 and 4: seeded ensembles run to t = 1e-2 in one captured graph
    (c3: 64 instances, plain FP64; c4: 528 instances, split precision),
    against the same instances run one at a time on the plain FP64 path, and
    every instance's result against the reference's own run of it.

    The one-at-a-time rate is sampled per size band (SIZE_BANDS), at least
    one instance each, spread over the band's sizes, and the bands are
    weighted by their share of the ensemble's zone-cycles: the time the
    instances would take one after another is sum(band zone-cycles / band
    rate)."""
    fx = json.loads((ROOT / "tests" / "golden" / "ensembles.json").read_text())
    cache = ROOT / "lulesh-accelerate_gb300" / "_build" / "batch_tuning.json"
    cache.parent.mkdir(exist_ok=True)
    out = {}
    for name, prec_name in (("c3", "fp64"), ("c4", "split")):
        prec = pkg.FP64 if prec_name == "fp64" else pkg.SPLIT
        sizes, scale = fx[name]["sizes"], fx[name]["e0_scale"]
        with pkg.Batch(sizes, scale, pkg.INIT_V2, prec) as w:        # warm-up + tuning
            w.autotune(str(cache))
            w.run(args.warmup)
        b = pkg.Batch(sizes, scale, pkg.INIT_V2, prec)
        b.autotune(str(cache))
        init = [b.instance(i) for i in range(b.n)]
        st = torch.cuda.ExternalStream(b.stream)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        l0 = b.kernel_launches
        barrier()
        e0.record(st)
        most = b.run()
        e1.record(st)
        barrier()
        ms = max_over_ranks(e0.elapsed_time(e1))
        zc = b.zone_cycles()
        final = [b.instance(i) for i in range(b.n)]
        launches = b.kernel_launches - l0
        tuning = b.tuning()
        b.close()

        # the same ensemble, its launch shapes re-timed whenever the running
        # instances' elements fall below half of those last tuned for (the
        # re-tuning inside the timed region)
        retuned = None
        if not args.no_retune:
            with pkg.Batch(sizes, scale, pkg.INIT_V2, prec) as rb:
                rb.autotune(str(cache))
                rst = torch.cuda.ExternalStream(rb.stream)
                r0, r1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                barrier()
                r0.record(rst)
                _, n_retunes = rb.run_retuned(chunk=args.retune_chunk, fraction=0.5)
                r1.record(rst)
                barrier()
                rms = max_over_ranks(r0.elapsed_time(r1))
                retuned = {"value": rb.zone_cycles() / (rms * 1e-3) * 1e-6, "unit": UNIT, "ms": rms,
                           "retunes": n_retunes, "chunk_cycles": args.retune_chunk,
                           "rule": "re-time the launch shapes when the running elements fall below half of "
                                   "those last tuned for"}

        # one at a time on the plain FP64 path, sampled per size band
        def solo(i):
            g = pkg.Lulesh(int(sizes[i]), pkg.INIT_V2, pkg.FP64)
            e = np.zeros(int(sizes[i]) ** 3)
            e[0] = init[i][1]
            g.set_field("e", e)
            sc = g.scalars
            sc.deltatime = init[i][0].deltatime
            g.scalars = sc
            gst = torch.cuda.ExternalStream(g.stream)
            a0, a1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a0.record(gst)
            n = g.run()
            a1.record(gst)
            torch.cuda.synchronize()
            g.close()
            return float(sizes[i]) ** 3 * n, a0.elapsed_time(a1)

        bands = []
        banded = [((lo, hi), sorted((i for i, x in enumerate(sizes) if lo <= x <= hi), key=lambda i: (sizes[i], i)))
                  for lo, hi in SIZE_BANDS]
        banded = [(bd, m) for bd, m in banded if m]
        budget_ms = 1e3 * args.solo_seconds / len(banded)
        est_ms = 0.0
        for (lo, hi), m in banded:
            band_zc = sum(float(sizes[i]) ** 3 * final[i][0].cycle for i in m)
            s_zc = s_ms = 0.0
            picked = []
            for j in spread_order(len(m)):
                z, t = solo(m[j])
                s_zc, s_ms = s_zc + z, s_ms + t
                picked.append(int(sizes[m[j]]))
                if s_ms > budget_ms:
                    break
            rate = s_zc / (s_ms * 1e-3) * 1e-6
            est_ms += band_zc / (rate * 1e6) * 1e3
            bands.append({"sizes": [lo, min(hi, max(sizes))], "instances": len(m), "sampled_sizes": picked,
                          "zone_cycle_share": band_zc / zc, "value": rate})
        solo_rate = zc / (est_ms * 1e-3) * 1e-6
        value = zc / (ms * 1e-3) * 1e-6
        leg = {"instances": len(sizes), "precision": prec_name, "elements": int(sum(int(x) ** 3 for x in sizes)),
               "seed": fx[name]["seed"], "cycles_max": most, "zone_cycles": zc, "ms": ms,
               "value": value, "unit": UNIT, "instances_per_s": len(sizes) / (ms * 1e-3),
               "one_at_a_time_fp64": {"value": solo_rate, "unit": UNIT, "bands": bands,
                                      "weighting": "each size band's sampled rate weighted by the band's share "
                                                   "of the ensemble's zone-cycles"},
               "speedup_vs_one_at_a_time_fp64": value / solo_rate, "gpu_launches": launches,
               "autotuned": tuning, "retuned": retuned}

        # every instance the reference ran, against its own answer
        refs = ref_runs.get(name, [])
        if refs:
            errs, cyc_diff = [], []
            for r in refs:
                i = r["index"]
                errs.append(abs(final[i][1] - r["origin_energy"]) / abs(r["origin_energy"]))
                cyc_diff.append(final[i][0].cycle - r["cycles"])
            leg["origin_energy_error_vs_reference"] = {
                "max": max(errs), "median": float(np.median(errs)), "instances_compared": len(refs),
                "instances_with_other_cycle_count": int(sum(1 for d in cyc_diff if d)),
                "largest_cycle_difference": int(max(abs(d) for d in cyc_diff)),
                "reference": f"tests/golden/reference_runs.json {name} (LULESH-OMP.cc per instance)"}
        out[name] = leg
    return out


def reduce_max(x: float, world: int) -> float:
    """Largest value over the ranks (the job lasts as long as its slowest rank)."""
    if world == 1:
        return x
    import torch
    import torch.distributed as dist

    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(units_per_rank: float, ms_per_rank: float, world: int) -> float:
    """Million units per second of the whole job: every rank ran one replica
    of the same work (weak scaling), timed by the slowest rank."""
    return world * units_per_rank / (reduce_max(ms_per_rank, world) * 1e-3) * 1e-6


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def config_for(args, ne, nn) -> dict:
    return {"workload": f"sedov_s{args.size}_{args.precision}", "s": args.size,
            "elements": ne, "nodes": nn, "init": "LULESH 2.0 (e0=3.948746e7*(s/45)^3)",
            "cycles_per_step": 1, "precision": args.precision,
            "l2": "no flush: the state (~5.4 GB) is far larger than the 129 MB L2",
            "parallelism": "replicas" if args.gpus > 1 else "single", "launch": args.launch}


def run_reference(args, world, rank):
    if rank != 0:
        return
    ne, nn = args.size ** 3, (args.size + 1) ** 3
    threads = os.cpu_count() or 1
    n = max(1, min(args.steps, args.cpu_cycles))
    cb = cpu_run(args.size, args.warmup, n, threads)
    line = {"impl": "reference", "metric": METRIC, "value": cb["value"], "unit": UNIT, "n_gpus": args.gpus,
            "steps": cb["cycles"], "warmup": args.warmup,
            "ms_per_step": 1e3 * cb["elapsed_s"] / max(cb["cycles"], 1), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": config_for(args, ne, nn),
            "cpu_baseline": {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample")},
            "e2e": {"value": cb["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=500, help="timed cycles")
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--size", type=int, default=192)
    ap.add_argument("--precision", default="fp64", choices=["fp64", "split"])
    ap.add_argument("--profile-cycles", type=int, default=20)
    ap.add_argument("--e2e-cycles", type=int, default=0, help="0: same as --steps")
    ap.add_argument("--copy-cycles", type=int, default=20,
                    help="cycles of the e2e variant that copies the whole Domain every cycle")
    ap.add_argument("--no-accuracy", action="store_true",
                    help="skip the 500-cycle runs compared with the reference's own")
    ap.add_argument("--no-ieee", action="store_true", help="skip the all-IEEE-FP64 leg")
    ap.add_argument("--no-retune", action="store_true", help="skip the re-tuned ensemble runs")
    ap.add_argument("--retune-chunk", type=int, default=200, help="cycles between re-tuning checks")
    ap.add_argument("--cpu-cycles", type=int, default=40,
                    help="cycles of the CPU baseline sample (about 10 s of the 16-core host at s=192)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-split", action="store_true", help="skip the split-precision leg")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched-ensemble legs")
    ap.add_argument("--no-regions", action="store_true", help="skip the LULESH 2.0 regions leg")
    ap.add_argument("--region-steps", type=int, default=100, help="timed cycles of the regions leg")
    ap.add_argument("--solo-seconds", type=float, default=8.0,
                    help="budget of the one-at-a-time sample of each batched leg")
    ap.add_argument("--launch", default="graph", choices=["graph", "direct"],
                    help="graph: the captured run loop (product path); direct: the same kernels "
                         "launched one by one (used for ncu captures)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    world, rank, local = dist_setup()

    if args.impl == "reference":
        run_reference(args, world, rank)
        return

    import numpy as np
    import torch

    import __graft_entry__ as ge

    pkg = ge.load_package()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    precision = pkg.FP64 if args.precision == "fp64" else pkg.SPLIT

    g = pkg.Lulesh(args.size, pkg.INIT_V2, precision)
    ne, nn = g.num_elem, g.num_node

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
            torch.cuda.synchronize()

    def max_over_ranks(x: float) -> float:
        return reduce_max(x, world)

    def timed(ctx, steps, clocks=None):
        """K cycles after W warm-up cycles; device ms on the library's stream."""
        run = ctx.run if args.launch == "graph" else (lambda n: ctx.run_profiled(n)[0])
        assert run(args.warmup) == args.warmup
        st = torch.cuda.ExternalStream(ctx.stream)
        l0 = ctx.kernel_launches
        barrier()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        if clocks is not None:
            clocks.__enter__()
        e0.record(st)
        done = run(steps)
        e1.record(st)
        barrier()
        if clocks is not None:
            clocks.__exit__(None, None, None)
        assert done == steps, (done, steps)
        return max_over_ranks(e0.elapsed_time(e1)), ctx.kernel_launches - l0

    def kernel_table(ctx, precision, traffic_key=None):
        """Per-kernel device time from a kernel-by-kernel pass, the roofline
        of the dominant kernel against the step's algorithmic bytes (K1, K2,
        K3), and the bytes per zone-cycle.  traffic_key names the entry of
        profiles/traffic.json measured for these kernels (default: precision)."""
        pc, kms = ctx.run_profiled(args.profile_cycles)
        per_launch = {k: v / max(pc, 1) for k, v in kms.items()}
        abytes = algorithmic_bytes(ne, nn, precision)
        sbytes = step_bytes(ne, nn, precision)
        peaks = measured_peaks()
        top = max(("elem_force", "node_update", "elem_kinematics", "elem_material"), key=lambda k: per_launch[k])
        part = SECTION8_KERNELS[top]
        part_ms = sum(per_launch[k] for k, v in SECTION8_KERNELS.items() if v == part)
        achieved = sbytes[part] / (part_ms * 1e-3) * 1e-9
        design_achieved = abytes[top] / (per_launch[top] * 1e-3) * 1e-9
        traffic = None
        fp64 = fp32 = None
        tf = ROOT / "profiles" / "traffic.json"
        if tf.exists():
            t = json.loads(tf.read_text()).get(traffic_key or precision, {}).get(top)
            if t:
                traffic = t["bytes_per_elem"] * ne
                units = nn if top == "node_update" else ne
                secs = per_launch[top] * 1e-3
                if "fp64_flops_per_unit" in t:
                    ach = t["fp64_flops_per_unit"] * units / secs * 1e-12
                    # DADD and DMUL occupy an FP64 issue slot like a DFMA: the
                    # pipe's utilisation is instructions / (DFMA slots)
                    inst_rate = t["fp64_inst_per_unit"] * units / secs
                    slot_rate = fp64_peak * 1e12 / 2.0
                    fp64 = {"bound": "fp64", "kernel": top, "achieved": ach, "peak": fp64_peak,
                            "unit": "TFLOP/s", "frac": ach / fp64_peak,
                            "issue_frac": inst_rate / slot_rate,
                            "peak_source": "measured FP64 FMA probe (lulesh_probe_fp64_peak)",
                            "flops_source": "per-unit FP64 work from the ncu capture in profiles/traffic.json"}
                if "fp32_inst_per_unit" in t:
                    # FP32 lane operations per second at the measured FFMA
                    # issue rate, SM count and median clock of the timed run
                    lane_rate = fp32_lanes_per_s()
                    fp32 = {"bound": "fp32", "kernel": top,
                            "achieved_ginst_per_s": t["fp32_inst_per_unit"] * units / secs * 1e-9,
                            "peak_ginst_per_s": lane_rate * 1e-9,
                            "issue_frac": t["fp32_inst_per_unit"] * units / secs / lane_rate,
                            "peak_source": "measured FP32 FMA probe (lulesh_probe_pipe_rates) x SMs x clock",
                            "inst_source": "per-unit FP32 instructions from the ncu capture in profiles/traffic.json"}
        roof = {"bound": "hbm", "kernel": top, "step_kernel": part, "achieved": achieved, "peak": peaks["hbm_gbs"],
                "unit": "GB/s", "frac": achieved / peaks["hbm_gbs"], "traffic": traffic,
                "peak_source": f"{peaks['source']} (MEASURED_PEAKS.json hbm_gbs)",
                "algorithmic_bytes_per_launch": sbytes[part],
                "algorithmic_bytes_source": f"the step's {part} traffic (48/node gathered, 4-byte indices, "
                                            "8-byte doubles; FP32 corner forces in split precision)",
                "design_bytes_per_launch": abytes[top], "design_achieved": design_achieved,
                "design_frac": design_achieved / peaks["hbm_gbs"], "fp64_issue": fp64, "fp32_issue": fp32}
        total = sum(per_launch.values())
        table = {k: {"ms": per_launch[k], "share": per_launch[k] / total,
                     "design_gbs": abytes[k] / (per_launch[k] * 1e-3) * 1e-9 if per_launch[k] > 0 else 0.0}
                 for k in KERNELS}
        cycle = {"bytes_per_zone_cycle": sum(sbytes.values()) / ne,
                 "design_bytes_per_zone_cycle": sum(abytes.values()) / ne,
                 "design_added_bytes_per_zone_cycle": (sum(abytes.values()) - sum(sbytes.values())) / ne}
        if precision == "fp64":
            cycle["geometry_cache_bytes_per_zone_cycle"] = 2 * 39 * 8
        return roof, table, cycle

    mesh = pkg.mesh_build(args.size, pkg.INIT_V2)
    fp64_peak = pkg.probe_fp64_peak()
    pipe_rates = pkg.probe_pipe_rates()
    n_sm = torch.cuda.get_device_properties(local).multi_processor_count

    def fp32_lanes_per_s():
        mhz = (clock_summary or {}).get("sm_mhz") or 2070.0
        return pipe_rates["ffma"] * n_sm * mhz * 1e6

    # ---- plain FP64: K cycles through the run-loop graph -----------------
    clocks = ClockSampler(local)
    ms, launches = timed(g, args.steps, clocks)       # already the slowest rank's time
    clock_summary = clocks.summary()
    value = world * ne * args.steps / (ms * 1e-3) * 1e-6
    roofline, kernels, cycle_bytes = kernel_table(g, args.precision)

    # ---- end to end through the C ABI with host buffers -------------------
    # (a) resident state, as a host that keeps its Domain on the device: the
    #     state goes up once before the first cycle and comes back once after
    #     the last; every cycle is two ABI calls, each returning its status
    #     (a 40-byte scalar read)
    e2e_cycles = args.e2e_cycles or args.steps
    pin = lambda n: torch.empty(n, dtype=torch.float64, pin_memory=True).numpy()
    host = pkg.Domain.empty(ne, nn, pinned=pin)
    g.download(host)
    state_bytes = sum(a.nbytes for a in host.arrays())
    scalar_bytes = 40   # lulesh_scalars-sized status read per call
    barrier()
    t0 = time.perf_counter()
    g.upload(host)
    for _ in range(e2e_cycles):
        g.time_increment()
        g.lagrange_leapfrog()
    g.download(host)
    barrier()
    e2e_s = max_over_ranks(time.perf_counter() - t0)
    e2e_value = world * ne * e2e_cycles / e2e_s * 1e-6
    # (b) the whole Domain across the FFI every cycle, as the functional step
    #     lulesh(domain) -> domain' of the Haskell host: upload, two calls,
    #     download, per cycle
    copy_cycles = max(1, min(args.copy_cycles, e2e_cycles))
    barrier()
    t0 = time.perf_counter()
    for _ in range(copy_cycles):
        g.upload(host)
        g.time_increment()
        g.lagrange_leapfrog()
        g.download(host)
    barrier()
    copy_s = max_over_ranks(time.perf_counter() - t0)
    e2e = {"value": e2e_value, "unit": UNIT, "cycles": e2e_cycles,
           "h2d_bytes_per_step": state_bytes / e2e_cycles,
           "d2h_bytes_per_step": (state_bytes + 2 * scalar_bytes * e2e_cycles) / e2e_cycles,
           "copies": "resident state: the Domain is uploaded once before the first cycle and downloaded once "
                     "after the last (bytes per step are those two copies spread over the cycles); every cycle "
                     "is a lulesh_time_increment + lulesh_lagrange_leapfrog call pair, each reading back its status",
           "timer": "host wall clock around upload + per-cycle ABI calls + download",
           "state_copied_every_cycle": {
               "value": world * ne * copy_cycles / copy_s * 1e-6, "unit": UNIT, "cycles": copy_cycles,
               "h2d_bytes_per_step": state_bytes, "d2h_bytes_per_step": state_bytes + 2 * scalar_bytes,
               "copies": "the whole Domain uploaded from pinned memory and downloaded every cycle"}}
    del host
    g.close()

    # ---- results at cycle 500 against the reference's own 500-cycle run ----
    ref_runs = load_reference_runs()
    accuracy = {}
    if args.size == 192 and "s192_c500" in ref_runs and not args.no_accuracy:
        for name, prec in (("fp64", pkg.FP64), ("fp64_ieee", pkg.FP64_IEEE), ("split", pkg.SPLIT)):
            if (name == "split" and args.no_split) or (name == "fp64_ieee" and args.no_ieee):
                continue
            accuracy[name] = accuracy_vs_reference(pkg, prec, mesh, ref_runs["s192_c500"])

    # ---- every operation in IEEE FP64, same workload ------------------------
    ieee = None
    if args.precision == "fp64" and not args.no_ieee:
        gi = pkg.Lulesh(args.size, pkg.INIT_V2, pkg.FP64_IEEE)
        ims, ilaunch = timed(gi, args.steps)
        ivalue = world * ne * args.steps / (ims * 1e-3) * 1e-6
        iroof, ikernels, _ = kernel_table(gi, "fp64", "fp64_ieee")
        gi.close()
        ieee = {"value": ivalue, "unit": UNIT, "ms_per_step": ims / args.steps, "gpu_launches": ilaunch,
                "value_over_ieee": value / ivalue, "errors_vs_reference": accuracy.get("fp64_ieee"),
                "roofline": iroof, "kernels": ikernels,
                "dtype": "f64: every operation IEEE FP64 (LULESH_PRECISION_FP64_IEEE)"}

    # ---- split precision on the same workload (config 2) ------------------
    split = None
    if args.precision == "fp64" and not args.no_split:
        gs = pkg.Lulesh(args.size, pkg.INIT_V2, pkg.SPLIT)
        sms, slaunch = timed(gs, args.steps)
        svalue = world * ne * args.steps / (sms * 1e-3) * 1e-6
        sroof, skernels, sbytes = kernel_table(gs, "split")
        gs.close()
        split = {"value": svalue, "unit": UNIT, "ms_per_step": sms / args.steps,
                 "speedup_vs_fp64": svalue / value, "gpu_launches": slaunch,
                 "errors_vs_reference": accuracy.get("split"),
                 "roofline": sroof, "kernels": skernels, **sbytes,
                 "dtype": "f32 geometry/forces/Q, f64 state/EOS/volume/vdov/dt"}

    batched = None
    if args.precision == "fp64" and not args.no_batch:
        batched = batch_legs(pkg, torch, args, barrier, max_over_ranks, ref_runs)

    regions = None
    if args.precision == "fp64" and not args.no_regions:
        regions = regions_leg(pkg, args, timed, value / world)
        if rank == 0 and not args.no_cpu:
            regions["cpu_baseline"] = lulesh2_run(args.size, 3, 11, 1, 1, os.cpu_count() or 1)

    cpu = None
    if rank == 0 and not args.no_cpu:
        cb = cpu_run(args.size, 2, args.cpu_cycles, os.cpu_count() or 1)
        cpu = {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample")}

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "arithmetic": "FP64 state, node update, EOS and time constraints; element geometry and forces "
                              "in double-float pairs of f32 (~48-bit significand) on the FP32 pipe, held to the "
                              "FP64 parity bar (fp64_ieee: every operation IEEE FP64)",
                "config": config_for(args, ne, nn), "roofline": roofline,
                "fp64": {"peak_tflops_probe": fp64_peak, "pipe_rates_per_sm_clk": pipe_rates,
                         "note": "the FP64 and FP32 pipes, not HBM, bound this path: see roofline.fp64_issue "
                                 "and roofline.fp32_issue"},
                **cycle_bytes,
                "kernels": kernels, "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": launches,
                "clocks": clock_summary, "accuracy_vs_reference": accuracy, "fp64_ieee": ieee, "split": split,
                "batched": batched, "regions": regions}
        line["summary"] = summary_of(line)
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def summary_of(line: dict) -> dict:
    """The legs' headline figures, repeated last so a truncated line keeps them."""
    out = {"fp64": round(line["value"], 1), "e2e": round(line["e2e"]["value"], 1),
           "hbm_frac_K1": round(line["roofline"]["frac"], 4)}
    acc = line.get("accuracy_vs_reference") or {}
    if "fp64" in acc:
        out["fp64_vs_reference"] = {"cycles_equal": acc["fp64"]["cycles_equal"],
                                    "origin_energy": acc["fp64"]["errors"]["origin_energy"]}
    if line.get("fp64_ieee"):
        out["fp64_ieee"] = round(line["fp64_ieee"]["value"], 1)
        if "fp64_ieee" in acc:
            out["fp64_ieee_vs_reference"] = {"cycles_equal": acc["fp64_ieee"]["cycles_equal"],
                                             "origin_energy": acc["fp64_ieee"]["errors"]["origin_energy"]}
    sp = line.get("split")
    if sp:
        out["split"] = round(sp["value"], 1)
        out["split_speedup"] = round(sp["speedup_vs_fp64"], 3)
        if sp.get("errors_vs_reference"):
            out["split_errors_vs_reference"] = sp["errors_vs_reference"]["errors"]
    for name, leg in (line.get("batched") or {}).items():
        out[name] = {"value": round(leg["value"], 1),
                     "speedup_vs_one_at_a_time_fp64": round(leg["speedup_vs_one_at_a_time_fp64"], 3)}
        if leg.get("retuned"):
            out[name]["retuned"] = round(leg["retuned"]["value"], 1)
        if leg.get("origin_energy_error_vs_reference"):
            e = leg["origin_energy_error_vs_reference"]
            out[name]["origin_energy_error_max"] = e["max"]
            out[name]["instances_compared"] = e["instances_compared"]
    if line.get("regions"):
        out["regions"] = round(line["regions"]["value"], 1)
    if line.get("cpu_baseline"):
        out["cpu_reference"] = round(line["cpu_baseline"]["value"], 2)
    return out


if __name__ == "__main__":
    main()
